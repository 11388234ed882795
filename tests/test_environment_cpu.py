"""CPU checks of the environment cube's layout and known answers of its oracle
(ENVIRONMENT_LUMINANCE, AtmosphereRenderer.glsl:248-275)."""
import numpy as np
import pytest

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import workloads as W


def test_level_offsets():
    lib = _abi.lib()
    off = 0
    for level in range(8):
        assert lib.skyr_environment_cube_level_offset(128, level) == off
        off += 6 * (128 >> level) ** 2
    assert lib.skyr_environment_cube_level_offset(128, 8) == off
    for bad_size, level in ((0, 0), (96, 0), (1024, 0), (128, 9), (128, -1)):
        assert lib.skyr_environment_cube_level_offset(bad_size, level) == 0


def test_oracle_zenith_texel_is_the_sky_view_top_row():
    """A 1-texel cube: the +Y face looks at the zenith of a camera on the +y
    axis, so its texel is the sky-view LUT's texel (0, 0) (cos_lat 1, cos_lon 1)."""
    p = W.earth_like_atmosphere()
    s = W.plain_lut_sizes()
    cam = W.Camera(position=(0.0, 1.0, 0.0))
    r = W.render_parameters(cam, 40.0)
    luts = orc.lut_set(p, r, s, 64)
    cube = orc.environment_cube(p, r, s, luts["transmittance"], luts["sky_view_luminance"],
                                luts["sky_view_transmittance"], 1)
    np.testing.assert_allclose(cube[2, 0, 0, :3], luts["sky_view_luminance"][0, 0, :3], rtol=1e-12)
    assert np.all(cube[..., 3] == 0)
    # the -Y face looks straight down: sky-view bottom row plus the lit ground
    assert np.all(cube[3, 0, 0, :3] > luts["sky_view_luminance"][-1, 0, :3])


def test_box_mip():
    lv = np.arange(6 * 4 * 4 * 4, dtype=np.float64).reshape(6, 4, 4, 4).astype(np.float16)
    m = orc.box_mip(lv)
    assert m.shape == (6, 2, 2, 4)
    np.testing.assert_array_equal(m[0, 0, 0], ((lv[0, 0, 0].astype(float) + lv[0, 0, 1]) + (lv[0, 1, 0] + lv[0, 1, 1])) / 4)


def _constant_cube(size, value=(0.5, 1.0, 2.0)):
    levels = size.bit_length()
    n = sum(6 * max(size >> l, 1) ** 2 for l in range(levels))
    c = np.zeros((n, 4))
    c[:, :3] = value
    return c, levels


def test_oracle_sh_and_prefilter_of_a_constant_cube():
    """Seamless sampling of a constant cube is the constant everywhere (edges,
    corners, every level), so the SH is c Y00 4 pi in the first coefficient and
    every prefiltered texel is c."""
    c, levels = _constant_cube(16)
    sh = orc.environment_sh(c, 16, levels)
    np.testing.assert_allclose(sh[0], np.array([0.5, 1.0, 2.0]) * 0.282095 * 4 * np.pi, rtol=1e-12)
    assert np.abs(sh[1:]).max() <= 1e-3 * np.abs(sh[0]).max()
    for n, r in ((16, 0.0), (8, 0.25), (2, 1.0)):
        pre = orc.environment_prefilter(c, 16, levels, n, r)
        np.testing.assert_allclose(pre, np.broadcast_to([0.5, 1.0, 2.0], pre.shape), rtol=1e-12)


def test_oracle_prefilter_roughness_zero_is_the_cube():
    """Roughness 0 draws one sample along the texel's own direction at LOD 0:
    the prefiltered level is the cube's level of the same size."""
    rng = np.random.default_rng(3)
    size = 8
    levels = size.bit_length()
    n = sum(6 * max(size >> l, 1) ** 2 for l in range(levels))
    c = np.zeros((n, 4))
    c[:, :3] = rng.uniform(0.1, 2.0, (n, 3))
    pre = orc.environment_prefilter(c, size, levels, size, 0.0)
    np.testing.assert_allclose(pre.reshape(-1, 3), c[:6 * size * size, :3], rtol=1e-9)
