"""GPU parity of the atmosphere LUT kernels against the FP64 CPU oracle,
called through the C ABI (libskyr.so).

Tolerance: <= 1e-3 maximum relative error per LUT texel and channel
(|gpu - oracle| / |oracle|, no absolute floor) for FP32 storage.  FP16 storage
adds its rounding (at most 2^-11 = 4.9e-4 relative) to the FP32 error (at most
1.4e-4 measured), so FP16 outputs are held to the same 1e-3 in the FP16 normal
range, and to the FP16 subnormal spacing (2^-24) below it, where the storage
can only hold multiples of that spacing.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import workloads as W
from skyrendering_gb300.atmosphere import Atmosphere, AtmosphereRenderer, LutSet, update_lut_set

pytestmark = pytest.mark.gpu

TOL = 1e-3
TOL_FP16 = 1e-3
FP16_MIN_NORMAL = 2.0 ** -14
FP16_SUBNORMAL_STEP = 2.0 ** -24
NAMES = ("transmittance", "multiscattering", "sky_view_luminance", "sky_view_transmittance",
         "aerial_perspective_luminance", "aerial_perspective_transmittance")


def as_np(luts, name, i=0):
    return getattr(luts, name)[i].float().cpu().numpy().astype(np.float64)


def max_rel(got, want):
    got, want = got[..., :3], want[..., :3]
    return float((np.abs(got - want) / np.maximum(np.abs(want), 1e-300)).max())


@pytest.mark.parametrize("zenith", W.SUN_ZENITHS_DEG)
def test_plain_lut_set_matches_fp64_oracle(ctx, zenith):
    p, s = W.earth_like_atmosphere(), W.plain_lut_sizes()
    r = W.render_parameters(W.frame_camera(), zenith)
    luts = update_lut_set(ctx, p, r, s)
    ctx.synchronize()
    ref = orc.lut_set(p, r, s, 64)
    errs = {n: max_rel(as_np(luts, n), ref[n]) for n in NAMES}
    print(f"zenith {zenith}: " + ", ".join(f"{k}={v:.2e}" for k, v in errs.items()))
    assert all(v <= TOL for v in errs.values()), errs
    # alpha channels: 1 for T / MS, 0 for the view LUTs
    assert np.all(as_np(luts, "transmittance")[..., 3] == 1.0)
    assert np.all(as_np(luts, "sky_view_luminance")[..., 3] == 0.0)


@pytest.mark.parametrize("zenith", W.SUN_ZENITHS_DEG)
def test_fp16_storage(ctx, zenith):
    p, s = W.earth_like_atmosphere(), W.plain_lut_sizes(_abi.SKYR_FORMAT_RGBA16F)
    r = W.render_parameters(W.frame_camera(), zenith)
    luts = update_lut_set(ctx, p, r, s)
    ctx.synchronize()
    assert luts.multiscattering.dtype.itemsize == 2
    ref = orc.lut_set(p, r, s, 64)
    assert max_rel(as_np(luts, "transmittance"), ref["transmittance"]) <= TOL
    for n in NAMES[1:]:
        got, want = as_np(luts, n)[..., :3], ref[n][..., :3]
        normal = np.abs(want) >= FP16_MIN_NORMAL
        # relative bound in the FP16 normal range; below it the storage can
        # only hold multiples of the subnormal spacing
        rel = (np.abs(got - want)[normal] / np.abs(want)[normal]).max()
        print(f"fp16 zenith {zenith} {n}: max rel {rel:.2e} over {int(normal.sum())} normal values")
        assert rel <= TOL_FP16, n
        assert np.abs(got - want)[~normal].max(initial=0.0) <= FP16_SUBNORMAL_STEP, n


def test_batched_sets_match_per_set_oracle(ctx):
    from tests.golden.make_atmosphere_golden import small_sizes

    params, renders = W.batched_lut_sets(8, seed=7)
    s = small_sizes()
    luts = update_lut_set(ctx, params, renders, s)
    ctx.synchronize()
    for i in range(8):
        ref = orc.lut_set(params[i], renders[i], s, 64)
        for n in NAMES:
            assert max_rel(as_np(luts, n, i), ref[n]) <= TOL, (i, n)


def test_split_entry_points_equal_lut_set(ctx):
    from tests.golden.make_atmosphere_golden import small_sizes

    p, s = W.earth_like_atmosphere(), small_sizes()
    r = W.render_parameters(W.frame_camera(), 85.0)
    a = Atmosphere(ctx, s).update_luts(p)
    a = AtmosphereRenderer(ctx, s).render_luts(p, r, a)
    b = update_lut_set(ctx, p, r, s)
    ctx.synchronize()
    for n in NAMES:
        np.testing.assert_array_equal(as_np(a, n), as_np(b, n))


def test_camera_in_space(ctx):
    from tests.golden.make_atmosphere_golden import small_sizes

    p, s = W.earth_like_atmosphere(), small_sizes()
    cam = W.Camera(position=(0.0, 300.0, 0.0), pitch=-60.0)
    r = W.render_parameters(cam, 45.0)
    luts = update_lut_set(ctx, p, r, s)
    ctx.synchronize()
    ref = orc.lut_set(p, r, s, 64)
    for n in NAMES:
        assert max_rel(as_np(luts, n), ref[n]) <= TOL, n


def test_golden_fixture(ctx):
    from tests.golden.make_atmosphere_golden import cases, small_sizes

    g = np.load(orc.HERE.parent / "tests" / "golden" / "atmosphere_small.npz")
    s = small_sizes()
    for tag, p, r in cases():
        luts = update_lut_set(ctx, p, r, s)
        ctx.synchronize()
        for n in NAMES:
            assert max_rel(as_np(luts, n), g[f"{tag}/{n}"]) <= TOL, (tag, n)


def test_vertical_transmittance_closed_form_gpu(ctx):
    p, s = W.earth_like_atmosphere(), W.plain_lut_sizes()
    p.transmittance_steps = 4000.0
    luts = Atmosphere(ctx, s).update_luts(p)
    ctx.synchronize()
    want = orc.transmittance_at(p, p.bottom_radius, 1.0)
    got = as_np(luts, "transmittance")[0, 0, :3]
    np.testing.assert_allclose(got, want, rtol=1e-4)


def test_size_independent_properties(ctx):
    # full-size batched run: transmittances in (0, 1], decreasing toward the
    # horizon along each transmittance row and with AP depth
    params, renders = W.batched_lut_sets(32, seed=3)
    s = W.plain_lut_sizes()
    luts = update_lut_set(ctx, params, renders, s)
    ctx.synchronize()
    t = luts.transmittance.cpu().numpy()[..., :3]
    assert np.all(t > 0) and np.all(t <= 1.0)
    assert np.all(np.diff(t, axis=2) <= 1e-6)
    apt = luts.aerial_perspective_transmittance.cpu().numpy()[..., :3]
    assert np.all(np.diff(apt, axis=1) <= 1e-6)
    for name in NAMES:
        assert np.isfinite(getattr(luts, name).cpu().numpy()).all(), name


def test_invalid_arguments(ctx):
    p, s = W.earth_like_atmosphere(), W.plain_lut_sizes()
    out = LutSet.allocate(s, 1, views=False)
    lib = _abi.lib()
    bad = W.plain_lut_sizes()
    bad.transmittance_width = 1
    rc = lib.skyr_update_luts(ctx.handle, C.byref(p), 1, C.byref(bad), C.c_void_p(out.transmittance.data_ptr()),
                              C.c_void_p(out.multiscattering.data_ptr()))
    assert rc == _abi.SKYR_EINVAL
    q = W.earth_like_atmosphere()
    q.mie_phase_g = math.nan
    rc = lib.skyr_update_luts(ctx.handle, C.byref(q), 1, C.byref(s), C.c_void_p(out.transmittance.data_ptr()),
                              C.c_void_p(out.multiscattering.data_ptr()))
    assert rc == _abi.SKYR_EINVAL and b"non-finite" in lib.skyr_last_error()
    rc = lib.skyr_update_luts(ctx.handle, C.byref(p), 0, C.byref(s), None, None)
    assert rc == _abi.SKYR_EINVAL
