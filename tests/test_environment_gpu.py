"""GPU parity of the environment luminance cube (include/skyr_environment.h).

* level 0 against the FP64 oracle on the same LUTs: per texel and channel
  |d| <= 2e-3 |w| + 2^-24 (RGBA16F storage: 4.9e-4 relative per rounding in
  the normal range, an absolute 2^-24 step below it), mean relative error
  <= 5e-4, for FP32 and FP16 LUTs and sun zeniths 30, 80 and 95 degrees;
* every mip level is bit-identical to the box filter of the level above
  (glGenerateTextureMipmap: FP32 mean of four half texels, rounded to half),
  for face sizes 1, 16, 128 and 512 and partial chains;
* bad sizes and level counts are refused.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import workloads as W
from skyrendering_gb300.atmosphere import environment_cube, update_lut_set

pytestmark = pytest.mark.gpu


def _luts(ctx, zenith, fmt=0):
    p = W.earth_like_atmosphere()
    s = W.plain_lut_sizes(fmt)
    r = W.render_parameters(W.frame_camera(), zenith)
    luts = update_lut_set(ctx, p, r, s)
    return p, r, s, luts


@pytest.mark.parametrize("zenith,fmt", [(30.0, 0), (80.0, 0), (95.0, 0), (45.0, 1)])
def test_level0_matches_oracle(ctx, zenith, fmt):
    p, r, s, luts = _luts(ctx, zenith, fmt)
    levels = environment_cube(ctx, p, r, s, luts, 128)
    ctx.synchronize()
    got = levels[0].float().cpu().numpy().astype(np.float64)
    want = orc.environment_cube(p, r, s, luts.transmittance[0].cpu().double().numpy(),
                                luts.sky_view_luminance[0].float().cpu().double().numpy(),
                                luts.sky_view_transmittance[0].float().cpu().double().numpy(), 128)
    g, w = got[..., :3], want[..., :3]
    # RGBA16F: relative steps of 2^-11 in the normal range, absolute steps of
    # 2^-24 below 2^-14 (a sun below the horizon leaves parts of the sky there)
    allowed = 2e-3 * np.abs(w) + 2.0 ** -24
    excess = (np.abs(g - w) / allowed).max()
    mean_rel = np.abs(g - w).sum() / np.abs(w).sum()
    print(f"zenith {zenith} fmt {fmt}: max |d| / (2e-3 |w| + 2^-24) = {excess:.2f}, mean rel {mean_rel:.2e}, "
          f"texels below the half normal range {(np.abs(w) < 2.0 ** -14).mean():.2f}")
    assert excess <= 1.0 and mean_rel <= 5e-4
    assert np.all(got[..., 3] == 0)


@pytest.mark.parametrize("size,levels", [(128, None), (512, None), (16, None), (1, None), (128, 3), (64, 6)])
def test_mips_are_the_box_filter(ctx, size, levels):
    p, r, s, luts = _luts(ctx, 45.0)
    lv = environment_cube(ctx, p, r, s, luts, size, levels)
    ctx.synchronize()
    n = size.bit_length() if levels is None else levels
    assert len(lv) == n
    for k in range(1, n):
        up = lv[k - 1].cpu().numpy()
        np.testing.assert_array_equal(lv[k].cpu().numpy(), orc.box_mip(up), err_msg=f"level {k}")


def test_invalid_arguments(ctx):
    p, r, s, luts = _luts(ctx, 45.0)
    for size, levels in ((96, 1), (1024, 1), (128, 9), (128, 0)):
        with pytest.raises(_abi.SkyrError):
            environment_cube(ctx, p, r, s, luts, size, levels)


def test_sh_and_prefilter_match_oracle(ctx):
    from skyrendering_gb300.atmosphere import environment_prefilter, environment_seamless, environment_sh

    p, r, s, luts = _luts(ctx, 60.0)
    total = _abi.lib().skyr_environment_cube_level_offset(128, 8)
    flat = torch.empty((total, 4), dtype=torch.float16, device="cuda")
    environment_cube(ctx, p, r, s, luts, 128, out=flat)
    seamless = environment_seamless(ctx, flat, 128, 8)
    sh = environment_sh(ctx, seamless, 128, 8)
    pre = environment_prefilter(ctx, seamless, 128, 8, 128, 5)
    ctx.synchronize()
    cube = flat.float().cpu().numpy().astype(np.float64)
    # the seamless copy: faces as stored, aprons from the adjacent faces (corners: mean of three)
    np.testing.assert_allclose(seamless.cpu().numpy(), orc.environment_seamless(cube, 128, 8), rtol=1e-6, atol=0)
    want = orc.environment_sh(cube, 128, 8)
    got = sh.cpu().numpy()[:, :3].astype(np.float64)
    err = np.abs(got - want).max() / np.abs(want).max()
    print(f"SH: max error {err:.2e} of the largest coefficient")
    assert err <= 1e-5 and np.all(sh.cpu().numpy()[:, 3] == 0)
    for k, lv in enumerate(pre):
        n = lv.shape[1]
        w = orc.environment_prefilter(cube, 128, 8, n, k / 4.0)
        g = lv.float().cpu().numpy().astype(np.float64)[..., :3]
        rel = np.abs(g - w) / np.maximum(np.abs(w), 1e-6 * np.abs(w).max())
        print(f"prefilter roughness {k / 4:.2f} ({n}^2): max rel {rel.max():.2e}, mean {rel.mean():.2e}")
        assert rel.mean() <= 5e-4 and rel.max() <= 3e-3
