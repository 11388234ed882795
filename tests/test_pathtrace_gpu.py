"""GPU parity of the voxel path tracer, the synthetic density grid and the
brick majorant grid against the CPU oracle, through the C ABI.

* grid: GPU (FP32 noise, FP16 storage) vs oracle (FP64) within one FP16 step;
* majorants: bit-exact against the oracle on the same FP16 grid, and a true
  bound of the trilinear extinction inside each brick;
* path tracing: the oracle draws the same random numbers (same hash, same FP32
  conversion) but its FP64 arithmetic lets paths diverge after a while, so the
  test is statistical -- per pixel and channel z = (mean_gpu - mean_oracle) /
  sqrt(var_gpu / N + var_oracle / N) over N frames, |z| <= 4.5 everywhere and
  mean z^2 <= 2 (a 3-sigma criterion with a multiple-comparison allowance).
"""
import math

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import workloads as W
from skyrendering_gb300.atmosphere import update_lut_set
from skyrendering_gb300.pathtrace import DensityGrid, PathTracer

pytestmark = pytest.mark.gpu
SMALL = (64, 80, 44)


def make_grid(ctx, dims=SMALL):
    origin, voxel = W.pt_grid_placement(dims)
    g = DensityGrid(*dims, origin=origin, voxel_size=voxel, density=1.0)
    g.generate(ctx, W.pt_grid_generator(dims)).normalize_extinction(ctx, W.PT_SIGMA_MAX)
    ctx.synchronize()
    return g


def test_grid_generator_matches_oracle(ctx):
    dims = (32, 40, 22)
    origin, voxel = W.pt_grid_placement(dims)
    g = DensityGrid(*dims, origin=origin, voxel_size=voxel, density=1.0).generate(ctx, W.pt_grid_generator(dims))
    ctx.synchronize()
    got = g.data.float().cpu().numpy().astype(np.float64)
    want = orc.grid_generate(W.pt_grid_generator(dims))
    step = np.maximum(np.abs(want), 2.0 ** -14) * 2.0 ** -10  # one FP16 step
    assert np.all(np.abs(got - want) <= step + 1e-6)
    assert (got > 0).mean() > 0.05


def test_majorants_exact_and_bounding(ctx):
    g = make_grid(ctx)
    half = g.data.cpu().numpy()
    got = g.majorant.cpu().numpy()
    np.testing.assert_array_equal(got, orc.grid_majorants(g.struct, half))
    # the brick majorant bounds the trilinear extinction anywhere in the brick
    vals = half.astype(np.float64) * g.struct.density
    nz, ny, nx = vals.shape
    rng = np.random.default_rng(1)
    p = rng.uniform(0, 1, size=(20000, 3)) * np.array([nx, ny, nz])  # grid units (x, y, z)
    q = p - 0.5
    i0 = np.floor(q).astype(int)
    f = q - i0
    pad = np.pad(vals, 1)
    s = np.zeros(len(p))
    for dz in (0, 1):
        for dy in (0, 1):
            for dx in (0, 1):
                w = (f[:, 0] if dx else 1 - f[:, 0]) * (f[:, 1] if dy else 1 - f[:, 1]) * (f[:, 2] if dz else 1 - f[:, 2])
                s += w * pad[i0[:, 2] + dz + 1, i0[:, 1] + dy + 1, i0[:, 0] + dx + 1]
    b = (p // g.struct.brick).astype(int)
    assert np.all(s <= got[b[:, 2], b[:, 1], b[:, 0]] * (1 + 1e-6))


class Scene:
    def __init__(self, ctx, dims=SMALL, width=128, height=128, env=_abi.SKYR_ENV_GROUND_MULTI_BOUNCE,
                 bricks=True, grid=None):
        self.atmo = W.earth_like_atmosphere()
        self.sizes = W.plain_lut_sizes()
        cam = W.pt_camera(width, height)
        self.render = W.render_parameters(cam, 45.0)
        self.luts = update_lut_set(ctx, self.atmo, self.render, self.sizes)
        self.grid = grid or make_grid(ctx, dims)
        self.cloud = W.pt_cloud_parameters(dims)
        self.pt = W.pt_parameters()
        self.pt.environment_lighting = env
        self.pt.use_brick_majorants = 1 if bricks else 0
        self.view = W.frame_view(cam, 45.0)
        self.tracer = PathTracer(ctx, self.pt, self.cloud, self.view, self.render, self.sizes, grid=self.grid,
                                 track_variance=True)
        ctx.synchronize()

    def host_luts(self):
        L = self.luts
        return {k: getattr(L, k)[0].float().cpu().double().numpy() for k in
                ("transmittance", "sky_view_luminance", "sky_view_transmittance", "aerial_perspective_luminance",
                 "aerial_perspective_transmittance")}

    def oracle(self, pixels, n_frames, frame_begin=1):
        return orc.pathtrace(self.atmo, self.cloud, None, None, self.grid.struct, self.grid.data.cpu().numpy(),
                             self.grid.majorant.cpu().numpy() if self.pt.use_brick_majorants else None, self.pt,
                             self.view, self.render, self.sizes, self.host_luts(), frame_begin, n_frames, pixels)


def zscores(sum_g, sq_g, sum_o, sq_o, n):
    mg, mo = sum_g / n, sum_o / n
    vg = np.maximum(sq_g / n - mg * mg, 0) / n
    vo = np.maximum(sq_o / n - mo * mo, 0) / n
    den = np.sqrt(vg + vo)
    z = np.where(den > 0, (mg - mo) / np.maximum(den, 1e-300), np.where(np.abs(mg - mo) > 1e-6, np.inf, 0.0))
    return z


def region_pixels(view, region):
    x0, y0, x1, y1 = region
    return np.array([y * view.width + x for y in range(y0, y1) for x in range(x0, x1)], dtype=np.int32)


@pytest.mark.parametrize("bricks", [True, False])
def test_pathtrace_matches_oracle_statistically(ctx, bricks):
    s = Scene(ctx, bricks=bricks)
    n = 1024
    region = (60, 58, 68, 62)  # 32 pixels looking into the cloud
    s.tracer.render(s.atmo, s.luts, n_frames=n, region=region)
    ctx.synchronize()
    px = region_pixels(s.view, region)
    acc = s.tracer.acc.cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    acc2 = s.tracer.acc_sq.cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    so, sqo = s.oracle(px, n)
    assert acc[:, 3].mean() / n < 0.5, "most paths should scatter in the cloud"
    z = zscores(acc, acc2, so, sqo, n)
    print(f"bricks={bricks}: max|z|={np.abs(z).max():.2f} mean z^2={np.mean(z * z):.2f}; "
          f"mean L gpu={acc[:, :3].mean() / n:.4e} oracle={so[:, :3].mean() / n:.4e}")
    assert np.abs(z).max() <= 4.5 and np.mean(z * z) <= 2.0


@pytest.mark.parametrize("env", [_abi.SKYR_ENV_OFF, _abi.SKYR_ENV_CONST_ENVIRONMENT_MAP,
                                 _abi.SKYR_ENV_GROUND_SINGLE_BOUNCE])
def test_environment_modes(ctx, env):
    s = Scene(ctx, env=env, width=64, height=64)
    n = 512
    region = (28, 28, 36, 32)
    s.tracer.render(s.atmo, s.luts, n_frames=n, region=region)
    ctx.synchronize()
    px = region_pixels(s.view, region)
    acc = s.tracer.acc.cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    acc2 = s.tracer.acc_sq.cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    so, sqo = s.oracle(px, n)
    z = zscores(acc, acc2, so, sqo, n)
    print(f"env={env}: max|z|={np.abs(z).max():.2f} mean z^2={np.mean(z * z):.2f}")
    assert np.abs(z).max() <= 4.5 and np.mean(z * z) <= 2.0


def test_brick_and_global_majorants_agree(ctx):
    grid = None
    res = []
    for bricks in (True, False):
        s = Scene(ctx, bricks=bricks, width=64, height=64, grid=grid)
        grid = s.grid
        s.tracer.render(s.atmo, s.luts, n_frames=512)
        ctx.synchronize()
        res.append((s.tracer.acc.double().cpu().numpy(), s.tracer.acc_sq.double().cpu().numpy()))
    (a, a2), (b, b2) = res
    z = zscores(a, a2, b, b2, 512)
    assert np.abs(z).max() <= 5.5 and np.mean(z * z) <= 1.5


def test_resolve_pass(ctx):
    s = Scene(ctx, width=32, height=32)
    s.tracer.render(s.atmo, s.luts, n_frames=4)
    bg = torch.rand((32, 32, 4), device="cuda").half()
    out = s.tracer.resolve(bg).float().cpu().numpy()
    acc = s.tracer.acc.cpu().numpy()
    want = bg.float().cpu().numpy()[..., :3] * (acc[..., 3:] / 4) + acc[..., :3] / 4
    np.testing.assert_allclose(out[..., :3], want, rtol=2e-3, atol=1e-4)


def test_pathtrace_invalid_arguments(ctx):
    import ctypes as C

    s = Scene(ctx, width=16, height=16)
    pt = W.pt_parameters()
    pt.environment_lighting = 9
    lib = _abi.lib()
    acc = torch.zeros((16, 16, 4), device="cuda")
    rc = lib.skyr_pathtrace(ctx.handle, C.byref(s.atmo), C.byref(s.cloud), None, None, C.byref(s.grid.struct),
                            C.byref(pt), C.byref(s.view), C.byref(s.render), C.byref(s.sizes),
                            C.c_void_p(s.luts.transmittance.data_ptr()), C.c_void_p(1), C.c_void_p(1),
                            C.c_void_p(1), C.c_void_p(1), 1, 1, None, C.c_void_p(acc.data_ptr()), None)
    assert rc == _abi.SKYR_EINVAL


def test_tracking_bound_reports_timeout(ctx):
    """A tracking bound far below what the scene needs ends the walks early and
    is reported as SKYR_ETIMEOUT by skyr_ctx_check_status; the default bound
    is not reached on the same scene (no fault, no hang either way)."""
    s = Scene(ctx, width=16, height=16)
    default = ctx.limits
    assert default.tracking_steps == 1 << 20 and default.copy_wait_cycles == 1 << 31
    tight = _abi.DeviceLimits.from_buffer_copy(default)
    tight.tracking_steps = 2
    ctx.limits = tight
    s.tracer.render(s.atmo, s.luts, n_frames=4)
    with pytest.raises(_abi.SkyrError) as exc:
        ctx.check_status()
    assert exc.value.status == _abi.SKYR_ETIMEOUT
    ctx.check_status()  # the status word was cleared by the report
    ctx.limits = default
    s.tracer.render(s.atmo, s.luts, n_frames=4)
    ctx.check_status()
    bad = _abi.DeviceLimits.from_buffer_copy(default)
    bad.tracking_steps = 0
    import ctypes as C

    assert _abi.lib().skyr_ctx_set_limits(ctx.handle, C.byref(bad)) == _abi.SKYR_EINVAL


def test_full_size_grid_matches_oracle_8192spp(ctx):
    """The voxel scene at its stated size: the seeded 512x640x352 FP16 grid of
    4-octave Worley fBm (seed 0x5EED, max extinction 40/km, 16^3 brick
    majorants), HG g = 0.857, albedo 1, up to 128 bounces, the sky-view
    environment with the ground bounce, a 1024x1024 view.  32 pixels looking
    into the cloud and 8 pixels grazing its edge (a 64-spp probe frame's
    never-scattered fraction between 0.3 and 0.7) are path-traced at 8192 spp
    and compared with the RNG-matched FP64 oracle by the same z-test; no walk
    may reach its tracking bound."""
    import ctypes as C

    dims = W.PT_GRID_DIMS
    grid = make_grid(ctx, dims)
    s = Scene(ctx, dims=dims, width=1024, height=1024, grid=grid)
    s.tracer.render(s.atmo, s.luts, n_frames=64)
    ctx.check_status()
    alpha = (s.tracer.acc[..., 3] / 64).cpu().numpy().reshape(-1)
    centre = region_pixels(s.view, (508, 508, 516, 512))
    edge = np.flatnonzero((alpha > 0.3) & (alpha < 0.7))
    assert len(edge) >= 8, "the probe frame should show the cloud's edge"
    edge = edge[np.linspace(0, len(edge) - 1, 8).astype(int)].astype(np.int32)
    px = np.concatenate([centre, edge]).astype(np.int32)
    n = 8192
    acc = torch.zeros((1024, 1024, 4), dtype=torch.float32, device="cuda")
    acc2 = torch.zeros_like(acc)
    dpx = torch.from_numpy(px).cuda()
    L = s.luts
    ptr = lambda t: C.c_void_p(t.data_ptr())
    _abi.call("skyr_pathtrace_pixels", ctx.handle, C.byref(s.atmo), C.byref(s.cloud), None, None,
              C.byref(grid.struct), C.byref(s.pt), C.byref(s.view), C.byref(s.render), C.byref(s.sizes),
              ptr(L.transmittance), ptr(L.sky_view_luminance), ptr(L.sky_view_transmittance),
              ptr(L.aerial_perspective_luminance), ptr(L.aerial_perspective_transmittance), 1, n, ptr(dpx),
              len(px), ptr(acc), ptr(acc2))
    ctx.check_status()  # no walk reached the tracking bound
    g = acc.cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    g2 = acc2.cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    so, sqo = s.oracle(px, n)
    assert g[:32, 3].mean() / n < 0.5, "the centre pixels should look into the cloud"
    z = zscores(g, g2, so, sqo, n)
    zc, ze = z[:32], z[32:]
    print(f"full grid 8192 spp: centre max|z|={np.abs(zc).max():.2f} mean z^2={np.mean(zc * zc):.2f}; "
          f"edge max|z|={np.abs(ze).max():.2f} mean z^2={np.mean(ze * ze):.2f}; "
          f"mean L gpu={g[:, :3].mean() / n:.4e} oracle={so[:, :3].mean() / n:.4e}")
    assert np.abs(z).max() <= 4.5 and np.mean(z * z) <= 2.0
