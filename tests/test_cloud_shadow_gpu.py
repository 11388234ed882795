"""GPU parity of the cloud shadow passes (include/skyr_cloud_shadow.h) and of
the shadow froxel's use in the raymarch, the path tracer and the surrogate.

* shadow map: GPU (FP32, stable ray-shell roots) against the FP64 oracle (the
  reference's formulas) on the same light frame, over sampled texels: mean
  relative error of the depth <= 1e-5, of the transmittance <= 1e-3, of the
  opacity (1 - T) <= 2e-3; with the temporal blend into the previous map too;
* blur: against the oracle's two passes over the GPU's raw map, to FP32
  rounding (max error 1e-6 of the map's range);
* froxel: against the oracle's froxel of the GPU's blurred map: mean |d| <= 0.5
  and max |d| <= 66 unorm16 steps (1e-3);
* consumers: the raymarch with a froxel (the passes' own, and a synthetic one
  that changes the frame by several percent) against the oracle with the same
  froxel at 1e-3 mean relative error; the path tracer by the same 3-sigma
  test as without a froxel;
* the whole chain computed by the oracle from scratch (its own light frame,
  map, blur, froxel and raymarch, all FP64) against the GPU's at 1e-3;
* a captured CUDA graph replays the passes bit-identically; bad arguments are
  refused.
"""
import numpy as np
import pytest
import torch

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import batch as B
from skyrendering_gb300 import cloud as CL
from skyrendering_gb300 import workloads as W
from skyrendering_gb300.atmosphere import Context

from .test_cloud_gpu import Frame, mean_rel
from .test_pathtrace_gpu import Scene, region_pixels, zscores

pytestmark = pytest.mark.gpu


def host_textures(f):
    return {k: (t.desc, t.data.cpu().numpy()) for k, t in f.tex.items()}


def synthetic_froxel(w=24, h=14, d=32, seed=5):
    """A smooth field in [0.15, 1] (uint16 [d][h][w])."""
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(np.arange(d), np.arange(h), np.arange(w), indexing="ij")
    a, b, c = rng.uniform(0, 6, 3)
    f = 0.575 + 0.425 * np.cos(x * 0.7 + a) * np.cos(y * 0.9 + b) * np.cos(z * 0.3 + c)
    return np.round(np.clip(f, 0, 1) * 65535).astype(np.uint16)


def device_froxel(arr: np.ndarray) -> torch.Tensor:
    return torch.from_numpy(np.ascontiguousarray(arr).view(np.int16)).cuda()


def attach(view, froxel_dev: torch.Tensor):
    d, h, w = froxel_dev.shape
    view.shadow_froxel = froxel_dev.data_ptr()
    view.shadow_froxel_width, view.shadow_froxel_height, view.shadow_froxel_depth = w, h, d
    return view


def froxel_host(t: torch.Tensor) -> np.ndarray:
    return t.cpu().numpy().view(np.uint16)


def map_errors(got, want):
    return {"depth": mean_rel(got[:, 0], want[:, 0]), "transmittance": mean_rel(got[:, 1], want[:, 1]),
            "opacity": mean_rel(1 - got[:, 1], 1 - want[:, 1])}


@pytest.mark.parametrize("zenith,azimuth", [(45.0, 60.0), (80.0, 200.0), (0.0, 0.0)])
def test_shadow_map_matches_oracle(ctx, zenith, azimuth):
    cam = W.frame_camera()
    f = Frame(ctx, cam, zenith, size=(320, 180))
    f.view.sun_direction_phi = azimuth
    sizes = CL.shadow_sizes(1920, 1080)
    sh = CL.CloudShadow(ctx, sizes)
    frame = sh.render(f.vc, f.atmo, f.view, f.bn)
    ctx.synchronize()
    raw = sh.raw_map.cpu().numpy().reshape(-1, 2).astype(np.float64)
    rng = np.random.default_rng(11)
    texels = np.sort(rng.choice(raw.shape[0], 6000, replace=False)).astype(np.int32)
    want = orc.shadow_map(f.atmo, f.cloud, f.material, host_textures(f), f.view, 512, 512, orc.frame_array(frame),
                          False, f.bn.cpu().numpy(), texels=texels)
    err = map_errors(raw[texels], want)
    print(f"zenith {zenith}: " + ", ".join(f"{k}={v:.2e}" for k, v in err.items()) +
          f"; shadowed texels {(want[:, 1] < 0.99).mean():.2f}")
    assert (want[:, 1] < 0.99).mean() > 0.05, "the map should hold cloud shadow"
    assert err["depth"] <= 1e-5 and err["transmittance"] <= 1e-3 and err["opacity"] <= 2e-3, err
    # blur: the oracle's two passes over the GPU's raw map
    blurred = sh.map.cpu().numpy().astype(np.float64)
    ob = orc.shadow_blur(sh.raw_map.cpu().numpy())
    for c in range(2):
        scale = np.abs(ob[..., c]).max()
        assert np.abs(blurred[..., c] - ob[..., c]).max() <= 1e-6 * scale + 1e-7, c
    # froxel: the oracle's froxel of the GPU's blurred map
    fx, _ = orc.shadow_froxel(f.atmo, f.cloud, f.material, host_textures(f), f.view, orc.frame_array(frame),
                              sh.map.cpu().numpy(), (sizes.froxel_width, sizes.froxel_height, sizes.froxel_depth))
    d = np.abs(froxel_host(sh.froxel).astype(np.int64) - fx.astype(np.int64))
    print(f"froxel: mean |d| {d.mean():.3f} max |d| {d.max()} (unorm16 steps); mean visibility "
          f"{fx.mean() / 65535:.3f}")
    assert d.mean() <= 0.5 and d.max() <= 66


def test_shadow_map_temporal_blend(ctx):
    cam = W.frame_camera()
    f = Frame(ctx, cam, 50.0, size=(320, 180))
    sizes = CL.shadow_sizes(1920, 1080)
    sh = CL.CloudShadow(ctx, sizes)
    sh.render(f.vc, f.atmo, f.view, f.bn)
    ctx.synchronize()
    prev_raw = sh.raw_map.cpu().numpy().copy()
    # next frame: the camera moved, the sun turned, the wind carried the clouds
    cam2 = W.Camera(position=(0.25, 1.1, 0.15), yaw=91.0, pitch=10.5)
    f2 = Frame(ctx, cam2, 51.0, size=(320, 180))
    f2.view.frame_id = 1.0
    wind = (0.04, 0.01)
    frame2 = sh.render(f2.vc, f2.atmo, f2.view, f2.bn, wind_delta=wind)
    ctx.synchronize()
    assert frame2.has_previous
    raw = sh.raw_map.cpu().numpy().reshape(-1, 2).astype(np.float64)
    rng = np.random.default_rng(12)
    texels = np.sort(rng.choice(raw.shape[0], 6000, replace=False)).astype(np.int32)
    fa = orc.frame_array(frame2)
    want = orc.shadow_map(f2.atmo, f2.cloud, f2.material, host_textures(f2), f2.view, 512, 512, fa, True,
                          f2.bn.cpu().numpy(), previous_map=prev_raw, texels=texels)
    err = map_errors(raw[texels], want)
    plain = orc.shadow_map(f2.atmo, f2.cloud, f2.material, host_textures(f2), f2.view, 512, 512, fa, False,
                           f2.bn.cpu().numpy(), texels=texels)
    blended = np.any(np.abs(want - plain) > 1e-9, axis=1).mean()
    print("blend: " + ", ".join(f"{k}={v:.2e}" for k, v in err.items()) + f"; blended texels {blended:.2f}")
    assert blended > 0.5, "most texels reproject into the previous map"
    assert err["depth"] <= 1e-5 and err["transmittance"] <= 1e-3 and err["opacity"] <= 2e-3, err
    # the oracle's own reprojection matrix agrees with the library's
    of, has = orc.light_frame(f2.atmo, f2.cloud, f2.view, 512, 512,
                              previous=orc.light_frame(f.atmo, f.cloud, f.view, 512, 512)[0], wind=wind)
    assert has
    np.testing.assert_allclose(fa[48:], of[48:], atol=2e-6)


def test_raymarch_with_froxel_matches_oracle(ctx):
    f = Frame(ctx, W.frame_camera(), 45.0)
    npx = f.view.width * f.view.height
    px = np.sort(np.random.default_rng(3).choice(npx, 60000, replace=False)).astype(np.int32)
    plain = f.rgba.float().cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    # a synthetic froxel that changes the frame visibly
    syn = synthetic_froxel()
    dev = device_froxel(syn)
    attach(f.view, dev)
    rgba, dist = f.vc.render(f.atmo, f.view, f.sizes, f.luts, f.bn)
    ctx.synchronize()
    g = rgba.float().cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    o, od = orc.cloud_render(f.atmo, f.cloud, f.material, host_textures(f), f.view, f.sizes,
                             f.luts.transmittance[0].cpu().double().numpy(),
                             f.luts.aerial_perspective_luminance[0].float().cpu().double().numpy(),
                             f.luts.aerial_perspective_transmittance[0].float().cpu().double().numpy(),
                             f.bn.cpu().numpy(), pixels=px, froxel=syn)
    change = mean_rel(g[:, :3], plain[:, :3])
    e = mean_rel(g[:, :3], o[:, :3])
    print(f"synthetic froxel: change {change:.2e}, luminance error {e:.2e}")
    assert change > 5e-3, "the froxel should change the frame"
    assert e <= 1e-3 and mean_rel(g[:, 3], o[:, 3]) <= 1e-3
    # the shadow passes' own froxel
    sh = CL.CloudShadow(ctx, CL.shadow_sizes(1920, 1080))
    sh.render(f.vc, f.atmo, CL.detach_froxel(f.view), f.bn)
    sh.attach(f.view)
    rgba, dist = f.vc.render(f.atmo, f.view, f.sizes, f.luts, f.bn)
    ctx.synchronize()
    g = rgba.float().cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    o, od = orc.cloud_render(f.atmo, f.cloud, f.material, host_textures(f), f.view, f.sizes,
                             f.luts.transmittance[0].cpu().double().numpy(),
                             f.luts.aerial_perspective_luminance[0].float().cpu().double().numpy(),
                             f.luts.aerial_perspective_transmittance[0].float().cpu().double().numpy(),
                             f.bn.cpu().numpy(), pixels=px, froxel=froxel_host(sh.froxel))
    e = mean_rel(g[:, :3], o[:, :3])
    print(f"pass froxel: change {mean_rel(g[:, :3], plain[:, :3]):.2e}, luminance error {e:.2e}")
    assert e <= 1e-3


def test_full_chain_matches_oracle(ctx):
    """Everything from the view on: the oracle derives its own light frame."""
    zenith = 60.0
    f = Frame(ctx, W.frame_camera(), zenith, size=(480, 270))
    sizes = CL.shadow_sizes(1920, 1080)
    sizes.map_width = sizes.map_height = 256
    sh = CL.CloudShadow(ctx, sizes)
    sh.render(f.vc, f.atmo, f.view, f.bn)
    sh.attach(f.view)
    rgba, dist = f.vc.render(f.atmo, f.view, f.sizes, f.luts, f.bn)
    ctx.synchronize()
    host = host_textures(f)
    of, _ = orc.light_frame(f.atmo, f.cloud, f.view, 256, 256)
    omap = orc.shadow_map(f.atmo, f.cloud, f.material, host, f.view, 256, 256, of, False, f.bn.cpu().numpy())
    oblur = orc.shadow_blur(omap.reshape(256, 256, 2))
    ofx, _ = orc.shadow_froxel(f.atmo, f.cloud, f.material, host, f.view, of, oblur,
                               (sizes.froxel_width, sizes.froxel_height, sizes.froxel_depth))
    d = np.abs(froxel_host(sh.froxel).astype(np.int64) - ofx.astype(np.int64))
    print(f"chain froxel: mean |d| {d.mean():.3f} max |d| {d.max()}; visibility {ofx.mean() / 65535:.3f}")
    assert d.mean() <= 2.0
    o, od = orc.cloud_render(f.atmo, f.cloud, f.material, host, f.view, f.sizes,
                             f.luts.transmittance[0].cpu().double().numpy(),
                             f.luts.aerial_perspective_luminance[0].float().cpu().double().numpy(),
                             f.luts.aerial_perspective_transmittance[0].float().cpu().double().numpy(),
                             f.bn.cpu().numpy(), froxel=ofx)
    g = rgba.float().cpu().numpy().reshape(-1, 4).astype(np.float64)
    err = (mean_rel(g[:, :3], o[:, :3]), mean_rel(g[:, 3], o[:, 3]))
    print(f"chain frame: luminance {err[0]:.2e} transmittance {err[1]:.2e}")
    assert max(err) <= 1e-3


def test_pathtrace_with_froxel_matches_oracle(ctx):
    s = Scene(ctx)
    n = 1024
    region = (60, 58, 68, 62)
    px = region_pixels(s.view, region)
    s.tracer.render(s.atmo, s.luts, n_frames=n, region=region)
    ctx.synchronize()
    plain = s.tracer.acc.cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    syn = synthetic_froxel(seed=9)
    dev = device_froxel(syn)
    attach(s.view, dev)
    s.tracer.reset()  # the same frames, so the same paths
    s.tracer.render(s.atmo, s.luts, n_frames=n, region=region)
    ctx.synchronize()
    acc = s.tracer.acc.cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    acc2 = s.tracer.acc_sq.cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
    so, sqo = orc.pathtrace(s.atmo, s.cloud, None, None, s.grid.struct, s.grid.data.cpu().numpy(),
                            s.grid.majorant.cpu().numpy(), s.pt, s.view, s.render, s.sizes, s.host_luts(), 1, n, px,
                            froxel=syn)
    z = zscores(acc, acc2, so, sqo, n)
    change = mean_rel(acc[:, :3], plain[:, :3])
    print(f"froxel: change {change:.2e}; max|z|={np.abs(z).max():.2f} mean z^2={np.mean(z * z):.2f}")
    assert change > 1e-4, "the froxel should change the accumulation"
    assert np.abs(z).max() <= 4.5 and np.mean(z * z) <= 2.0


@pytest.fixture()
def sctx(cuda):
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        c = Context(s)
        yield c
        c.close()


def test_graph_replay_and_invalid_arguments(sctx):
    f = Frame(sctx, W.frame_camera(), 45.0, size=(160, 90))
    sizes = CL.shadow_sizes(1920, 1080)
    sh = CL.CloudShadow(sctx, sizes)
    sh.render(f.vc, f.atmo, f.view, f.bn, blend=False)
    sctx.synchronize()
    ref = (sh.raw_map.clone(), sh.map.clone(), sh.froxel.clone())
    frame = sh.frame
    raw, smap = torch.zeros_like(ref[0]), torch.zeros_like(ref[1])
    fx = torch.zeros_like(ref[2])
    args = (sctx.handle, _abi.C.byref(f.atmo), _abi.C.byref(f.cloud), _abi.C.byref(f.material),
            _abi.C.byref(f.vc.textures), _abi.C.byref(f.view), _abi.C.byref(sizes), _abi.C.byref(frame))
    with B.capture(sctx) as cap:
        _abi.call("skyr_cloud_shadow_render", *args, _abi.C.c_void_p(f.bn.data_ptr()), None,
                  _abi.C.c_void_p(raw.data_ptr()), _abi.C.c_void_p(smap.data_ptr()), _abi.C.c_void_p(fx.data_ptr()))
    cap.graph.launch()
    cap.graph.launch()
    sctx.synchronize()
    assert torch.equal(raw, ref[0]) and torch.equal(smap, ref[1]) and torch.equal(fx, ref[2])
    cap.graph.close()
    bn = _abi.C.c_void_p(f.bn.data_ptr())
    r0, s0, x0 = (_abi.C.c_void_p(t.data_ptr()) for t in (raw, smap, fx))
    with pytest.raises(_abi.SkyrError):  # the raw map is also the previous one
        _abi.call("skyr_cloud_shadow_render", *args, bn, r0, r0, s0, x0)
    with pytest.raises(_abi.SkyrError):  # a froxel without the blurred map
        _abi.call("skyr_cloud_shadow_render", *args, bn, None, r0, None, x0)
    bad = _abi.CloudShadowSizes.from_buffer_copy(sizes)
    bad.froxel_depth = 600
    with pytest.raises(_abi.SkyrError):
        _abi.call("skyr_cloud_shadow_render", sctx.handle, _abi.C.byref(f.atmo), _abi.C.byref(f.cloud),
                  _abi.C.byref(f.material), _abi.C.byref(f.vc.textures), _abi.C.byref(f.view), _abi.C.byref(bad),
                  _abi.C.byref(frame), bn, None, r0, s0, x0)
    # a view whose froxel has no size
    v = _abi.CloudView.from_buffer_copy(f.view)
    v.shadow_froxel = fx.data_ptr()
    v.shadow_froxel_width = 0
    with pytest.raises(_abi.SkyrError):
        f.vc.render(f.atmo, v, f.sizes, f.luts, f.bn)
