"""GPU parity of the quarter-resolution cloud pass (include/skyr_cloud_quarter.h)
against the FP64 oracle, pass by pass on the GPU's own intermediate buffers
and as a whole chain.

* checkerboard depth: bit-exact (max / min of the same floats);
* index: the same texel chosen (mismatch <= 1e-3 of texels), linear depth
  within 1e-6;
* quarter raymarch at the chosen checkerboard texels: mean relative error
  <= 1e-3 (luminance, transmittance, distance);
* reconstruct, without and with history (a moved camera, wind, the previous
  frame's reconstruction): mean relative error <= 1e-3 (RGBA16F storage);
* upscale and composite into the HDR target: mean relative error <= 1e-3;
* the chain on an empty depth buffer at 1920x1080 (oracle: its own index,
  raymarch, reconstruct and upscale): mean relative error <= 1e-3;
* a synthetic depth buffer (the Earth's surface and a near occluder) drives
  the depth-aware paths; viewport 480x270 gives odd half / quarter sizes;
* graph replay is bit-identical, and so is the raymarch with 2, 4 or 8 lanes
  per ray; bad arguments are refused;
* the quarter-pass autotuner times all 288 launch shapes on the pass itself and
  keeps the fastest, which renders the same texels as the default shape.
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

pytestmark = pytest.mark.gpu
Z_NEAR, Z_FAR = 0.3, 50000.0  # the workload Camera's planes


def synthetic_depth(cam: W.Camera, w: int, h: int, R: float) -> np.ndarray:
    """GL window depth of the Earth's surface below the horizon and of a near
    occluder 2.5 km away in a screen rectangle; 1 (empty) elsewhere."""
    vp = cam.view_projection()
    ivp = np.linalg.inv(vp)
    ys, xs = np.mgrid[0:h, 0:w]
    ndc = np.stack([(xs + 0.5) / w * 2 - 1, (ys + 0.5) / h * 2 - 1, np.zeros_like(xs, float), np.ones_like(xs, float)],
                   -1)
    p = ndc @ ivp.T
    p = p[..., :3] / p[..., 3:]
    o = np.asarray(cam.position, dtype=np.float64)
    d = p - o
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    c = o - np.array([0.0, -R, 0.0])
    b = d @ c
    disc = b * b - (c @ c - R * R)
    t = np.where((disc > 0) & (b < 0), -b - np.sqrt(np.maximum(disc, 0)), np.inf)
    occ = (xs > 0.3 * w) & (xs < 0.45 * w) & (ys > 0.35 * h) & (ys < 0.75 * h)
    t = np.where(occ, 2.5, t)
    hit = np.isfinite(t)
    q = o + d * np.where(hit, t, 1.0)[..., None]
    clip = np.concatenate([q, np.ones_like(q[..., :1])], -1) @ vp.T
    depth = np.where(hit, 0.5 * clip[..., 2] / clip[..., 3] + 0.5, 1.0)
    return depth.astype(np.float32)


def host_textures(f):
    return {k: (t.desc, t.data.cpu().numpy()) for k, t in f.tex.items()}


def half4(t: torch.Tensor) -> np.ndarray:
    return t.float().cpu().numpy().astype(np.float64)


class Quarter:
    def __init__(self, ctx, cam, w, h, zenith=45.0, depth=True):
        self.f = Frame(ctx, cam, zenith, size=(w, h))
        self.w, self.h = w, h
        self.depth_np = synthetic_depth(cam, w, h, self.f.atmo.bottom_radius) if depth else None
        self.depth = None if self.depth_np is None else torch.from_numpy(self.depth_np).cuda()
        self.vp = CL.CloudViewport(ctx, w, h)
        rng = np.random.default_rng(8)
        self.hdr_in = torch.from_numpy(rng.uniform(0.0, 4.0, (h, w, 4)).astype(np.float16)).cuda()

    def render(self, view=None, wind=None, history=True):
        f = self.f
        self.hdr = self.hdr_in.clone()
        frame = self.vp.render(f.vc, f.atmo, view or f.view, f.sizes, f.luts, f.bn, depth=self.depth, hdr=self.hdr,
                               wind_delta=wind, z_near=Z_NEAR, z_far=Z_FAR, history=history)
        torch.cuda.synchronize()
        return frame

    def luts(self):
        L = self.f.luts
        return (L.transmittance[0].cpu().double().numpy(),
                L.aerial_perspective_luminance[0].float().cpu().double().numpy(),
                L.aerial_perspective_transmittance[0].float().cpu().double().numpy())


def check_passes(q: Quarter, frame, view, previous=None):
    f, vp = q.f, q.vp
    cb = vp.checkerboard.cpu().numpy()
    np.testing.assert_array_equal(cb, orc.checkerboard(q.depth_np, q.w, q.h))
    idx = vp.index.cpu().numpy()
    oidx = orc.index_gen(cb, q.w, q.h, Z_NEAR, Z_FAR, frame.base_shading_index)
    mism = (idx[..., 0] != oidx[..., 0]).mean()
    assert mism <= 1e-3, mism
    same = idx[..., 0] == oidx[..., 0]
    np.testing.assert_allclose(idx[..., 1][same], oidx[..., 1][same], rtol=1e-6)
    rgba, dist = orc.render_quarter(f.atmo, f.cloud, f.material, host_textures(f), view, f.sizes, *q.luts(),
                                    f.bn.cpu().numpy(), idx, cb)
    g = half4(vp.render_rgba).reshape(-1, 4)
    gd = vp.render_distance.cpu().numpy().reshape(-1).astype(np.float64)
    e_render = (mean_rel(g[:, :3], rgba[:, :3]), mean_rel(g[:, 3], rgba[:, 3]), mean_rel(gd, dist))
    rec = orc.reconstruct(f.atmo, f.cloud, f.material, host_textures(f), view, frame, cb, idx,
                          half4(vp.render_rgba), vp.render_distance.cpu().numpy(), previous)
    grec = half4(vp.reconstruction)
    e_rec = (mean_rel(grec[..., :3], rec[..., :3]), mean_rel(grec[..., 3], rec[..., 3]))
    up = orc.upscale(q.w, q.h, q.depth_np, Z_NEAR, Z_FAR, cb, grec, half4(q.hdr_in))
    ghdr = half4(q.hdr)
    e_up = mean_rel(ghdr[..., :3], up[..., :3])
    assert np.array_equal(ghdr[..., 3], half4(q.hdr_in)[..., 3])
    print(f"index mismatch {mism:.1e}; render {e_render[0]:.2e}/{e_render[1]:.2e}/{e_render[2]:.2e}; "
          f"reconstruct {e_rec[0]:.2e}/{e_rec[1]:.2e}; upscale {e_up:.2e}")
    assert max(e_render) <= 1e-3 and max(e_rec) <= 1e-3 and e_up <= 1e-3
    return rec


def test_passes_match_oracle_with_depth_buffer(ctx):
    cam = W.frame_camera()
    q = Quarter(ctx, cam, 480, 270)
    frame = q.render()
    assert not frame.has_previous
    # the synthetic depth makes both checkerboard choices and edges appear
    cb = q.vp.checkerboard.cpu().numpy()
    assert (cb < 1).mean() > 0.2 and (cb == 1).mean() > 0.2
    check_passes(q, frame, q.f.view)


def test_temporal_frame_with_history_matches_oracle(ctx):
    cam = W.frame_camera()
    q = Quarter(ctx, cam, 480, 270)
    q.render()
    prev_rec = half4(q.vp.reconstruction)
    cam2 = W.Camera(position=(0.05, 1.0, 0.03), yaw=90.3, pitch=10.1, width=480, height=270)
    view2 = W.frame_view(cam2, 45.0, width=480, height=270)
    view2.frame_id = 1.0
    frame = q.render(view=view2, wind=(0.01, 0.0))
    assert frame.has_previous and frame.base_shading_index == 1
    rec = check_passes(q, frame, view2, previous=prev_rec)
    # history matters: the reconstruction without it differs
    f = q.f
    nohist = _abi.CloudTemporalFrame.from_buffer_copy(frame)
    nohist.has_previous = 0
    plain = orc.reconstruct(f.atmo, f.cloud, f.material, host_textures(f), view2, nohist,
                            q.vp.checkerboard.cpu().numpy(), q.vp.index.cpu().numpy(), half4(q.vp.render_rgba),
                            q.vp.render_distance.cpu().numpy(), None)
    # (where the neighbourhood is uniform -- clear sky -- the clamp pins the
    # history to this frame's value, so only cloudy texels can change)
    changed = np.any(np.abs(rec - plain) > 1e-6 * (1 + np.abs(plain)), axis=-1)
    cloudy = plain[..., 3] < 0.999
    print(f"texels changed by the history: {changed.mean():.2f} (cloudy {cloudy.mean():.2f})")
    assert changed[cloudy].mean() > 0.5


def test_chain_1080p_empty_depth_matches_oracle(ctx):
    cam = W.frame_camera()
    q = Quarter(ctx, cam, 1920, 1080, depth=False)
    frame = q.render()
    f = q.f
    cb = orc.checkerboard(None, 1920, 1080)
    idx = orc.index_gen(cb, 1920, 1080, Z_NEAR, Z_FAR, frame.base_shading_index)
    rgba, dist = orc.render_quarter(f.atmo, f.cloud, f.material, host_textures(f), f.view, f.sizes, *q.luts(),
                                    f.bn.cpu().numpy(), idx, cb)
    rec = orc.reconstruct(f.atmo, f.cloud, f.material, host_textures(f), f.view, frame, cb, idx,
                          rgba.reshape(270, 480, 4), dist.reshape(270, 480), None)
    up = orc.upscale(1920, 1080, None, Z_NEAR, Z_FAR, cb, rec, half4(q.hdr_in))
    g = half4(q.hdr)
    e = (mean_rel(g[..., :3], up[..., :3]), mean_rel(half4(q.vp.reconstruction), rec))
    cloud = (half4(q.vp.reconstruction)[..., 3] < 0.99).mean()
    print(f"chain: hdr {e[0]:.2e}, reconstruction {e[1]:.2e}; cloudy texels {cloud:.2f}")
    assert cloud > 0.05 and max(e) <= 1e-3


@pytest.fixture()
def sctx(cuda):
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        c = Context(s)
        yield c
        c.close()


def test_graph_replay_and_invalid_arguments(sctx):
    import ctypes as C

    cam = W.frame_camera()
    q = Quarter(sctx, cam, 320, 180)
    frame = q.render(history=False)
    ref = [t.clone() for t in (q.vp.checkerboard, q.vp.index, q.vp.render_rgba, q.vp.render_distance,
                               q.vp.reconstruction, q.hdr)]
    f = q.f
    q.vp.current = 1 - q.vp.current  # write the same buffer again
    b = q.vp.buffers(history=False)
    hdr = q.hdr_in.clone()
    args = (sctx.handle, C.byref(f.atmo), C.byref(f.vc.params), C.byref(f.vc.material), C.byref(f.vc.textures),
            C.byref(f.view), C.byref(f.sizes), C.c_void_p(f.luts.transmittance.data_ptr()),
            C.c_void_p(f.luts.aerial_perspective_luminance.data_ptr()),
            C.c_void_p(f.luts.aerial_perspective_transmittance.data_ptr()), C.c_void_p(f.bn.data_ptr()),
            C.c_void_p(q.depth.data_ptr()), C.byref(frame), C.byref(b))
    with B.capture(sctx) as cap:
        _abi.call("skyr_cloud_render_quarter", *args, C.c_void_p(hdr.data_ptr()))
    for _ in range(2):
        hdr.copy_(q.hdr_in)
        cap.graph.launch()
    sctx.synchronize()
    got = [q.vp.checkerboard, q.vp.index, q.vp.render_rgba, q.vp.render_distance,
           q.vp.reconstruct[1 - q.vp.current], hdr]
    for a, r in zip(got, ref):
        assert torch.equal(a, r)
    cap.graph.close()
    # the checkerboard raymarch with 2, 4 or 8 lanes per ray: the same texels bit for bit
    for g in (2, 4, 8):
        B.set_tuning(sctx, cloud_ray_lanes=g, cloud_tile_width=8)
        hdr.copy_(q.hdr_in)
        _abi.call("skyr_cloud_render_quarter", *args, C.c_void_p(hdr.data_ptr()))
        sctx.synchronize()
        for a, r in zip((q.vp.render_rgba, q.vp.render_distance, hdr), (ref[2], ref[3], ref[5])):
            assert torch.equal(a, r), g
    B.set_tuning(sctx, cloud_ray_lanes=1)
    bad = _abi.CloudQuarterBuffers.from_buffer_copy(b)
    bad.previous_reconstruct = bad.reconstruct
    with pytest.raises(_abi.SkyrError):
        _abi.call("skyr_cloud_render_quarter", *args[:-1], C.byref(bad), None)
    bad = _abi.CloudQuarterBuffers.from_buffer_copy(b)
    bad.render_rgba = None
    with pytest.raises(_abi.SkyrError):
        _abi.call("skyr_cloud_render_quarter", *args[:-1], C.byref(bad), None)


def test_quarter_autotuner(sctx):
    cam = W.frame_camera()
    q = Quarter(sctx, cam, 640, 360, depth=False)
    q.render(history=False)
    f = q.f
    best, times = q.vp.autotune(f.vc, f.atmo, f.view, f.sizes, f.luts, f.bn, z_near=Z_NEAR, z_far=Z_FAR, reps=2)
    key = B.cloud_tuning_key(best)
    assert key in B.CLOUD_CANDIDATES and len(times) == len(B.CLOUD_CANDIDATES)
    assert all(t > 0 for t in times)
    assert min(times) == pytest.approx(times[B.CLOUD_CANDIDATES.index(key)])
    assert B.cloud_tuning_key(B.tuning(sctx)) == key
    # the chosen shape renders the same texels as the default one
    B.set_tuning(sctx, cloud_ray_lanes=1, cloud_tile_width=8, cloud_block_warps_x=2, cloud_blocks_per_sm=5)
    q.vp.frames = 0
    q.render(history=False)
    got_default = q.vp.render_rgba.clone()
    B.set_tuning(sctx, cloud_tile_width=best.cloud_tile_width, cloud_block_warps_x=best.cloud_block_warps_x,
                 cloud_blocks_per_sm=best.cloud_blocks_per_sm, cloud_ray_lanes=best.cloud_ray_lanes)
    q.vp.frames = 0
    q.render(history=False)
    assert torch.equal(q.vp.render_rgba, got_default)
