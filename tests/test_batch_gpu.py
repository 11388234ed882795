"""GPU checks of the batched path (include/skyr_batch.h): prepared LUT batches,
launch-shape tuning, the autotuners, multi-view raymarches and CUDA graphs.

* a prepared batch and skyr_update_lut_set run the same kernels on the same
  constants: bit-identical LUTs;
* lanes per texel change only the order of the per-ray sums: LUTs within 2e-6
  relative (FP32) / one FP16 step (FP16) of the default;
* the raymarch's warp-tile shape, register budget and lanes per ray change
  only which lane computes a step and how it is scheduled (with 2 or 4 lanes
  per ray the steps are folded in step order with the same FP32 operations):
  the 288 shapes give bit-identical frames;
* views rendered together (forked streams) or replayed from a CUDA graph are
  bit-identical to one skyr_cloud_render per view;
* a seeded subset of the batched workload (perturbed atmospheres, altitudes up
  to 10 km, sun zeniths up to 95 deg, uneven view sizes) matches the FP64
  oracle to 1e-3 mean relative error on sampled pixels.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import batch as B
from skyrendering_gb300 import workloads as W
from skyrendering_gb300.atmosphere import Context, LutSet, update_lut_set
from skyrendering_gb300.cloud import (NoiseTexture, VolumetricCloud, blue_noise_tile, prepare_textures,
                                      textures_struct)

pytestmark = pytest.mark.gpu


@pytest.fixture()
def sctx(cuda):
    """A context on its own stream (graph capture needs a created stream);
    torch works on the same stream."""
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        c = Context(s)
        yield c
        c.close()


class Clouds:
    def __init__(self, ctx):
        self.cloud = W.frame_cloud_parameters()
        self.material = W.frame_material()
        self.tex = {"cloud_map": NoiseTexture(W.cloud_map_desc()).generate(ctx),
                    "detail": NoiseTexture(W.base_noise_desc()).generate(ctx)}
        prepare_textures(ctx, self.material.type, self.tex)
        self.textures = textures_struct(**self.tex)
        self.bn = blue_noise_tile().cuda()
        self.vc = VolumetricCloud(ctx, self.cloud, self.material, self.textures)


def _set(luts: LutSet, s: int) -> LutSet:
    return LutSet(luts.transmittance[s:s + 1], luts.multiscattering[s:s + 1], luts.sky_view_luminance[s:s + 1],
                  luts.sky_view_transmittance[s:s + 1], luts.aerial_perspective_luminance[s:s + 1],
                  luts.aerial_perspective_transmittance[s:s + 1])


def _luts_equal(a: LutSet, b: LutSet):
    for k in ("transmittance", "multiscattering", "sky_view_luminance", "sky_view_transmittance",
              "aerial_perspective_luminance", "aerial_perspective_transmittance"):
        assert torch.equal(getattr(a, k), getattr(b, k)), k


@pytest.mark.parametrize("fmt", [0, 1])
def test_lut_batch_matches_update_lut_set(sctx, fmt):
    params, renders = W.batched_lut_sets(8)
    sizes = W.plain_lut_sizes(fmt)
    ref = update_lut_set(sctx, params, renders, sizes)
    got = LutSet.allocate(sizes, 8)
    b = B.LutBatch(sctx, params, renders, 8, sizes)
    b.launch(got)
    sctx.synchronize()
    _luts_equal(got, ref)
    b.close()


@pytest.mark.parametrize("lanes", [2, 4, 16])
def test_lut_lanes_variants(sctx, lanes):
    params, renders = W.batched_lut_sets(6)
    sizes = W.plain_lut_sizes(0)
    ref = update_lut_set(sctx, params, renders, sizes)
    B.set_tuning(sctx, transmittance_lanes=lanes, view_lanes=lanes)
    got = update_lut_set(sctx, params, renders, sizes)
    sctx.synchronize()
    for k in ("transmittance", "multiscattering", "sky_view_luminance", "aerial_perspective_luminance",
              "aerial_perspective_transmittance"):
        torch.testing.assert_close(getattr(got, k), getattr(ref, k), rtol=2e-6, atol=1e-12, msg=k)


def test_cloud_tile_shapes_are_identical(sctx):
    cl = Clouds(sctx)
    atmo, sizes = W.earth_like_atmosphere(), W.plain_lut_sizes()
    cam = W.frame_camera()
    luts = update_lut_set(sctx, atmo, W.render_parameters(cam, 45.0), sizes)
    view = W.frame_view(cam, 45.0, width=320, height=180)
    ref_rgba, ref_dist = cl.vc.render(atmo, view, sizes, luts, cl.bn)
    ref_rgba, ref_dist = ref_rgba.clone(), ref_dist.clone()
    for w, bx, occ, g in B.CLOUD_CANDIDATES:
        B.set_tuning(sctx, cloud_tile_width=w, cloud_block_warps_x=bx, cloud_blocks_per_sm=occ, cloud_ray_lanes=g)
        rgba, dist = cl.vc.render(atmo, view, sizes, luts, cl.bn)
        sctx.synchronize()
        assert torch.equal(rgba, ref_rgba), (w, bx, occ, g)
        assert torch.equal(dist, ref_dist), (w, bx, occ, g)


def _batched(ctx, n_sets=6, n_views=5, fmt=1):
    params, renders, views, sov = W.batched_frame(n_sets, n_views, seed=0xBA7C)
    sizes = W.plain_lut_sizes(fmt)
    luts = LutSet.allocate(sizes, n_sets)
    b = B.LutBatch(ctx, params, renders, n_sets, sizes)
    return params, renders, views, sov, sizes, luts, b


def test_render_views_and_graph_match_single_views(sctx):
    cl = Clouds(sctx)
    params, renders, views, sov, sizes, luts, b = _batched(sctx)
    n_views = len(sov)
    b.launch(luts)
    out = B.ViewOutputs(views, n_views)
    B.render_views(sctx, params, len(params), sov, cl.cloud, cl.material, cl.textures, views, n_views, sizes, luts,
                   cl.bn, out)
    sctx.synchronize()
    refs = []
    for i in range(n_views):
        r, d = cl.vc.render(params[sov[i]], views[i], sizes, _set(luts, sov[i]), cl.bn)
        refs.append((r.clone(), d.clone()))
    sctx.synchronize()
    for i in range(n_views):
        assert torch.equal(out.rgba[i], refs[i][0]), i
        assert torch.equal(out.dist[i], refs[i][1]), i
    # the same work captured into one graph and replayed twice
    luts2 = LutSet.allocate(sizes, len(params))
    out2 = B.ViewOutputs(views, n_views)
    with B.capture(sctx) as cap:
        b.launch(luts2)
        B.render_views(sctx, params, len(params), sov, cl.cloud, cl.material, cl.textures, views, n_views, sizes,
                       luts2, cl.bn, out2)
    for _ in range(2):
        cap.graph.launch()
    sctx.synchronize()
    _luts_equal(luts2, luts)
    for i in range(n_views):
        assert torch.equal(out2.rgba[i], refs[i][0]), i
        assert torch.equal(out2.dist[i], refs[i][1]), i
    cap.graph.close()
    b.close()


def test_autotuners(sctx):
    params, renders = W.batched_lut_sets(16)
    sizes = W.plain_lut_sizes(1)
    luts = LutSet.allocate(sizes, 16)
    best, times = B.autotune_luts(sctx, params, renders, 16, sizes, luts, reps=2)
    assert best.transmittance_lanes in (2, 4, 8, 16) and best.view_lanes in (2, 4, 8, 16)
    assert len(times) == 8 and all(t > 0 for t in times)
    assert min(times[:4]) == pytest.approx(times[[2, 4, 8, 16].index(best.transmittance_lanes)])
    assert min(times[4:]) == pytest.approx(times[4 + [2, 4, 8, 16].index(best.view_lanes)])
    got = B.tuning(sctx)
    assert (got.transmittance_lanes, got.view_lanes) == (best.transmittance_lanes, best.view_lanes)
    cl = Clouds(sctx)
    atmo = W.earth_like_atmosphere()
    cam = W.frame_camera()
    l1 = update_lut_set(sctx, atmo, W.render_parameters(cam, 45.0), sizes)
    view = W.frame_view(cam, 45.0, width=640, height=360)
    rgba = torch.empty((360, 640, 4), dtype=torch.float16, device="cuda")
    dist = torch.empty((360, 640), dtype=torch.float32, device="cuda")
    best, times = B.autotune_cloud(sctx, atmo, cl.cloud, cl.material, cl.textures, view, sizes, l1, cl.bn, rgba,
                                   dist, reps=2)
    key = B.cloud_tuning_key(best)
    assert key in B.CLOUD_CANDIDATES and len(times) == len(B.CLOUD_CANDIDATES) == 288
    assert min(times) == pytest.approx(times[B.CLOUD_CANDIDATES.index(key)])


def _mean_rel(got, want):
    return float(np.abs(got - want).sum() / max(np.abs(want).sum(), 1e-300))


def test_batched_subset_matches_oracle(sctx):
    cl = Clouds(sctx)
    params, renders, views, sov, sizes, luts, b = _batched(sctx, n_sets=4, n_views=3, fmt=0)
    b.launch(luts)
    out = B.ViewOutputs(views, 3)
    B.render_views(sctx, params, 4, sov, cl.cloud, cl.material, cl.textures, views, 3, sizes, luts, cl.bn, out)
    sctx.synchronize()
    host = {k: (t.desc, t.data.cpu().numpy()) for k, t in cl.tex.items()}
    rng = np.random.default_rng(3)
    for i in range(3):
        v = views[i]
        npx = v.width * v.height
        px = np.sort(rng.choice(npx, 1500, replace=False)).astype(np.int32)
        s = sov[i]
        rgba, dist = orc.cloud_render(params[s], cl.cloud, cl.material, host, v, sizes,
                                      luts.transmittance[s].cpu().double().numpy(),
                                      luts.aerial_perspective_luminance[s].cpu().double().numpy(),
                                      luts.aerial_perspective_transmittance[s].cpu().double().numpy(),
                                      cl.bn.cpu().numpy(), pixels=px)
        g = out.rgba[i].float().cpu().numpy().reshape(-1, 4)[px].astype(np.float64)
        gd = out.dist[i].cpu().numpy().reshape(-1)[px].astype(np.float64)
        e = (_mean_rel(g[:, :3], rgba[:, :3]), _mean_rel(g[:, 3], rgba[:, 3]), _mean_rel(gd, dist))
        print(f"view {i} {v.width}x{v.height}: luminance {e[0]:.2e} transmittance {e[1]:.2e} distance {e[2]:.2e}")
        assert max(e) <= 1e-3, (i, e)
    b.close()


def test_invalid_arguments(sctx):
    with pytest.raises(_abi.SkyrError):
        B.set_tuning(sctx, transmittance_lanes=5)
    with pytest.raises(_abi.SkyrError):
        B.set_tuning(sctx, view_lanes=1)
    with pytest.raises(_abi.SkyrError):
        B.set_tuning(sctx, cloud_tile_width=64)
    with pytest.raises(_abi.SkyrError):
        B.set_tuning(sctx, cloud_ray_lanes=3)
    with pytest.raises(_abi.SkyrError):
        B.set_tuning(sctx, cloud_ray_lanes=16)
    cl = Clouds(sctx)
    params, renders, views, sov, sizes, luts, b = _batched(sctx, n_sets=2, n_views=2)
    out = B.ViewOutputs(views, 2)
    with pytest.raises(_abi.SkyrError):  # view 1 names LUT set 2 of 2
        B.render_views(sctx, params, 2, [0, 2], cl.cloud, cl.material, cl.textures, views, 2, sizes, luts, cl.bn,
                       out)
    # graph capture on a context bound to the legacy default stream is refused
    legacy = Context(torch.cuda.default_stream())
    assert legacy.stream.cuda_stream == 0
    assert _abi.lib().skyr_graph_begin(legacy.handle) == _abi.SKYR_EINVAL
    legacy.close()
    b.close()
