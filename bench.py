"""Benchmark of the atmosphere-LUT / volumetric-cloud hot path on one GB300.

The timed step (value, e2e) is one plain 1920x1080 frame, one
skyr_render_frame call replayed from a CUDA graph captured once through the
public API (skyr_graph_*):
  * the whole LUT set (transmittance 256x64 / 40 samples, multi-scattering
    32x32 / 64 directions x 20 samples, sky-view 192x108 / 30 samples, aerial
    perspective 32^3 / 40 samples over 32 km), then
  * the per-pixel cloud raymarch (layer 1.5-4.0 km, Material1, 50/km,
    64 primary steps, 6 light-march steps, seeded blue-noise jitter), launched
    as a programmatic dependent of the LUT set's last pass.
The split into the two parts (lut_set_us, cloud_frame_ms) is timed from the
two calls (skyr_update_lut_set, skyr_cloud_render) captured as two graphs.
Noise textures (512^2 RG8 weather map, 128^3 RGBA8 base noise) are generated
once before timing, as the reference regenerates them only when their
parameters change.  Inputs are seeded synthetic (skyrendering_gb300/workloads.py).

The third part of the metric, the surrogate against the path tracer on the
512x640x352 voxel cloud, is measured after the timed frames and reported under
"surrogate" (GPU times at 1024^2, errors at 256^2 against a path-traced
reference, the path tracer's spp and time at the surrogate's error).  The
batched workload (256 parameter sets, 64 views of uneven size, one CUDA graph
with autotuned launch shapes) is reported under "batched", and the cloud
shadow passes (shadow map, blur, shadow froxel) with the shadowed frame under
"shadow".  The reference's production cloud pass (quarter-resolution raymarch,
temporal reconstruction, upscale) and the production frame built on it (LUT
set + shadow passes + quarter pass) are under "quarter".

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  --impl reference times the CPU restatement of the
reference's shader math (the reference itself is GLSL for an OpenGL driver,
which these machines cannot run) on the host cores.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "LUT-set regen µs; 1080p cloud frame ms; surrogate vs path-trace GPU time @2% err"
UNIT = "ms per 1920x1080 frame (LUT set + cloud raymarch)"
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2
SUN_ZENITH = 45.0
# FP32 operations of one density evaluation (SampleSigmaT of Material1 with its
# sample position, VolumetricCloudDefaultMaterial1.glsl:14-29), counted from the
# reference formulas with GL's bilinear filter written out (FMA = 2):
#   sample position 6, CalHeight01 14, GetUVWLod of the cloud map 18, bilinear
#   R 17, coverage / height terms 9                                   -> 64
# Every evaluation runs these.  One that passes the coverage test also runs
# GetUVWLod of the detail texture 18, trilinear R 33 and the detail terms 15
# (66 more); the counted launch reports how many do (DETAIL_FLOPS).
COVERAGE_FLOPS = 64
DETAIL_FLOPS = 66


def cloud_tile(tile_width: int, ray_lanes: int) -> str:
    """The pixel tile of one raymarch warp for a tuning's tile width and lanes per ray."""
    w = min(tile_width, 32 // ray_lanes)
    return f"{w}x{32 // ray_lanes // w}"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=30)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="skyr", choices=["skyr", "reference"])
    ap.add_argument("--cpu-sample-s", type=float, default=12.0)
    ap.add_argument("--no-shadow", action="store_true", help="skip the cloud shadow-pass leg")
    ap.add_argument("--no-quarter", action="store_true", help="skip the quarter-resolution cloud-pass leg")
    ap.add_argument("--no-surrogate", action="store_true",
                    help="leave out the voxel-cloud leg (surrogate vs path tracer) of the metric")
    ap.add_argument("--no-batched", action="store_true",
                    help="leave out the batched 256-set / 64-view graph measurement")
    return ap.parse_args()


def max_over_ranks(value: float, device: str) -> float:
    """The largest of the ranks' values (replicas: the slowest rank sets the step time)."""
    import torch

    t = torch.tensor([value], dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t.item())


def dist_env():
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.file = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.file, stderr=subprocess.DEVNULL)
        except FileNotFoundError:
            self.proc = None
        time.sleep(0.4)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait(timeout=5)

    def summary(self):
        self.file.flush()
        rows = [r.split(",") for r in Path(self.file.name).read_text().splitlines() if r.strip()]
        os.unlink(self.file.name)
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx.append(float(r[2]))
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() in ("active", "1"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


def reference_blue_noise():
    """The reference's 64x64 blue-noise jitter tile (data/BlueNoise/64_64/HDR_L_0.png,
    committed as tests/golden/blue_noise_64x64.npy) as its GL_R16 values / 65535."""
    import numpy as np

    raw = np.load(ROOT / "tests" / "golden" / "blue_noise_64x64.npy")
    return (raw.astype(np.float64) / 65535.0).astype(np.float32)


def ncu_capture(kernel: str) -> dict:
    """The committed ncu figures of one launch of `kernel` (profiles/dram_bytes_per_launch.json)."""
    f = ROOT / "profiles" / "dram_bytes_per_launch.json"
    return json.loads(f.read_text()).get(kernel, {}) if f.exists() else {}


def ncu_traffic(kernel: str):
    """dram__bytes_read.sum + dram__bytes_write.sum of one launch of `kernel`
    from the committed ncu capture (profiles/dram_bytes_per_launch.json)."""
    f = ROOT / "profiles" / "dram_bytes_per_launch.json"
    if f.exists():
        e = json.loads(f.read_text()).get(kernel)
        return None if e is None else e.get("bytes")
    return None


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
class FrameState:
    def __init__(self, ctx):
        import torch

        from skyrendering_gb300 import workloads as W
        from skyrendering_gb300.atmosphere import LutSet
        from skyrendering_gb300.cloud import NoiseTexture, VolumetricCloud, prepare_textures, textures_struct

        self.W = W
        self.ctx = ctx
        self.atmo = W.earth_like_atmosphere()
        self.sizes = W.plain_lut_sizes()
        self.cam = W.frame_camera()
        self.render = W.render_parameters(self.cam, SUN_ZENITH)
        self.luts = LutSet.allocate(self.sizes, 1)
        self.tex = {"cloud_map": NoiseTexture(W.cloud_map_desc()).generate(ctx),
                    "detail": NoiseTexture(W.base_noise_desc()).generate(ctx)}
        self.material = W.frame_material()
        prepare_textures(ctx, self.material.type, self.tex)
        self.bn_host = torch.from_numpy(reference_blue_noise()).pin_memory()
        self.bn = self.bn_host.cuda()
        self.view = W.frame_view(self.cam, SUN_ZENITH)
        self.vc = VolumetricCloud(ctx, W.frame_cloud_parameters(), self.material, textures_struct(**self.tex))
        h, w = self.view.height, self.view.width
        self.rgba = torch.empty((h, w, 4), dtype=torch.float16, device="cuda")
        self.dist = torch.empty((h, w), dtype=torch.float32, device="cuda")

    def luts_step(self):
        from skyrendering_gb300.atmosphere import update_lut_set

        update_lut_set(self.ctx, self.atmo, self.render, self.sizes, self.luts)

    def cloud_step(self):
        self.vc.render(self.atmo, self.view, self.sizes, self.luts, self.bn, out_rgba=self.rgba,
                       out_distance=self.dist)

    def frame_step(self, out_rgba=None, out_distance=None, on_host=False):
        """The LUT set and the raymarch in one call (skyr_render_frame)."""
        self.vc.render_frame(self.atmo, self.render, self.view, self.sizes, self.luts, self.bn,
                             out_rgba=self.rgba if out_rgba is None else out_rgba,
                             out_distance=self.dist if out_distance is None else out_distance, on_host=on_host)


def surrogate_vs_pathtracer(ctx, small: int = 256, ref_spp: int = 16384, big: int = 1024):
    """The voxel-cloud leg of the metric: GPU time of the surrogate-shaded image
    against the plain path tracer at equal error.

    * times (CUDA events, on the context's stream): the surrogate raymarch at
      big x big, the feature lattice it needs, one path-traced frame at big x big
      (a 16-frame call / 16);
    * errors at small x small against a 2 x ref_spp path-traced reference:
      surrogate, single scattering only (no network), and the path tracer at
      64 / 256 / 1024 spp; the spp at which the path tracer reaches the
      surrogate's error is interpolated in log-log between those points;
    * the reference's own noise: the relative L1 between its two halves, and
      half of that as an estimate of the noise of their mean (which every
      error above includes).
    """
    import math

    import torch

    from skyrendering_gb300 import surrogate as S
    from skyrendering_gb300 import surrogate_train as T
    from skyrendering_gb300.pathtrace import PathTracer

    model = S.load_model(S.MODEL_PATH)
    net = model.packed(ctx)
    table = torch.from_numpy(model.error_table).cuda()
    stream = ctx.stream
    ev = lambda: torch.cuda.Event(enable_timing=True)

    def timed(fn, reps=5):
        fn()
        e0, e1 = ev(), ev()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    out = {"image": f"{big}x{big}", "grid": "512x640x352 FP16, max extinction 40/km, 16^3 brick majorants",
           "network": "103-64-64-64-64-3 BF16 (the 43 configured inputs, the view ray's far-side transmittance, a "
                      "35-point sun-oriented density stencil from the grid's mip levels 2-6 and a 24-point "
                      "view-oriented one from levels 3-6), 128-step raymarch",
           "target_rel_l1": 0.02}
    sc = T.Scene(ctx, size=big)
    grid = sc.grid(0x5EED)
    fv = sc.lattice(grid)
    sp = S.parameters(error_table=table)
    out["lattice_ms"] = timed(lambda: sc.lattice(grid), reps=3)
    out["surrogate_ms"] = timed(lambda: S.render(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.sizes, sc.luts,
                                                 fv, net, sp))
    tr = PathTracer(ctx, sc.pt, sc.cloud, sc.view, sc.env, sc.sizes, grid=grid)
    out["pt_ms_per_spp"] = timed(lambda: tr.render(sc.atmo, sc.luts, 16), reps=2) / 16.0
    del tr, fv
    # errors at the small size
    sm = T.Scene(ctx, size=small)
    fvs = sm.lattice(grid)
    sur, _ = S.render(ctx, sm.atmo, sm.cloud, grid, sm.pt, sm.view, sm.sizes, sm.luts, fvs, net, sp)
    ss, _ = S.render(ctx, sm.atmo, sm.cloud, grid, sm.pt, sm.view, sm.sizes, sm.luts, fvs, None,
                     S.parameters(use_network=0))

    def pt_image(frames, begin):
        t = PathTracer(ctx, sm.pt, sm.cloud, sm.view, sm.env, sm.sizes, grid=grid)
        t.frames = begin
        t.render(sm.atmo, sm.luts, frames)
        return t.acc / frames

    half_a, half_b = pt_image(ref_spp, 1000000), pt_image(ref_spp, 2000000)
    ref = (half_a + half_b) / 2
    out["reference"] = f"{small}x{small}, 2 x {ref_spp} spp"
    out["reference_halves_rel_l1"] = halves = S.relative_l1(half_a, half_b)
    out["reference_noise_rel_l1_estimate"] = 0.5 * halves
    del half_a, half_b
    out["rel_l1_surrogate"] = e_s = S.relative_l1(sur, ref)
    out["rel_l1_single_scattering_only"] = S.relative_l1(ss, ref)
    pts = [(n, S.relative_l1(pt_image(n, 3000000 + n), ref)) for n in (64, 256, 1024)]
    out["rel_l1_pt"] = {str(n): e for n, e in pts}
    # log-log interpolation (or extrapolation from the last two points)
    (n0, e0), (n1, e1) = (pts[-2], pts[-1]) if e_s < pts[1][1] else (pts[0], pts[1])
    slope = math.log(e1 / e0) / math.log(n1 / n0)
    spp = n0 * math.exp(math.log(e_s / e0) / slope) if slope < 0 else float("nan")
    out["pt_spp_for_equal_error"] = spp
    out["pt_ms_equal_error"] = spp * out["pt_ms_per_spp"]
    surrogate_total = out["surrogate_ms"] + out["lattice_ms"]
    out["speedup_equal_error"] = out["pt_ms_equal_error"] / surrogate_total
    out["speedup_equal_error_static_lattice"] = out["pt_ms_equal_error"] / out["surrogate_ms"]
    out["meets_target"] = bool(e_s <= 0.02 and out["speedup_equal_error"] >= 20.0)
    ctx.check_status()
    return out


def batched_frames(ctx, reps: int = 5, n_sets: int = 256, n_views: int = 64):
    """The batched workload (256 perturbed parameter sets, 64 views of uneven
    size) as one CUDA graph: the prepared LUT batch (FP16 storage) followed by
    the 64 raymarches fanned out over the context's streams.  Launch shapes are
    picked by the autotuners first (LUT passes on the batch, raymarch on a
    1920x1080 view of it)."""
    import torch

    from skyrendering_gb300 import batch as B
    from skyrendering_gb300 import workloads as W
    from skyrendering_gb300.atmosphere import LutSet
    from skyrendering_gb300.cloud import NoiseTexture, prepare_textures, textures_struct

    stream = ctx.stream
    params, renders, views, sov = W.batched_frame(n_sets, n_views)
    sizes = W.plain_lut_sizes(1)
    cloud, material = W.frame_cloud_parameters(), W.frame_material()
    tex = {"cloud_map": NoiseTexture(W.cloud_map_desc()).generate(ctx),
           "detail": NoiseTexture(W.base_noise_desc()).generate(ctx)}
    prepare_textures(ctx, material.type, tex)
    textures = textures_struct(**tex)
    bn = torch.from_numpy(reference_blue_noise()).cuda()
    luts = LutSet.allocate(sizes, n_sets)
    lut_best, lut_times = B.autotune_luts(ctx, params, renders, n_sets, sizes, luts, reps=3)
    k = next(i for i in range(n_views) if views[i].width == 1920) if any(
        views[i].width == 1920 for i in range(n_views)) else 0
    probe_rgba = torch.empty((views[k].height, views[k].width, 4), dtype=torch.float16, device="cuda")
    probe_dist = torch.empty((views[k].height, views[k].width), dtype=torch.float32, device="cuda")
    one = LutSet(luts.transmittance[sov[k]:sov[k] + 1], luts.multiscattering[sov[k]:sov[k] + 1],
                 luts.sky_view_luminance[sov[k]:sov[k] + 1], luts.sky_view_transmittance[sov[k]:sov[k] + 1],
                 luts.aerial_perspective_luminance[sov[k]:sov[k] + 1],
                 luts.aerial_perspective_transmittance[sov[k]:sov[k] + 1])
    cloud_best, cloud_times = B.autotune_cloud(ctx, params[sov[k]], cloud, material, textures, views[k], sizes, one,
                                               bn, probe_rgba, probe_dist, reps=3)
    del probe_rgba, probe_dist
    lb = B.LutBatch(ctx, params, renders, n_sets, sizes)
    out = B.ViewOutputs(views, n_views)
    with B.capture(ctx) as lut_cap:
        lb.launch(luts)
    with B.capture(ctx) as cap:
        lb.launch(luts)
        B.render_views(ctx, params, n_sets, sov, cloud, material, textures, views, n_views, sizes, luts, bn, out)

    def timed(g):
        for _ in range(3):
            g.launch()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            g.launch()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    lut_ms = timed(lut_cap.graph)
    graph_ms = timed(cap.graph)
    ctx.check_status()
    px = out.pixels
    res = {"sets": n_sets, "views": n_views, "view_pixels": px, "lut_storage": "RGBA16F",
           "graph_ms": graph_ms, "lut_batch_ms": lut_ms, "lut_us_per_set": lut_ms * 1000.0 / n_sets,
           "raymarch_ms": graph_ms - lut_ms, "raymarch_gpix_per_s": px / ((graph_ms - lut_ms) * 1e-3) / 1e9,
           "graph_launches": 1, "kernels_per_graph": 3 + n_views,
           "tuning": {"transmittance_lanes": lut_best.transmittance_lanes, "view_lanes": lut_best.view_lanes,
                      "cloud_tile_width": cloud_best.cloud_tile_width,
                      "cloud_block_warps_x": cloud_best.cloud_block_warps_x,
                      "cloud_blocks_per_sm": cloud_best.cloud_blocks_per_sm,
                      "cloud_ray_lanes": cloud_best.cloud_ray_lanes},
           "autotune_lut_ms": {"transmittance_lanes_2_4_8_16": lut_times[:4], "view_lanes_2_4_8_16": lut_times[4:]},
           "autotune_cloud_ms": {f"{cloud_tile(w, g)}/{bx}/{occ}/{g}": t
                                 for (w, bx, occ, g), t in zip(B.CLOUD_CANDIDATES, cloud_times)}}
    cap.graph.close()
    lut_cap.graph.close()
    lb.close()
    return res


def shadow_passes(ctx, fs, lut_graph, reps: int = 20, cpu: bool = True):
    """The cloud shadow passes of a 1920x1080 frame (VolumetricCloud::RenderShadow:
    512^2 (depth, T) map blended into the previous frame's, 9-tap separable
    blur, 160x90x128 R16 shadow froxel) on the frame workload: each pass timed
    alone (CUDA events, back-to-back launches), the three as one CUDA graph,
    and the shadowed frame -- LUT set + shadow passes + the raymarch reading
    the froxel -- with L2 flushed between frames.  The FP64 oracle's time for
    the same passes on the host cores (sampled map texels, scaled) is beside it."""
    import ctypes as C

    import torch

    from skyrendering_gb300 import _abi
    from skyrendering_gb300 import batch as B
    from skyrendering_gb300 import cloud as CL
    from skyrendering_gb300.atmosphere import _ptr

    stream = ctx.stream
    sizes = CL.shadow_sizes(1920, 1080)
    sh = CL.CloudShadow(ctx, sizes)
    sh.render(fs.vc, fs.atmo, fs.view, fs.bn)  # the first frame: nothing to blend into
    view = _abi.CloudView.from_buffer_copy(fs.view)
    view.frame_id = 1.0
    wind = (0.01, 0.0)
    frame = CL.light_frame(fs.atmo, fs.vc.params, view, sizes, previous=sh.frame, wind_delta=wind)
    prev, cur = sh.raw[sh.current], sh.raw[1 - sh.current]
    base = (ctx.handle, C.byref(fs.atmo), C.byref(fs.vc.params), C.byref(fs.vc.material), C.byref(fs.vc.textures),
            C.byref(view), C.byref(sizes), C.byref(frame), _ptr(fs.bn), _ptr(prev), _ptr(cur))

    def launch(stage):  # 1: the map, 2: + blur, 3: + froxel
        _abi.call("skyr_cloud_shadow_render", *base, _ptr(sh.map) if stage >= 2 else None,
                  _ptr(sh.froxel) if stage >= 3 else None)

    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    t_map = timed(lambda: launch(1))
    t_map_blur = timed(lambda: launch(2))
    t_all = timed(lambda: launch(3))
    with B.capture(ctx) as cap:
        launch(3)
    shadow_graph = cap.graph
    t_graph = timed(shadow_graph.launch)
    fview = sh.attach(_abi.CloudView.from_buffer_copy(fs.view))
    with B.capture(ctx) as ccap:
        fs.vc.render(fs.atmo, fview, fs.sizes, fs.luts, fs.bn, out_rgba=fs.rgba, out_distance=fs.dist)
    cloud_graph = ccap.graph
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(4)] for _ in range(reps)]
    for _ in range(3):
        lut_graph.launch()
        shadow_graph.launch()
        cloud_graph.launch()
    torch.cuda.synchronize()
    for i in range(reps):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        lut_graph.launch()
        ev[i][1].record(stream)
        shadow_graph.launch()
        ev[i][2].record(stream)
        cloud_graph.launch()
        ev[i][3].record(stream)
    torch.cuda.synchronize()
    ctx.check_status()
    frame_ms = statistics.mean(a.elapsed_time(d) for a, _, _, d in ev)
    shadow_in_frame = statistics.mean(b.elapsed_time(c) for _, b, c, _ in ev)
    cloud_in_frame = statistics.mean(c.elapsed_time(d) for _, _, c, d in ev)
    mw, mh = sizes.map_width, sizes.map_height
    fw, fh, fd = sizes.froxel_width, sizes.froxel_height, sizes.froxel_depth
    sun_z = math.cos(math.radians(SUN_ZENITH))
    steps = int(12.0 - 6.0 * sun_z)  # light-ray samples per map texel (the sun's local z ~ cos(zenith))
    blur_ms = t_map_blur - t_map
    froxel_ms = t_all - t_map_blur
    res = {"map": f"{mw}x{mh} float2, temporal blend", "froxel": f"{fw}x{fh}x{fd} unorm16",
           "map_ms": t_map, "blur_ms": blur_ms, "froxel_ms": froxel_ms, "passes_ms": t_all,
           "passes_graph_ms": t_graph,
           "map_density_evaluations": mw * mh * steps,
           "map_density_evaluations_per_s": mw * mh * steps / (t_map * 1e-3),
           "blur_bytes": 2 * mw * mh * 8, "blur_gb_per_s": 2 * mw * mh * 8 / max(blur_ms * 1e-3, 1e-9) / 1e9,
           "froxel_bytes": mw * mh * 8 + fw * fh * fd * 2,
           "froxel_gb_per_s": (mw * mh * 8 + fw * fh * fd * 2) / max(froxel_ms * 1e-3, 1e-9) / 1e9,
           "shadowed_frame_ms": frame_ms, "shadow_in_frame_ms": shadow_in_frame,
           "raymarch_with_froxel_ms": cloud_in_frame,
           "note": "per-pass times are differences of back-to-back launches (map; map+blur; all three); "
                   "the shadowed frame replays three graphs with L2 flushed between frames"}
    if cpu:
        import numpy as np

        from oracle import oracle as orc

        host = {k: (t.desc, t.data.cpu().numpy()) for k, t in fs.tex.items()}
        fa = orc.frame_array(frame)
        threads = os.cpu_count() or 1
        texels = np.arange(0, mw * mh, 64, dtype=np.int32)
        t0 = time.perf_counter()
        orc.shadow_map(fs.atmo, fs.vc.params, fs.vc.material, host, view, mw, mh, fa, True, fs.bn.cpu().numpy(),
                       previous_map=prev.cpu().numpy(), texels=texels, nthreads=threads)
        t_map_cpu = (time.perf_counter() - t0) * (mw * mh) / len(texels)
        smap = sh.map.cpu().numpy()
        t0 = time.perf_counter()
        orc.shadow_blur(cur.cpu().numpy())
        t_blur_cpu = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.shadow_froxel(fs.atmo, fs.vc.params, fs.vc.material, host, view, fa, smap, (fw, fh, fd),
                          nthreads=threads)
        t_fx_cpu = time.perf_counter() - t0
        res["cpu_oracle"] = {"passes_ms": (t_map_cpu + t_blur_cpu + t_fx_cpu) * 1e3, "map_ms": t_map_cpu * 1e3,
                             "blur_ms": t_blur_cpu * 1e3, "froxel_ms": t_fx_cpu * 1e3, "cores": threads,
                             "kind": "port", "precision": "f64",
                             "sample": f"{len(texels)} of {mw * mh} map texels scaled; full blur and froxel"}
    shadow_graph.close()
    cloud_graph.close()
    return res


def quarter_pass(ctx, fs, lut_graph, reps: int = 20):
    """The reference's production cloud pass at 1920x1080 (VolumetricCloud::Render):
    checkerboard depth, index, the raymarch of 480x270 checkerboard texels,
    the temporal reconstruction at 960x540 and the upscale composited into an
    RGBA16F HDR target, on an empty depth buffer in steady state (the previous
    frame's reconstruction as history).  Timed as one CUDA graph with and
    without the upscale, and inside the production frame: LUT set +
    environment cube + shadow passes + quarter pass reading the shadow froxel,
    L2 flushed between frames."""
    import ctypes as C

    import torch

    from skyrendering_gb300 import _abi
    from skyrendering_gb300 import batch as B
    from skyrendering_gb300 import cloud as CL
    from skyrendering_gb300.atmosphere import _ptr

    stream = ctx.stream
    W_, H_ = fs.view.width, fs.view.height
    zn, zf = fs.cam.z_near, fs.cam.z_far
    frame_tuning = B.tuning(ctx)
    vp = CL.CloudViewport(ctx, W_, H_)
    hdr = torch.zeros((H_, W_, 4), dtype=torch.float16, device="cuda")
    vp.render(fs.vc, fs.atmo, fs.view, fs.sizes, fs.luts, fs.bn, hdr=hdr, z_near=zn, z_far=zf)
    # the quarter pass's raymarch has 1/16 of the rays: its own launch shape, autotuned on the
    # pass itself and kept in the context while its graphs are captured
    q_tuned, _ = vp.autotune(fs.vc, fs.atmo, fs.view, fs.sizes, fs.luts, fs.bn, z_near=zn, z_far=zf, reps=5)
    sh = CL.CloudShadow(ctx, CL.shadow_sizes(W_, H_))
    sh.render(fs.vc, fs.atmo, fs.view, fs.bn)
    view = _abi.CloudView.from_buffer_copy(fs.view)
    view.frame_id = 1.0
    frame = CL.temporal_frame(fs.atmo, view, vp.previous_view, None, zn, zf, 1)
    b = vp.buffers(history=True)
    L = fs.luts

    def call(v, out_hdr):
        _abi.call("skyr_cloud_render_quarter", ctx.handle, C.byref(fs.atmo), C.byref(fs.vc.params),
                  C.byref(fs.vc.material), C.byref(fs.vc.textures), C.byref(v), C.byref(fs.sizes),
                  _ptr(L.transmittance), _ptr(L.aerial_perspective_luminance),
                  _ptr(L.aerial_perspective_transmittance), _ptr(fs.bn), None, C.byref(frame), C.byref(b),
                  _ptr(out_hdr))

    with B.capture(ctx) as cap:
        call(view, hdr)
    full = cap.graph
    with B.capture(ctx) as cap:
        call(view, None)
    no_upscale = cap.graph
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(g):
        for _ in range(3):
            g.launch()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(reps):
            g.launch()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    t_full, t_no_up = timed(full), timed(no_upscale)
    # the production frame: LUT set, shadow passes, quarter pass reading the froxel
    shadow_frame = CL.light_frame(fs.atmo, fs.vc.params, view, sh.sizes, previous=sh.frame)
    prev, cur = sh.raw[sh.current], sh.raw[1 - sh.current]
    with B.capture(ctx) as cap:
        _abi.call("skyr_cloud_shadow_render", ctx.handle, C.byref(fs.atmo), C.byref(fs.vc.params),
                  C.byref(fs.vc.material), C.byref(fs.vc.textures), C.byref(view), C.byref(sh.sizes),
                  C.byref(shadow_frame), _ptr(fs.bn), _ptr(prev), _ptr(cur), _ptr(sh.map), _ptr(sh.froxel))
    shadow_graph = cap.graph
    # AtmosphereRenderer::Render's environment cube (128^2 x 6 RGBA16F + mips) and IBL::Precompute (SH,
    # 5 prefiltered roughness levels), every frame in the reference
    from skyrendering_gb300.atmosphere import (environment_cube, environment_prefilter, environment_seamless,
                                               environment_sh)

    env_out = torch.empty((_abi.lib().skyr_environment_cube_level_offset(128, 8), 4), dtype=torch.float16,
                          device="cuda")
    env_seam = torch.empty((_abi.lib().skyr_environment_seamless_level_offset(128, 8), 4), dtype=torch.float32,
                           device="cuda")
    env_sh = torch.empty((9, 4), dtype=torch.float32, device="cuda")
    env_pre = torch.empty((_abi.lib().skyr_environment_cube_level_offset(128, 5), 4), dtype=torch.float16,
                          device="cuda")
    with B.capture(ctx) as cap:
        environment_cube(ctx, fs.atmo, fs.render, fs.sizes, fs.luts, 128, out=env_out)
        environment_seamless(ctx, env_out, 128, 8, out=env_seam)
        environment_sh(ctx, env_seam, 128, 8, out=env_sh)
        environment_prefilter(ctx, env_seam, 128, 8, 128, 5, out=env_pre)
    env_graph = cap.graph
    t_env = timed(env_graph)
    fview = sh.attach(_abi.CloudView.from_buffer_copy(view))
    with B.capture(ctx) as cap:
        call(fview, hdr)
    quarter_graph = cap.graph
    _abi.call("skyr_ctx_set_tuning", ctx.handle, C.byref(frame_tuning))
    # AtmosphereRenderer's full-screen composite (reference defaults: per-pixel raymarch, 40 dithered samples;
    # seeded star map; the cloud shadow froxel) into the HDR target the cloud upscale composites onto
    from skyrendering_gb300.atmosphere import composite, composite_parameters

    stars = torch.from_numpy(fs.W.star_map()).cuda()
    cp = composite_parameters()
    with B.capture(ctx) as cap:
        composite(ctx, fs.atmo, fs.render, cp, fs.sizes, fs.luts, W_, H_, blue_noise=fs.bn, star_map=stars,
                  shadow_froxel=sh.froxel, shadow_froxel_max_distance=fs.vc.params.shadow_froxel_max_distance,
                  out=hdr)
    composite_graph = cap.graph
    t_composite = timed(composite_graph)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    order = [("lut_set", lut_graph), ("shadow_passes", shadow_graph), ("environment_cube_and_ibl", env_graph),
             ("atmosphere_composite", composite_graph), ("quarter_cloud_pass", quarter_graph)]
    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(len(order) + 1)] for _ in range(reps)]
    for _ in range(3):
        for _, g in order:
            g.launch()
    torch.cuda.synchronize()
    for i in range(reps):
        flush.fill_(float(i))
        ev[i][0].record(stream)
        for k, (_, g) in enumerate(order):
            g.launch()
            ev[i][k + 1].record(stream)
    torch.cuda.synchronize()
    ctx.check_status()
    res = {"viewport": f"{W_}x{H_}", "raymarch": f"{W_ // 4}x{H_ // 4} checkerboard texels",
           "reconstruct": f"{W_ // 2}x{H_ // 2}", "depth": "empty (1)", "history": "previous reconstruction",
           "pass_ms": t_full, "pass_without_upscale_ms": t_no_up, "upscale_ms": t_full - t_no_up,
           "environment_and_ibl_us": t_env * 1000.0, "atmosphere_composite_ms": t_composite,
           "production_frame_ms": statistics.mean(e[0].elapsed_time(e[-1]) for e in ev),
           "production_frame_parts_ms": {
               name: statistics.mean(e[k].elapsed_time(e[k + 1]) for e in ev) for k, (name, _) in enumerate(order)},
           "kernels_per_pass": 5,
           "raymarch_tuning": {"tile": cloud_tile(q_tuned.cloud_tile_width, q_tuned.cloud_ray_lanes),
                               "block_warps_x": q_tuned.cloud_block_warps_x,
                               "blocks_per_sm": q_tuned.cloud_blocks_per_sm,
                               "ray_lanes": q_tuned.cloud_ray_lanes},
           "note": "production frame = the reference's per-frame GPU work of the sky and clouds, in its order: LUT "
                   "set, cloud shadow passes, environment cube (128^2 x 6 + mips, SH, 5 prefiltered levels), "
                   "full-screen atmosphere composite (per-pixel raymarch), quarter-resolution cloud pass with the "
                   "froxel composited onto it; five CUDA graphs, L2 flushed between frames"}
    for g in (full, no_upscale, shadow_graph, quarter_graph, env_graph, composite_graph):
        g.close()
    return res


def run_skyr(args):
    import ctypes as C

    import torch

    from skyrendering_gb300 import _abi
    from skyrendering_gb300.atmosphere import Context, _ptr

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = Context(stream)
    fs = FrameState(ctx)
    # launch shapes from the autotuners, on this frame's own workload (setup, untimed)
    from skyrendering_gb300 import batch as B

    lut_tuned, _ = B.autotune_luts(ctx, fs.atmo, fs.render, 1, fs.sizes, fs.luts, reps=5)
    cloud_tuned, _ = B.autotune_cloud(ctx, fs.atmo, fs.vc.params, fs.vc.material, fs.vc.textures, fs.view, fs.sizes,
                                      fs.luts, fs.bn, fs.rgba, fs.dist, reps=5)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    kernels_per_step = 4  # transmittance, multi-scattering, sky-view + AP, cloud raymarch (in 2 graphs)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(max(args.warmup, 3)):
        fs.luts_step()
        fs.cloud_step()
    barrier()
    # the production form of the step: one skyr_render_frame call (the LUT set,
    # then the raymarch as a programmatic dependent of its last pass) captured
    # once into a CUDA graph (skyr_graph_*), replayed every frame.  The two parts
    # captured as two graphs (skyr_update_lut_set, skyr_cloud_render) give the
    # per-component split.
    with B.capture(ctx) as frame_cap:
        fs.frame_step()
    with B.capture(ctx) as lut_cap:
        fs.luts_step()
    with B.capture(ctx) as cloud_cap:
        fs.cloud_step()
    frame_graph, lut_graph, cloud_graph = frame_cap.graph, lut_cap.graph, cloud_cap.graph
    for _ in range(3):
        frame_graph.launch()
        lut_graph.launch()
        cloud_graph.launch()
    barrier()

    ev = [[torch.cuda.Event(enable_timing=True) for _ in range(2)] for _ in range(args.steps)]
    split_ev = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))  # evict L2 between steps (outside the timed interval)
            ev[i][0].record(stream)
            frame_graph.launch()
            ev[i][1].record(stream)
        barrier()
        wall = time.perf_counter() - wall0
        # the split: the same step as two graph launches with an event between them
        for i in range(args.steps):
            flush.fill_(float(i))
            split_ev[i][0].record(stream)
            lut_graph.launch()
            split_ev[i][1].record(stream)
            cloud_graph.launch()
            split_ev[i][2].record(stream)
        barrier()
        # e2e through the public API with host buffers: the blue-noise tile
        # H2D from pinned memory (parameter blocks travel by value in the
        # launches), then skyr_render_frame with the frame's two outputs in
        # pinned host memory: its raymarch stores every pixel into the mapped
        # host buffers, so the D2H bytes move while the kernel runs.  The whole
        # step is one CUDA graph (the copy a memcpy node).
        host_rgba = torch.empty(fs.rgba.shape, dtype=fs.rgba.dtype, pin_memory=True)
        host_dist = torch.empty(fs.dist.shape, dtype=fs.dist.dtype, pin_memory=True)

        def e2e_body():
            fs.bn.copy_(fs.bn_host, non_blocking=True)
            fs.frame_step(out_rgba=host_rgba, out_distance=host_dist, on_host=True)

        try:
            with B.capture(ctx) as e2e_cap:
                e2e_body()
            e2e_graph = e2e_cap.graph
            e2e_step, e2e_form = e2e_graph.launch, "one CUDA graph"
        except Exception as exc:  # capture refused: the same calls, launched directly
            print(f"bench: e2e graph capture failed ({exc}); launching directly", file=sys.stderr)
            e2e_graph, e2e_step, e2e_form = None, e2e_body, "direct launches"

        for _ in range(3):
            e2e_step()
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            e2e_step()
        e1.record(stream)
        barrier()
    e2e_ms = e0.elapsed_time(e1) / args.steps
    lut_ms = [a.elapsed_time(b) for a, b, _ in split_ev]
    cloud_ms = [b.elapsed_time(c) for _, b, c in split_ev]
    frame_ms = [a.elapsed_time(b) for a, b in ev]
    ms = statistics.mean(frame_ms)
    if world > 1:
        ms = max_over_ranks(ms, "cuda")

    # work counters of one frame (instrumented launch, outside the timing):
    # raymarch samples, density evaluations, evaluations past the coverage test
    counters = torch.zeros(3, dtype=torch.int64, device="cuda")
    L = fs.luts
    _abi.call("skyr_cloud_render_counted", ctx.handle, C.byref(fs.atmo), C.byref(fs.vc.params),
              C.byref(fs.vc.material), C.byref(fs.vc.textures), C.byref(fs.view), C.byref(fs.sizes),
              _ptr(L.transmittance), _ptr(L.aerial_perspective_luminance), _ptr(L.aerial_perspective_transmittance),
              _ptr(fs.bn), None, _ptr(fs.rgba), _ptr(fs.dist), _ptr(counters))
    torch.cuda.synchronize()
    samples, evals, detail_evals = (int(x) for x in counters.cpu())
    # the frame the e2e steps left in host memory is the device frame of the timed
    # launch shape, bit for bit (the counted launch above ran its own instance)
    cloud_graph.launch()
    torch.cuda.synchronize()
    e2e_matches = bool(torch.equal(host_rgba.view(torch.int16), fs.rgba.cpu().view(torch.int16)) and
                       torch.equal(host_dist.view(torch.int32), fs.dist.cpu().view(torch.int32)))
    if e2e_graph is not None:
        e2e_graph.close()

    clocks = clk.summary()
    hbm_peak, peak_kind = peaks()
    npx = fs.view.width * fs.view.height
    # algorithmic bytes of one raymarch launch: the outputs (8 B RGBA16F + 4 B
    # R32F per pixel) plus one read of every input it samples (weather map
    # level 0 RG, base noise level 0 R, the transmittance LUT, both AP volumes)
    tex_bytes = 512 * 512 * 2 + 128 ** 3 * 1
    lut_bytes = 256 * 64 * 16 + 2 * 32 ** 3 * 16
    alg_bytes = npx * 12 + tex_bytes + lut_bytes
    cloud_mean = statistics.mean(cloud_ms)
    achieved = alg_bytes / (cloud_mean * 1e-3) / 1e9
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    fp32_peak = sms * 128 * 2 * sm_mhz * 1e6 / 1e12  # TFLOP/s: FP32 lanes x FMA x sampled clock
    flops = evals * COVERAGE_FLOPS + detail_evals * DETAIL_FLOPS
    fp32_achieved = flops / (cloud_mean * 1e-3) / 1e12
    result = {
        "metric": METRIC,
        "value": ms,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded Earth-like atmosphere and Perlin-Worley cloud textures, 1 km camera, "
                "60 deg FOV, sun zenith 45 deg, seeded 64x64 blue noise)",
        "config": {"workload": "plain 1920x1080 frame: LUT set (T 256x64x40, MS 32x32x64x20, SV 192x108x30, "
                               "AP 32^3x40 over 32 km) + per-pixel cloud raymarch (layer 1.5-4.0 km, "
                               "Material1 50/km, 64 steps, 6 light steps)",
                   "l2": "flushed between timed steps (512 MB write outside the timed interval)",
                   "parallelism": f"replicas x{world}",
                   "launch": "one CUDA graph per step (skyr_render_frame: LUT set + raymarch, the raymarch a "
                             "programmatic dependent of the LUT set's last pass), captured once; lut_set_us and "
                             "cloud_frame_ms from the two parts captured as two graphs (skyr_update_lut_set, "
                             "skyr_cloud_render), timed in a second loop of as many steps with an event between "
                             "the launches",
                   "tuning": {"transmittance_lanes": lut_tuned.transmittance_lanes,
                              "view_lanes": lut_tuned.view_lanes,
                              "cloud_tile": cloud_tile(cloud_tuned.cloud_tile_width, cloud_tuned.cloud_ray_lanes),
                              "cloud_block_warps_x": cloud_tuned.cloud_block_warps_x,
                              "cloud_blocks_per_sm": cloud_tuned.cloud_blocks_per_sm,
                              "cloud_ray_lanes": cloud_tuned.cloud_ray_lanes}},
        "lut_set_us": statistics.mean(lut_ms) * 1000.0,
        "cloud_frame_ms": cloud_mean,
        "components": {"lut_set_us": statistics.mean(lut_ms) * 1000.0, "cloud_frame_ms": cloud_mean,
                       "two_graph_frame_ms": statistics.mean(a.elapsed_time(c) for a, _, c in split_ev),
                       "raymarch_samples": samples, "density_evaluations": evals,
                       "density_evaluations_past_coverage": detail_evals,
                       "density_evaluations_per_s": evals / (cloud_mean * 1e-3)},
        "e2e": {"value": e2e_ms, "unit": UNIT, "h2d_bytes_per_step": fs.bn_host.numel() * 4,
                "d2h_bytes_per_step": host_rgba.numel() * 2 + host_dist.numel() * 4,
                "path": f"{e2e_form} per step: blue-noise tile H2D (pinned) + skyr_render_frame with host "
                        "outputs (LUT set, then the raymarch as a programmatic dependent of its last pass, storing "
                        "the frame into mapped pinned host buffers while it runs)",
                "matches_device_frame": e2e_matches},
        "gpu_launches": kernels_per_step * args.steps,
        "roofline": {"kernel": "cloud_render_kernel", "bound": "fp32", "achieved": fp32_achieved,
                     "peak": fp32_peak, "unit": "TFLOP/s", "frac": fp32_achieved / fp32_peak,
                     "peak_kind": f"nominal: {sms} SMs (queried) x 128 FP32 lanes x 2 x median sampled SM clock",
                     "traffic": ncu_traffic("cloud_render_kernel"),
                     "algorithmic_flops_per_launch": flops,
                     "flops_per_evaluation": {"coverage": COVERAGE_FLOPS, "past_coverage": DETAIL_FLOPS},
                     "note": "algorithmic FP32 FLOPs of the counted density evaluations of one frame (reference "
                             "formulas, texture filters written out) over the launch's CUDA-event time"},
        "roofline_hbm": {"kernel": "cloud_render_kernel", "bound": "hbm", "achieved": achieved,
                         "peak": hbm_peak, "unit": "GB/s", "frac": achieved / hbm_peak, "peak_kind": peak_kind,
                         "algorithmic_bytes_per_launch": alg_bytes,
                         "note": "compulsory bytes; the textures are read from L1 / L2, so HBM is not the bound"},
        "roofline_issue": roofline_issue(cloud_mean, sm_mhz, cloud_tuned, sms),
        "clocks": clocks,
        "wall_s": wall,
    }
    if not args.no_shadow:
        result["shadow"] = shadow_passes(ctx, fs, lut_graph, cpu=(rank == 0 and world == 1))
    if not args.no_quarter:
        result["quarter"] = quarter_pass(ctx, fs, lut_graph)
    if not args.no_surrogate:
        result["surrogate"] = surrogate_vs_pathtracer(ctx)
    if not args.no_batched:
        result["batched"] = batched_frames(ctx)
    if rank == 0:
        if world == 1:
            result["cpu_baseline"] = cpu_baseline(args.cpu_sample_s)
        print(json.dumps(result))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# CPU baseline / reference arm: the FP32 restatement of the shader math
# (oracle/, test infrastructure; timed, never shipped) on the host cores, on a
# bounded sample scaled to a full frame.
# ---------------------------------------------------------------------------
_HOST_TEXTURES = {}


def cpu_frame_ms(sample_s: float, threads: int):
    import numpy as np

    from oracle import oracle as orc
    from skyrendering_gb300 import workloads as W

    atmo, sizes, cam = W.earth_like_atmosphere(), W.plain_lut_sizes(), W.frame_camera()
    render = W.render_parameters(cam, SUN_ZENITH)
    t0 = time.perf_counter()
    luts = orc.lut_set(atmo, render, sizes, 32, nthreads=threads)
    lut_s = time.perf_counter() - t0
    if not _HOST_TEXTURES:  # generated once, like the GPU arm's textures
        _HOST_TEXTURES["cloud_map"] = (W.cloud_map_desc(), orc.noise_generate(W.cloud_map_desc(), 32, threads))
        _HOST_TEXTURES["detail"] = (W.base_noise_desc(), orc.noise_generate(W.base_noise_desc(), 32, threads))
    host = dict(_HOST_TEXTURES)
    view = W.frame_view(cam, SUN_ZENITH)
    bn = reference_blue_noise()
    npx = view.width * view.height
    args = (W.frame_cloud_parameters(), W.frame_material(), host, view, sizes, luts["transmittance"],
            luts["aerial_perspective_luminance"], luts["aerial_perspective_transmittance"], bn)
    stride = 4096
    done, spent = 0, 0.0
    while spent < max(sample_s - lut_s, 0.5) and stride >= 1:
        px = np.arange(done % stride, npx, stride, dtype=np.int32)
        t0 = time.perf_counter()
        orc.cloud_render(atmo, *args, pixels=px, precision=32, nthreads=threads)
        el = time.perf_counter() - t0
        spent += el
        done += len(px)
        stride = max(stride // 2, 1)
    cloud_s = spent / done * npx
    return (lut_s + cloud_s) * 1000.0, done, lut_s * 1e3


def roofline_issue(cloud_ms: float, sm_mhz: float, tuned, sms: int) -> dict:
    """The raymarch against instruction issue: the warp instructions of one
    launch (ncu capture of the same frame and launch shape,
    profiles/dram_bytes_per_launch.json) over the launch's CUDA-event time,
    against the SMs (queried) x 4 schedulers x one issue per cycle at the
    sampled clock."""
    cap = ncu_capture("cloud_render_kernel")
    shape = {"cloud_tile": cloud_tile(tuned.cloud_tile_width, tuned.cloud_ray_lanes),
             "cloud_block_warps_x": tuned.cloud_block_warps_x, "cloud_blocks_per_sm": tuned.cloud_blocks_per_sm,
             "cloud_ray_lanes": tuned.cloud_ray_lanes}
    inst = cap.get("warp_instructions")
    if not inst:
        return {"kernel": "cloud_render_kernel", "achieved": None, "note": "no committed ncu instruction count"}
    achieved = inst / (cloud_ms * 1e-3) / 1e9
    peak = sms * 4 * sm_mhz * 1e6 / 1e9
    return {"kernel": "cloud_render_kernel", "bound": "issue", "achieved": achieved, "peak": peak,
            "unit": "G warp-instructions/s", "frac": achieved / peak, "warp_instructions_per_launch": inst,
            "capture_shape": cap.get("tuning"), "timed_shape": shape, "same_shape": cap.get("tuning") == shape,
            "note": f"peak = {sms} SMs x 4 schedulers x 1 instruction/cycle x median SM clock"}


def cpu_baseline(sample_s: float):
    threads = os.cpu_count() or 1
    ms, n, lut_ms = cpu_frame_ms(sample_s, threads)
    return {"value": ms, "unit": UNIT, "cores": threads, "kind": "port",
            "lut_set_ms": lut_ms,
            "sample": f"one full LUT set + {n} raymarched pixels ({n / 2073600:.2f} frames' worth, strided "
                      f"passes over the 1920x1080 frame) in FP32 on {threads} threads, scaled to one frame"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    per = max(2.0, min(args.cpu_sample_s, 150.0 / max(args.steps + args.warmup, 1)))
    for _ in range(args.warmup):
        cpu_frame_ms(1.0, threads)
    vals, ns = [], []
    for _ in range(args.steps):
        ms, n, _l = cpu_frame_ms(per, threads)
        vals.append(ms)
        ns.append(n)
    v = statistics.mean(vals)
    sample = (f"per step: one full LUT set + ~{int(statistics.mean(ns))} raymarched pixels in FP32 on "
              f"{threads} threads (oracle/ restatement of the reference shaders), scaled to 1920x1080")
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": v, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32", "data": "synthetic (same seeded inputs as the skyr arm)",
        "config": {"workload": "plain 1920x1080 frame: LUT set + per-pixel cloud raymarch (as the skyr arm)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_skyr(a)
