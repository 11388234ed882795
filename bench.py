"""Benchmark of the atmosphere-LUT / volumetric-cloud hot path on one GB300.

A step is one full plain frame of the 1920x1080 workload: the whole LUT set
(transmittance 256x64 / 40 samples, multi-scattering 32x32 / 64 directions x
20 samples, sky-view 192x108 / 30 samples, aerial perspective 32^3 / 40
samples over 32 km) followed by the per-pixel cloud raymarch.  Inputs are
seeded synthetic (no dataset); see skyrendering_gb300/workloads.py.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

Prints one JSON line.  --impl reference times the CPU restatement of the
reference's shader math (the reference itself is GLSL for an OpenGL driver,
which this machine cannot run) on the host cores.
"""
from __future__ import annotations

import argparse
import json
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
L2_FLUSH_BYTES = 512 << 20  # > 129 MB L2


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="skyr", choices=["skyr", "reference"])
    ap.add_argument("--cpu-sample-s", type=float, default=15.0)
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


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
        time.sleep(0.3)
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


def measured_peaks():
    f = ROOT / "MEASURED_PEAKS.json"
    if f.exists():
        d = json.loads(f.read_text())
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
def run_skyr(args):
    import torch

    from skyrendering_gb300 import _abi
    from skyrendering_gb300 import workloads as W
    from skyrendering_gb300.atmosphere import Context, LutSet, update_lut_set

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = Context(stream)

    p = W.earth_like_atmosphere()
    sizes = W.plain_lut_sizes()
    cam = W.frame_camera()
    render = W.render_parameters(cam, 45.0)
    luts = LutSet.allocate(sizes, 1)
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")

    def step():
        update_lut_set(ctx, p, render, sizes, luts)

    kernels_per_step = 3
    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    with ClockSampler(local) as clk:
        barrier()
        wall0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(float(i))  # evict L2 between steps (not timed)
            starts[i].record(stream)
            step()
            ends[i].record(stream)
        barrier()
        wall = time.perf_counter() - wall0
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    ms = statistics.mean(step_ms)
    if world > 1:
        t = torch.tensor([ms], device="cuda")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = float(t.item())

    # e2e: public API with host buffers: parameter blocks H2D (pinned) and the
    # LUT outputs D2H (pinned) inside the timed region
    host_out = {n: torch.empty(getattr(luts, n).shape, dtype=getattr(luts, n).dtype, pin_memory=True)
                for n in ("transmittance", "multiscattering", "sky_view_luminance", "sky_view_transmittance",
                          "aerial_perspective_luminance", "aerial_perspective_transmittance")}
    d2h = sum(t.numel() * t.element_size() for t in host_out.values())
    import ctypes as C
    h2d = C.sizeof(p) + C.sizeof(render)

    def e2e_step():
        update_lut_set(ctx, p, render, sizes, luts)
        for n, t in host_out.items():
            t.copy_(getattr(luts, n), non_blocking=True)

    for _ in range(3):
        e2e_step()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        e2e_step()
    e1.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e0.elapsed_time(e1) / args.steps

    clocks = clk.summary()
    result = {
        "metric": METRIC,
        "value": ms * 1000.0,
        "unit": "us per LUT set",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": False,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic (seeded Earth-like atmosphere, 1 km camera, sun zenith 45 deg)",
        "config": {"workload": "plain LUT set: T 256x64x40, MS 32x32x64x20, SV 192x108x30, AP 32^3x40 over 32 km",
                   "l2": "flushed between timed steps (512 MB write)", "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e_ms * 1000.0, "unit": "us per LUT set", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h},
        "gpu_launches": kernels_per_step * args.steps,
        "clocks": clocks,
        "wall_s": wall,
    }
    if rank == 0:
        if world == 1:
            result["cpu_baseline"] = cpu_baseline(args.cpu_sample_s)
        print(json.dumps(result))
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()


# ---------------------------------------------------------------------------
# CPU baseline / reference arm: the FP32 restatement of the shader math on the
# host cores (oracle/, test infrastructure; timed, never shipped)
# ---------------------------------------------------------------------------
def cpu_lut_set_us(sample_s: float, threads: int):
    from oracle import oracle as orc
    from skyrendering_gb300 import workloads as W

    p = W.earth_like_atmosphere()
    s = W.plain_lut_sizes()
    r = W.render_parameters(W.frame_camera(), 45.0)
    orc.lut_set(p, r, s, 32, nthreads=threads)  # warm-up / build
    n, t0 = 0, time.perf_counter()
    while True:
        orc.lut_set(p, r, s, 32, nthreads=threads)
        n += 1
        el = time.perf_counter() - t0
        if el >= sample_s or n >= 1000:
            break
    return el / n * 1e6, n


def cpu_baseline(sample_s: float):
    threads = os.cpu_count() or 1
    us, n = cpu_lut_set_us(sample_s, threads)
    return {"value": us, "unit": "us per LUT set", "cores": threads, "kind": "port",
            "sample": f"{n} full plain LUT sets in FP32 on {threads} threads (~{sample_s:.0f} s)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    vals = []
    for _ in range(max(args.warmup, 0)):
        cpu_lut_set_us(0.5, threads)
    for _ in range(args.steps):
        us, _n = cpu_lut_set_us(min(args.cpu_sample_s, 120.0 / max(args.steps, 1)), threads)
        vals.append(us)
    v = statistics.mean(vals)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": "us per LUT set", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": v / 1000.0, "higher_is_better": False,
        "dtype": "f32", "data": "synthetic", "config": {"workload": "plain LUT set (as the skyr arm)"},
        "cpu_baseline": {"value": v, "unit": "us per LUT set", "cores": threads, "kind": "port",
                         "sample": "FP32 restatement of the reference shaders (oracle/), all host threads"},
        "e2e": {"value": v, "unit": "us per LUT set", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }))


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_skyr(a)
