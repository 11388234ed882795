"""Fixed hot-path cases for profilers: set one case up, run it a given number of
times on one stream, synchronise and exit 0.

    python -m skyrendering_gb300.profile_cases luts  --iters 3
    python -m skyrendering_gb300.profile_cases cloud --iters 3
    python -m skyrendering_gb300.profile_cases pt    --iters 2 [--global-majorant] [--size 1024] [--frames 4]
    python -m skyrendering_gb300.profile_cases surrogate --iters 3 [--size 1024]
    python -m skyrendering_gb300.profile_cases lattice --iters 2
    python -m skyrendering_gb300.profile_cases mlp --iters 3
    python -m skyrendering_gb300.profile_cases shadow --iters 3
    python -m skyrendering_gb300.profile_cases quarter --iters 3
    python -m skyrendering_gb300.profile_cases environment --iters 3
    python -m skyrendering_gb300.profile_cases composite --iters 3

--tuning W,BX,OCC,LANES sets the cloud raymarch's launch shape (tile width,
block warps x, blocks per SM, lanes per ray) before the case is set up;
--lut-lanes T,V the lanes per transmittance texel and per sky-view /
aerial-perspective ray of the LUT passes.

Cases (seeded synthetic inputs from workloads.py):
  luts   the plain LUT set (T 256x64, MS 32x32, SV 192x108, AP 32^3) of the
         1 km / 60 deg / sun-zenith-45 frame;
  cloud  that LUT set once, then the 1920x1080 per-pixel cloud raymarch;
  pt     the 512x640x352 FP16 Worley-fBm grid (max extinction 40/km), its 16^3
         brick majorants and the LUT set once, then `frames` path-traced
         frames of the size x size view per iteration, in one launch (128
         bounces, HG 0.857).
  surrogate  the committed network's 128-step surrogate raymarch of that grid
         (size x size, feature lattice built once);
  lattice the feature lattice of that grid for the scene's sun;
  mlp    one Adam training step of the network on a 16384-sample batch of
         seeded random records.
  shadow the cloud shadow passes of the 1920x1080 frame (512^2 map blended
         into the previous frame's, blur, 160x90x128 froxel).
  composite the full-screen atmosphere composite of that frame (1920x1080,
         per-pixel raymarch of 40 dithered samples, star map, no objects);
  environment the environment cube of that frame's LUT set (128^2 x 6 +
         mips), its SH coefficients and 5 prefiltered roughness levels;
  quarter the quarter-resolution cloud pass of that frame (checkerboard,
         index, 480x270 raymarch, 960x540 reconstruction with history,
         upscale into an HDR target; empty depth buffer).
The per-iteration CUDA-event time is printed for orientation; it is not a
benchmark figure (bench.py is).
"""
from __future__ import annotations

import argparse

import torch

from . import workloads as W
from .atmosphere import Context, LutSet, update_lut_set
from .cloud import NoiseTexture, VolumetricCloud, blue_noise_tile, prepare_textures, textures_struct
from .pathtrace import DensityGrid, PathTracer

SUN_ZENITH = 45.0


def lut_case(ctx, cam):
    atmo, sizes = W.earth_like_atmosphere(), W.plain_lut_sizes()
    render = W.render_parameters(cam, SUN_ZENITH)
    luts = LutSet.allocate(sizes, 1)
    return atmo, sizes, render, luts, lambda: update_lut_set(ctx, atmo, render, sizes, luts)


def cloud_case(ctx):
    cam = W.frame_camera()
    atmo, sizes, render, luts, lut_step = lut_case(ctx, cam)
    lut_step()
    tex = {"cloud_map": NoiseTexture(W.cloud_map_desc()).generate(ctx),
           "detail": NoiseTexture(W.base_noise_desc()).generate(ctx)}
    material = W.frame_material()
    prepare_textures(ctx, material.type, tex)
    bn = blue_noise_tile().cuda()
    view = W.frame_view(cam, SUN_ZENITH)
    vc = VolumetricCloud(ctx, W.frame_cloud_parameters(), material, textures_struct(**tex))
    rgba = torch.empty((view.height, view.width, 4), dtype=torch.float16, device="cuda")
    dist = torch.empty((view.height, view.width), dtype=torch.float32, device="cuda")
    return lambda: vc.render(atmo, view, sizes, luts, bn, out_rgba=rgba, out_distance=dist)


def pt_case(ctx, size: int, global_majorant: bool, frames: int):
    cam = W.pt_camera(size, size)
    atmo, sizes, render, luts, lut_step = lut_case(ctx, cam)
    lut_step()
    origin, voxel = W.pt_grid_placement()
    grid = DensityGrid(*W.PT_GRID_DIMS, origin=origin, voxel_size=voxel, density=1.0)
    grid.generate(ctx, W.pt_grid_generator()).normalize_extinction(ctx, W.PT_SIGMA_MAX)
    pt = W.pt_parameters()
    pt.use_brick_majorants = 0 if global_majorant else 1
    tracer = PathTracer(ctx, pt, W.pt_cloud_parameters(), W.frame_view(cam, SUN_ZENITH), render, sizes, grid=grid)
    return lambda: tracer.render(atmo, luts, frames)


def surrogate_case(ctx, size: int, what: str):
    from . import surrogate as S
    from . import surrogate_train as T

    sc = T.Scene(ctx, size=size)
    grid = sc.grid(W.SEED)
    if what == "lattice":
        return lambda: sc.lattice(grid)
    fv = sc.lattice(grid)
    model = S.load_model(S.MODEL_PATH)
    net = model.packed(ctx)
    table = torch.from_numpy(model.error_table).cuda()
    sp = S.parameters(error_table=table)
    out = torch.empty((size, size, 4), dtype=torch.float32, device="cuda")
    err = torch.empty((size, size), dtype=torch.float32, device="cuda")
    keep = (table, fv)
    return lambda: (S.render(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.sizes, sc.luts, fv, net, sp, out, err),
                    keep)


def mlp_case(ctx):
    from . import mlp

    g = torch.Generator(device="cuda").manual_seed(5)
    x = torch.rand((16384, mlp.INPUTS), device="cuda", generator=g)
    rec = mlp.to_records(x)
    t = torch.rand((16384, 3), device="cuda", generator=g) + 0.5
    tr = mlp.Trainer(ctx, mlp.init_params(1), mlp.hparams())
    return lambda: (tr.step(rec, t), tr)


def shadow_case(ctx):
    from .cloud import CloudShadow, shadow_sizes

    cam = W.frame_camera()
    tex = {"cloud_map": NoiseTexture(W.cloud_map_desc()).generate(ctx),
           "detail": NoiseTexture(W.base_noise_desc()).generate(ctx)}
    material = W.frame_material()
    prepare_textures(ctx, material.type, tex)
    bn = blue_noise_tile().cuda()
    view = W.frame_view(cam, SUN_ZENITH)
    vc = VolumetricCloud(ctx, W.frame_cloud_parameters(), material, textures_struct(**tex))
    sh = CloudShadow(ctx, shadow_sizes(1920, 1080))
    sh.render(vc, W.earth_like_atmosphere(), view, bn)
    atmo = W.earth_like_atmosphere()
    return lambda: sh.render(vc, atmo, view, bn, wind_delta=(0.01, 0.0))


def quarter_case(ctx):
    from .cloud import CloudViewport

    cam = W.frame_camera()
    atmo, sizes, render, luts, lut_step = lut_case(ctx, cam)
    lut_step()
    tex = {"cloud_map": NoiseTexture(W.cloud_map_desc()).generate(ctx),
           "detail": NoiseTexture(W.base_noise_desc()).generate(ctx)}
    material = W.frame_material()
    prepare_textures(ctx, material.type, tex)
    bn = blue_noise_tile().cuda()
    view = W.frame_view(cam, SUN_ZENITH)
    vc = VolumetricCloud(ctx, W.frame_cloud_parameters(), material, textures_struct(**tex))
    vp = CloudViewport(ctx, view.width, view.height)
    hdr = torch.zeros((view.height, view.width, 4), dtype=torch.float16, device="cuda")
    vp.render(vc, atmo, view, sizes, luts, bn, hdr=hdr, z_near=cam.z_near, z_far=cam.z_far)

    def step():
        view.frame_id = float((int(view.frame_id) + 1) & 0xFF)
        vp.render(vc, atmo, view, sizes, luts, bn, hdr=hdr, z_near=cam.z_near, z_far=cam.z_far)

    return step


def environment_case(ctx):
    from .atmosphere import environment_cube, environment_prefilter, environment_seamless, environment_sh

    atmo, sizes, render, luts, lut_step = lut_case(ctx, W.frame_camera())
    lut_step()
    total = sum(6 * (128 >> l) ** 2 for l in range(8))
    out = torch.empty((total, 4), dtype=torch.float16, device="cuda")
    seam = torch.empty((sum(6 * ((128 >> l) + 2) ** 2 for l in range(8)), 4), dtype=torch.float32, device="cuda")
    sh = torch.empty((9, 4), dtype=torch.float32, device="cuda")
    pre = torch.empty((sum(6 * (128 >> l) ** 2 for l in range(5)), 4), dtype=torch.float16, device="cuda")

    def step():
        environment_cube(ctx, atmo, render, sizes, luts, 128, out=out)
        environment_seamless(ctx, out, 128, 8, out=seam)
        environment_sh(ctx, seam, 128, 8, out=sh)
        environment_prefilter(ctx, seam, 128, 8, 128, 5, out=pre)

    return step


def composite_case(ctx):
    from .atmosphere import composite, composite_parameters

    cam = W.frame_camera()
    atmo, sizes, render, luts, lut_step = lut_case(ctx, cam)
    lut_step()
    bn = blue_noise_tile().cuda()
    stars = torch.from_numpy(W.star_map()).cuda()
    out = torch.empty((cam.height, cam.width, 4), dtype=torch.float16, device="cuda")
    cp = composite_parameters()
    return lambda: composite(ctx, atmo, render, cp, sizes, luts, cam.width, cam.height, blue_noise=bn,
                             star_map=stars, out=out)


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("case", choices=["luts", "cloud", "pt", "surrogate", "lattice", "mlp", "shadow", "quarter", "environment", "composite"])
    ap.add_argument("--iters", type=int, default=3)
    ap.add_argument("--size", type=int, default=1024)
    ap.add_argument("--global-majorant", action="store_true")
    ap.add_argument("--frames", type=int, default=4)
    ap.add_argument("--tuning", default=None, help="W,BX,OCC,LANES of the cloud raymarch")
    ap.add_argument("--lut-lanes", default=None, help="T,V lanes of the transmittance and view LUT passes")
    a = ap.parse_args(argv)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    ctx = Context(stream)
    if a.tuning:
        from . import batch as B

        w, bx, occ, g = (int(v) for v in a.tuning.split(","))
        B.set_tuning(ctx, cloud_tile_width=w, cloud_block_warps_x=bx, cloud_blocks_per_sm=occ, cloud_ray_lanes=g)
    if a.lut_lanes:
        from . import batch as B

        tl, vl = (int(v) for v in a.lut_lanes.split(","))
        B.set_tuning(ctx, transmittance_lanes=tl, view_lanes=vl)
    if a.case == "luts":
        step = lut_case(ctx, W.frame_camera())[-1]
    elif a.case == "cloud":
        step = cloud_case(ctx)
    elif a.case == "pt":
        step = pt_case(ctx, a.size, a.global_majorant, a.frames)
    elif a.case in ("surrogate", "lattice"):
        step = surrogate_case(ctx, a.size, a.case)
    elif a.case == "shadow":
        step = shadow_case(ctx)
    elif a.case == "quarter":
        step = quarter_case(ctx)
    elif a.case == "environment":
        step = environment_case(ctx)
    elif a.case == "composite":
        step = composite_case(ctx)
    else:
        step = mlp_case(ctx)
    torch.cuda.synchronize()
    for i in range(a.iters):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        torch.cuda.synchronize()
        print(f"{a.case} iteration {i}: {e0.elapsed_time(e1):.3f} ms")
    ctx.check_status()
    ctx.close()


if __name__ == "__main__":
    main()
