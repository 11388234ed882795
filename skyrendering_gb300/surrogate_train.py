"""Train the multiple-scattering surrogate on path-traced targets.

    python -m skyrendering_gb300.surrogate_train [--clouds 600] [--points 20000] [--paths 128]
                                                 [--epochs 192] [--out model.npz]

For each of `clouds` seeded synthetic clouds (the voxel scene's generator with
seeds 1000, 1001, ...; the evaluation cloud 0x5EED is not among them) the grid
is generated and normalised to a largest extinction of 40/km, its feature
lattice is built for the scene's sun, `points` training points are drawn (half
first collisions of outside rays, half uniform in the cloud) and each gets the
mean of `paths` path-traced order >= 2 radiance estimates as its target.
Validation clouds (seeds 900..) get 8x the paths.  The network is trained with
Adam (lr 1e-3 with a cosine decay to 5e-5, batch 16384, relative L2 loss with
eps 1e-2) by the tensor-core kernels of libskyr; the validation relative L1
error, overall and per error bin (the table of skyr_surrogate_parameters), is
stored with the parameters and drives the renderer's error estimate.
"""
from __future__ import annotations

import argparse
import time

import numpy as np
import torch

from . import mlp
from . import surrogate as S
from . import workloads as W
from .atmosphere import Context, update_lut_set
from .pathtrace import DensityGrid

SUN_ZENITH = 45.0
STRIDE = 4
SIGMA_REF = W.PT_SIGMA_MAX


class Scene:
    """The voxel scene's atmosphere, LUTs, camera frame and path-tracer settings."""

    def __init__(self, ctx: Context, size: int = 1024, dims=W.PT_GRID_DIMS):
        self.ctx = ctx
        self.dims = dims
        self.atmo = W.earth_like_atmosphere()
        self.sizes = W.plain_lut_sizes()
        self.cam = W.pt_camera(size, size)
        self.env = W.render_parameters(self.cam, SUN_ZENITH)
        self.luts = update_lut_set(ctx, self.atmo, self.env, self.sizes)
        self.view = W.frame_view(self.cam, SUN_ZENITH)
        self.cloud = W.pt_cloud_parameters(dims)
        self.pt = W.pt_parameters()

    def grid(self, seed: int) -> DensityGrid:
        origin, voxel = W.pt_grid_placement(self.dims)
        g = DensityGrid(*self.dims, origin=origin, voxel_size=voxel, density=1.0)
        return g.generate(self.ctx, W.pt_grid_generator(self.dims, seed=seed)).normalize_extinction(
            self.ctx, W.PT_SIGMA_MAX)

    def lattice(self, grid: DensityGrid) -> S.FeatureVolume:
        return S.FeatureVolume(grid, STRIDE, SIGMA_REF).build(self.ctx, self.atmo, self.cloud, self.view)


def cloud_samples(scene: Scene, seed: int, n_points: int, n_paths: int):
    grid = scene.grid(seed)
    fv = scene.lattice(grid)
    pts = S.sample_points(scene.ctx, grid, n_points, seed * 7919 + 17, W.PT_SIGMA_MAX)
    rec = S.records(scene.ctx, fv, pts)
    lab = S.point_radiance(scene.ctx, scene.atmo, scene.cloud, grid, scene.pt, scene.view, scene.env, scene.sizes,
                           scene.luts, pts, n_paths, frame_begin=1 + seed * 4099)
    return rec, lab


def dataset(scene: Scene, seeds, n_points: int, n_paths: int):
    recs, labs = [], []
    for s in seeds:
        r, l = cloud_samples(scene, s, n_points, n_paths)
        recs.append(r)
        labs.append(l)
    scene.ctx.check_status()
    return torch.cat(recs), torch.cat(labs)


def validation_error(net: mlp.PackedMLP, rec: torch.Tensor, lab: torch.Tensor) -> float:
    """Relative L1 of the network on labelled points: sum |y - t| / sum |t|."""
    y = net.infer(rec)
    return float((y - lab).abs().sum() / lab.abs().sum().clamp_min(1e-30))


def train(ctx: Context, rec: torch.Tensor, lab: torch.Tensor, val_rec: torch.Tensor, val_lab: torch.Tensor,
          epochs: int, batch: int = 16384, lr: float = 1e-3, seed: int = 7, loss_eps: float = 1e-2,
          cosine: bool = True, log=print):
    """Adam from lr (cosine decay to lr / 20 over the epochs when `cosine`)."""
    import math

    label_scale = float(lab.mean().item())
    h = mlp.hparams(learning_rate=lr, label_scale=label_scale, loss_epsilon=loss_eps)
    tr = mlp.Trainer(ctx, mlp.init_params(seed), h)
    n = rec.shape[0]
    gen = torch.Generator(device="cuda").manual_seed(seed)
    loss = torch.zeros(1, device="cuda")
    curve = []
    for ep in range(epochs):
        if cosine:
            tr.set_learning_rate(lr * (0.05 + 0.95 * 0.5 * (1.0 + math.cos(math.pi * ep / max(epochs, 1)))))
        perm = torch.randperm(n, device="cuda", generator=gen)
        loss.zero_()
        steps = n // batch
        tr.epoch(rec, lab, perm, batch, loss)  # the batches gathered inside the gradient kernel
        ve = validation_error(tr.packed(), val_rec, val_lab)
        curve.append((ep, float(loss.item()) / max(steps, 1), ve))
        log(f"epoch {ep}: train loss {curve[-1][1]:.5f}  validation rel L1 {ve:.4f}")
    params = tr.params().cpu().numpy()
    tr.close()
    return params, label_scale, curve


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--clouds", type=int, default=600)
    ap.add_argument("--val-clouds", type=int, default=8)
    ap.add_argument("--points", type=int, default=20000)
    ap.add_argument("--paths", type=int, default=128)
    ap.add_argument("--epochs", type=int, default=192)
    ap.add_argument("--out", default="surrogate_model.npz")
    a = ap.parse_args(argv)
    torch.cuda.set_device(0)
    ctx = Context()
    scene = Scene(ctx)
    t0 = time.time()
    rec, lab = dataset(scene, range(1000, 1000 + a.clouds), a.points, a.paths)
    vrec, vlab = dataset(scene, range(900, 900 + a.val_clouds), a.points // 4, a.paths * 8)
    torch.cuda.synchronize()
    t1 = time.time()
    print(f"data: {rec.shape[0]} training / {vrec.shape[0]} validation points in {t1 - t0:.1f} s")
    params, scale, curve = train(ctx, rec, lab, vrec, vlab, a.epochs)
    torch.cuda.synchronize()
    t2 = time.time()
    net = mlp.PackedMLP.from_params(ctx, params, scale)
    verr = validation_error(net, vrec, vlab)
    table = S.calibrate_error_table(ctx, net, vrec, vlab).cpu().numpy()
    print(f"training: {a.epochs} epochs in {t2 - t1:.1f} s; validation relative L1 {verr:.4f}")
    print("error table (rows: local extinction bins, columns: near-sun extinction bins):")
    print(np.array2string(table.reshape(S.BINS, S.BINS), precision=3))
    meta = {"clouds": a.clouds, "points_per_cloud": a.points, "paths": a.paths, "epochs": a.epochs,
            "val_clouds": a.val_clouds, "curve": curve, "data_s": t1 - t0, "train_s": t2 - t1}
    S.save_model(a.out, params, scale, verr, meta, table)
    ctx.close()


if __name__ == "__main__":
    main()
