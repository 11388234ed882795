"""Host side of the multiple-scattering surrogate (include/skyr_surrogate.h):
feature lattice, training points, records and path-traced targets, and the
surrogate-shaded render with its path-traced fallback.

No counterpart in the reference: the network stands in for the multiple-
scattering heuristic of VolumetricCloudRender.comp:125-130, and the plain path
tracer (VolumetricCloudPathTracing.comp) is both its training-data source and
its fallback.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from pathlib import Path

import numpy as np
import torch

from . import _abi, mlp
from .atmosphere import Context, LutSet, _ptr
from .mlp import RECORD, PackedMLP
from .pathtrace import DensityGrid


class FeatureVolume:
    """Feature lattice of one (grid, sun direction) pair."""

    def __init__(self, grid: DensityGrid, stride: int = 4, sigma_ref: float = 40.0):
        self.struct = _abi.FeatureVolume()
        n = _abi.lib().skyr_feature_volume_bytes(C.byref(grid.struct), stride, C.byref(self.struct))
        if n == 0:
            raise ValueError("bad grid or stride")
        self.buf = torch.empty(n, dtype=torch.uint8, device="cuda")
        self.struct.data = self.buf.data_ptr()
        self.struct.sigma_ref = sigma_ref
        self.grid = grid

    def build(self, ctx: Context, atmosphere, cloud, view) -> "FeatureVolume":
        _abi.call("skyr_feature_volume_build", ctx.handle, C.byref(atmosphere), C.byref(cloud),
                  C.byref(self.grid.struct), C.byref(view), C.byref(self.struct))
        return self


def sample_points(ctx: Context, grid: DensityGrid, n: int, seed: int, sigma_max: float,
                  sigma_min: float = 0.5) -> torch.Tensor:
    pts = torch.empty((n, 6), dtype=torch.float32, device="cuda")
    _abi.call("skyr_surrogate_sample_points", ctx.handle, C.byref(grid.struct), C.c_float(sigma_max),
              C.c_float(sigma_min), C.c_uint64(seed), n, _ptr(pts))
    return pts


def records(ctx: Context, fv: FeatureVolume, points: torch.Tensor) -> torch.Tensor:
    rec = torch.empty((points.shape[0], RECORD), dtype=torch.bfloat16, device="cuda")
    _abi.call("skyr_surrogate_records", ctx.handle, C.byref(fv.grid.struct), C.byref(fv.struct), _ptr(points),
              points.shape[0], _ptr(rec))
    return rec


def point_radiance(ctx: Context, atmosphere, cloud, grid: DensityGrid, pt, view, env_view, sizes, luts: LutSet,
                   points: torch.Tensor, n_paths: int, frame_begin: int = 1) -> torch.Tensor:
    """Path-traced order >= 2 in-scattered radiance at the points (mean of n_paths)."""
    out = torch.zeros((points.shape[0], 3), dtype=torch.float32, device="cuda")
    _abi.call("skyr_pathtrace_points", ctx.handle, C.byref(atmosphere), C.byref(cloud), C.byref(grid.struct),
              C.byref(pt), C.byref(view), C.byref(env_view), C.byref(sizes), _ptr(luts.transmittance),
              _ptr(luts.sky_view_luminance), _ptr(luts.sky_view_transmittance),
              _ptr(luts.aerial_perspective_luminance), _ptr(luts.aerial_perspective_transmittance), frame_begin,
              n_paths, _ptr(points), points.shape[0], _ptr(out))
    return out.div_(float(n_paths))


def parameters(error_table: torch.Tensor | None = None, **kw) -> _abi.SurrogateParameters:
    """Raymarch settings; `error_table` (device float[64]) is referenced, keep it alive."""
    p = _abi.SurrogateParameters()
    _abi.call("skyr_surrogate_parameters_default", C.byref(p))
    for k, v in kw.items():
        setattr(p, k, v)
    if error_table is not None:
        p.error_table = error_table.data_ptr()
    return p


BINS = _abi.SKYR_SURROGATE_ERROR_BINS


def error_bins(ctx: Context, rec: torch.Tensor) -> torch.Tensor:
    bins = torch.empty(rec.shape[0], dtype=torch.int32, device="cuda")
    _abi.call("skyr_surrogate_error_bins", ctx.handle, _ptr(rec), rec.shape[0], _ptr(bins))
    return bins


def calibrate_error_table(ctx: Context, net: PackedMLP, rec: torch.Tensor, lab: torch.Tensor,
                          min_count: int = 50) -> torch.Tensor:
    """Relative L1 of the network per error bin on labelled points (bins with
    fewer than min_count points take the overall value)."""
    y = net.infer(rec)
    e = (y - lab).abs().sum(1).double()
    m = lab.abs().sum(1).double()
    b = error_bins(ctx, rec).long()
    n = BINS * BINS
    se = torch.zeros(n, dtype=torch.float64, device="cuda").index_add_(0, b, e)
    sm = torch.zeros(n, dtype=torch.float64, device="cuda").index_add_(0, b, m)
    cnt = torch.zeros(n, dtype=torch.float64, device="cuda").index_add_(0, b, torch.ones_like(e))
    overall = float(e.sum() / m.sum().clamp_min(1e-30))
    table = torch.where((cnt >= min_count) & (sm > 0), se / sm.clamp_min(1e-30), torch.full_like(se, overall))
    return table.float().contiguous()


def render(ctx: Context, atmosphere, cloud, grid: DensityGrid, pt, view, sizes, luts: LutSet, fv: FeatureVolume,
           net: PackedMLP | None, sp: _abi.SurrogateParameters, out: torch.Tensor | None = None,
           err: torch.Tensor | None = None):
    """(rgba [h][w][4] = luminance, transmittance; error estimate [h][w])."""
    h, w = view.height, view.width
    out = out if out is not None else torch.empty((h, w, 4), dtype=torch.float32, device="cuda")
    err = err if err is not None else torch.empty((h, w), dtype=torch.float32, device="cuda")
    _abi.call("skyr_surrogate_render", ctx.handle, C.byref(atmosphere), C.byref(cloud), C.byref(grid.struct),
              C.byref(pt), C.byref(view), C.byref(sizes), _ptr(luts.transmittance),
              _ptr(luts.aerial_perspective_luminance), _ptr(luts.aerial_perspective_transmittance), C.byref(fv.struct),
              _ptr(net.buf) if net is not None else None, C.byref(sp), _ptr(out), _ptr(err))
    return out, err


def pathtrace_pixels(ctx: Context, atmosphere, cloud, grid: DensityGrid, pt, view, env_view, sizes, luts: LutSet,
                     pixels: torch.Tensor, n_frames: int, acc: torch.Tensor, frame_begin: int = 1):
    """Add n_frames path-traced frames of the listed pixels (int32 y * w + x) to acc."""
    _abi.call("skyr_pathtrace_pixels", ctx.handle, C.byref(atmosphere), C.byref(cloud), None, None,
              C.byref(grid.struct), C.byref(pt), C.byref(view), C.byref(env_view), C.byref(sizes),
              _ptr(luts.transmittance), _ptr(luts.sky_view_luminance), _ptr(luts.sky_view_transmittance),
              _ptr(luts.aerial_perspective_luminance), _ptr(luts.aerial_perspective_transmittance), frame_begin,
              n_frames, _ptr(pixels), pixels.shape[0], _ptr(acc), None)


def luminance(rgb: torch.Tensor) -> torch.Tensor:
    return rgb[..., 0] * 0.2126 + rgb[..., 1] * 0.7152 + rgb[..., 2] * 0.0722


def relative_l1(img: torch.Tensor, ref: torch.Tensor) -> float:
    """Image relative L1 error of the rgb luminance: sum |img - ref| / sum |ref|."""
    a, b = img[..., :3].double(), ref[..., :3].double()
    return float((a - b).abs().sum() / b.abs().sum().clamp_min(1e-30))


@dataclass
class FallbackResult:
    image: torch.Tensor  # [h][w][4] luminance rgb, transmittance
    flagged: int         # pixels path traced
    frames: int          # path-traced frames per flagged pixel


def render_with_fallback(ctx: Context, atmosphere, cloud, grid: DensityGrid, pt, view, env_view, sizes,
                         luts: LutSet, fv: FeatureVolume, net: PackedMLP, sp: _abi.SurrogateParameters,
                         threshold: float, fallback_frames: int, floor: float = 1e-3) -> FallbackResult:
    """`sp` should carry the calibrated error table (parameters(error_table=...))."""
    """Surrogate image; pixels whose estimated relative error exceeds `threshold`
    are path traced with `fallback_frames` frames instead."""
    img, err = render(ctx, atmosphere, cloud, grid, pt, view, sizes, luts, fv, net, sp)
    lum = luminance(img[..., :3]).clamp_min(floor)
    mask = (err / lum) > threshold
    pix = torch.nonzero(mask.reshape(-1), as_tuple=False).reshape(-1).to(torch.int32)
    n = int(pix.numel())
    if n and fallback_frames > 0:
        acc = torch.zeros((view.height, view.width, 4), dtype=torch.float32, device="cuda")
        pathtrace_pixels(ctx, atmosphere, cloud, grid, pt, view, env_view, sizes, luts, pix, fallback_frames, acc)
        flat = img.reshape(-1, 4)
        flat[pix.long()] = acc.reshape(-1, 4)[pix.long()] / float(fallback_frames)
    return FallbackResult(img, n, fallback_frames)


def save_model(path, params: np.ndarray, label_scale: float, network_error: float, meta: dict,
               error_table: np.ndarray | None = None):
    table = np.full(BINS * BINS, network_error, np.float32) if error_table is None else error_table
    np.savez(path, params=np.asarray(params, dtype=np.float32), label_scale=np.float32(label_scale),
             network_error=np.float32(network_error), error_table=np.asarray(table, dtype=np.float32),
             meta=np.array(repr(meta)))


@dataclass
class Model:
    params: np.ndarray
    label_scale: float
    network_error: float
    error_table: np.ndarray
    meta: str

    def packed(self, ctx: Context) -> PackedMLP:
        return PackedMLP.from_params(ctx, self.params, self.label_scale)


def load_model(path) -> Model:
    d = np.load(path, allow_pickle=False)
    if d["params"].size != mlp.PARAMS:
        raise ValueError(f"{path}: a network of {d['params'].size} parameters, this build's has {mlp.PARAMS}")
    table = d["error_table"] if "error_table" in d.files else np.full(BINS * BINS, float(d["network_error"]),
                                                                        np.float32)
    return Model(d["params"], float(d["label_scale"]), float(d["network_error"]), table, str(d["meta"]))


MODEL_PATH = Path(__file__).resolve().parent / "data" / "surrogate_model.npz"
