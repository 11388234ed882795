"""Host side of include/skyr_batch.h: launch-shape tuning and the autotuners,
prepared LUT batches, multi-view raymarches and CUDA-graph capture.

No reference counterpart: the reference regenerates one parameter set per frame
and picks its compute local sizes by hand (src/Base/src/GLReloadableProgram.cpp:43-62).
"""
from __future__ import annotations

import ctypes as C
from contextlib import contextmanager

import numpy as np
import torch

from . import _abi
from .atmosphere import Context, LutSet, _ptr

TILE_CANDIDATES = ((4, 1), (4, 2), (4, 4), (8, 1), (8, 2), (8, 4), (16, 1), (16, 2), (16, 4), (32, 1), (32, 2),
                   (32, 4))
OCCUPANCY_CANDIDATES = (5, 6, 7, 8, 9, 10)
RAY_LANE_CANDIDATES = (1, 2, 4, 8)
# (tile width, block warps x, blocks per SM, ray lanes) in the order of skyr_autotune_cloud's times
CLOUD_CANDIDATES = tuple((w, bx, occ, g) for g in RAY_LANE_CANDIDATES for occ in OCCUPANCY_CANDIDATES
                         for w, bx in TILE_CANDIDATES)


def cloud_tuning_key(t: _abi.Tuning) -> tuple:
    """The CLOUD_CANDIDATES entry of a tuning."""
    return (t.cloud_tile_width, t.cloud_block_warps_x, t.cloud_blocks_per_sm, t.cloud_ray_lanes)


def tuning(ctx: Context) -> _abi.Tuning:
    t = _abi.Tuning()
    _abi.call("skyr_ctx_get_tuning", ctx.handle, C.byref(t))
    return t


def set_tuning(ctx: Context, **kw) -> _abi.Tuning:
    t = tuning(ctx)
    for k, v in kw.items():
        setattr(t, k, v)
    _abi.call("skyr_ctx_set_tuning", ctx.handle, C.byref(t))
    return t


def _luts_args(luts: LutSet):
    return (_ptr(luts.transmittance), _ptr(luts.multiscattering), _ptr(luts.sky_view_luminance),
            _ptr(luts.sky_view_transmittance), _ptr(luts.aerial_perspective_luminance),
            _ptr(luts.aerial_perspective_transmittance))


def autotune_luts(ctx: Context, params, renders, n: int, sizes, luts: LutSet, reps: int = 5):
    """(chosen tuning, times ms: transmittance lanes 2/4/8/16, view lanes 2/4/8/16)."""
    best = _abi.Tuning()
    times = (C.c_float * 8)()
    _abi.call("skyr_autotune_luts", ctx.handle, params, renders, n, C.byref(sizes), *_luts_args(luts), reps,
              C.byref(best), times)
    return best, list(times)


def autotune_cloud(ctx: Context, atmosphere, cloud, material, textures, view, sizes, luts: LutSet, blue_noise,
                   out_rgba, out_dist, reps: int = 3):
    """(chosen tuning, times ms per CLOUD_CANDIDATES entry)."""
    best = _abi.Tuning()
    times = (C.c_float * _abi.SKYR_CLOUD_TUNE_CANDIDATES)()
    _abi.call("skyr_autotune_cloud", ctx.handle, C.byref(atmosphere), C.byref(cloud), C.byref(material),
              C.byref(textures), C.byref(view), C.byref(sizes), _ptr(luts.transmittance),
              _ptr(luts.aerial_perspective_luminance), _ptr(luts.aerial_perspective_transmittance), _ptr(blue_noise),
              _ptr(out_rgba), _ptr(out_dist), reps, C.byref(best), times)
    return best, list(times)


class LutBatch:
    """Per-set constants uploaded once; launch() only enqueues the passes."""

    def __init__(self, ctx: Context, params, renders, n: int, sizes):
        self.ctx = ctx
        self._b = C.c_void_p()
        _abi.call("skyr_lut_batch_create", ctx.handle, params, renders, n, C.byref(sizes), C.byref(self._b))

    def launch(self, luts: LutSet):
        _abi.call("skyr_lut_batch_launch", self._b, *_luts_args(luts))

    def close(self):
        if self._b:
            _abi.call("skyr_lut_batch_destroy", self._b)
            self._b = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class ViewOutputs:
    """Per-view RGBA16F / R32F outputs and the pointer arrays the ABI takes."""

    def __init__(self, views, n: int):
        self.rgba = [torch.empty((views[i].height, views[i].width, 4), dtype=torch.float16, device="cuda")
                     for i in range(n)]
        self.dist = [torch.empty((views[i].height, views[i].width), dtype=torch.float32, device="cuda")
                     for i in range(n)]
        self.rgba_ptrs = (C.c_void_p * n)(*[t.data_ptr() for t in self.rgba])
        self.dist_ptrs = (C.c_void_p * n)(*[t.data_ptr() for t in self.dist])

    @property
    def pixels(self) -> int:
        return sum(t.shape[0] * t.shape[1] for t in self.dist)


def render_views(ctx: Context, atmospheres, n_sets: int, set_of_view, cloud, material, textures, views, n_views: int,
                 sizes, luts: LutSet, blue_noise, out: ViewOutputs):
    sov = (C.c_int * n_views)(*set_of_view[:n_views])
    _abi.call("skyr_cloud_render_views", ctx.handle, atmospheres, n_sets, sov, C.byref(cloud), C.byref(material),
              C.byref(textures), views, n_views, C.byref(sizes), _ptr(luts.transmittance),
              _ptr(luts.aerial_perspective_luminance), _ptr(luts.aerial_perspective_transmittance), _ptr(blue_noise),
              out.rgba_ptrs, out.dist_ptrs)


class Graph:
    """A captured, instantiated CUDA graph of a context's calls."""

    def __init__(self, ctx: Context, handle: C.c_void_p):
        self.ctx, self._g = ctx, handle

    def launch(self):
        _abi.call("skyr_graph_launch", self._g)

    def close(self):
        if self._g:
            _abi.call("skyr_graph_destroy", self._g)
            self._g = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


@contextmanager
def capture(ctx: Context):
    """with capture(ctx) as cap: <skyr calls on ctx>  ->  cap.graph"""

    class _Cap:
        graph: Graph | None = None

    cap = _Cap()
    _abi.call("skyr_graph_begin", ctx.handle)
    ok = False
    try:
        yield cap
        ok = True
    finally:
        h = C.c_void_p()
        st = _abi.lib().skyr_graph_end(ctx.handle, C.byref(h))
        if ok:
            _abi.check(st, "skyr_graph_end")
            cap.graph = Graph(ctx, h)
