"""The allocation-free LUT-set entry point, skyr_update_lut_set_noalloc.

It exists for hosts that cannot let this library allocate device memory: an
engine that hands out every device byte from its own pool or budget, or a
frame loop that must not take cudaMalloc / cudaFree (cudaFree synchronises the
device).  It keeps its per-set constants in a static device table of
SKYR_NOALLOC_MAX_SETS sets instead of a table it would cudaMalloc.

The test calls it through the C ABI twice in a row, with different inputs, and
checks each result against the allocating entry point skyr_update_lut_set
within the LUT tolerance of the other tests (1e-3 maximum relative error per
texel); the second call shows that the shared table is rewritten, not reused
stale.  It also checks the capacity limit.  This file sorts last so that a run
stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

from skyrendering_gb300 import _abi
from skyrendering_gb300 import workloads as W
from skyrendering_gb300.atmosphere import LutSet, _ptr, update_lut_set

pytestmark = pytest.mark.gpu
TOL = 1e-3
NAMES = ("transmittance", "multiscattering", "sky_view_luminance", "sky_view_transmittance",
         "aerial_perspective_luminance", "aerial_perspective_transmittance")


def small_sizes():
    s = W.plain_lut_sizes()
    s.transmittance_width, s.transmittance_height = 64, 16
    s.multiscattering_width, s.multiscattering_height = 16, 16
    s.sky_view_width, s.sky_view_height = 48, 27
    s.aerial_perspective_width = s.aerial_perspective_height = s.aerial_perspective_depth = 16
    return s


def call_noalloc(ctx, params, renders, n, sizes, out):
    return _abi.lib().skyr_update_lut_set_noalloc(
        ctx.handle, params, renders, n, C.byref(sizes), _ptr(out.transmittance), _ptr(out.multiscattering),
        _ptr(out.sky_view_luminance), _ptr(out.sky_view_transmittance), _ptr(out.aerial_perspective_luminance),
        _ptr(out.aerial_perspective_transmittance))


def max_rel(a, b):
    a, b = a[..., :3].astype(np.float64), b[..., :3].astype(np.float64)
    return float((np.abs(a - b) / np.maximum(np.abs(b), 1e-300)).max())


def test_noalloc_matches_allocating_entry_point_on_two_calls(ctx):
    sizes = small_sizes()
    n = 12
    for seed in (21, 22):
        params, renders = W.batched_lut_sets(n, seed=seed)
        want = update_lut_set(ctx, params, renders, sizes)
        got = LutSet.allocate(sizes, n)
        rc = call_noalloc(ctx, params, renders, n, sizes, got)
        assert rc == _abi.SKYR_OK, _abi.lib().skyr_last_error()
        ctx.synchronize()
        for name in NAMES:
            g = getattr(got, name).float().cpu().numpy()
            w = getattr(want, name).float().cpu().numpy()
            assert max_rel(g, w) <= TOL, (seed, name)


def test_noalloc_rejects_more_sets_than_its_table_holds(ctx):
    sizes = small_sizes()
    n = _abi.SKYR_NOALLOC_MAX_SETS + 1
    params = (_abi.AtmosphereParameters * n)()
    renders = (_abi.AtmosphereRenderParameters * n)()
    out = LutSet.allocate(sizes, 1)
    rc = call_noalloc(ctx, params, renders, n, sizes, out)
    assert rc == _abi.SKYR_EINVAL
    assert b"capacity" in _abi.lib().skyr_last_error()
