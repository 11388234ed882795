"""The allocation-free LUT-set entry point, skyr_update_lut_set_noalloc.

It exists for hosts that cannot let this library allocate device memory: an
engine that hands out every device byte from its own pool or budget, or a
frame loop that must not take cudaMalloc / cudaFree (cudaFree synchronises the
device).  It keeps its per-set constants in a static device table of
SKYR_NOALLOC_MAX_SETS sets instead of a table it would cudaMalloc.

The tests call it through the C ABI and check:
  * two calls in a row, with different inputs, against the allocating entry
    point skyr_update_lut_set within the LUT tolerance of the other tests
    (1e-3 maximum relative error per texel), in RGBA32F and RGBA16F storage;
    the second call shows that the shared table is rewritten, not reused stale;
  * a call with only one view-LUT pair, as skyr_update_lut_set allows;
  * that repeated calls leave the device's free memory unchanged (no
    allocation by the call), once a first call has loaded its kernels;
  * the capacity limit, and that a set rejected late in a call is reported.
This file sorts last so that a run stopping at the first failure has run every
other test first.
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


def small_sizes(fmt=_abi.SKYR_FORMAT_RGBA32F):
    s = W.plain_lut_sizes(fmt)
    s.transmittance_width, s.transmittance_height = 64, 16
    s.multiscattering_width, s.multiscattering_height = 16, 16
    s.sky_view_width, s.sky_view_height = 48, 27
    s.aerial_perspective_width = s.aerial_perspective_height = s.aerial_perspective_depth = 16
    return s


def call_noalloc(ctx, params, renders, n, sizes, out, sky_view=True, aerial_perspective=True):
    sv = (_ptr(out.sky_view_luminance), _ptr(out.sky_view_transmittance)) if sky_view else (None, None)
    ap = ((_ptr(out.aerial_perspective_luminance), _ptr(out.aerial_perspective_transmittance))
          if aerial_perspective else (None, None))
    return _abi.lib().skyr_update_lut_set_noalloc(
        ctx.handle, params, renders, n, C.byref(sizes), _ptr(out.transmittance), _ptr(out.multiscattering), *sv, *ap)


def max_rel(a, b):
    a, b = a[..., :3].astype(np.float64), b[..., :3].astype(np.float64)
    return float((np.abs(a - b) / np.maximum(np.abs(b), 1e-300)).max())


@pytest.mark.parametrize("fmt", [_abi.SKYR_FORMAT_RGBA32F, _abi.SKYR_FORMAT_RGBA16F], ids=["rgba32f", "rgba16f"])
def test_noalloc_matches_allocating_entry_point_on_two_calls(ctx, fmt):
    sizes = small_sizes(fmt)
    n = 20  # more than one 16-set upload chunk
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


def test_noalloc_takes_one_view_pair_like_the_allocating_entry_point(ctx):
    sizes = small_sizes()
    n = 3
    params, renders = W.batched_lut_sets(n, seed=23)
    want = update_lut_set(ctx, params, renders, sizes)
    got = LutSet.allocate(sizes, n)
    got.sky_view_luminance.fill_(-1.0)
    rc = call_noalloc(ctx, params, renders, n, sizes, got, sky_view=False)
    assert rc == _abi.SKYR_OK, _abi.lib().skyr_last_error()
    ctx.synchronize()
    for name in ("transmittance", "multiscattering", "aerial_perspective_luminance",
                 "aerial_perspective_transmittance"):
        assert max_rel(getattr(got, name).cpu().numpy(), getattr(want, name).cpu().numpy()) <= TOL, name
    assert bool((got.sky_view_luminance == -1.0).all())  # the left-out LUT is not written
    rc = _abi.lib().skyr_update_lut_set_noalloc(ctx.handle, params, renders, n, C.byref(sizes),
                                                _ptr(got.transmittance), _ptr(got.multiscattering),
                                                _ptr(got.sky_view_luminance), None, None, None)
    assert rc == _abi.SKYR_EINVAL


def test_noalloc_calls_leave_free_device_memory_unchanged(ctx, cuda):
    torch = cuda
    n = _abi.SKYR_NOALLOC_MAX_SETS
    params, renders = W.batched_lut_sets(n, seed=24)
    outs = {f: (small_sizes(f), LutSet.allocate(small_sizes(f), n))
            for f in (_abi.SKYR_FORMAT_RGBA32F, _abi.SKYR_FORMAT_RGBA16F)}
    for sizes, out in outs.values():  # first calls: kernels loaded, the table's address looked up
        assert call_noalloc(ctx, params, renders, n, sizes, out) == _abi.SKYR_OK, _abi.lib().skyr_last_error()
    ctx.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for k in (1, 17, n):
        for sizes, out in outs.values():
            assert call_noalloc(ctx, params, renders, k, sizes, out) == _abi.SKYR_OK
    ctx.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0


def test_noalloc_rejects_more_sets_than_its_table_holds(ctx):
    sizes = small_sizes()
    n = _abi.SKYR_NOALLOC_MAX_SETS + 1
    params = (_abi.AtmosphereParameters * n)()
    renders = (_abi.AtmosphereRenderParameters * n)()
    out = LutSet.allocate(sizes, 1)
    rc = call_noalloc(ctx, params, renders, n, sizes, out)
    assert rc == _abi.SKYR_EINVAL
    assert b"capacity" in _abi.lib().skyr_last_error()


def test_noalloc_reports_a_bad_set_after_the_first_upload_chunk(ctx):
    sizes = small_sizes()
    n = 40
    params, renders = W.batched_lut_sets(n, seed=25)
    params[33].bottom_radius = float("nan")
    out = LutSet.allocate(sizes, n)
    rc = call_noalloc(ctx, params, renders, n, sizes, out)
    assert rc == _abi.SKYR_EINVAL
    assert b"33" in _abi.lib().skyr_last_error()
