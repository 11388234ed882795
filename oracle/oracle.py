"""ctypes wrapper of the CPU oracle — TEST INFRASTRUCTURE ONLY.

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may use
this module, and only as the checker / the timed CPU baseline.  The product
(skyrendering_gb300) never imports it.

Parity status: unpinned — the reference ships no tests or golden vectors and
its GLSL path cannot run here; the oracle is pinned by analytic known-answer
tests only (see tests/test_oracle_kat.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "liboracle.so"

_lib = None


def build() -> Path:
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(str(LIB))
        _declare(_lib)
    return _lib


def threads() -> int:
    return int(os.environ.get("SKYR_ORACLE_THREADS", os.cpu_count() or 1))


P = C.c_void_p
D = C.POINTER(C.c_double)


def _declare(lb):
    lb.oracle_lut_set.restype = C.c_int
    lb.oracle_lut_set.argtypes = [P, P, P, C.c_int, C.c_int, D, D, D, D, D, D]
    lb.oracle_multiscattering.restype = C.c_int
    lb.oracle_multiscattering.argtypes = [P, P, D, C.c_int, D]
    lb.oracle_view_luts.restype = C.c_int
    lb.oracle_view_luts.argtypes = [P, P, P, D, D, C.c_int, D, D, D, D]
    lb.oracle_transmittance_at.restype = C.c_int
    lb.oracle_transmittance_at.argtypes = [P, C.c_double, C.c_double, D]
    _declare_ext(lb)


_EXT = []


def _declare_ext(lb):
    for fn in _EXT:
        fn(lb)


def _dp(a: np.ndarray | None):
    if a is None:
        return None
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(D)


def _ref(x):
    return C.cast(C.byref(x), P) if x is not None else None


def lut_set(params, render, sizes, precision: int = 64, views: bool = True, nthreads: int | None = None):
    """Whole LUT set of one parameter set (dict of float64 arrays, RGBA, x fastest)."""
    t = np.zeros((sizes.transmittance_height, sizes.transmittance_width, 4))
    ms = np.zeros((sizes.multiscattering_height, sizes.multiscattering_width, 4))
    out = {"transmittance": t, "multiscattering": ms}
    svl = svt = apl = apt = None
    if views:
        svl = np.zeros((sizes.sky_view_height, sizes.sky_view_width, 4))
        svt = np.zeros_like(svl)
        shape = (sizes.aerial_perspective_depth, sizes.aerial_perspective_height, sizes.aerial_perspective_width, 4)
        apl = np.zeros(shape)
        apt = np.zeros(shape)
        out.update(sky_view_luminance=svl, sky_view_transmittance=svt, aerial_perspective_luminance=apl,
                   aerial_perspective_transmittance=apt)
    rc = lib().oracle_lut_set(_ref(params), _ref(render) if views else None, _ref(sizes), precision,
                              nthreads or threads(), _dp(t), _dp(ms), _dp(svl), _dp(svt), _dp(apl), _dp(apt))
    assert rc == 0
    return out


def multiscattering_from(params, sizes, transmittance: np.ndarray, nthreads: int | None = None) -> np.ndarray:
    t = np.ascontiguousarray(transmittance, dtype=np.float64)
    ms = np.zeros((sizes.multiscattering_height, sizes.multiscattering_width, 4))
    assert lib().oracle_multiscattering(_ref(params), _ref(sizes), _dp(t), nthreads or threads(), _dp(ms)) == 0
    return ms


def view_luts_from(params, render, sizes, transmittance, multiscattering, nthreads: int | None = None):
    t = np.ascontiguousarray(transmittance, dtype=np.float64)
    m = np.ascontiguousarray(multiscattering, dtype=np.float64)
    svl = np.zeros((sizes.sky_view_height, sizes.sky_view_width, 4))
    svt = np.zeros_like(svl)
    shape = (sizes.aerial_perspective_depth, sizes.aerial_perspective_height, sizes.aerial_perspective_width, 4)
    apl, apt = np.zeros(shape), np.zeros(shape)
    assert lib().oracle_view_luts(_ref(params), _ref(render), _ref(sizes), _dp(t), _dp(m), nthreads or threads(),
                                  _dp(svl), _dp(svt), _dp(apl), _dp(apt)) == 0
    return {"sky_view_luminance": svl, "sky_view_transmittance": svt, "aerial_perspective_luminance": apl,
            "aerial_perspective_transmittance": apt}


def transmittance_at(params, r: float, mu: float) -> np.ndarray:
    out = np.zeros(3)
    assert lib().oracle_transmittance_at(_ref(params), r, mu, _dp(out)) == 0
    return out
