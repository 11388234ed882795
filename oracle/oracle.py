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


def _host_view(view, froxel, keep):
    """Copy of a skyr_cloud_view whose shadow froxel is the host array `froxel`
    (uint16 [depth][height][width]) or none, so that a device pointer never
    reaches the oracle."""
    if view is None:
        return None
    v = type(view).from_buffer_copy(view)
    if froxel is None:
        v.shadow_froxel = None
        v.shadow_froxel_width = v.shadow_froxel_height = v.shadow_froxel_depth = 0
    else:
        a = np.ascontiguousarray(froxel, dtype=np.uint16)
        assert a.ndim == 3
        keep.append(a)
        v.shadow_froxel = a.ctypes.data
        v.shadow_froxel_depth, v.shadow_froxel_height, v.shadow_froxel_width = a.shape
    return v


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


# ---------------------------------------------------------------------------
# noise and cloud raymarch
# ---------------------------------------------------------------------------
U8 = C.POINTER(C.c_uint8)
I32 = C.POINTER(C.c_int)
F32 = C.POINTER(C.c_float)


def _declare_cloud(lb):
    lb.oracle_noise_generate.restype = C.c_int
    lb.oracle_noise_generate.argtypes = [P, C.c_int, C.c_int, U8]
    lb.oracle_noise_mips.restype = C.c_int
    lb.oracle_noise_mips.argtypes = [P, U8]
    lb.oracle_noise_values.restype = C.c_int
    lb.oracle_noise_values.argtypes = [P, C.c_int, I32, C.c_int, D]
    lb.oracle_wang_hash.restype = C.c_uint32
    lb.oracle_wang_hash.argtypes = [C.c_uint32]
    lb.oracle_pcg_hash.restype = C.c_uint32
    lb.oracle_pcg_hash.argtypes = [C.c_uint32]
    lb.oracle_cloud_render.restype = C.c_int
    lb.oracle_cloud_render.argtypes = [P, P, P, P, P, P, D, D, D, F32, F32, I32, C.c_int, C.c_int, C.c_int, D, D]


_EXT.append(_declare_cloud)


def noise_bytes(desc) -> int:
    total, m = 0, max(desc.width, desc.height, desc.depth)
    levels = m.bit_length()
    for l in range(levels):
        total += max(desc.width >> l, 1) * max(desc.height >> l, 1) * max(desc.depth >> l, 1) * desc.channels
    return total


def noise_generate(desc, precision: int = 64, nthreads: int | None = None) -> np.ndarray:
    out = np.zeros(noise_bytes(desc), dtype=np.uint8)
    assert lib().oracle_noise_generate(_ref(desc), precision, nthreads or threads(),
                                       out.ctypes.data_as(U8)) == 0
    return out


def noise_mips(desc, tex: np.ndarray) -> np.ndarray:
    """Rebuild levels 1.. from level 0 of `tex` (copy)."""
    out = np.ascontiguousarray(tex, dtype=np.uint8).copy()
    assert lib().oracle_noise_mips(_ref(desc), out.ctypes.data_as(U8)) == 0
    return out


def noise_values(desc, channel: int, idx: np.ndarray) -> np.ndarray:
    idx = np.ascontiguousarray(idx, dtype=np.int32)
    out = np.zeros(len(idx))
    assert lib().oracle_noise_values(_ref(desc), channel, idx.ctypes.data_as(I32), len(idx), _dp(out)) == 0
    return out


def wang_hash(x: int) -> int:
    return lib().oracle_wang_hash(x)


def pcg_hash(x: int) -> int:
    return lib().oracle_pcg_hash(x)


def cloud_render(atmo, cloud, material, textures_host: dict, view, sizes, transmittance, ap_lum, ap_trans,
                 blue_noise, depth=None, pixels=None, precision: int = 64, nthreads: int | None = None,
                 froxel: np.ndarray | None = None):
    """Raymarch pixels (flat indices, or all) of `view` with host textures.

    textures_host maps 'cloud_map' / 'detail' / 'displacement' / 'voxel' to
    (desc, uint8 array); `froxel` is the view's shadow froxel on the host."""
    import skyrendering_gb300._abi as A  # struct layout only

    t = A.CloudTextures()
    keep = []
    view = _host_view(view, froxel, keep)
    for name in ("cloud_map", "detail", "displacement", "voxel"):
        if name in textures_host:
            desc, arr = textures_host[name]
            arr = np.ascontiguousarray(arr, dtype=np.uint8)
            keep.append(arr)
            setattr(t, name, arr.ctypes.data)
            setattr(t, name + "_desc", desc)
    n = view.width * view.height if pixels is None else len(pixels)
    px = None if pixels is None else np.ascontiguousarray(pixels, dtype=np.int32)
    rgba = np.zeros((n, 4))
    dist = np.zeros(n)
    bn = np.ascontiguousarray(blue_noise, dtype=np.float32)
    dp = None if depth is None else np.ascontiguousarray(depth, dtype=np.float32)
    tl = np.ascontiguousarray(transmittance, dtype=np.float64)
    al = np.ascontiguousarray(ap_lum, dtype=np.float64)
    at = np.ascontiguousarray(ap_trans, dtype=np.float64)
    rc = lib().oracle_cloud_render(_ref(atmo), _ref(cloud), _ref(material), _ref(t), _ref(view), _ref(sizes),
                                   _dp(tl), _dp(al), _dp(at), bn.ctypes.data_as(F32),
                                   None if dp is None else dp.ctypes.data_as(F32),
                                   None if px is None else px.ctypes.data_as(I32), n, precision,
                                   nthreads or threads(), _dp(rgba), _dp(dist))
    assert rc == 0
    return rgba, dist


# ---------------------------------------------------------------------------
# path tracer
# ---------------------------------------------------------------------------
U16 = C.POINTER(C.c_uint16)
FP = C.POINTER(C.c_float)


def _declare_pt(lb):
    lb.oracle_grid_generate.restype = C.c_int
    lb.oracle_grid_generate.argtypes = [P, C.c_int, C.c_int, D]
    lb.oracle_grid_majorants.restype = C.c_int
    lb.oracle_grid_majorants.argtypes = [P, U16, FP]
    lb.oracle_pathtrace.restype = C.c_int
    lb.oracle_pathtrace.argtypes = [P, P, P, P, P, P, P, P, P, D, D, D, D, D, C.c_uint, C.c_int, I32, C.c_int,
                                    C.c_int, C.c_int, D, D]


_EXT.append(_declare_pt)


def grid_generate(gen, precision: int = 64, nthreads: int | None = None) -> np.ndarray:
    out = np.zeros((gen.nz, gen.ny, gen.nx))
    assert lib().oracle_grid_generate(_ref(gen), precision, nthreads or threads(), _dp(out)) == 0
    return out


def grid_majorants(grid_struct, data_half: np.ndarray) -> np.ndarray:
    d = np.ascontiguousarray(data_half).view(np.uint16)
    b = grid_struct.brick
    shape = tuple((n + b - 1) // b for n in (grid_struct.nz, grid_struct.ny, grid_struct.nx))
    out = np.zeros(shape, dtype=np.float32)
    assert lib().oracle_grid_majorants(_ref(grid_struct), d.ctypes.data_as(U16), out.ctypes.data_as(FP)) == 0
    return out


def pathtrace(atmo, cloud, material, textures_host: dict | None, grid_struct, grid_half: np.ndarray | None,
              majorant: np.ndarray | None, pt, view, env_view, sizes, luts: dict, frame_begin: int, n_frames: int,
              pixels, precision: int = 64, nthreads: int | None = None, froxel: np.ndarray | None = None):
    """Per-pixel (sum, sum of squares) of n_frames path-traced frames."""
    import skyrendering_gb300._abi as A

    keep = []
    view = _host_view(view, froxel, keep)
    env_view = _host_view(env_view, None, keep)
    t = A.CloudTextures()
    for name, (desc, arr) in (textures_host or {}).items():
        arr = np.ascontiguousarray(arr, dtype=np.uint8)
        keep.append(arr)
        setattr(t, name, arr.ctypes.data)
        setattr(t, name + "_desc", desc)
    g = None
    if grid_struct is not None:
        g = A.DensityGrid()
        C.memmove(C.byref(g), C.byref(grid_struct), C.sizeof(g))
        gh = np.ascontiguousarray(grid_half).view(np.uint16)
        keep.append(gh)
        g.data = gh.ctypes.data
        if majorant is not None:
            mj = np.ascontiguousarray(majorant, dtype=np.float32)
            keep.append(mj)
            g.majorant = mj.ctypes.data
        else:
            g.majorant = None
    px = np.ascontiguousarray(pixels, dtype=np.int32)
    n = len(px)
    s, sq = np.zeros((n, 4)), np.zeros((n, 4))
    arrs = [np.ascontiguousarray(luts[k], dtype=np.float64) for k in
            ("transmittance", "sky_view_luminance", "sky_view_transmittance", "aerial_perspective_luminance",
             "aerial_perspective_transmittance")]
    mat = material if material is not None else None
    rc = lib().oracle_pathtrace(_ref(atmo), _ref(cloud), _ref(mat) if mat is not None else _ref(A.CloudMaterial()),
                                _ref(t), _ref(g) if g is not None else None, _ref(pt), _ref(view), _ref(env_view),
                                _ref(sizes), *[_dp(a) for a in arrs], frame_begin, n_frames,
                                px.ctypes.data_as(I32), n, precision, nthreads or threads(), _dp(s), _dp(sq))
    assert rc == 0
    return s, sq


# ---------------------------------------------------------------------------
# surrogate network
# ---------------------------------------------------------------------------
def _declare_mlp(lb):
    lb.oracle_mlp_predict.restype = C.c_int
    lb.oracle_mlp_predict.argtypes = [FP, FP, C.c_int, C.c_int, C.c_int, D]
    lb.oracle_mlp_gradient.restype = C.c_double
    lb.oracle_mlp_gradient.argtypes = [FP, FP, FP, C.c_int, C.c_double, C.c_double, C.c_int, D]
    lb.oracle_mlp_adam.restype = None
    lb.oracle_mlp_adam.argtypes = [D, D, D, D, C.c_int, C.c_double, C.c_double, C.c_double, C.c_double, C.c_int]
    lb.oracle_mlp_param_count.restype = C.c_int


_EXT.append(_declare_mlp)


def _fp(a: np.ndarray):
    assert a.dtype == np.float32 and a.flags.c_contiguous
    return a.ctypes.data_as(FP)


def mlp_predict(params: np.ndarray, x: np.ndarray, mirror: bool = True, nthreads: int | None = None) -> np.ndarray:
    """FP64 forward of the surrogate network: x[n][103] -> y[n][3]."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    xx = np.ascontiguousarray(x, dtype=np.float32)
    y = np.zeros((len(xx), 3))
    assert lib().oracle_mlp_predict(_fp(p), _fp(xx), len(xx), int(mirror), nthreads or threads(), _dp(y)) == 0
    return y


def mlp_gradient(params: np.ndarray, x: np.ndarray, t: np.ndarray, label_scale: float = 1.0,
                 loss_eps: float = 1e-2, mirror: bool = True):
    """(loss, gradient[19331]) of the mean relative-L2 loss, FP64."""
    p = np.ascontiguousarray(params, dtype=np.float32)
    xx = np.ascontiguousarray(x, dtype=np.float32)
    tt = np.ascontiguousarray(t, dtype=np.float32)
    g = np.zeros(lib().oracle_mlp_param_count())
    loss = lib().oracle_mlp_gradient(_fp(p), _fp(xx), _fp(tt), len(xx), label_scale, loss_eps, int(mirror), _dp(g))
    return loss, g


def mlp_adam(p: np.ndarray, m: np.ndarray, v: np.ndarray, g: np.ndarray, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8,
             step: int = 1):
    """In-place FP64 Adam step on float64 arrays."""
    for a in (p, m, v, g):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    lib().oracle_mlp_adam(_dp(p), _dp(m), _dp(v), _dp(g), len(p), lr, b1, b2, eps, step)


# ---------------------------------------------------------------------------
# surrogate: grid lookups, point-source paths, the surrogate raymarch
# ---------------------------------------------------------------------------
def _declare_surrogate(lb):
    lb.oracle_grid_sigma.restype = C.c_int
    lb.oracle_grid_sigma.argtypes = [P, D, C.c_int, D]
    lb.oracle_point_radiance.restype = C.c_int
    lb.oracle_point_radiance.argtypes = [P, P, P, P, P, P, P, D, D, D, D, D, C.c_uint, C.c_int, D, C.c_int, C.c_int,
                                         D, D]
    lb.oracle_surrogate_render.restype = C.c_int
    lb.oracle_surrogate_render.argtypes = [P, P, P, P, P, P, D, D, D, C.POINTER(C.c_uint8), P, FP, C.c_double, C.c_int, C.c_int,
                                           C.c_double, C.c_double, I32, C.c_int, C.c_int, D, D]


_EXT.append(_declare_surrogate)


def _grid_copy(grid_struct, data_half, keep):
    import skyrendering_gb300._abi as A

    g = A.DensityGrid()
    C.memmove(C.byref(g), C.byref(grid_struct), C.sizeof(g))
    gh = np.ascontiguousarray(data_half).view(np.uint16)
    keep.append(gh)
    g.data = gh.ctypes.data
    g.majorant = None
    return g


def grid_sigma(grid_struct, data_half: np.ndarray, points: np.ndarray) -> np.ndarray:
    """FP64 trilinear extinction of the FP16 grid at points[n][3]."""
    keep = []
    g = _grid_copy(grid_struct, data_half, keep)
    pts = np.ascontiguousarray(points, dtype=np.float64)
    out = np.zeros(len(pts))
    assert lib().oracle_grid_sigma(_ref(g), _dp(pts), len(pts), _dp(out)) == 0
    return out


def _lut_arrays(luts: dict, names):
    return [np.ascontiguousarray(luts[k], dtype=np.float64) for k in names]


def point_radiance(atmo, cloud, grid_struct, data_half, pt, view, env_view, sizes, luts: dict, frame_begin: int,
                   n_paths: int, points: np.ndarray, nthreads: int | None = None):
    """Per point (sum, sum of squares) of n_paths point-source path radiances."""
    keep = []
    view = _host_view(view, None, keep)
    env_view = _host_view(env_view, None, keep)
    g = _grid_copy(grid_struct, data_half, keep)
    arrs = _lut_arrays(luts, ("transmittance", "sky_view_luminance", "sky_view_transmittance",
                              "aerial_perspective_luminance", "aerial_perspective_transmittance"))
    pts = np.ascontiguousarray(points, dtype=np.float64)
    s, sq = np.zeros((len(pts), 3)), np.zeros((len(pts), 3))
    rc = lib().oracle_point_radiance(_ref(atmo), _ref(cloud), _ref(g), _ref(pt), _ref(view), _ref(env_view),
                                     _ref(sizes), *[_dp(a) for a in arrs], frame_begin, n_paths, _dp(pts), len(pts),
                                     nthreads or threads(), _dp(s), _dp(sq))
    assert rc == 0
    return s, sq


def surrogate_render(atmo, cloud, grid_struct, data_half, pt, view, sizes, luts: dict, lattice: np.ndarray, fv,
                     params: np.ndarray, out_scale: float, steps: int, use_network: bool, min_t: float,
                     rel_err: float, pixels, nthreads: int | None = None, froxel: np.ndarray | None = None):
    """FP64 surrogate raymarch of listed pixels over the GPU-built lattice bytes:
    (out[n][4] = rgb, transmittance; err[n])."""
    keep = []
    view = _host_view(view, froxel, keep)
    g = _grid_copy(grid_struct, data_half, keep)
    arrs = _lut_arrays(luts, ("transmittance", "aerial_perspective_luminance", "aerial_perspective_transmittance"))
    raw = np.ascontiguousarray(lattice, dtype=np.uint8)  # records, optical depths, mip levels
    p = np.ascontiguousarray(params, dtype=np.float32)
    px = np.ascontiguousarray(pixels, dtype=np.int32)
    out, err = np.zeros((len(px), 4)), np.zeros(len(px))
    rc = lib().oracle_surrogate_render(_ref(atmo), _ref(cloud), _ref(g), _ref(pt), _ref(view), _ref(sizes),
                                       *[_dp(a) for a in arrs], raw.ctypes.data_as(C.POINTER(C.c_uint8)),
                                       _ref(fv), p.ctypes.data_as(FP), out_scale, steps, int(use_network), min_t,
                                       rel_err, px.ctypes.data_as(I32), len(px), nthreads or threads(), _dp(out),
                                       _dp(err))
    assert rc == 0
    return out, err


# ---------------------------------------------------------------------------
# cloud shadow passes
# ---------------------------------------------------------------------------
def _declare_shadow(lb):
    lb.oracle_cloud_light_frame.restype = C.c_int
    lb.oracle_cloud_light_frame.argtypes = [P, P, P, C.c_int, C.c_int, D, FP, D]
    lb.oracle_cloud_shadow_map.restype = C.c_int
    lb.oracle_cloud_shadow_map.argtypes = [P, P, P, P, P, C.c_int, C.c_int, D, C.c_int, F32, D, I32, C.c_int,
                                           C.c_int, D]
    lb.oracle_cloud_shadow_blur.restype = C.c_int
    lb.oracle_cloud_shadow_blur.argtypes = [C.c_int, C.c_int, D, D]
    lb.oracle_cloud_shadow_froxel.restype = C.c_int
    lb.oracle_cloud_shadow_froxel.argtypes = [P, P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, D, D,
                                              C.c_int, U16, D]


_EXT.append(_declare_shadow)


def _textures_struct(textures_host: dict | None, keep):
    import skyrendering_gb300._abi as A  # struct layout only

    t = A.CloudTextures()
    for name, (desc, arr) in (textures_host or {}).items():
        arr = np.ascontiguousarray(arr, dtype=np.uint8)
        keep.append(arr)
        setattr(t, name, arr.ctypes.data)
        setattr(t, name + "_desc", desc)
    return t


def frame_array(frame) -> np.ndarray:
    """A skyr_cloud_light_frame as the oracle's 4 x 16 doubles (light VP,
    inverse, model, reprojection), column-major."""
    return np.concatenate([np.array(frame.light_view_projection[:]), np.array(frame.inverse_light_view_projection[:]),
                           np.array(frame.model[:]), np.array(frame.shadow_map_reproject[:])]).astype(np.float64)


def light_frame(atmo, cloud, view, map_w: int, map_h: int, previous: np.ndarray | None = None,
                wind=None) -> tuple[np.ndarray, bool]:
    """FP64 light transform of a view: (4 x 16 doubles, has_previous)."""
    keep = []
    v = _host_view(view, None, keep)
    out = np.zeros(64)
    prev = None if previous is None else np.ascontiguousarray(previous, dtype=np.float64)
    w = None if wind is None else np.ascontiguousarray(wind, dtype=np.float32)
    has = lib().oracle_cloud_light_frame(_ref(atmo), _ref(cloud), _ref(v), map_w, map_h, _dp(prev),
                                         None if w is None else w.ctypes.data_as(FP), _dp(out))
    return out, bool(has)


def shadow_map(atmo, cloud, material, textures_host, view, map_w: int, map_h: int, frame: np.ndarray,
               has_previous: bool, blue_noise, previous_map=None, texels=None, nthreads: int | None = None):
    """Shadow-map texels (flat indices y * map_w + x, or all): [n][2] (depth, T)."""
    keep = []
    t = _textures_struct(textures_host, keep)
    v = _host_view(view, None, keep)
    fr = np.ascontiguousarray(frame, dtype=np.float64)
    bn = np.ascontiguousarray(blue_noise, dtype=np.float32)
    pm = None if previous_map is None else np.ascontiguousarray(previous_map, dtype=np.float64).reshape(-1)
    n = map_w * map_h if texels is None else len(texels)
    tx = None if texels is None else np.ascontiguousarray(texels, dtype=np.int32)
    out = np.zeros((n, 2))
    rc = lib().oracle_cloud_shadow_map(_ref(atmo), _ref(cloud), _ref(material), _ref(t), _ref(v), map_w, map_h,
                                       _dp(fr), int(has_previous), bn.ctypes.data_as(F32), _dp(pm),
                                       None if tx is None else tx.ctypes.data_as(I32), n, nthreads or threads(),
                                       _dp(out))
    assert rc == 0
    return out


def shadow_blur(raw: np.ndarray) -> np.ndarray:
    """Both blur passes of an [h][w][2] map."""
    r = np.ascontiguousarray(raw, dtype=np.float64)
    h, w = r.shape[:2]
    out = np.zeros_like(r)
    assert lib().oracle_cloud_shadow_blur(w, h, _dp(r.reshape(-1)), _dp(out.reshape(-1))) == 0
    return out


def shadow_froxel(atmo, cloud, material, textures_host, view, frame: np.ndarray, shadow_map_hw2: np.ndarray,
                  froxel_size, nthreads: int | None = None):
    """The R16 shadow froxel [d][h][w] (uint16) and its running means before the
    store (float64) from a blurred [h][w][2] map."""
    keep = []
    t = _textures_struct(textures_host, keep)
    v = _host_view(view, None, keep)
    fr = np.ascontiguousarray(frame, dtype=np.float64)
    m = np.ascontiguousarray(shadow_map_hw2, dtype=np.float64)
    mh, mw = m.shape[:2]
    fw, fh, fd = froxel_size
    out = np.zeros((fd, fh, fw), dtype=np.uint16)
    exact = np.zeros((fd, fh, fw))
    rc = lib().oracle_cloud_shadow_froxel(_ref(atmo), _ref(cloud), _ref(material), _ref(t), _ref(v), mw, mh, fw,
                                          fh, fd, _dp(fr), _dp(m.reshape(-1)), nthreads or threads(),
                                          out.ctypes.data_as(U16), _dp(exact.reshape(-1)))
    assert rc == 0
    return out, exact


# ---------------------------------------------------------------------------
# quarter-resolution cloud pass
# ---------------------------------------------------------------------------
def _declare_quarter(lb):
    lb.oracle_cloud_checkerboard.restype = C.c_int
    lb.oracle_cloud_checkerboard.argtypes = [F32, C.c_int, C.c_int, D]
    lb.oracle_cloud_index.restype = C.c_int
    lb.oracle_cloud_index.argtypes = [D, C.c_int, C.c_int, C.c_float, C.c_float, C.c_int, D]
    lb.oracle_cloud_render_quarter.restype = C.c_int
    lb.oracle_cloud_render_quarter.argtypes = [P, P, P, P, P, P, D, D, D, F32, D, D, I32, C.c_int, C.c_int, D, D]
    lb.oracle_cloud_reconstruct.restype = C.c_int
    lb.oracle_cloud_reconstruct.argtypes = [P, P, P, P, P, FP, C.c_float, C.c_float, C.c_int, D, D, D, D, D, C.c_int,
                                            D]
    lb.oracle_cloud_upscale.restype = C.c_int
    lb.oracle_cloud_upscale.argtypes = [C.c_int, C.c_int, F32, C.c_float, C.c_float, D, D, D, C.c_int, D]


_EXT.append(_declare_quarter)


def _f64(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _f32p(a, keep):
    if a is None:
        return None
    a = np.ascontiguousarray(a, dtype=np.float32)
    keep.append(a)
    return a.ctypes.data_as(F32)


def checkerboard(depth, w: int, h: int) -> np.ndarray:
    """Checkerboard depth [h/2][w/2] of a window depth [h][w] (None: 1)."""
    keep = []
    out = np.zeros((h // 2, w // 2))
    assert lib().oracle_cloud_checkerboard(_f32p(depth, keep), w, h, _dp(out)) == 0
    return out


def index_gen(cb, w: int, h: int, z_near: float, z_far: float, base: int) -> np.ndarray:
    """[qh][qw][2] (index, linear depth) from a checkerboard depth [h/2][w/2]."""
    c = _f64(cb)
    out = np.zeros(((h // 2) // 2, (w // 2) // 2, 2))
    assert lib().oracle_cloud_index(_dp(c), w, h, z_near, z_far, base, _dp(out)) == 0
    return out


def render_quarter(atmo, cloud, material, textures_host, view, sizes, transmittance, ap_lum, ap_trans, blue_noise,
                   index, cb, pixels=None, froxel=None, nthreads: int | None = None):
    """Raymarch quarter texels (flat y * qw + x, or all) at their checkerboard texels."""
    keep = []
    t = _textures_struct(textures_host, keep)
    v = _host_view(view, froxel, keep)
    qw, qh = (view.width // 2) // 2, (view.height // 2) // 2
    n = qw * qh if pixels is None else len(pixels)
    px = None if pixels is None else np.ascontiguousarray(pixels, dtype=np.int32)
    rgba, dist = np.zeros((n, 4)), np.zeros(n)
    bn = np.ascontiguousarray(blue_noise, dtype=np.float32)
    ix, c = _f64(index).reshape(-1), _f64(cb).reshape(-1)
    arrs = [_f64(transmittance), _f64(ap_lum), _f64(ap_trans)]
    rc = lib().oracle_cloud_render_quarter(_ref(atmo), _ref(cloud), _ref(material), _ref(t), _ref(v), _ref(sizes),
                                           *[_dp(a) for a in arrs], bn.ctypes.data_as(F32), _dp(ix), _dp(c),
                                           None if px is None else px.ctypes.data_as(I32), n, nthreads or threads(),
                                           _dp(rgba), _dp(dist))
    assert rc == 0
    return rgba, dist


def reconstruct(atmo, cloud, material, textures_host, view, frame, cb, index, render, rdist, previous,
                nthreads: int | None = None) -> np.ndarray:
    """[h/2][w/2][4] reconstruction; `frame` a skyr_cloud_temporal_frame; previous None: no history."""
    keep = []
    t = _textures_struct(textures_host, keep)
    v = _host_view(view, None, keep)
    hw, hh = view.width // 2, view.height // 2
    out = np.zeros((hh, hw, 4))
    rp = np.ascontiguousarray(frame.reproject[:], dtype=np.float32)
    prev = None if previous is None else _f64(previous).reshape(-1)
    args = [_f64(a).reshape(-1) for a in (cb, index, render, rdist)]
    rc = lib().oracle_cloud_reconstruct(_ref(atmo), _ref(cloud), _ref(material), _ref(t), _ref(v),
                                        rp.ctypes.data_as(FP), frame.z_near, frame.z_far,
                                        int(bool(frame.has_previous)), *[_dp(a) for a in args], _dp(prev),
                                        nthreads or threads(), _dp(out.reshape(-1)))
    assert rc == 0
    return out


def upscale(w: int, h: int, depth, z_near: float, z_far: float, cb, rec, hdr_in,
            nthreads: int | None = None) -> np.ndarray:
    """[h][w][4]: the upscaled reconstruction composited over hdr_in."""
    keep = []
    out = np.zeros((h, w, 4))
    args = [_f64(a).reshape(-1) for a in (cb, rec, hdr_in)]
    rc = lib().oracle_cloud_upscale(w, h, _f32p(depth, keep), z_near, z_far, *[_dp(a) for a in args],
                                    nthreads or threads(), _dp(out.reshape(-1)))
    assert rc == 0
    return out


# ---------------------------------------------------------------------------
# environment cube
# ---------------------------------------------------------------------------
def _declare_env(lb):
    lb.oracle_environment_cube.restype = C.c_int
    lb.oracle_environment_cube.argtypes = [P, P, P, D, D, D, C.c_int, C.c_int, D]
    lb.oracle_environment_seamless.restype = C.c_int
    lb.oracle_environment_seamless.argtypes = [D, C.c_int, C.c_int, D]
    lb.oracle_environment_sh.restype = C.c_int
    lb.oracle_environment_sh.argtypes = [D, C.c_int, C.c_int, D]
    lb.oracle_environment_prefilter.restype = C.c_int
    lb.oracle_environment_prefilter.argtypes = [D, C.c_int, C.c_int, C.c_int, C.c_double, C.c_int, D]


_EXT.append(_declare_env)


def environment_cube(params, render, sizes, transmittance, sky_view_luminance, sky_view_transmittance, size: int,
                     nthreads: int | None = None) -> np.ndarray:
    """Level 0 of the environment cube: [6][size][size][4] (a = 0)."""
    arrs = [_f64(a).reshape(-1) for a in (transmittance, sky_view_luminance, sky_view_transmittance)]
    out = np.zeros((6, size, size, 4))
    rc = lib().oracle_environment_cube(_ref(params), _ref(render), _ref(sizes), *[_dp(a) for a in arrs], size,
                                       nthreads or threads(), _dp(out.reshape(-1)))
    assert rc == 0
    return out


def box_mip(level: np.ndarray) -> np.ndarray:
    """glGenerateTextureMipmap's 2x2 box filter of [6][s][s][4] half values,
    rounded to half: the next level."""
    a = level.astype(np.float64)
    m = ((a[:, 0::2, 0::2] + a[:, 0::2, 1::2]) + (a[:, 1::2, 0::2] + a[:, 1::2, 1::2])) * 0.25
    return m.astype(np.float16)


def environment_sh(cube_texels: np.ndarray, size: int, levels: int) -> np.ndarray:
    """[9][3] SH coefficients of a cube given as its flat texels ([n][4], all levels)."""
    c = _f64(cube_texels).reshape(-1)
    out = np.zeros((9, 3))
    assert lib().oracle_environment_sh(_dp(c), size, levels, _dp(out.reshape(-1))) == 0
    return out


def environment_prefilter(cube_texels: np.ndarray, size: int, levels: int, n: int, roughness: float,
                          nthreads: int | None = None) -> np.ndarray:
    """[6][n][n][3]: one prefiltered level of side n."""
    c = _f64(cube_texels).reshape(-1)
    out = np.zeros((6, n, n, 3))
    assert lib().oracle_environment_prefilter(_dp(c), size, levels, n, roughness, nthreads or threads(),
                                              _dp(out.reshape(-1))) == 0
    return out


def environment_seamless(cube_texels: np.ndarray, size: int, levels: int) -> np.ndarray:
    """The seamless copy ([n][4], apron texels from the adjacent faces) of a cube's flat texels."""
    c = _f64(cube_texels).reshape(-1)
    total = sum(6 * (max(size >> l, 1) + 2) ** 2 for l in range(levels))
    out = np.zeros((total, 4))
    assert lib().oracle_environment_seamless(_dp(c), size, levels, _dp(out.reshape(-1))) == 0
    return out


# ---------------------------------------------------------------------------
# full-screen composite
# ---------------------------------------------------------------------------
def _declare_composite(lb):
    lb.oracle_atmosphere_composite.restype = C.c_int
    lb.oracle_atmosphere_composite.argtypes = [P, P, P, P, D, D, D, D, D, D, P, I32, C.c_int, C.c_int, D]


_EXT.append(_declare_composite)


def atmosphere_composite(params, render, cp, sizes, luts: dict, width: int, height: int, blue_noise=None, depth=None,
                         object_luminance=None, star_map=None, froxel=None, froxel_max_distance: float = 20.0,
                         pixels=None, nthreads: int | None = None) -> np.ndarray:
    """The composite of listed pixels (or all): [n][4].  luts: name -> array
    (transmittance, multiscattering, sky_view_*, aerial_perspective_*)."""
    import skyrendering_gb300._abi as A  # struct layout only

    keep = []
    inp = A.CompositeInputs()
    inp.width, inp.height = width, height

    def host(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt)
        keep.append(a)
        return a.ctypes.data

    inp.depth = host(depth, np.float32)
    inp.object_luminance = host(object_luminance, np.float32)
    inp.blue_noise = host(blue_noise, np.float32)
    if star_map is not None:
        inp.star_map = host(star_map, np.uint8)
        inp.star_height, inp.star_width = star_map.shape[:2]
    if froxel is not None:
        inp.shadow_froxel = host(froxel, np.uint16)
        inp.froxel_depth, inp.froxel_height, inp.froxel_width = froxel.shape
        inp.shadow_froxel_max_distance = froxel_max_distance
    names = ("transmittance", "multiscattering", "sky_view_luminance", "sky_view_transmittance",
             "aerial_perspective_luminance", "aerial_perspective_transmittance")
    arrs = [None if luts.get(k) is None else _f64(luts[k]).reshape(-1) for k in names]
    n = width * height if pixels is None else len(pixels)
    px = None if pixels is None else np.ascontiguousarray(pixels, dtype=np.int32)
    out = np.zeros((n, 4))
    rc = lib().oracle_atmosphere_composite(_ref(params), _ref(render), _ref(cp), _ref(sizes), *[_dp(a) for a in arrs],
                                           _ref(inp), None if px is None else px.ctypes.data_as(I32), n,
                                           nthreads or threads(), _dp(out))
    assert rc == 0
    return out
