"""Host-side mirror of the reference's atmosphere classes over the C ABI.

* ``Atmosphere.update_luts`` ~ Atmosphere::UpdateLuts
  (src/SkyRendering/Atmosphere.cpp:101-124): transmittance + multi-scattering.
* ``AtmosphereRenderer.render_luts`` ~ the SKY_VIEW / AERIAL_PERSPECTIVE passes
  of AtmosphereRenderer::Render (src/SkyRendering/AtmosphereRenderer.cpp:164-233).
* ``update_lut_set`` runs both for one or many (parameter set, view) pairs.

Device memory comes from torch (plumbing only); every kernel is a libskyr.so
kernel.  Errors raise ``SkyrError`` carrying the C status.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass

import torch

from . import _abi


class Context:
    """A skyr_ctx bound to a CUDA stream (default: torch's current stream)."""

    def __init__(self, stream: torch.cuda.Stream | None = None, device: int | None = None):
        if not torch.cuda.is_available():
            raise RuntimeError("skyrendering_gb300 requires a CUDA device")
        if device is not None:
            torch.cuda.set_device(device)
        self.stream = stream if stream is not None else torch.cuda.current_stream()
        self._ctx = C.c_void_p()
        _abi.call("skyr_ctx_create", C.c_void_p(self.stream.cuda_stream), C.byref(self._ctx))

    @property
    def handle(self) -> C.c_void_p:
        return self._ctx

    def synchronize(self) -> None:
        _abi.call("skyr_ctx_synchronize", self._ctx)

    def check_status(self) -> None:
        """Synchronise and raise SkyrError if a kernel of this context raised
        its device status word (a tracking walk that hit its iteration cap)."""
        _abi.call("skyr_ctx_check_status", self._ctx)

    @property
    def limits(self) -> _abi.DeviceLimits:
        """The bounds of this context's device loops (skyr_device_limits)."""
        out = _abi.DeviceLimits()
        _abi.call("skyr_ctx_get_limits", self._ctx, C.byref(out))
        return out

    @limits.setter
    def limits(self, value: _abi.DeviceLimits) -> None:
        _abi.call("skyr_ctx_set_limits", self._ctx, C.byref(value))

    def close(self) -> None:
        if self._ctx:
            _abi.call("skyr_ctx_destroy", self._ctx)
            self._ctx = C.c_void_p()

    def __del__(self):  # best effort
        try:
            self.close()
        except Exception:
            pass


def _ptr(t: torch.Tensor | None) -> C.c_void_p:
    return C.c_void_p(0 if t is None else t.data_ptr())


def texel_channels(fmt: int):
    return (torch.float16, 4) if fmt == _abi.SKYR_FORMAT_RGBA16F else (torch.float32, 4)


@dataclass
class LutSet:
    """Device LUTs of n parameter sets, shaped (n, [D,] H, W, 4)."""

    transmittance: torch.Tensor
    multiscattering: torch.Tensor
    sky_view_luminance: torch.Tensor | None = None
    sky_view_transmittance: torch.Tensor | None = None
    aerial_perspective_luminance: torch.Tensor | None = None
    aerial_perspective_transmittance: torch.Tensor | None = None

    @staticmethod
    def allocate(sizes: _abi.LutSizes, n: int = 1, views: bool = True, device="cuda") -> "LutSet":
        dt, c = texel_channels(sizes.format)
        t = torch.empty((n, sizes.transmittance_height, sizes.transmittance_width, 4), dtype=torch.float32,
                        device=device)
        ms = torch.empty((n, sizes.multiscattering_height, sizes.multiscattering_width, c), dtype=dt, device=device)
        out = LutSet(t, ms)
        if views:
            out.sky_view_luminance = torch.empty((n, sizes.sky_view_height, sizes.sky_view_width, c), dtype=dt,
                                                 device=device)
            out.sky_view_transmittance = torch.empty_like(out.sky_view_luminance)
            shape = (n, sizes.aerial_perspective_depth, sizes.aerial_perspective_height,
                     sizes.aerial_perspective_width, c)
            out.aerial_perspective_luminance = torch.empty(shape, dtype=dt, device=device)
            out.aerial_perspective_transmittance = torch.empty_like(out.aerial_perspective_luminance)
        return out


def _as_array(items, ctype):
    if isinstance(items, ctype):
        arr = (ctype * 1)()
        arr[0] = items
        return arr, 1
    if isinstance(items, C.Array):
        return items, len(items)
    arr = (ctype * len(items))(*items)
    return arr, len(items)


class Atmosphere:
    """Atmosphere (src/SkyRendering/Atmosphere.h:70-92)."""

    def __init__(self, ctx: Context, sizes: _abi.LutSizes):
        self.ctx, self.sizes = ctx, sizes

    def update_luts(self, params, out: LutSet | None = None) -> LutSet:
        arr, n = _as_array(params, _abi.AtmosphereParameters)
        out = out or LutSet.allocate(self.sizes, n, views=False)
        _abi.call("skyr_update_luts", self.ctx.handle, arr, n, C.byref(self.sizes), _ptr(out.transmittance),
                  _ptr(out.multiscattering))
        return out


class AtmosphereRenderer:
    """LUT passes of AtmosphereRenderer (src/SkyRendering/AtmosphereRenderer.h:86-132)."""

    def __init__(self, ctx: Context, sizes: _abi.LutSizes):
        self.ctx, self.sizes = ctx, sizes

    def render_luts(self, params, render, luts: LutSet) -> LutSet:
        pa, n = _as_array(params, _abi.AtmosphereParameters)
        ra, m = _as_array(render, _abi.AtmosphereRenderParameters)
        if n != m:
            raise ValueError("one render parameter block per atmosphere parameter set")
        if luts.sky_view_luminance is None:
            full = LutSet.allocate(self.sizes, n, views=True)
            full.transmittance, full.multiscattering = luts.transmittance, luts.multiscattering
            luts = full
        _abi.call("skyr_render_view_luts", self.ctx.handle, pa, ra, n, C.byref(self.sizes),
                  _ptr(luts.transmittance), _ptr(luts.multiscattering), _ptr(luts.sky_view_luminance),
                  _ptr(luts.sky_view_transmittance), _ptr(luts.aerial_perspective_luminance),
                  _ptr(luts.aerial_perspective_transmittance))
        return luts


def update_lut_set(ctx: Context, params, render, sizes: _abi.LutSizes, out: LutSet | None = None) -> LutSet:
    pa, n = _as_array(params, _abi.AtmosphereParameters)
    ra, m = _as_array(render, _abi.AtmosphereRenderParameters)
    if n != m:
        raise ValueError("one render parameter block per atmosphere parameter set")
    out = out or LutSet.allocate(sizes, n, views=True)
    _abi.call("skyr_update_lut_set", ctx.handle, pa, ra, n, C.byref(sizes), _ptr(out.transmittance),
              _ptr(out.multiscattering), _ptr(out.sky_view_luminance), _ptr(out.sky_view_transmittance),
              _ptr(out.aerial_perspective_luminance), _ptr(out.aerial_perspective_transmittance))
    return out


def environment_cube_levels(face_size: int) -> list[tuple[int, int]]:
    """(offset in half4 texels, side) of each level of a face_size cube."""
    n = face_size.bit_length()
    return [(_abi.lib().skyr_environment_cube_level_offset(face_size, l), max(face_size >> l, 1)) for l in range(n)]


def environment_cube(ctx: Context, atmosphere: _abi.AtmosphereParameters,
                     render: _abi.AtmosphereRenderParameters, sizes: _abi.LutSizes, luts: "LutSet",
                     face_size: int = 128, levels: int | None = None, out: torch.Tensor | None = None,
                     set_index: int = 0) -> list[torch.Tensor]:
    """AtmosphereRenderer's environment luminance cube (128^2 x 6 RGBA16F in the
    reference) with its box-filtered mip chain: one [6][s][s][4] half view per level."""
    n = face_size.bit_length() if levels is None else levels
    total = _abi.lib().skyr_environment_cube_level_offset(face_size, n)
    if total == 0:
        raise _abi.SkyrError(_abi.SKYR_EINVAL, "environment_cube", "bad face size or level count")
    if out is None:
        out = torch.empty((total, 4), dtype=torch.float16, device="cuda")
    s = set_index
    _abi.call("skyr_environment_cube", ctx.handle, C.byref(atmosphere), C.byref(render), C.byref(sizes),
              _ptr(luts.transmittance[s]), _ptr(luts.sky_view_luminance[s]), _ptr(luts.sky_view_transmittance[s]),
              face_size, n, _ptr(out))
    views = []
    for off, side in environment_cube_levels(face_size)[:n]:
        views.append(out[off:off + 6 * side * side].view(6, side, side, 4))
    return views


def environment_seamless(ctx: Context, cube: torch.Tensor, face_size: int, levels: int,
                         out: torch.Tensor | None = None) -> torch.Tensor:
    """The cube's seamless copy (each face with a one-texel apron from its
    neighbours), float4 texels: the input of the IBL passes."""
    total = _abi.lib().skyr_environment_seamless_level_offset(face_size, levels)
    if total == 0:
        raise _abi.SkyrError(_abi.SKYR_EINVAL, "environment_seamless", "bad face size or level count")
    if out is None:
        out = torch.empty((total, 4), dtype=torch.float32, device="cuda")
    _abi.call("skyr_environment_seamless", ctx.handle, _ptr(cube), face_size, levels, _ptr(out))
    return out


def environment_sh(ctx: Context, seamless: torch.Tensor, face_size: int, levels: int,
                   out: torch.Tensor | None = None) -> torch.Tensor:
    """IBL's 9 spherical-harmonic radiance coefficients: [9][4] float (a = 0)."""
    if out is None:
        out = torch.empty((9, 4), dtype=torch.float32, device="cuda")
    _abi.call("skyr_environment_sh", ctx.handle, _ptr(seamless), face_size, levels, _ptr(out))
    return out


def environment_prefilter(ctx: Context, seamless: torch.Tensor, face_size: int, levels: int, resolution: int = 128,
                          roughness_count: int = 5, out: torch.Tensor | None = None) -> list[torch.Tensor]:
    """IBL's GGX-prefiltered radiance (128^2 cube, 5 roughness levels in the
    reference): one [6][s][s][4] half view per roughness level."""
    total = _abi.lib().skyr_environment_cube_level_offset(resolution, roughness_count)
    if total == 0:
        raise _abi.SkyrError(_abi.SKYR_EINVAL, "environment_prefilter", "bad resolution or roughness count")
    if out is None:
        out = torch.empty((total, 4), dtype=torch.float16, device="cuda")
    _abi.call("skyr_environment_prefilter", ctx.handle, _ptr(seamless), face_size, levels, resolution,
              roughness_count, _ptr(out))
    return [out[off:off + 6 * side * side].view(6, side, side, 4)
            for off, side in environment_cube_levels(resolution)[:roughness_count]]


def composite_parameters(**overrides) -> _abi.CompositeParameters:
    """AtmosphereRenderer's composite parameters (reference defaults: per-pixel
    raymarch of 40 dithered samples, star scale 0.005), with overrides."""
    cp = _abi.CompositeParameters()
    _abi.call("skyr_composite_parameters_default", C.byref(cp))
    for k, v in overrides.items():
        setattr(cp, k, v)
    return cp


def composite(ctx: Context, atmosphere: _abi.AtmosphereParameters, render: _abi.AtmosphereRenderParameters,
              parameters: _abi.CompositeParameters, sizes: _abi.LutSizes, luts: "LutSet", width: int, height: int,
              blue_noise: torch.Tensor | None = None, depth: torch.Tensor | None = None,
              object_luminance: torch.Tensor | None = None, star_map: torch.Tensor | None = None,
              shadow_froxel: torch.Tensor | None = None, shadow_froxel_max_distance: float = 20.0,
              out: torch.Tensor | None = None, set_index: int = 0) -> torch.Tensor:
    """The full-screen atmosphere composite (AtmosphereRenderer's
    ATMOSPHERE_RENDER pass) into a [height][width][4] half HDR target.
    star_map: uint8 [h][w][3] sRGB; shadow_froxel: int16 words [d][h][w]."""
    if out is None:
        out = torch.empty((height, width, 4), dtype=torch.float16, device="cuda")
    inp = _abi.CompositeInputs()
    inp.width, inp.height = width, height
    inp.depth = None if depth is None else depth.data_ptr()
    inp.object_luminance = None if object_luminance is None else object_luminance.data_ptr()
    inp.blue_noise = None if blue_noise is None else blue_noise.data_ptr()
    if star_map is not None:
        inp.star_map = star_map.data_ptr()
        inp.star_height, inp.star_width = star_map.shape[0], star_map.shape[1]
    if shadow_froxel is not None:
        inp.shadow_froxel = shadow_froxel.data_ptr()
        inp.froxel_depth, inp.froxel_height, inp.froxel_width = shadow_froxel.shape
        inp.shadow_froxel_max_distance = shadow_froxel_max_distance
    s = set_index
    L = luts
    _abi.call("skyr_atmosphere_composite", ctx.handle, C.byref(atmosphere), C.byref(render), C.byref(parameters),
              C.byref(sizes), _ptr(L.transmittance[s]), _ptr(L.multiscattering[s]), _ptr(L.sky_view_luminance[s]),
              _ptr(L.sky_view_transmittance[s]), _ptr(L.aerial_perspective_luminance[s]),
              _ptr(L.aerial_perspective_transmittance[s]), C.byref(inp), _ptr(out))
    return out
