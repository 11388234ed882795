"""Host-side mirror of the reference's volumetric-cloud classes over the C ABI.

* ``NoiseTexture`` ~ DynamicTexture (src/SkyRendering/VolumetricCloudDefaultMaterial.h:20-55):
  a generated UNORM8 texture with its mip chain, regenerated when its
  parameters change (GenerateIfParameterChanged).
* ``VolumetricCloud.render`` ~ the raymarch pass of VolumetricCloud::Render
  (src/SkyRendering/VolumetricCloud.cpp:361-385) at full resolution.
* ``CloudShadow`` ~ VolumetricCloud::RenderShadow (VolumetricCloud.cpp:282-325)
  with its state: the raw shadow maps used in turn, the blurred map, the
  shadow froxel and the previous frame's light transform.
* ``CloudViewport`` ~ VolumetricCloud::Render's quarter-resolution pass with
  its ViewportData (VolumetricCloud.cpp:120-136,327-423): checkerboard depth,
  index, quarter-resolution raymarch, temporal reconstruction, upscale.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _abi
from .atmosphere import Context, LutSet, _ptr


class NoiseTexture:
    def __init__(self, desc: _abi.NoiseTextureDesc, device="cuda"):
        self.desc = desc
        lib = _abi.lib()
        self.levels = lib.skyr_noise_texture_levels(C.byref(desc))
        if self.levels == 0:
            _abi.check(_abi.SKYR_EINVAL, "skyr_noise_texture_levels")
        self.nbytes = lib.skyr_noise_level_offset(C.byref(desc), self.levels)
        self.data = torch.empty(self.nbytes, dtype=torch.uint8, device=device)
        self.expanded = None
        self.expanded_channels = 0
        self._sampler = C.c_void_p()
        self._sampler_ctx = None
        self._generated = None

    def level_offset(self, level: int) -> int:
        return _abi.lib().skyr_noise_level_offset(C.byref(self.desc), level)

    def level(self, level: int) -> torch.Tensor:
        """Level `level` as a (channels, d, h, w) view."""
        d = self.desc
        w, h, dd = max(d.width >> level, 1), max(d.height >> level, 1), max(d.depth >> level, 1)
        o = self.level_offset(level)
        return self.data[o:o + w * h * dd * d.channels].view(d.channels, dd, h, w)

    def generate(self, ctx: Context) -> "NoiseTexture":
        _abi.call("skyr_noise_generate", ctx.handle, C.byref(self.desc), _ptr(self.data))
        self._generated = bytes(self.desc)
        if self.expanded is not None:
            self.expand(ctx, self.expanded_channels)
        if self._sampler:  # the same handle, refreshed: textures structs that hold it stay valid
            _abi.call("skyr_noise_sampler_update", ctx.handle, self._sampler, _ptr(self.data))
        return self

    def make_sampler(self, ctx: Context) -> "NoiseTexture":
        """(Re)build the hardware sampler of channel 0 of level 0 (skyr_noise_sampler):
        GL LINEAR / REPEAT / UNORM8 filtering in the texture units."""
        self.close_sampler()
        _abi.call("skyr_noise_sampler_create", ctx.handle, C.byref(self.desc), _ptr(self.data), 0,
                  C.byref(self._sampler))
        self._sampler_ctx = ctx
        return self

    @property
    def sampler(self) -> int:
        """The LINEAR level-0 sampler's texture-object handle, 0 without one."""
        return int(_abi.lib().skyr_noise_sampler_handle(self._sampler)) if self._sampler else 0

    @property
    def sampler_nearest(self) -> int:
        """The NEAREST every-level sampler's texture-object handle, 0 without one."""
        return int(_abi.lib().skyr_noise_sampler_nearest_handle(self._sampler)) if self._sampler else 0

    def close_sampler(self) -> None:
        if self._sampler:
            if self._sampler_ctx is not None:
                self._sampler_ctx.synchronize()  # no launch in flight may still read it
            _abi.call("skyr_noise_sampler_destroy", self._sampler)
            self._sampler = C.c_void_p()

    def __del__(self):  # best effort
        try:
            self.close_sampler()
        except Exception:
            pass

    def expand(self, ctx: Context, channels: int) -> "NoiseTexture":
        """Build the filtering layout of level 0 for the first `channels` channels."""
        n = _abi.lib().skyr_noise_expanded_bytes(C.byref(self.desc), channels)
        if n == 0:
            _abi.check(_abi.SKYR_EINVAL, "skyr_noise_expanded_bytes")
        if self.expanded is None or self.expanded.numel() != n:
            self.expanded = torch.empty(n, dtype=torch.uint8, device=self.data.device)
        _abi.call("skyr_noise_expand", ctx.handle, C.byref(self.desc), _ptr(self.data), channels,
                  _ptr(self.expanded))
        self.expanded_channels = channels
        return self

    def generate_if_parameter_changed(self, ctx: Context) -> bool:
        if self._generated != bytes(self.desc):
            self.generate(ctx)
            return True
        return False


def textures_struct(cloud_map: NoiseTexture | None = None, detail: NoiseTexture | None = None,
                    displacement: NoiseTexture | None = None, voxel: NoiseTexture | None = None):
    t = _abi.CloudTextures()
    # The struct holds raw device pointers and sampler handles: it keeps the
    # textures alive, so a sampler is not destroyed (nor a buffer reused) while
    # a renderer that holds the struct can still launch with it.
    t._owners = [x for x in (cloud_map, detail, displacement, voxel) if x is not None]
    for name, tex in (("cloud_map", cloud_map), ("detail", detail), ("displacement", displacement),
                      ("voxel", voxel)):
        if tex is not None:
            setattr(t, name, tex.data.data_ptr())
            setattr(t, name + "_desc", tex.desc)
            if tex.expanded is not None:
                setattr(t, name + "_expanded", tex.expanded.data_ptr())
                setattr(t, name + "_expanded_channels", tex.expanded_channels)
            if name in ("cloud_map", "detail") and tex.sampler:
                setattr(t, name + "_sampler", tex.sampler)
                setattr(t, name + "_sampler_nearest", tex.sampler_nearest)
    return t


# channels of each texture that a material's SampleSigmaT filters at level 0
MATERIAL_CHANNELS = {
    _abi.SKYR_MATERIAL_DEFAULT1: {"cloud_map": 1, "detail": 1},
    _abi.SKYR_MATERIAL_DEFAULT0: {"cloud_map": 2, "detail": 1, "displacement": 4},
    _abi.SKYR_MATERIAL_MINIMAL: {},
    _abi.SKYR_MATERIAL_VOXEL: {},
}


def prepare_textures(ctx: Context, material_type: int, textures: dict, samplers: bool = True) -> dict:
    """Expand the level-0 channels that `material_type` filters (exact re-layout) and,
    for Material1 with `samplers`, build the hardware samplers of its two textures."""
    for name, ch in MATERIAL_CHANNELS[material_type].items():
        if name in textures and textures[name].expanded_channels < ch:
            textures[name].expand(ctx, ch)
        if samplers and material_type == _abi.SKYR_MATERIAL_DEFAULT1 and name in textures and \
                not textures[name].sampler:
            textures[name].make_sampler(ctx)
    return textures


class VolumetricCloud:
    """VolumetricCloud (src/SkyRendering/VolumetricCloud.h:16-193): parameters,
    material and the textures its material samples."""

    def __init__(self, ctx: Context, params: _abi.CloudParameters, material: _abi.CloudMaterial,
                 textures: _abi.CloudTextures):
        self.ctx, self.params, self.material, self.textures = ctx, params, material, textures

    def render(self, atmosphere: _abi.AtmosphereParameters, view: _abi.CloudView, sizes: _abi.LutSizes,
               luts: LutSet, blue_noise: torch.Tensor, depth: torch.Tensor | None = None,
               out_rgba: torch.Tensor | None = None, out_distance: torch.Tensor | None = None):
        if out_rgba is None:
            out_rgba = torch.empty((view.height, view.width, 4), dtype=torch.float16, device="cuda")
        if out_distance is None:
            out_distance = torch.empty((view.height, view.width), dtype=torch.float32, device="cuda")
        _abi.call("skyr_cloud_render", self.ctx.handle, C.byref(atmosphere), C.byref(self.params),
                  C.byref(self.material), C.byref(self.textures), C.byref(view), C.byref(sizes),
                  _ptr(luts.transmittance), _ptr(luts.aerial_perspective_luminance),
                  _ptr(luts.aerial_perspective_transmittance), _ptr(blue_noise), _ptr(depth), _ptr(out_rgba),
                  _ptr(out_distance))
        return out_rgba, out_distance

    def render_to_host(self, atmosphere: _abi.AtmosphereParameters, view: _abi.CloudView, sizes: _abi.LutSizes,
                       luts: LutSet, blue_noise: torch.Tensor, depth: torch.Tensor | None = None,
                       out_rgba: torch.Tensor | None = None, out_distance: torch.Tensor | None = None):
        """render() with the frame stored by the kernel straight into pinned
        host tensors (skyr_cloud_render_to_host); valid once the context's
        stream has passed the call."""
        if out_rgba is None:
            out_rgba = torch.empty((view.height, view.width, 4), dtype=torch.float16, pin_memory=True)
        if out_distance is None:
            out_distance = torch.empty((view.height, view.width), dtype=torch.float32, pin_memory=True)
        _abi.call("skyr_cloud_render_to_host", self.ctx.handle, C.byref(atmosphere), C.byref(self.params),
                  C.byref(self.material), C.byref(self.textures), C.byref(view), C.byref(sizes),
                  _ptr(luts.transmittance), _ptr(luts.aerial_perspective_luminance),
                  _ptr(luts.aerial_perspective_transmittance), _ptr(blue_noise), _ptr(depth), _ptr(out_rgba),
                  _ptr(out_distance))
        return out_rgba, out_distance

    def render_frame(self, atmosphere: _abi.AtmosphereParameters, render: _abi.AtmosphereRenderParameters,
                     view: _abi.CloudView, sizes: _abi.LutSizes, luts: LutSet, blue_noise: torch.Tensor,
                     depth: torch.Tensor | None = None, out_rgba: torch.Tensor | None = None,
                     out_distance: torch.Tensor | None = None, on_host: bool = False):
        """One frame (skyr_render_frame): the LUT set of (atmosphere, render)
        into `luts` (set 0), then render() -- or render_to_host() with
        `on_host` -- reading it, the raymarch overlapping the LUT set's end."""
        if out_rgba is None:
            out_rgba = (torch.empty((view.height, view.width, 4), dtype=torch.float16, pin_memory=True) if on_host
                        else torch.empty((view.height, view.width, 4), dtype=torch.float16, device="cuda"))
        if out_distance is None:
            out_distance = (torch.empty((view.height, view.width), dtype=torch.float32, pin_memory=True) if on_host
                            else torch.empty((view.height, view.width), dtype=torch.float32, device="cuda"))
        _abi.call("skyr_render_frame", self.ctx.handle, C.byref(atmosphere), C.byref(render), C.byref(sizes),
                  _ptr(luts.transmittance), _ptr(luts.multiscattering), _ptr(luts.sky_view_luminance),
                  _ptr(luts.sky_view_transmittance), _ptr(luts.aerial_perspective_luminance),
                  _ptr(luts.aerial_perspective_transmittance), C.byref(self.params), C.byref(self.material),
                  C.byref(self.textures), C.byref(view), _ptr(blue_noise), _ptr(depth), _ptr(out_rgba),
                  _ptr(out_distance), 1 if on_host else 0)
        return out_rgba, out_distance


def shadow_sizes(viewport_width: int, viewport_height: int) -> _abi.CloudShadowSizes:
    """512 x 512 map, (w / 12) x (h / 12) x 128 froxel (VolumetricCloud.cpp:52,134-135)."""
    s = _abi.CloudShadowSizes()
    _abi.call("skyr_cloud_shadow_sizes_default", viewport_width, viewport_height, C.byref(s))
    return s


def light_frame(atmosphere: _abi.AtmosphereParameters, params: _abi.CloudParameters, view: _abi.CloudView,
                sizes: _abi.CloudShadowSizes, previous: _abi.CloudLightFrame | None = None,
                wind_delta=None) -> _abi.CloudLightFrame:
    """The light transform of VolumetricCloud::Update for a view (host only)."""
    out = _abi.CloudLightFrame()
    wind = None if wind_delta is None else (C.c_float * 2)(*wind_delta)
    _abi.call("skyr_cloud_light_frame_derive", C.byref(atmosphere), C.byref(params), C.byref(view), C.byref(sizes),
              None if previous is None else C.byref(previous), wind, C.byref(out))
    return out


class CloudShadow:
    """Shadow-pass state of one viewport (VolumetricCloud.h:106-115,
    VolumetricCloud.cpp:102-113,134-135): two raw (depth, transmittance) maps
    used in turn, so that each frame blends into the previous one, the
    blurred map and the R16 shadow froxel ([depth][height][width], stored as
    int16 words, read as uint16)."""

    def __init__(self, ctx: Context, sizes: _abi.CloudShadowSizes):
        self.ctx, self.sizes = ctx, sizes
        h, w = sizes.map_height, sizes.map_width
        self.raw = [torch.zeros((h, w, 2), dtype=torch.float32, device="cuda") for _ in range(2)]
        self.map = torch.zeros((h, w, 2), dtype=torch.float32, device="cuda")
        self.froxel = torch.zeros((sizes.froxel_depth, sizes.froxel_height, sizes.froxel_width), dtype=torch.int16,
                                  device="cuda")
        self.frame: _abi.CloudLightFrame | None = None  # the last frame's light transform
        self.current = 0  # index of the raw map written last

    def render(self, cloud: "VolumetricCloud", atmosphere: _abi.AtmosphereParameters, view: _abi.CloudView,
               blue_noise: torch.Tensor, wind_delta=None, blend: bool = True) -> _abi.CloudLightFrame:
        """RenderShadow for `view`: derive this frame's light transform, write
        the other raw map (blended with the last one unless `blend` is False or
        this is the first frame), blur it and rebuild the froxel."""
        frame = light_frame(atmosphere, cloud.params, view, self.sizes, self.frame if blend else None, wind_delta)
        k = 1 - self.current
        previous = self.raw[self.current] if (blend and self.frame is not None) else None
        _abi.call("skyr_cloud_shadow_render", self.ctx.handle, C.byref(atmosphere), C.byref(cloud.params),
                  C.byref(cloud.material), C.byref(cloud.textures), C.byref(view), C.byref(self.sizes),
                  C.byref(frame), _ptr(blue_noise), _ptr(previous), _ptr(self.raw[k]), _ptr(self.map),
                  _ptr(self.froxel))
        self.frame, self.current = frame, k
        return frame

    @property
    def raw_map(self) -> torch.Tensor:
        return self.raw[self.current]

    def attach(self, view: _abi.CloudView) -> _abi.CloudView:
        """Point `view` at this froxel (the raymarch, path tracer and surrogate
        then scale their aerial-perspective luminance by its visibility)."""
        view.shadow_froxel = self.froxel.data_ptr()
        view.shadow_froxel_width = self.sizes.froxel_width
        view.shadow_froxel_height = self.sizes.froxel_height
        view.shadow_froxel_depth = self.sizes.froxel_depth
        return view


def detach_froxel(view: _abi.CloudView) -> _abi.CloudView:
    view.shadow_froxel = None
    view.shadow_froxel_width = view.shadow_froxel_height = view.shadow_froxel_depth = 0
    return view


def temporal_frame(atmosphere: _abi.AtmosphereParameters, view: _abi.CloudView,
                   previous_view: _abi.CloudView | None = None, wind_delta=None, z_near: float = 0.1,
                   z_far: float = 1000.0, frame_index: int = 0) -> _abi.CloudTemporalFrame:
    """The temporal constants of VolumetricCloud::Update (host only); the
    planes default to the reference Camera's (Camera.h:39-40)."""
    out = _abi.CloudTemporalFrame()
    wind = None if wind_delta is None else (C.c_float * 2)(*wind_delta)
    _abi.call("skyr_cloud_temporal_frame_derive", C.byref(atmosphere), C.byref(view),
              None if previous_view is None else C.byref(previous_view), wind, z_near, z_far, frame_index,
              C.byref(out))
    return out


class CloudViewport:
    """The buffers of one viewport (ViewportData): half-resolution checkerboard
    depth and two reconstructions used in turn, quarter-resolution index,
    raymarch output and distance."""

    def __init__(self, ctx: Context, width: int, height: int):
        self.ctx, self.width, self.height = ctx, width, height
        hw, hh = width // 2, height // 2
        qw, qh = hw // 2, hh // 2
        dev = dict(device="cuda")
        self.checkerboard = torch.zeros((hh, hw), dtype=torch.float32, **dev)
        self.index = torch.zeros((qh, qw, 2), dtype=torch.float32, **dev)
        self.render_rgba = torch.zeros((qh, qw, 4), dtype=torch.float16, **dev)
        self.render_distance = torch.zeros((qh, qw), dtype=torch.float32, **dev)
        self.reconstruct = [torch.zeros((hh, hw, 4), dtype=torch.float16, **dev) for _ in range(2)]
        self.current = 0        # the reconstruction written last
        self.frames = 0
        self.previous_view: _abi.CloudView | None = None

    def buffers(self, history: bool = True) -> _abi.CloudQuarterBuffers:
        b = _abi.CloudQuarterBuffers()
        b.checkerboard_depth = self.checkerboard.data_ptr()
        b.index_linear_depth = self.index.data_ptr()
        b.render_rgba = self.render_rgba.data_ptr()
        b.render_distance = self.render_distance.data_ptr()
        k = 1 - self.current
        b.previous_reconstruct = self.reconstruct[self.current].data_ptr() if (history and self.frames) else None
        b.reconstruct = self.reconstruct[k].data_ptr()
        return b

    @property
    def reconstruction(self) -> torch.Tensor:
        return self.reconstruct[self.current]

    def render(self, cloud: "VolumetricCloud", atmosphere: _abi.AtmosphereParameters, view: _abi.CloudView,
               sizes: _abi.LutSizes, luts: LutSet, blue_noise: torch.Tensor, depth: torch.Tensor | None = None,
               hdr: torch.Tensor | None = None, wind_delta=None, z_near: float = 0.1, z_far: float = 1000.0,
               history: bool = True) -> _abi.CloudTemporalFrame:
        """One frame of VolumetricCloud::Render (all five passes; the upscale
        composites into `hdr` when given) and the swap of the reconstructions."""
        assert view.width == self.width and view.height == self.height
        prev = self.previous_view if (history and self.frames) else None
        # uBaseShadingIndex and the raymarch's jitter both follow the view's frame id
        frame = temporal_frame(atmosphere, view, prev, wind_delta, z_near, z_far, int(view.frame_id))
        b = self.buffers(history)
        _abi.call("skyr_cloud_render_quarter", self.ctx.handle, C.byref(atmosphere), C.byref(cloud.params),
                  C.byref(cloud.material), C.byref(cloud.textures), C.byref(view), C.byref(sizes),
                  _ptr(luts.transmittance), _ptr(luts.aerial_perspective_luminance),
                  _ptr(luts.aerial_perspective_transmittance), _ptr(blue_noise), _ptr(depth), C.byref(frame),
                  C.byref(b), _ptr(hdr))
        self.current = 1 - self.current
        self.frames += 1
        self.previous_view = _abi.CloudView.from_buffer_copy(view)
        return frame

    def autotune(self, cloud: "VolumetricCloud", atmosphere: _abi.AtmosphereParameters, view: _abi.CloudView,
                 sizes: _abi.LutSizes, luts: LutSet, blue_noise: torch.Tensor, depth: torch.Tensor | None = None,
                 z_near: float = 0.1, z_far: float = 1000.0, reps: int = 5):
        """skyr_autotune_cloud_quarter on this viewport's passes (the next
        frame's, with history once a frame exists): keeps the fastest launch
        shape in the context; returns (tuning, times ms per CLOUD_CANDIDATES
        entry).  Writes the buffers of the next frame without swapping."""
        assert view.width == self.width and view.height == self.height
        prev = self.previous_view if self.frames else None
        frame = temporal_frame(atmosphere, view, prev, None, z_near, z_far, int(view.frame_id))
        b = self.buffers(True)
        best = _abi.Tuning()
        times = (C.c_float * _abi.SKYR_CLOUD_TUNE_CANDIDATES)()
        _abi.call("skyr_autotune_cloud_quarter", self.ctx.handle, C.byref(atmosphere), C.byref(cloud.params),
                  C.byref(cloud.material), C.byref(cloud.textures), C.byref(view), C.byref(sizes),
                  _ptr(luts.transmittance), _ptr(luts.aerial_perspective_luminance),
                  _ptr(luts.aerial_perspective_transmittance), _ptr(blue_noise), _ptr(depth), C.byref(frame),
                  C.byref(b), reps, C.byref(best), times)
        return best, list(times)


def blue_noise_tile(seed: int = 0x5EED) -> torch.Tensor:
    """Seeded 64x64 blue-noise tile (host float32)."""
    out = (C.c_float * 4096)()
    _abi.call("skyr_blue_noise_generate", C.c_uint32(seed), out)
    return torch.frombuffer(bytearray(out), dtype=torch.float32).view(64, 64).clone()
