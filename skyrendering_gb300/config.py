"""Loader of the reference's application configuration files (bin/config*.json)
into this library's parameter blocks.

The reference saves and loads its state with rapidjson through cppreflection
(AppWindow's config load, src/SkyRendering/AppWindow.cpp:30-47;
src/Base/include/Serialization.h:1-7):

* every FIELD_DECLARE'd member is a key named as the member (private members
  keep their trailing underscore: ``bottom_altitude_``); a nested serialisable
  object is a nested JSON object; glm vectors are JSON arrays;
* a member path declared with dots is one flattened key
  (``"cloud_map_.buffer.uDensity.base_frequency"``,
  VolumetricCloudDefaultMaterial.h:103-122);
* enums are their enumerator names (``"NEAREST_MIPMAP_NEAREST"``, Samplers.h:20-25);
* a polymorphic member is ``{"type": "class <Name>", "data": {...}}``, the
  subclass picked by name from the factory of IVolumetricCloudMaterial
  (src/SkyRendering/IVolumetricCloudMaterial.cpp:7-12);
* a member absent from the file keeps its C++ default.

``load(path_or_dict)`` returns a ReferenceConfig with the skyr structs
(atmosphere, render, cloud, material, noise descriptions, LUT sizes, composite
parameters) and the camera.  Keys the reference's schema knows but this path
does not use (post-process, SMAA, window flags, the moon) are listed in
``ignored``; keys the schema does not know are listed in ``unknown`` and,
with ``strict=True``, raise ConfigError.  Nothing here needs the CUDA
library: the defaults are the reference's C++ member initialisers, restated
in DEFAULTS below (a test checks them against skyr_*_default).
"""
from __future__ import annotations

import ctypes as C
import json
import math
from dataclasses import dataclass, field
from pathlib import Path

import numpy as np

from . import _abi


class ConfigError(ValueError):
    """A configuration the loader cannot map (bad type, unknown material, unknown key in strict mode)."""


# ---------------------------------------------------------------------------
# The reference's defaults (C++ member initialisers)
# ---------------------------------------------------------------------------
# AtmosphereParameters (src/SkyRendering/Atmosphere.h:13-38)
ATMOSPHERE_DEFAULTS = {
    "solar_illuminance": (1.0, 1.0, 1.0), "sun_angular_radius": 0.5334 * 0.5, "bottom_radius": 6360.0,
    "thickness": 6420.0 - 6360.0, "ground_albedo": (0.4, 0.4, 0.4), "rayleigh_exponential_distribution": 8.0,
    "rayleigh_scattering_scale": 0.0331, "rayleigh_scattering": (0.175287, 0.409607, 1.0),
    "mie_exponential_distribution": 1.2, "mie_phase_g": 0.8, "mie_scattering_scale": 0.003996,
    "mie_scattering": (1.0, 1.0, 1.0), "mie_absorption_scale": 0.000444, "mie_absorption": (1.0, 1.0, 1.0),
    "ozone_center_altitude": 25.0, "ozone_width": 15.0, "ozone_absorption_scale": 0.001881,
    "ozone_absorption": (0.345561, 1.0, 0.045189), "transmittance_steps": 40.0, "multiscattering_steps": 30.0,
    "multiscattering_mask": 1.0,
}
# AtmosphereRenderParameters (src/SkyRendering/AtmosphereRenderer.h:13-19)
RENDER_DEFAULTS = {
    "sun_direction_theta": 70.0, "sun_direction_phi": 180.0, "star_luminance_scale": 0.005,
    "raymarching_steps": 40.0, "sky_view_lut_steps": 40.0, "aerial_perspective_lut_steps": 40.0,
    "aerial_perspective_lut_max_distance": 100.0,
}
# AtmosphereRenderInitParameters (src/SkyRendering/AtmosphereRenderer.h:43-52)
INIT_DEFAULTS = {
    "pcss_enable": True, "volumetric_light_enable": True, "moon_shadow_enable": False,
    "raymarching_dither_sample_point_enable": True, "use_sky_view_lut": False,
    "sky_view_lut_dither_sample_point_enable": False, "use_aerial_perspective_lut": False,
    "aerial_perspective_lut_dither_sample_point_enable": False, "aerial_perspective_lut_depth": 32,
}
# VolumetricCloud (src/SkyRendering/VolumetricCloud.h:20-35); the phase lobes are the
# constants of VolumetricCloudRender.comp:125-127 (not serialised)
CLOUD_DEFAULTS = {
    "bottom_altitude": 2.0, "thickness": 2.0, "max_raymarch_distance": 30.0, "max_raymarch_steps": 128.0,
    "max_visible_distance": 120.0, "env_color": (1.0, 1.0, 1.0), "env_color_scale": 0.1,
    "sun_illuminance_scale": 1.0, "shadow_steps": 5.0, "shadow_distance": 2.0, "shadow_froxel_max_distance": 20.0,
    "sun_multiscattering_sigma_scale": 0.3, "env_multiscattering_sigma_scale": 0.5, "env_bottom_visibility": 0.4,
    "env_sun_height_curve_exp": 1.0, "phase_g_forward": 0.85, "phase_g_back": -0.15, "phase_back_scale": 2.16,
    "shadow_map_max_distance": 20.0,
}
# VolumetricCloudDefaultMaterialCommon (VolumetricCloudDefaultMaterial.h:126-133, .cpp:37-64),
# Material1 (.h:199-205), Material0 (.h:165-166), VolumetricCloudVoxelMaterial.h:32-35,
# VolumetricCloudMinimalMaterial.h:26
MATERIAL_DEFAULTS = {
    "lod_bias": 2.75, "density": 15.0, "cloud_map_repeat_size": 18.99, "detail_repeat_size": 5.33,
    "displacement_repeat_size": 3.51, "minfilter2d": 0, "minfilter3d": 0, "minfilter_displacement": 0,
    "detail_base": 0.67, "detail_scale": 1.86, "base_density_threshold": 0.4, "base_height_hardness": 6.0,
    "base_edge_hardness": 6.0, "height_cut": 0.9, "edge_cut": 0.8, "detail_param": (0.4, 0.0),
    "displacement_scale": 1.0, "voxel_base": (0.0, 0.0), "voxel_width": (2.0, 2.0),
}
MATERIAL_DENSITY = {_abi.SKYR_MATERIAL_VOXEL: 20.0, _abi.SKYR_MATERIAL_MINIMAL: 0.5}
# NoiseCreateInfo defaults of the three generated textures (VolumetricCloudDefaultMaterial.h:66-84)
NOISE_DEFAULTS = {
    "cloud_map_.buffer.uDensity": (0, 3, 0.35, 0.75), "cloud_map_.buffer.uHeight": (0, 5, 0.8, 0.4),
    "detail_.buffer.uPerlin": (0, 7, 0.23, 1.0), "detail_.buffer.uWorley": (0, 11, 1.0, 0.0),
    "displacement_.buffer.uPerlin": (0, 6, 0.25, 0.75),
}
# Camera (src/Base/include/Camera.h:33-35,57-66)
CAMERA_DEFAULTS = {"fovy": 45.0, "zNear": 0.1, "zFar": 1000.0, "position_": (0.0, 0.0, 0.0),
                   "front_": (0.0, 0.0, 0.0), "right_": (0.0, 0.0, 0.0), "up_": (0.0, 0.0, 0.0), "yaw_": 0.0,
                   "pitch_": 0.0, "aspect_": 1.0}
# texture sizes and LUT sizes the reference creates (VolumetricCloudDefaultMaterial.cpp:40-72;
# NoiseGen.comp:25,41: 8 fBm octaves; Atmosphere.cpp:11-12; AtmosphereRenderer.cpp:15-20)
CLOUD_MAP_SIZE, DETAIL_SIZE, DISPLACEMENT_SIZE, NOISE_OCTAVES = 512, 128, 128, 8
LUT_SIZES = {"transmittance": (256, 64), "multiscattering": (32, 32), "sky_view": (128, 128),
             "aerial_perspective": (32, 32)}

MATERIAL_TYPES = {
    "class VolumetricCloudDefaultMaterial0": _abi.SKYR_MATERIAL_DEFAULT0,
    "class VolumetricCloudDefaultMaterial1": _abi.SKYR_MATERIAL_DEFAULT1,
    "class VolumetricCloudMinimalMaterial": _abi.SKYR_MATERIAL_MINIMAL,
    "class VolumetricCloudVoxelMaterial": _abi.SKYR_MATERIAL_VOXEL,
}
MIPMAP_MIN = {"NEAREST_MIPMAP_NEAREST": _abi.SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST,
              "LINEAR_MIPMAP_NEAREST": _abi.SKYR_MIPMAP_LINEAR_MIPMAP_NEAREST,
              "NEAREST_MIPMAP_LINEAR": _abi.SKYR_MIPMAP_NEAREST_MIPMAP_LINEAR,
              "LINEAR_MIPMAP_LINEAR": _abi.SKYR_MIPMAP_LINEAR_MIPMAP_LINEAR}

# Serialised members of the top-level AppWindow object and of the sections this
# path does not use (AppWindow.h, PostProcess.h, Earth.h moon_status).
_TOP_KEYS_IGNORED = {"anisotropy_enable_", "camera_speed_", "draw_debug_textures_enable_", "draw_gui_enable_",
                     "draw_help_enable_", "full_screen_", "post_process_parameters_", "smaa_option_",
                     "vsync_enable_"}
_CLOUD_KEYS = {"bottom_altitude_": "bottom_altitude", "thickness_": "thickness",
               "max_raymarch_distance_": "max_raymarch_distance", "max_raymarch_steps_": "max_raymarch_steps",
               "max_visible_distance_": "max_visible_distance", "env_color_": "env_color",
               "env_color_scale_": "env_color_scale", "sun_illuminance_scale_": "sun_illuminance_scale",
               "shadow_steps_": "shadow_steps", "shadow_distance_": "shadow_distance",
               "shadow_map_max_distance": "shadow_map_max_distance",
               "shadow_froxel_max_distance": "shadow_froxel_max_distance",
               "sun_multiscattering_sigma_scale": "sun_multiscattering_sigma_scale",
               "env_multiscattering_sigma_scale": "env_multiscattering_sigma_scale",
               "env_bottom_visibility": "env_bottom_visibility", "env_sun_height_curve_exp": "env_sun_height_curve_exp"}
_COMMON_KEYS = {"density_": "density", "lod_bias_": "lod_bias", "cloud_map_.texture.repeat_size": "cloud_map_repeat_size",
                "detail_.texture.repeat_size": "detail_repeat_size",
                "displacement_.texture.repeat_size": "displacement_repeat_size"}
_COMMON_ENUMS = {"minfilter2d_": "minfilter2d", "minfilter3d_": "minfilter3d",
                 "minfilter_displacement_": "minfilter_displacement"}
_COMMON_EXTRA = {"wind_speed_": 0.05, "detail_wind_magnify_": 1.0}  # the caller's wind offsets per frame
_MATERIAL1_KEYS = {"base_density_threshold_": "base_density_threshold", "base_height_hardness_": "base_height_hardness",
                   "base_edge_hardness_": "base_edge_hardness", "detail_base_": "detail_base",
                   "detail_scale_": "detail_scale", "height_cut_": "height_cut", "edge_cut_": "edge_cut"}
_MATERIAL0_KEYS = {"detail_param_": "detail_param", "displacement_scale_": "displacement_scale"}
_VOXEL_KEYS = {"density_": "density", "lod_bias_": "lod_bias", "base_": "voxel_base", "width_": "voxel_width"}


def _set(struct, name: str, value) -> None:
    cur = getattr(struct, name)
    if isinstance(cur, C.Array):
        vals = list(value) if isinstance(value, (list, tuple)) else None
        if vals is None or len(vals) != len(cur):
            raise ConfigError(f"{name}: expected {len(cur)} numbers, got {value!r}")
        cur[:] = [float(v) for v in vals]
    elif isinstance(cur, int):
        if isinstance(value, bool) or not isinstance(value, (int, float)) or float(value) != int(value):
            raise ConfigError(f"{name}: expected an integer, got {value!r}")
        setattr(struct, name, int(value))
    else:
        if isinstance(value, bool) or not isinstance(value, (int, float)) or not math.isfinite(float(value)):
            raise ConfigError(f"{name}: expected a finite number, got {value!r}")
        setattr(struct, name, float(value))


def _fill(struct, defaults: dict):
    for k, v in defaults.items():
        _set(struct, k, v)
    return struct


def atmosphere_defaults() -> _abi.AtmosphereParameters:
    """The reference's AtmosphereParameters defaults, without the CUDA library."""
    return _fill(_abi.AtmosphereParameters(), ATMOSPHERE_DEFAULTS)


def cloud_defaults() -> _abi.CloudParameters:
    """The reference's VolumetricCloud defaults, without the CUDA library."""
    return _fill(_abi.CloudParameters(), CLOUD_DEFAULTS)


def material_defaults(kind: int) -> _abi.CloudMaterial:
    """The reference's defaults of one material type, without the CUDA library."""
    m = _fill(_abi.CloudMaterial(), MATERIAL_DEFAULTS)
    m.type = kind
    m.density = MATERIAL_DENSITY.get(kind, m.density)
    return m


def _noise_info(values) -> _abi.NoiseCreateInfo:
    ci = _abi.NoiseCreateInfo()
    ci.seed, ci.base_frequency, ci.remap_min, ci.remap_max = int(values[0]), int(values[1]), float(values[2]), \
        float(values[3])
    return ci


def _noise_descs(noise: dict) -> dict:
    """The reference's three generated textures (VolumetricCloudDefaultMaterial.cpp:40-72)."""
    def desc(w, h, d, channels):
        out = _abi.NoiseTextureDesc()
        out.width, out.height, out.depth, out.octaves, out.channels = w, h, d, NOISE_OCTAVES, len(channels)
        for i, (kind, a, b) in enumerate(channels):
            out.channel[i].kind = kind
            out.channel[i].a = a
            if b is not None:
                out.channel[i].b = b
        return out

    cm = desc(CLOUD_MAP_SIZE, CLOUD_MAP_SIZE, 1,
              [(_abi.SKYR_NOISE_PERLIN, _noise_info(noise["cloud_map_.buffer.uDensity"]), None),
               (_abi.SKYR_NOISE_WORLEY, _noise_info(noise["cloud_map_.buffer.uHeight"]), None)])
    dt = desc(DETAIL_SIZE, DETAIL_SIZE, DETAIL_SIZE,
              [(_abi.SKYR_NOISE_PERLIN_WORLEY, _noise_info(noise["detail_.buffer.uPerlin"]),
                _noise_info(noise["detail_.buffer.uWorley"]))])
    s, f, lo, hi = noise["displacement_.buffer.uPerlin"]
    # DISPLACEMENT_GEN: four Perlin fBm channels with seeds seed .. seed + 3 (NoiseGen.comp:57-74)
    dp = desc(DISPLACEMENT_SIZE, DISPLACEMENT_SIZE, 1,
              [(_abi.SKYR_NOISE_PERLIN, _noise_info((int(s) + i, f, lo, hi)), None) for i in range(4)])
    return {"cloud_map": cm, "detail": dt, "displacement": dp}


@dataclass
class ReferenceCamera:
    """Camera (src/Base/include/Camera.h): serialised vectors as the file holds them."""

    position: tuple
    front: tuple
    up: tuple
    fovy: float
    aspect: float
    z_near: float
    z_far: float

    def view_projection(self, aspect: float | None = None) -> np.ndarray:
        """ProjectionMatrix() * ViewMatrix() (Camera.cpp:13-19), row-major numpy."""
        from .workloads import look_at, perspective

        p = np.asarray(self.position, dtype=np.float64)
        view = look_at(p, p + np.asarray(self.front, dtype=np.float64), self.up)
        return perspective(self.fovy, self.aspect if aspect is None else aspect, self.z_near, self.z_far) @ view


@dataclass
class ReferenceConfig:
    atmosphere: _abi.AtmosphereParameters
    render: _abi.AtmosphereRenderParameters
    composite: _abi.CompositeParameters
    cloud: _abi.CloudParameters
    material: _abi.CloudMaterial
    noise: dict
    lut_sizes: _abi.LutSizes
    camera: ReferenceCamera
    init: dict
    extra: dict = field(default_factory=dict)
    ignored: list = field(default_factory=list)
    unknown: list = field(default_factory=list)

    def view(self, width: int, height: int, frame_id: float = 0.0) -> _abi.CloudView:
        """A skyr_cloud_view of this configuration's camera and sun for a width x height viewport
        (the projection takes the viewport's aspect, as AppWindow sets it from the window)."""
        from .workloads import column_major

        v = _abi.CloudView()
        v.camera_position[:] = [float(x) for x in self.camera.position]
        v.view_projection[:] = column_major(self.camera.view_projection(width / height))
        v.fovy = self.camera.fovy
        v.viewport_width, v.viewport_height, v.width, v.height = width, height, width, height
        v.sun_direction_theta, v.sun_direction_phi = self.render.sun_direction_theta, self.render.sun_direction_phi
        v.frame_id = frame_id
        v.aerial_perspective_lut_max_distance = self.render.aerial_perspective_lut_max_distance
        return v

    def render_parameters(self, width: int, height: int) -> _abi.AtmosphereRenderParameters:
        """The render parameters with the camera's view-projection for a width x height viewport."""
        from .workloads import column_major

        r = _abi.AtmosphereRenderParameters.from_buffer_copy(self.render)
        r.view_projection[:] = column_major(self.camera.view_projection(width / height))
        return r


class _Reader:
    def __init__(self, strict: bool):
        self.strict, self.unknown, self.ignored = strict, [], []

    def obj(self, d, path: str) -> dict:
        if not isinstance(d, dict):
            raise ConfigError(f"{path}: expected an object, got {type(d).__name__}")
        return d

    def unknown_key(self, path: str) -> None:
        if self.strict:
            raise ConfigError(f"unknown key {path}")
        self.unknown.append(path)


def _load_material(r: _Reader, node, extra: dict):
    node = r.obj(node, "volumetric_cloud_.material")
    kind_name = node.get("type")
    if kind_name not in MATERIAL_TYPES:
        raise ConfigError(f"volumetric_cloud_.material.type: unknown material {kind_name!r} "
                          f"(known: {', '.join(sorted(MATERIAL_TYPES))})")
    for k in node:
        if k not in ("type", "data"):
            r.unknown_key(f"volumetric_cloud_.material.{k}")
    kind = MATERIAL_TYPES[kind_name]
    m = material_defaults(kind)
    noise = dict(NOISE_DEFAULTS)
    data = r.obj(node.get("data", {}), "volumetric_cloud_.material.data")
    base = "volumetric_cloud_.material.data"
    own = {_abi.SKYR_MATERIAL_DEFAULT1: _MATERIAL1_KEYS, _abi.SKYR_MATERIAL_DEFAULT0: _MATERIAL0_KEYS,
           _abi.SKYR_MATERIAL_VOXEL: _VOXEL_KEYS, _abi.SKYR_MATERIAL_MINIMAL: {"density_": "density"}}[kind]
    for k, v in data.items():
        if k == "materail_common_" and kind in (_abi.SKYR_MATERIAL_DEFAULT0, _abi.SKYR_MATERIAL_DEFAULT1):
            for ck, cv in r.obj(v, f"{base}.{k}").items():
                path = f"{base}.{k}.{ck}"
                stem, _, leaf = ck.rpartition(".")
                if ck in _COMMON_KEYS:
                    _set(m, _COMMON_KEYS[ck], cv)
                elif ck in _COMMON_ENUMS:
                    if cv not in MIPMAP_MIN:
                        raise ConfigError(f"{path}: unknown filter {cv!r}")
                    setattr(m, _COMMON_ENUMS[ck], MIPMAP_MIN[cv])
                elif ck in _COMMON_EXTRA:
                    _set_extra(extra, ck.rstrip("_"), cv, path)
                elif stem in NOISE_DEFAULTS and leaf in ("seed", "base_frequency", "remap_min", "remap_max"):
                    vals = list(noise[stem])
                    i = ("seed", "base_frequency", "remap_min", "remap_max").index(leaf)
                    if leaf in ("seed", "base_frequency") and (isinstance(cv, bool) or not isinstance(cv, int)):
                        raise ConfigError(f"{path}: expected an integer, got {cv!r}")
                    if not isinstance(cv, (int, float)) or isinstance(cv, bool):
                        raise ConfigError(f"{path}: expected a number, got {cv!r}")
                    vals[i] = cv
                    noise[stem] = tuple(vals)
                else:
                    r.unknown_key(path)
        elif k in own:
            _set(m, own[k], v)
        else:
            r.unknown_key(f"{base}.{k}")
    return m, _noise_descs(noise)


def _set_extra(extra: dict, name: str, value, path: str) -> None:
    if isinstance(value, bool) or not isinstance(value, (int, float)):
        raise ConfigError(f"{path}: expected a number, got {value!r}")
    extra[name] = float(value)


def load(source, strict: bool = False) -> ReferenceConfig:
    """Parse one of the reference's configuration files (a path, JSON text or an
    already-parsed dict) into skyr parameter blocks."""
    if isinstance(source, dict):
        doc = source
    else:
        src = str(source).lstrip()
        text = src if src.startswith(("{", "[")) else Path(source).read_text()
        try:
            doc = json.loads(text)
        except json.JSONDecodeError as exc:
            raise ConfigError(f"not JSON: {exc}") from exc
    r = _Reader(strict)
    doc = r.obj(doc, "<root>")
    atmo = atmosphere_defaults()
    render = _abi.AtmosphereRenderParameters()
    render_vals = dict(RENDER_DEFAULTS)
    init = dict(INIT_DEFAULTS)
    cloud = cloud_defaults()
    material, noise = None, None
    extra = {k.rstrip("_"): v for k, v in _COMMON_EXTRA.items()}
    cam = dict(CAMERA_DEFAULTS)
    for k, v in doc.items():
        if k == "earth_":
            for ek, ev in r.obj(v, k).items():
                if ek == "parameters":
                    for pk, pv in r.obj(ev, f"{k}.{ek}").items():
                        if pk in ATMOSPHERE_DEFAULTS:
                            _set(atmo, pk, pv)
                        else:
                            r.unknown_key(f"{k}.{ek}.{pk}")
                elif ek == "moon_status":
                    r.ignored.append(f"{k}.{ek}")
                else:
                    r.unknown_key(f"{k}.{ek}")
        elif k == "atmosphere_render_parameters_":
            for rk, rv in r.obj(v, k).items():
                if rk not in RENDER_DEFAULTS:
                    r.unknown_key(f"{k}.{rk}")
                elif isinstance(rv, bool) or not isinstance(rv, (int, float)) or not math.isfinite(float(rv)):
                    raise ConfigError(f"{k}.{rk}: expected a finite number, got {rv!r}")
                else:
                    render_vals[rk] = float(rv)
        elif k == "atmosphere_render_init_parameters_":
            for ik, iv in r.obj(v, k).items():
                if ik not in INIT_DEFAULTS:
                    r.unknown_key(f"{k}.{ik}")
                elif ik == "aerial_perspective_lut_depth":
                    if isinstance(iv, bool) or not isinstance(iv, int) or not 2 <= iv <= 8192:
                        raise ConfigError(f"{k}.{ik}: expected an integer in [2, 8192], got {iv!r}")
                    init[ik] = iv
                elif not isinstance(iv, bool):
                    raise ConfigError(f"{k}.{ik}: expected true or false, got {iv!r}")
                else:
                    init[ik] = iv
        elif k == "volumetric_cloud_":
            for ck, cv in r.obj(v, k).items():
                if ck == "material":
                    material, noise = _load_material(r, cv, extra)
                elif ck in _CLOUD_KEYS:
                    _set(cloud, _CLOUD_KEYS[ck], cv)
                else:
                    r.unknown_key(f"{k}.{ck}")
        elif k == "camera_":
            for ck, cv in r.obj(v, k).items():
                if ck not in CAMERA_DEFAULTS:
                    r.unknown_key(f"{k}.{ck}")
                    continue
                want = CAMERA_DEFAULTS[ck]
                if isinstance(want, tuple):
                    if not isinstance(cv, list) or len(cv) != 3 or not all(
                            isinstance(x, (int, float)) and not isinstance(x, bool) for x in cv):
                        raise ConfigError(f"{k}.{ck}: expected 3 numbers, got {cv!r}")
                    cam[ck] = tuple(float(x) for x in cv)
                elif isinstance(cv, bool) or not isinstance(cv, (int, float)):
                    raise ConfigError(f"{k}.{ck}: expected a number, got {cv!r}")
                else:
                    cam[ck] = float(cv)
        elif k in _TOP_KEYS_IGNORED:
            r.ignored.append(k)
        else:
            r.unknown_key(k)
    if material is None:  # VolumetricCloud's default material (VolumetricCloud.cpp:55)
        material = material_defaults(_abi.SKYR_MATERIAL_DEFAULT0)
        noise = _noise_descs(NOISE_DEFAULTS)
    for name in ("sun_direction_theta", "sun_direction_phi", "sky_view_lut_steps", "aerial_perspective_lut_steps",
                 "aerial_perspective_lut_max_distance"):
        setattr(render, name, render_vals[name])
    render.camera_position[:] = list(cam["position_"])
    cam_doc = doc.get("camera_", {})
    if "front_" not in cam_doc and "up_" not in cam_doc:
        # Camera::UpdateVectors from yaw and pitch (Camera.cpp:33-37)
        from .workloads import theta_phi_direction

        front = theta_phi_direction(math.radians(90.0 - cam["pitch_"]), math.radians(cam["yaw_"]))
        right = np.cross(front, [0.0, 1.0, 0.0])
        right /= np.linalg.norm(right)
        up = np.cross(right, front)
        cam["front_"], cam["up_"] = tuple(front), tuple(up / np.linalg.norm(up))
    camera = ReferenceCamera(position=cam["position_"], front=cam["front_"], up=cam["up_"], fovy=cam["fovy"],
                             aspect=cam["aspect_"], z_near=cam["zNear"], z_far=cam["zFar"])
    if np.linalg.norm(camera.front) == 0 or np.linalg.norm(camera.up) == 0:
        raise ConfigError("camera_: front_ and up_ must be non-zero vectors")
    from .workloads import column_major

    render.view_projection[:] = column_major(camera.view_projection())
    comp = _abi.CompositeParameters()
    comp.star_luminance_scale = render_vals["star_luminance_scale"]
    comp.raymarching_steps = render_vals["raymarching_steps"]
    comp.use_sky_view_lut = int(init["use_sky_view_lut"])
    comp.use_aerial_perspective_lut = int(init["use_aerial_perspective_lut"])
    comp.dither_sample_point = int(init["raymarching_dither_sample_point_enable"])
    sizes = _abi.LutSizes()
    sizes.transmittance_width, sizes.transmittance_height = LUT_SIZES["transmittance"]
    sizes.multiscattering_width, sizes.multiscattering_height = LUT_SIZES["multiscattering"]
    sizes.sky_view_width, sizes.sky_view_height = LUT_SIZES["sky_view"]
    sizes.aerial_perspective_width, sizes.aerial_perspective_height = LUT_SIZES["aerial_perspective"]
    sizes.aerial_perspective_depth = init["aerial_perspective_lut_depth"]
    sizes.format = _abi.SKYR_FORMAT_RGBA32F
    return ReferenceConfig(atmosphere=atmo, render=render, composite=comp, cloud=cloud, material=material,
                           noise=noise, lut_sizes=sizes, camera=camera, init=init, extra=extra, ignored=r.ignored,
                           unknown=r.unknown)


def struct_dict(s) -> dict:
    """A ctypes parameter block as a plain dict (arrays as lists, nested blocks as dicts)."""
    out = {}
    for name, _ in s._fields_:
        v = getattr(s, name)
        if isinstance(v, C.Array):
            out[name] = [struct_dict(x) if isinstance(x, C.Structure) else x for x in v]
        elif isinstance(v, C.Structure):
            out[name] = struct_dict(v)
        else:
            out[name] = v
    return out


def struct_from_dict(kind, d: dict):
    """The inverse of struct_dict: a ctypes parameter block of type `kind` from a field dict."""
    s = kind()
    for name, ftype in kind._fields_:
        if name not in d:
            raise ConfigError(f"{kind.__name__}: missing field {name}")
        v = d[name]
        cur = getattr(s, name)
        if isinstance(cur, C.Array):
            for i, x in enumerate(v):
                if isinstance(x, dict):
                    cur[i] = struct_from_dict(type(cur[i]), x)
                else:
                    cur[i] = x
        elif isinstance(cur, C.Structure):
            setattr(s, name, struct_from_dict(type(cur), v))
        else:
            setattr(s, name, v)
    return s


def from_blocks(d: dict) -> ReferenceConfig:
    """A ReferenceConfig from the plain field dicts of its blocks (the form of
    tests/golden/reference_configs.json)."""
    cam = d["camera"]
    return ReferenceConfig(
        atmosphere=struct_from_dict(_abi.AtmosphereParameters, d["atmosphere"]),
        render=struct_from_dict(_abi.AtmosphereRenderParameters, d["render"]),
        composite=struct_from_dict(_abi.CompositeParameters, d["composite"]),
        cloud=struct_from_dict(_abi.CloudParameters, d["cloud"]),
        material=struct_from_dict(_abi.CloudMaterial, d["material"]),
        noise={k: struct_from_dict(_abi.NoiseTextureDesc, v) for k, v in d["noise"].items()},
        lut_sizes=struct_from_dict(_abi.LutSizes, d["lut_sizes"]),
        camera=ReferenceCamera(position=tuple(cam["position"]), front=tuple(cam["front"]), up=tuple(cam["up"]),
                               fovy=cam["fovy"], aspect=cam["aspect"], z_near=cam["z_near"], z_far=cam["z_far"]),
        init=dict(d["init"]), extra=dict(d.get("extra", {})))
