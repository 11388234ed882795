"""ctypes mirror of include/skyr.h and loader of the in-tree libskyr.so.

There is no fallback: if libskyr.so is missing or cannot be loaded, every call
raises.  The structs below must match include/skyr.h field for field; the
layout is checked against ``skyr_struct_size`` at load time.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libskyr.so"

SKYR_OK, SKYR_EINVAL, SKYR_ENOMEM, SKYR_ECUDA, SKYR_ETIMEOUT, SKYR_ENOTSUP = range(6)
SKYR_FORMAT_RGBA32F, SKYR_FORMAT_RGBA16F = 0, 1
SKYR_LUT_TRANSMITTANCE, SKYR_LUT_MULTISCATTERING, SKYR_LUT_SKY_VIEW, SKYR_LUT_AERIAL_PERSPECTIVE = range(4)

f3 = C.c_float * 3
f16 = C.c_float * 16


class AtmosphereParameters(C.Structure):
    """skyr_atmosphere_parameters (AtmosphereParameters, src/SkyRendering/Atmosphere.h:10-38)."""

    _fields_ = [
        ("solar_illuminance", f3),
        ("sun_angular_radius", C.c_float),
        ("bottom_radius", C.c_float),
        ("thickness", C.c_float),
        ("ground_albedo", f3),
        ("rayleigh_exponential_distribution", C.c_float),
        ("rayleigh_scattering_scale", C.c_float),
        ("rayleigh_scattering", f3),
        ("mie_exponential_distribution", C.c_float),
        ("mie_phase_g", C.c_float),
        ("mie_scattering_scale", C.c_float),
        ("mie_scattering", f3),
        ("mie_absorption_scale", C.c_float),
        ("mie_absorption", f3),
        ("ozone_center_altitude", C.c_float),
        ("ozone_width", C.c_float),
        ("ozone_absorption_scale", C.c_float),
        ("ozone_absorption", f3),
        ("transmittance_steps", C.c_float),
        ("multiscattering_steps", C.c_float),
        ("multiscattering_mask", C.c_float),
    ]


class AtmosphereRenderParameters(C.Structure):
    """skyr_atmosphere_render_parameters (src/SkyRendering/AtmosphereRenderer.h:12-35)."""

    _fields_ = [
        ("sun_direction_theta", C.c_float),
        ("sun_direction_phi", C.c_float),
        ("sky_view_lut_steps", C.c_float),
        ("aerial_perspective_lut_steps", C.c_float),
        ("aerial_perspective_lut_max_distance", C.c_float),
        ("camera_position", f3),
        ("view_projection", f16),
    ]


class LutSizes(C.Structure):
    """skyr_lut_sizes."""

    _fields_ = [
        ("transmittance_width", C.c_int),
        ("transmittance_height", C.c_int),
        ("multiscattering_width", C.c_int),
        ("multiscattering_height", C.c_int),
        ("sky_view_width", C.c_int),
        ("sky_view_height", C.c_int),
        ("aerial_perspective_width", C.c_int),
        ("aerial_perspective_height", C.c_int),
        ("aerial_perspective_depth", C.c_int),
        ("format", C.c_int),
    ]


class DeviceLimits(C.Structure):
    """skyr_device_limits: bounds of the device loops (skyr_ctx_set_limits)."""

    _fields_ = [("tracking_steps", C.c_int32), ("reserved", C.c_int32), ("copy_wait_cycles", C.c_int64)]


# struct id (skyr_struct_size) -> ctypes type; extended by later modules
STRUCT_IDS: dict[int, type] = {0: AtmosphereParameters, 1: AtmosphereRenderParameters, 2: LutSizes,
                               21: DeviceLimits}

P = C.c_void_p
_SIGNATURES = {
    "skyr_abi_version": (C.c_int, []),
    "skyr_status_string": (C.c_char_p, [C.c_int]),
    "skyr_last_error": (C.c_char_p, []),
    "skyr_struct_size": (C.c_size_t, [C.c_int]),
    "skyr_ctx_create": (C.c_int, [P, C.POINTER(P)]),
    "skyr_ctx_destroy": (C.c_int, [P]),
    "skyr_ctx_synchronize": (C.c_int, [P]),
    "skyr_ctx_check_status": (C.c_int, [P]),
    "skyr_device_limits_default": (C.c_int, [C.POINTER(DeviceLimits)]),
    "skyr_ctx_set_limits": (C.c_int, [P, C.POINTER(DeviceLimits)]),
    "skyr_ctx_get_limits": (C.c_int, [P, C.POINTER(DeviceLimits)]),
    "skyr_atmosphere_parameters_default": (C.c_int, [C.POINTER(AtmosphereParameters)]),
    "skyr_lut_bytes": (C.c_size_t, [C.POINTER(LutSizes), C.c_int]),
    "skyr_update_luts": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.c_int, C.POINTER(LutSizes), P, P]),
    "skyr_render_view_luts": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(AtmosphereRenderParameters),
                                        C.c_int, C.POINTER(LutSizes), P, P, P, P, P, P]),
    "skyr_update_lut_set": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(AtmosphereRenderParameters),
                                      C.c_int, C.POINTER(LutSizes), P, P, P, P, P, P]),
}

_lib = None


class SkyrError(RuntimeError):
    def __init__(self, status: int, where: str, message: str):
        self.status = status
        super().__init__(f"{where}: {status_name(status)}: {message}")


def register(signatures: dict) -> None:
    """Add signatures of entry points declared by later modules of skyr.h."""
    _SIGNATURES.update(signatures)
    if _lib is not None:
        _bind(_lib, signatures)


def _bind(lib, sigs):
    for name, (res, args) in sigs.items():
        fn = getattr(lib, name)  # AttributeError: symbol missing from the build
        fn.restype = res
        fn.argtypes = args


def lib():
    """The loaded libskyr.so; raises if it is missing (no fallback path)."""
    global _lib
    if _lib is None:
        path = Path(os.environ.get("SKYR_LIB", LIB_PATH))
        if not path.exists():
            raise RuntimeError(
                f"{path} not found: build the CUDA extension first "
                "(python -c 'import __graft_entry__ as g; g.build()')")
        lb = C.CDLL(str(path))
        _bind(lb, _SIGNATURES)
        for sid, st in STRUCT_IDS.items():
            n = lb.skyr_struct_size(sid)
            if n != C.sizeof(st):
                raise RuntimeError(f"ABI mismatch: {st.__name__} is {C.sizeof(st)} bytes in Python, {n} in C")
        _lib = lb
    return _lib


def status_name(status: int) -> str:
    try:
        return lib().skyr_status_string(status).decode()
    except Exception:  # pragma: no cover - only when the library itself is missing
        return str(status)


def check(status: int, where: str) -> None:
    if status != SKYR_OK:
        msg = lib().skyr_last_error().decode(errors="replace")
        raise SkyrError(status, where, msg)


def call(name: str, *args) -> None:
    check(getattr(lib(), name)(*args), name)


def exported_symbols() -> list[str]:
    return sorted(_SIGNATURES)


# ---------------------------------------------------------------------------
# skyr_cloud.h
# ---------------------------------------------------------------------------
SKYR_NOISE_PERLIN, SKYR_NOISE_WORLEY, SKYR_NOISE_PERLIN_WORLEY, SKYR_NOISE_ZERO = range(4)
SKYR_MATERIAL_DEFAULT0, SKYR_MATERIAL_DEFAULT1, SKYR_MATERIAL_MINIMAL, SKYR_MATERIAL_VOXEL = range(4)
(SKYR_MIPMAP_NEAREST_MIPMAP_NEAREST, SKYR_MIPMAP_LINEAR_MIPMAP_NEAREST, SKYR_MIPMAP_NEAREST_MIPMAP_LINEAR,
 SKYR_MIPMAP_LINEAR_MIPMAP_LINEAR) = range(4)
f2 = C.c_float * 2


class NoiseCreateInfo(C.Structure):
    """skyr_noise_create_info (NoiseCreateInfo, src/SkyRendering/VolumetricCloudDefaultMaterial.h:57-64)."""

    _fields_ = [("seed", C.c_int), ("base_frequency", C.c_int), ("remap_min", C.c_float), ("remap_max", C.c_float)]


class NoiseChannel(C.Structure):
    _fields_ = [("kind", C.c_int), ("a", NoiseCreateInfo), ("b", NoiseCreateInfo)]


class NoiseTextureDesc(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("depth", C.c_int), ("channels", C.c_int),
                ("octaves", C.c_int), ("channel", NoiseChannel * 4)]


class CloudMaterial(C.Structure):
    """skyr_cloud_material (the IVolumetricCloudMaterial implementations)."""

    _fields_ = [
        ("type", C.c_int),
        ("density", C.c_float), ("lod_bias", C.c_float),
        ("cloud_map_repeat_size", C.c_float), ("detail_repeat_size", C.c_float),
        ("displacement_repeat_size", C.c_float),
        ("offset_from_first", f2), ("detail_offset_from_first", f2),
        ("minfilter2d", C.c_int), ("minfilter3d", C.c_int), ("minfilter_displacement", C.c_int),
        ("base_density_threshold", C.c_float), ("base_height_hardness", C.c_float),
        ("base_edge_hardness", C.c_float), ("detail_base", C.c_float), ("detail_scale", C.c_float),
        ("height_cut", C.c_float), ("edge_cut", C.c_float),
        ("detail_param", f2), ("displacement_scale", C.c_float),
        ("voxel_base", f2), ("voxel_width", f2),
    ]


class CloudTextures(C.Structure):
    _fields_ = [("cloud_map", C.c_void_p), ("cloud_map_desc", NoiseTextureDesc),
                ("detail", C.c_void_p), ("detail_desc", NoiseTextureDesc),
                ("displacement", C.c_void_p), ("displacement_desc", NoiseTextureDesc),
                ("voxel", C.c_void_p), ("voxel_desc", NoiseTextureDesc),
                ("cloud_map_expanded", C.c_void_p), ("detail_expanded", C.c_void_p),
                ("displacement_expanded", C.c_void_p), ("voxel_expanded", C.c_void_p),
                ("cloud_map_expanded_channels", C.c_int), ("detail_expanded_channels", C.c_int),
                ("displacement_expanded_channels", C.c_int), ("voxel_expanded_channels", C.c_int),
                ("cloud_map_sampler", C.c_uint64), ("detail_sampler", C.c_uint64),
                ("cloud_map_sampler_nearest", C.c_uint64), ("detail_sampler_nearest", C.c_uint64)]


class CloudParameters(C.Structure):
    """skyr_cloud_parameters (VolumetricCloud fields, src/SkyRendering/VolumetricCloud.h:20-55)."""

    _fields_ = [
        ("bottom_altitude", C.c_float), ("thickness", C.c_float), ("max_raymarch_distance", C.c_float),
        ("max_raymarch_steps", C.c_float), ("max_visible_distance", C.c_float), ("env_color", f3),
        ("env_color_scale", C.c_float), ("sun_illuminance_scale", C.c_float), ("shadow_steps", C.c_float),
        ("shadow_distance", C.c_float), ("shadow_froxel_max_distance", C.c_float),
        ("sun_multiscattering_sigma_scale", C.c_float), ("env_multiscattering_sigma_scale", C.c_float),
        ("env_bottom_visibility", C.c_float), ("env_sun_height_curve_exp", C.c_float),
        ("phase_g_forward", C.c_float), ("phase_g_back", C.c_float), ("phase_back_scale", C.c_float),
        ("shadow_map_max_distance", C.c_float),
    ]


class CloudView(C.Structure):
    _fields_ = [("camera_position", f3), ("view_projection", f16), ("fovy", C.c_float),
                ("viewport_width", C.c_int), ("viewport_height", C.c_int), ("width", C.c_int),
                ("height", C.c_int), ("sun_direction_theta", C.c_float), ("sun_direction_phi", C.c_float),
                ("frame_id", C.c_float), ("aerial_perspective_lut_max_distance", C.c_float),
                ("shadow_froxel", C.c_void_p), ("shadow_froxel_width", C.c_int), ("shadow_froxel_height", C.c_int),
                ("shadow_froxel_depth", C.c_int)]


STRUCT_IDS.update({3: NoiseTextureDesc, 4: CloudMaterial, 5: CloudTextures, 6: CloudParameters, 7: CloudView})
_SIGNATURES.update({
    "skyr_noise_texture_levels": (C.c_int, [C.POINTER(NoiseTextureDesc)]),
    "skyr_noise_level_offset": (C.c_size_t, [C.POINTER(NoiseTextureDesc), C.c_int]),
    "skyr_noise_generate": (C.c_int, [P, C.POINTER(NoiseTextureDesc), P]),
    "skyr_cloud_material_default": (C.c_int, [C.c_int, C.POINTER(CloudMaterial)]),
    "skyr_noise_sampler_create": (C.c_int, [P, C.POINTER(NoiseTextureDesc), P, C.c_int, C.POINTER(P)]),
    "skyr_noise_sampler_update": (C.c_int, [P, P, P]),
    "skyr_noise_sampler_destroy": (C.c_int, [P]),
    "skyr_noise_sampler_handle": (C.c_uint64, [P]),
    "skyr_noise_sampler_nearest_handle": (C.c_uint64, [P]),
    "skyr_cloud_parameters_default": (C.c_int, [C.POINTER(CloudParameters)]),
    "skyr_cloud_render": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                    C.POINTER(CloudMaterial), C.POINTER(CloudTextures), C.POINTER(CloudView),
                                    C.POINTER(LutSizes), P, P, P, P, P, P, P]),
    "skyr_blue_noise_generate": (C.c_int, [C.c_uint32, C.POINTER(C.c_float)]),
    "skyr_noise_expanded_bytes": (C.c_size_t, [C.POINTER(NoiseTextureDesc), C.c_int]),
    "skyr_noise_expand": (C.c_int, [P, C.POINTER(NoiseTextureDesc), P, C.c_int, P]),
})
_SIGNATURES["skyr_cloud_render_to_host"] = (
    C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters), C.POINTER(CloudMaterial),
              C.POINTER(CloudTextures), C.POINTER(CloudView), C.POINTER(LutSizes), P, P, P, P, P, P, P])
_SIGNATURES["skyr_render_frame"] = (
    C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(AtmosphereRenderParameters), C.POINTER(LutSizes),
              P, P, P, P, P, P, C.POINTER(CloudParameters), C.POINTER(CloudMaterial), C.POINTER(CloudTextures),
              C.POINTER(CloudView), P, P, P, P, C.c_int])
_SIGNATURES["skyr_cloud_render_counted"] = (
    C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters), C.POINTER(CloudMaterial),
              C.POINTER(CloudTextures), C.POINTER(CloudView), C.POINTER(LutSizes), P, P, P, P, P, P, P, P])

# ---------------------------------------------------------------------------
# skyr_cloud_shadow.h
# ---------------------------------------------------------------------------
class CloudShadowSizes(C.Structure):
    _fields_ = [("map_width", C.c_int), ("map_height", C.c_int), ("froxel_width", C.c_int),
                ("froxel_height", C.c_int), ("froxel_depth", C.c_int)]


class CloudLightFrame(C.Structure):
    _fields_ = [("light_view_projection", f16), ("inverse_light_view_projection", f16), ("model", f16),
                ("shadow_map_reproject", f16), ("has_previous", C.c_int)]


STRUCT_IDS.update({15: CloudShadowSizes, 16: CloudLightFrame})
_SIGNATURES.update({
    "skyr_cloud_shadow_sizes_default": (C.c_int, [C.c_int, C.c_int, C.POINTER(CloudShadowSizes)]),
    "skyr_cloud_light_frame_derive": (C.c_int, [C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                                C.POINTER(CloudView), C.POINTER(CloudShadowSizes),
                                                C.POINTER(CloudLightFrame), C.POINTER(C.c_float),
                                                C.POINTER(CloudLightFrame)]),
    "skyr_cloud_shadow_render": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                           C.POINTER(CloudMaterial), C.POINTER(CloudTextures), C.POINTER(CloudView),
                                           C.POINTER(CloudShadowSizes), C.POINTER(CloudLightFrame), P, P, P, P, P]),
})


# ---------------------------------------------------------------------------
# skyr_cloud_quarter.h
# ---------------------------------------------------------------------------
class CloudTemporalFrame(C.Structure):
    _fields_ = [("reproject", f16), ("z_near", C.c_float), ("z_far", C.c_float), ("base_shading_index", C.c_int),
                ("has_previous", C.c_int)]


class CloudQuarterBuffers(C.Structure):
    _fields_ = [("checkerboard_depth", P), ("index_linear_depth", P), ("render_rgba", P), ("render_distance", P),
                ("previous_reconstruct", P), ("reconstruct", P)]


STRUCT_IDS.update({17: CloudTemporalFrame, 18: CloudQuarterBuffers})
_SIGNATURES.update({
    "skyr_cloud_temporal_frame_derive": (C.c_int, [C.POINTER(AtmosphereParameters), C.POINTER(CloudView),
                                                   C.POINTER(CloudView), C.POINTER(C.c_float), C.c_float, C.c_float,
                                                   C.c_int, C.POINTER(CloudTemporalFrame)]),
    "skyr_cloud_render_quarter": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                            C.POINTER(CloudMaterial), C.POINTER(CloudTextures), C.POINTER(CloudView),
                                            C.POINTER(LutSizes), P, P, P, P, P, C.POINTER(CloudTemporalFrame),
                                            C.POINTER(CloudQuarterBuffers), P]),
    "skyr_autotune_cloud_quarter": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                              C.POINTER(CloudMaterial), C.POINTER(CloudTextures),
                                              C.POINTER(CloudView), C.POINTER(LutSizes), P, P, P, P, P,
                                              C.POINTER(CloudTemporalFrame), C.POINTER(CloudQuarterBuffers), C.c_int,
                                              P, P]),
})


# ---------------------------------------------------------------------------
# skyr_environment.h
# ---------------------------------------------------------------------------
_SIGNATURES.update({
    "skyr_environment_cube_level_offset": (C.c_size_t, [C.c_int, C.c_int]),
    "skyr_environment_cube": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(AtmosphereRenderParameters),
                                        C.POINTER(LutSizes), P, P, P, C.c_int, C.c_int, P]),
    "skyr_environment_seamless_level_offset": (C.c_size_t, [C.c_int, C.c_int]),
    "skyr_environment_seamless": (C.c_int, [P, P, C.c_int, C.c_int, P]),
    "skyr_environment_sh": (C.c_int, [P, P, C.c_int, C.c_int, P]),
    "skyr_environment_prefilter": (C.c_int, [P, P, C.c_int, C.c_int, C.c_int, C.c_int, P]),
})


# ---------------------------------------------------------------------------
# skyr_composite.h
# ---------------------------------------------------------------------------
class CompositeParameters(C.Structure):
    _fields_ = [("star_luminance_scale", C.c_float), ("raymarching_steps", C.c_float),
                ("use_sky_view_lut", C.c_int), ("use_aerial_perspective_lut", C.c_int),
                ("dither_sample_point", C.c_int)]


class CompositeInputs(C.Structure):
    _fields_ = [("width", C.c_int), ("height", C.c_int), ("depth", P), ("object_luminance", P),
                ("blue_noise", P), ("star_map", P), ("star_width", C.c_int), ("star_height", C.c_int),
                ("shadow_froxel", P), ("froxel_width", C.c_int), ("froxel_height", C.c_int),
                ("froxel_depth", C.c_int), ("shadow_froxel_max_distance", C.c_float)]


STRUCT_IDS.update({19: CompositeParameters, 20: CompositeInputs})
_SIGNATURES.update({
    "skyr_composite_parameters_default": (C.c_int, [C.POINTER(CompositeParameters)]),
    "skyr_atmosphere_composite": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(AtmosphereRenderParameters),
                                            C.POINTER(CompositeParameters), C.POINTER(LutSizes), P, P, P, P, P, P,
                                            C.POINTER(CompositeInputs), P]),
})


# allocation-free LUT set (static device scratch, SKYR_NOALLOC_MAX_SETS sets)
SKYR_NOALLOC_MAX_SETS = 256
_SIGNATURES["skyr_update_lut_set_noalloc"] = (
    C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(AtmosphereRenderParameters), C.c_int,
              C.POINTER(LutSizes), P, P, P, P, P, P])


# ---------------------------------------------------------------------------
# skyr_pathtrace.h
# ---------------------------------------------------------------------------
SKYR_PRNG_WANG_HASH, SKYR_PRNG_PCG_HASH = 0, 1
SKYR_ENV_OFF, SKYR_ENV_CONST_ENVIRONMENT_MAP, SKYR_ENV_GROUND_SINGLE_BOUNCE, SKYR_ENV_GROUND_MULTI_BOUNCE = range(4)


class DensityGrid(C.Structure):
    _fields_ = [("data", C.c_void_p), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("origin", f3),
                ("voxel_size", C.c_float), ("density", C.c_float), ("majorant", C.c_void_p), ("brick", C.c_int)]


class GridGenerator(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int), ("seed", C.c_int), ("base_frequency", C.c_int),
                ("octaves", C.c_int), ("center", f3), ("radii", f3), ("inner", C.c_float),
                ("threshold", C.c_float)]


class PathtraceParameters(C.Structure):
    """skyr_pathtrace_parameters (PathTracing::InitParam, src/SkyRendering/VolumetricCloud.h:104-114)."""

    _fields_ = [("max_bounces", C.c_int), ("region_box_half_width", C.c_float), ("importance_sampling", C.c_int),
                ("forward_phase_g", C.c_float), ("back_phase_g", C.c_float),
                ("forward_scattering_ratio", C.c_float), ("prng", C.c_int), ("environment_lighting", C.c_int),
                ("sigma_t_max", C.c_float), ("use_brick_majorants", C.c_int)]


STRUCT_IDS.update({8: DensityGrid, 9: GridGenerator, 10: PathtraceParameters})
_SIGNATURES.update({
    "skyr_pathtrace_parameters_default": (C.c_int, [C.POINTER(PathtraceParameters)]),
    "skyr_grid_bytes": (C.c_size_t, [C.c_int, C.c_int, C.c_int]),
    "skyr_grid_generate": (C.c_int, [P, C.POINTER(GridGenerator), P]),
    "skyr_grid_brick_count": (C.c_int, [C.c_int, C.c_int]),
    "skyr_grid_majorants": (C.c_int, [P, C.POINTER(DensityGrid), P]),
    "skyr_pathtrace": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                 C.POINTER(CloudMaterial), C.POINTER(CloudTextures), C.POINTER(DensityGrid),
                                 C.POINTER(PathtraceParameters), C.POINTER(CloudView),
                                 C.POINTER(AtmosphereRenderParameters), C.POINTER(LutSizes), P, P, P, P, P,
                                 C.c_uint, C.c_int, P, P, P]),
    "skyr_pathtrace_resolve": (C.c_int, [P, P, C.c_int, C.c_int, C.c_uint, P, P]),
    "skyr_pathtrace_pixels": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                        C.POINTER(CloudMaterial), C.POINTER(CloudTextures), C.POINTER(DensityGrid),
                                        C.POINTER(PathtraceParameters), C.POINTER(CloudView),
                                        C.POINTER(AtmosphereRenderParameters), C.POINTER(LutSizes), P, P, P, P, P,
                                        C.c_uint, C.c_int, P, C.c_int, P, P]),
    "skyr_pathtrace_points": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                        C.POINTER(DensityGrid), C.POINTER(PathtraceParameters), C.POINTER(CloudView),
                                        C.POINTER(AtmosphereRenderParameters), C.POINTER(LutSizes), P, P, P, P, P,
                                        C.c_uint, C.c_int, P, C.c_int, P]),
})


# ---------------------------------------------------------------------------
# skyr_mlp.h
# ---------------------------------------------------------------------------
SKYR_MLP_INPUTS, SKYR_MLP_RECORD, SKYR_MLP_WIDTH, SKYR_MLP_OUTPUTS, SKYR_MLP_PARAMS = 103, 112, 64, 3, 19331


class MlpHparams(C.Structure):
    _fields_ = [("learning_rate", C.c_float), ("beta1", C.c_float), ("beta2", C.c_float), ("epsilon", C.c_float),
                ("label_scale", C.c_float), ("loss_epsilon", C.c_float)]


STRUCT_IDS.update({11: MlpHparams})
_SIGNATURES.update({
    "skyr_mlp_hparams_default": (C.c_int, [C.POINTER(MlpHparams)]),
    "skyr_mlp_param_count": (C.c_size_t, []),
    "skyr_mlp_packed_bytes": (C.c_size_t, []),
    "skyr_mlp_init_params": (C.c_int, [C.c_uint64, P]),
    "skyr_mlp_pack": (C.c_int, [P, P, C.c_float, P]),
    "skyr_mlp_infer": (C.c_int, [P, P, P, C.c_int, P]),
    "skyr_mlp_gradient": (C.c_int, [P, P, C.POINTER(MlpHparams), P, P, C.c_int, P, P]),
    "skyr_mlp_trainer_create": (C.c_int, [P, P, C.POINTER(MlpHparams), C.POINTER(P)]),
    "skyr_mlp_trainer_destroy": (C.c_int, [P]),
    "skyr_mlp_train_step": (C.c_int, [P, P, P, C.c_int, P]),
    "skyr_mlp_trainer_params": (P, [P]),
    "skyr_mlp_trainer_packed": (P, [P]),
    "skyr_mlp_trainer_steps": (C.c_int, [P]),
    "skyr_mlp_trainer_copy_params": (C.c_int, [P, P]),
    "skyr_mlp_trainer_copy_packed": (C.c_int, [P, P]),
    "skyr_mlp_train_epoch": (C.c_int, [P, P, P, C.c_int, P, C.c_int, C.c_int, P]),
    "skyr_mlp_trainer_save_state": (C.c_int, [P, P, P, P, C.POINTER(C.c_int)]),
    "skyr_mlp_trainer_load_state": (C.c_int, [P, P, P, P, C.c_int]),
    "skyr_mlp_trainer_set_learning_rate": (C.c_int, [P, C.c_float]),
})


# ---------------------------------------------------------------------------
# skyr_surrogate.h
# ---------------------------------------------------------------------------
class FeatureVolume(C.Structure):
    _fields_ = [("data", P), ("stride", C.c_int), ("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("sigma_ref", C.c_float), ("sun", C.c_float * 3)]


class SurrogateParameters(C.Structure):
    _fields_ = [("steps", C.c_int), ("use_network", C.c_int), ("network_error", C.c_float),
                ("min_transmittance", C.c_float), ("error_table", P)]


SKYR_SURROGATE_ERROR_BINS = 8


STRUCT_IDS.update({12: FeatureVolume, 13: SurrogateParameters})
_SIGNATURES.update({
    "skyr_surrogate_parameters_default": (C.c_int, [C.POINTER(SurrogateParameters)]),
    "skyr_feature_volume_bytes": (C.c_size_t, [C.POINTER(DensityGrid), C.c_int, C.POINTER(FeatureVolume)]),
    "skyr_feature_volume_build": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                            C.POINTER(DensityGrid), C.POINTER(CloudView), C.POINTER(FeatureVolume)]),
    "skyr_surrogate_sample_points": (C.c_int, [P, C.POINTER(DensityGrid), C.c_float, C.c_float, C.c_uint64, C.c_int,
                                               P]),
    "skyr_surrogate_records": (C.c_int, [P, C.POINTER(DensityGrid), C.POINTER(FeatureVolume), P, C.c_int, P]),
    "skyr_surrogate_error_bins": (C.c_int, [P, P, C.c_int, P]),
    "skyr_surrogate_render": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                        C.POINTER(DensityGrid), C.POINTER(PathtraceParameters), C.POINTER(CloudView),
                                        C.POINTER(LutSizes), P, P, P, C.POINTER(FeatureVolume), P,
                                        C.POINTER(SurrogateParameters), P, P]),
})


# ---------------------------------------------------------------------------
# skyr_batch.h
# ---------------------------------------------------------------------------
SKYR_CLOUD_TILE_CANDIDATES = 12
SKYR_CLOUD_TUNE_CANDIDATES = 288


class Tuning(C.Structure):
    _fields_ = [("transmittance_lanes", C.c_int), ("view_lanes", C.c_int), ("cloud_tile_width", C.c_int),
                ("cloud_block_warps_x", C.c_int), ("cloud_blocks_per_sm", C.c_int), ("cloud_ray_lanes", C.c_int)]


STRUCT_IDS.update({14: Tuning})
_SIGNATURES.update({
    "skyr_tuning_default": (C.c_int, [C.POINTER(Tuning)]),
    "skyr_ctx_set_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "skyr_ctx_get_tuning": (C.c_int, [P, C.POINTER(Tuning)]),
    "skyr_autotune_luts": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(AtmosphereRenderParameters),
                                     C.c_int, C.POINTER(LutSizes), P, P, P, P, P, P, C.c_int, C.POINTER(Tuning), P]),
    "skyr_autotune_cloud": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(CloudParameters),
                                      C.POINTER(CloudMaterial), C.POINTER(CloudTextures), C.POINTER(CloudView),
                                      C.POINTER(LutSizes), P, P, P, P, P, P, C.c_int, C.POINTER(Tuning), P]),
    "skyr_lut_batch_create": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.POINTER(AtmosphereRenderParameters),
                                        C.c_int, C.POINTER(LutSizes), C.POINTER(P)]),
    "skyr_lut_batch_launch": (C.c_int, [P, P, P, P, P, P, P]),
    "skyr_lut_batch_destroy": (C.c_int, [P]),
    "skyr_cloud_render_views": (C.c_int, [P, C.POINTER(AtmosphereParameters), C.c_int, P, C.POINTER(CloudParameters),
                                          C.POINTER(CloudMaterial), C.POINTER(CloudTextures), C.POINTER(CloudView),
                                          C.c_int, C.POINTER(LutSizes), P, P, P, P, P, P]),
    "skyr_graph_begin": (C.c_int, [P]),
    "skyr_graph_end": (C.c_int, [P, C.POINTER(P)]),
    "skyr_graph_launch": (C.c_int, [P]),
    "skyr_graph_destroy": (C.c_int, [P]),
})
