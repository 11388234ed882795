"""Seeded synthetic workloads: the parameter sets, cameras and sizes of the
benchmark and parity configurations, built on the reference's own parameter
surface (bin/config.json fields) and conventions:

* world space is y-up with the Earth centre at (0, -bottom_radius, 0)
  (src/SkyRendering/Earth.h:37);
* cameras follow Camera::UpdateVectors / ViewMatrix / ProjectionMatrix
  (src/Base/src/Camera.cpp:13-37): glm::lookAt + glm::perspective, OpenGL
  clip space (z in [-1, 1]), column-major matrices;
* sun direction from (zenith theta, azimuth phi) by FromThetaPhiToDirection
  (src/Base/src/Utils.cpp:23-31).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

from . import _abi

SEED = 0x5EED
SUN_ZENITHS_DEG = (0.0, 45.0, 85.0, 90.0, 95.0)


def theta_phi_direction(theta_rad: float, phi_rad: float) -> np.ndarray:
    return np.array([math.cos(phi_rad) * math.sin(theta_rad), math.cos(theta_rad),
                     math.sin(phi_rad) * math.sin(theta_rad)])


def perspective(fovy_deg: float, aspect: float, z_near: float, z_far: float) -> np.ndarray:
    """glm::perspective (right-handed, clip z in [-1, 1]); row-major numpy (row, col)."""
    t = math.tan(math.radians(fovy_deg) * 0.5)
    m = np.zeros((4, 4))
    m[0, 0] = 1.0 / (aspect * t)
    m[1, 1] = 1.0 / t
    m[2, 2] = -(z_far + z_near) / (z_far - z_near)
    m[3, 2] = -1.0
    m[2, 3] = -(2.0 * z_far * z_near) / (z_far - z_near)
    return m


def look_at(eye, center, up) -> np.ndarray:
    """glm::lookAt (right-handed); row-major numpy (row, col)."""
    eye, center, up = (np.asarray(v, dtype=np.float64) for v in (eye, center, up))
    f = center - eye
    f /= np.linalg.norm(f)
    s = np.cross(f, up)
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[0, :3], m[1, :3], m[2, :3] = s, u, -f
    m[0, 3], m[1, 3], m[2, 3] = -s @ eye, -u @ eye, f @ eye
    return m


def column_major(m: np.ndarray) -> list[float]:
    return [float(x) for x in np.asarray(m, dtype=np.float32).flatten(order="F")]


@dataclass
class Camera:
    """Camera (src/Base/include/Camera.h:10-67): yaw/pitch in degrees, y-up world."""

    position: tuple = (0.0, 1.0, 0.0)
    yaw: float = 90.0
    pitch: float = 10.0
    fovy: float = 60.0
    width: int = 1920
    height: int = 1080
    z_near: float = 0.3
    z_far: float = 50000.0

    def vectors(self):
        # Camera::UpdateVectors (src/Base/src/Camera.cpp:33-37)
        front = theta_phi_direction(math.radians(90.0 - self.pitch), math.radians(self.yaw))
        right = np.cross(front, [0.0, 1.0, 0.0])
        right /= np.linalg.norm(right)
        up = np.cross(right, front)
        up /= np.linalg.norm(up)
        return front, right, up

    def view_projection(self) -> np.ndarray:
        front, _, up = self.vectors()
        pos = np.asarray(self.position, dtype=np.float64)
        proj = perspective(self.fovy, self.width / self.height, self.z_near, self.z_far)
        return proj @ look_at(pos, pos + front, up)


def atmosphere_defaults() -> _abi.AtmosphereParameters:
    """The reference's AtmosphereParameters defaults (config.py restates them; equal to
    skyr_atmosphere_parameters_default, checked on the CPU)."""
    from .config import atmosphere_defaults as reference_defaults

    return reference_defaults()


def C_ref(x):
    import ctypes
    return ctypes.byref(x)


def earth_like_atmosphere() -> _abi.AtmosphereParameters:
    """Earth-like atmosphere of the plain-LUT workload: R 6360 km, top 6460 km,
    Rayleigh (5.802, 13.558, 33.1)e-3/km H 8 km, Mie scattering 3.996e-3/km and
    extinction 4.40e-3/km H 1.2 km g 0.8, ozone (0.650, 1.881, 0.085)e-3/km tent
    at 25 km half-width 15 km, ground albedo 0.3, 40 transmittance samples and 20
    multi-scattering samples.  Expressed through the reference's own fields: the
    Mie extinction target sets mie_absorption_scale = 0.404e-3."""
    p = atmosphere_defaults()
    p.thickness = 100.0
    p.ground_albedo[:] = [0.3, 0.3, 0.3]
    p.mie_absorption_scale = 0.000404
    p.transmittance_steps = 40.0
    p.multiscattering_steps = 20.0
    return p


def plain_lut_sizes(fmt: int = _abi.SKYR_FORMAT_RGBA32F) -> _abi.LutSizes:
    s = _abi.LutSizes()
    s.transmittance_width, s.transmittance_height = 256, 64
    s.multiscattering_width, s.multiscattering_height = 32, 32
    s.sky_view_width, s.sky_view_height = 192, 108
    s.aerial_perspective_width = s.aerial_perspective_height = s.aerial_perspective_depth = 32
    s.format = fmt
    return s


def render_parameters(cam: Camera, sun_zenith_deg: float, sun_azimuth_deg: float = 60.0,
                      sky_view_steps: float = 30.0, ap_steps: float = 40.0,
                      ap_max_distance: float = 32.0) -> _abi.AtmosphereRenderParameters:
    r = _abi.AtmosphereRenderParameters()
    r.sun_direction_theta = sun_zenith_deg
    r.sun_direction_phi = sun_azimuth_deg
    r.sky_view_lut_steps = sky_view_steps
    r.aerial_perspective_lut_steps = ap_steps
    r.aerial_perspective_lut_max_distance = ap_max_distance
    r.camera_position[:] = list(cam.position)
    r.view_projection[:] = column_major(cam.view_projection())
    return r


def frame_camera() -> Camera:
    """The 1920x1080 frame camera: 1 km altitude, 60 degree vertical FOV,
    pitched 10 degrees up toward +z."""
    return Camera()


def _batched_sets(n: int, seed: int):
    """(params, cameras, sun zeniths, sun azimuths) of the batched workload."""
    rng = np.random.default_rng(seed)
    base = earth_like_atmosphere()
    params = (_abi.AtmosphereParameters * n)()
    cams, zen, azi = [], [], []
    lo, hi = math.log(0.5), math.log(1.5)
    import ctypes
    for i in range(n):
        p = params[i]
        ctypes.memmove(ctypes.byref(p), ctypes.byref(base), ctypes.sizeof(base))
        kr, km, ko = np.exp(rng.uniform(lo, hi, size=3))
        p.rayleigh_scattering_scale = base.rayleigh_scattering_scale * kr
        p.mie_scattering_scale = base.mie_scattering_scale * km
        p.mie_absorption_scale = base.mie_absorption_scale * km
        p.ozone_absorption_scale = base.ozone_absorption_scale * ko
        p.mie_phase_g = rng.uniform(0.6, 0.9)
        cams.append(Camera(position=(0.0, float(rng.uniform(0.0, 10.0)), 0.0), yaw=float(rng.uniform(0, 360)),
                           pitch=float(rng.uniform(-5.0, 30.0))))
        zen.append(float(rng.uniform(0.0, 95.0)))
        azi.append(float(rng.uniform(0.0, 360.0)))
    return params, cams, zen, azi


def batched_lut_sets(n: int = 256, seed: int = SEED):
    """n parameter sets: Rayleigh, Mie and ozone coefficients each scaled by a
    log-uniform factor in [0.5, 1.5] of the Earth-like set, Mie g ~ U[0.6, 0.9];
    each set paired with a view at altitude U[0, 10] km, sun zenith U[0, 95] deg,
    sun azimuth U[0, 360) deg."""
    params, cams, zen, azi = _batched_sets(n, seed)
    renders = (_abi.AtmosphereRenderParameters * n)()
    for i in range(n):
        renders[i] = render_parameters(cams[i], zen[i], azi[i])
    return params, renders


VIEW_SIZES = ((640, 360), (1280, 720), (1920, 1080), (3840, 2160))


def batched_frame(n_sets: int = 256, n_views: int = 64, seed: int = SEED):
    """The batched workload: n_sets parameter sets (as batched_lut_sets) and
    n_views views of sizes drawn uniformly from VIEW_SIZES; view i looks
    through the camera and sun of set i (its aspect ratio set to the view's).
    Returns (params, renders, views, set_of_view)."""
    params, cams, zen, azi = _batched_sets(n_sets, seed)
    rng = np.random.default_rng(seed + 1)
    views = (_abi.CloudView * n_views)()
    for i in range(n_views):
        w, h = VIEW_SIZES[int(rng.integers(len(VIEW_SIZES)))]
        c = cams[i]
        cams[i] = Camera(position=c.position, yaw=c.yaw, pitch=c.pitch, fovy=60.0, width=w, height=h)
        views[i] = frame_view(cams[i], zen[i], azi[i])
    renders = (_abi.AtmosphereRenderParameters * n_sets)()
    for i in range(n_sets):
        renders[i] = render_parameters(cams[i], zen[i], azi[i])
    return params, renders, views, list(range(n_views))


# ---------------------------------------------------------------------------
# Cloud frame workload (1920x1080, layer 1.5-4.0 km)
# ---------------------------------------------------------------------------
def noise_info(seed, freq, rmin, rmax):
    ci = _abi.NoiseCreateInfo()
    ci.seed, ci.base_frequency, ci.remap_min, ci.remap_max = seed, freq, rmin, rmax
    return ci


def noise_desc(w, h, d, channels, octaves=3):
    desc = _abi.NoiseTextureDesc()
    desc.width, desc.height, desc.depth, desc.octaves = w, h, d, octaves
    desc.channels = len(channels)
    for i, (kind, a, b) in enumerate(channels):
        desc.channel[i].kind = kind
        desc.channel[i].a = a
        if b is not None:
            desc.channel[i].b = b
    return desc


def cloud_map_desc(size=512, octaves=3):
    """Weather / cloud map (CLOUD_MAP_GEN, NoiseGen.comp:77-92): R = Perlin fBm
    coverage-density, G = Worley fBm cloud type; CloudMapBuffer defaults
    (VolumetricCloudDefaultMaterial.h:66-71)."""
    return noise_desc(size, size, 1, [(_abi.SKYR_NOISE_PERLIN, noise_info(0, 3, 0.35, 0.75), None),
                                      (_abi.SKYR_NOISE_WORLEY, noise_info(0, 5, 0.8, 0.4), None)], octaves)


def base_noise_desc(size=128, octaves=3):
    """128^3 RGBA8 base noise: R = Perlin-Worley (DETAIL_MAP_GEN, NoiseGen.comp:95-104,
    DetailBuffer defaults VolumetricCloudDefaultMaterial.h:73-78), G/B/A = Worley
    fBm at base frequencies 8, 16, 32.  The reference materials read channel R."""
    return noise_desc(size, size, size, [
        (_abi.SKYR_NOISE_PERLIN_WORLEY, noise_info(0, 7, 0.23, 1.0), noise_info(0, 11, 1.0, 0.0)),
        (_abi.SKYR_NOISE_WORLEY, noise_info(1, 8, 1.0, 0.0), None),
        (_abi.SKYR_NOISE_WORLEY, noise_info(2, 16, 1.0, 0.0), None),
        (_abi.SKYR_NOISE_WORLEY, noise_info(3, 32, 1.0, 0.0), None)], octaves)


def detail_noise_desc(size=32, octaves=3):
    """32^3 RGBA8 Worley detail noise (base frequencies 2, 4, 8, 16).  Generated
    for the frame's texture set; the reference's material formulas do not
    sample a second 3D texture."""
    return noise_desc(size, size, size, [(_abi.SKYR_NOISE_WORLEY, noise_info(4 + i, 2 << i, 1.0, 0.0), None)
                                         for i in range(4)], octaves)


def displacement_desc(size=128, octaves=3):
    """DISPLACEMENT_GEN (NoiseGen.comp:57-74): 4 Perlin fBm channels, seeds s..s+3
    (DisplacementBuffer defaults, VolumetricCloudDefaultMaterial.h:80-84)."""
    return noise_desc(size, size, 1, [(_abi.SKYR_NOISE_PERLIN, noise_info(i, 6, 0.25, 0.75), None)
                                      for i in range(4)], octaves)


def frame_cloud_parameters() -> _abi.CloudParameters:
    """Cloud layer 1.5-4.0 km, 64 primary steps, 6 light-march steps,
    dual-lobe HG g = 0.8 / -0.3; the other fields are the reference defaults
    (src/SkyRendering/VolumetricCloud.h:20-35)."""
    from .config import cloud_defaults

    c = cloud_defaults()
    c.bottom_altitude, c.thickness = 1.5, 2.5
    c.max_raymarch_steps = 64.0
    c.shadow_steps = 6.0
    c.phase_g_forward, c.phase_g_back = 0.8, -0.3
    return c


def frame_material(kind: int = None) -> _abi.CloudMaterial:
    """VolumetricCloudDefaultMaterial1 defaults with density 50/km (0.05/m)."""
    from .config import material_defaults

    kind = _abi.SKYR_MATERIAL_DEFAULT1 if kind is None else kind
    m = material_defaults(kind)
    if kind in (_abi.SKYR_MATERIAL_DEFAULT0, _abi.SKYR_MATERIAL_DEFAULT1):
        m.density = 50.0
    return m


def frame_view(cam: Camera, sun_zenith_deg: float, sun_azimuth_deg: float = 60.0,
               ap_max_distance: float = 32.0, width=None, height=None) -> _abi.CloudView:
    v = _abi.CloudView()
    v.camera_position[:] = list(cam.position)
    v.view_projection[:] = column_major(cam.view_projection())
    v.fovy = cam.fovy
    v.viewport_width, v.viewport_height = cam.width, cam.height
    v.width, v.height = width or cam.width, height or cam.height
    v.sun_direction_theta, v.sun_direction_phi = sun_zenith_deg, sun_azimuth_deg
    v.frame_id = 0.0
    v.aerial_perspective_lut_max_distance = ap_max_distance
    return v


# ---------------------------------------------------------------------------
# Voxel path-tracer scene: a synthetic dense FP16 grid spanning 1 km along its
# longest axis, max extinction 40/km, 1.5 km in front of the camera
# ---------------------------------------------------------------------------
PT_GRID_DIMS = (512, 640, 352)  # x, y (horizontal), z (up)
PT_EXTENT_KM = 1.0  # along the longest axis (640 voxels)
PT_SIGMA_MAX = 40.0


def pt_grid_generator(dims=PT_GRID_DIMS, seed=0x5EED) -> _abi.GridGenerator:
    """Seeded 4-octave Worley fBm inside a soft ellipsoid."""
    g = _abi.GridGenerator()
    g.nx, g.ny, g.nz = dims
    g.seed, g.base_frequency, g.octaves = seed, 4, 4
    g.center[:] = [0.5, 0.5, 0.45]
    g.radii[:] = [0.46, 0.46, 0.42]
    g.inner, g.threshold = 0.55, 0.15
    return g


def pt_grid_placement(dims=PT_GRID_DIMS):
    """(origin, voxel_size) of the grid in the local z-up cloud frame (km)."""
    voxel = PT_EXTENT_KM / max(dims)
    ex, ey, ez = (n * voxel for n in dims)
    return (1.5, -0.5 * ey, 1.5), voxel


def pt_cloud_parameters(dims=PT_GRID_DIMS) -> _abi.CloudParameters:
    c = frame_cloud_parameters()
    origin, voxel = pt_grid_placement(dims)
    c.bottom_altitude = origin[2]
    c.thickness = dims[2] * voxel
    return c


def pt_parameters() -> _abi.PathtraceParameters:
    """HG g = 0.857 single lobe, albedo 1, up to 128 bounces, brick majorants."""
    p = _abi.PathtraceParameters()
    _abi.call("skyr_pathtrace_parameters_default", C_ref(p))
    p.forward_phase_g = 0.857
    p.forward_scattering_ratio = 1.0
    p.region_box_half_width = 3.0
    p.sigma_t_max = PT_SIGMA_MAX
    p.max_bounces = 128
    return p


def pt_camera(width=1024, height=1024) -> Camera:
    """Mid-cloud altitude, looking along local +x (world -z) at the grid."""
    origin, voxel = pt_grid_placement()
    alt = origin[2] + 0.5 * PT_GRID_DIMS[2] * voxel
    return Camera(position=(0.0, alt, 0.0), yaw=-90.0, pitch=0.0, fovy=35.0, width=width, height=height,
                  z_near=0.01, z_far=1000.0)


# ---------------------------------------------------------------------------
# Full-screen composite inputs: a seeded star map (the reference loads
# data/NASA/starmap_2020_4k.jpg) and a depth buffer with the Earth's surface
# and one near occluder
# ---------------------------------------------------------------------------
def star_map(width: int = 1024, height: int = 512, n_stars: int = 6000, seed: int = SEED) -> np.ndarray:
    """sRGB8 RGB texels [height][width][3]: a faint band and n_stars point stars
    of random magnitude and colour temperature."""
    rng = np.random.default_rng(seed)
    img = np.zeros((height, width, 3), dtype=np.float64)
    v = (np.arange(height) + 0.5) / height
    img += (0.03 * np.exp(-((v - 0.5) / 0.08) ** 2))[:, None, None]
    ys, xs = rng.integers(0, height, n_stars), rng.integers(0, width, n_stars)
    mag = rng.uniform(0.05, 1.0, n_stars) ** 3
    tint = rng.uniform(-0.2, 0.2, n_stars)
    col = np.stack([1.0 + tint, np.ones(n_stars), 1.0 - tint], -1) * mag[:, None]
    np.add.at(img, (ys, xs), col)
    return np.round(np.clip(img, 0.0, 1.0) * 255.0).astype(np.uint8)


def ground_depth(cam: Camera, width: int, height: int, R: float, occluder: bool = True) -> np.ndarray:
    """GL window depth [height][width] of the Earth's surface below the horizon
    and, when `occluder`, of a screen rectangle 2.5 km away; 1 elsewhere."""
    vp = cam.view_projection()
    ivp = np.linalg.inv(vp)
    ys, xs = np.mgrid[0:height, 0:width]
    ndc = np.stack([(xs + 0.5) / width * 2 - 1, (ys + 0.5) / height * 2 - 1, np.zeros(xs.shape),
                    np.ones(xs.shape)], -1)
    p = ndc @ ivp.T
    p = p[..., :3] / p[..., 3:]
    o = np.asarray(cam.position, dtype=np.float64)
    d = p - o
    d /= np.linalg.norm(d, axis=-1, keepdims=True)
    c = o - np.array([0.0, -R, 0.0])
    b = d @ c
    disc = b * b - (c @ c - R * R)
    t = np.where((disc > 0) & (b < 0), -b - np.sqrt(np.maximum(disc, 0)), np.inf)
    if occluder:
        occ = (xs > 0.3 * width) & (xs < 0.45 * width) & (ys > 0.35 * height) & (ys < 0.75 * height)
        t = np.where(occ, 2.5, t)
    hit = np.isfinite(t)
    q = o + d * np.where(hit, t, 1.0)[..., None]
    clip = np.concatenate([q, np.ones_like(q[..., :1])], -1) @ vp.T
    return np.where(hit, 0.5 * clip[..., 2] / clip[..., 3] + 0.5, 1.0).astype(np.float32)
