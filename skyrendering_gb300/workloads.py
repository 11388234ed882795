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
    p = _abi.AtmosphereParameters()
    _abi.call("skyr_atmosphere_parameters_default", C_ref(p))
    return p


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


def batched_lut_sets(n: int = 256, seed: int = SEED):
    """n parameter sets: Rayleigh, Mie and ozone coefficients each scaled by a
    log-uniform factor in [0.5, 1.5] of the Earth-like set, Mie g ~ U[0.6, 0.9];
    each set paired with a view at altitude U[0, 10] km, sun zenith U[0, 95] deg,
    sun azimuth U[0, 360) deg."""
    rng = np.random.default_rng(seed)
    base = earth_like_atmosphere()
    params = (_abi.AtmosphereParameters * n)()
    renders = (_abi.AtmosphereRenderParameters * n)()
    lo, hi = math.log(0.5), math.log(1.5)
    for i in range(n):
        p = params[i]
        import ctypes
        ctypes.memmove(ctypes.byref(p), ctypes.byref(base), ctypes.sizeof(base))
        kr, km, ko = np.exp(rng.uniform(lo, hi, size=3))
        p.rayleigh_scattering_scale = base.rayleigh_scattering_scale * kr
        p.mie_scattering_scale = base.mie_scattering_scale * km
        p.mie_absorption_scale = base.mie_absorption_scale * km
        p.ozone_absorption_scale = base.ozone_absorption_scale * ko
        p.mie_phase_g = rng.uniform(0.6, 0.9)
        cam = Camera(position=(0.0, float(rng.uniform(0.0, 10.0)), 0.0), yaw=float(rng.uniform(0, 360)),
                     pitch=float(rng.uniform(-5.0, 30.0)))
        renders[i] = render_parameters(cam, float(rng.uniform(0.0, 95.0)), float(rng.uniform(0.0, 360.0)))
    return params, renders
