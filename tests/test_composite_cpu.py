"""CPU checks of the full-screen atmosphere composite (include/skyr_composite.h):
the reference defaults, argument checks, and known answers of the oracle's
restatement of the ATMOSPHERE_RENDER shader (AtmosphereRenderer.glsl:325-432)
with an almost empty atmosphere (transmittance 1):

* looking at the sun's centre: solar illuminance / (pi r^2), the limb
  darkening factor 1; at the limb the factor goes to 0;
* a constant star map: the star luminance scale times the sRGB-decoded value;
* an object pixel: the given object luminance;
* with no depth buffer and the LUT switches off, every pixel is raymarched.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import workloads as W
from skyrendering_gb300.atmosphere import composite_parameters


def _thin_atmosphere():
    p = W.earth_like_atmosphere()
    p.rayleigh_scattering_scale = 1e-9
    p.mie_scattering_scale = 1e-9
    p.mie_absorption_scale = 0.0
    p.ozone_absorption_scale = 0.0
    return p


def _luts(p, r, s):
    return orc.lut_set(p, r, s, 64)


def test_defaults_and_invalid_arguments():
    cp = composite_parameters()
    assert (cp.star_luminance_scale, cp.raymarching_steps) == (pytest.approx(0.005), 40.0)
    assert (cp.use_sky_view_lut, cp.use_aerial_perspective_lut, cp.dither_sample_point) == (0, 0, 1)
    lib = _abi.lib()
    p, s = W.earth_like_atmosphere(), W.plain_lut_sizes()
    r = W.render_parameters(W.frame_camera(), 45.0)
    inp = _abi.CompositeInputs()
    inp.width = inp.height = 8
    assert lib.skyr_atmosphere_composite(None, C.byref(p), C.byref(r), C.byref(cp), C.byref(s), None, None, None,
                                         None, None, None, C.byref(inp), None) == _abi.SKYR_EINVAL


def test_oracle_sun_disc():
    p = _thin_atmosphere()
    s = W.plain_lut_sizes()
    zenith, azimuth = 50.0, 30.0
    cam = W.Camera(position=(0.0, 1.0, 0.0), yaw=azimuth, pitch=90.0 - zenith, width=1, height=1)
    r = W.render_parameters(cam, zenith, azimuth)
    luts = _luts(p, r, s)
    cp = composite_parameters(dither_sample_point=0)
    out = orc.atmosphere_composite(p, r, cp, s, luts, 1, 1)
    sar = math.radians(p.sun_angular_radius)
    want = np.array(p.solar_illuminance[:]) / (math.pi * sar * sar)
    np.testing.assert_allclose(out[0, :3], want, rtol=1e-5)
    assert out[0, 3] == 1.0
    # at 0.999 of the disc's radius the limb darkening has taken most of it away
    cam.yaw = azimuth + math.degrees(sar) * 0.999 / math.sin(math.radians(zenith))
    r = W.render_parameters(cam, zenith, azimuth)
    edge = orc.atmosphere_composite(p, r, cp, s, luts, 1, 1)
    assert np.all(edge[0, :3] < 0.5 * want)


def test_oracle_constant_star_map_and_object():
    p = _thin_atmosphere()
    s = W.plain_lut_sizes()
    cam = W.Camera(position=(0.0, 1.0, 0.0), yaw=90.0, pitch=60.0, width=8, height=6)
    r = W.render_parameters(cam, 95.0, 200.0)  # the sun below the horizon, out of view
    luts = _luts(p, r, s)
    cp = composite_parameters(dither_sample_point=0)
    stars = np.full((16, 32, 3), 128, dtype=np.uint8)
    out = orc.atmosphere_composite(p, r, cp, s, luts, 8, 6, star_map=stars)
    c = 128 / 255.0
    lin = ((c + 0.055) / 1.055) ** 2.4
    np.testing.assert_allclose(out[:, :3], cp.star_luminance_scale * lin, rtol=1e-6)
    # an object at depth 0.99 everywhere: its luminance, the stars hidden
    depth = np.full((6, 8), 0.99, dtype=np.float32)
    obj = np.zeros((48, 4), dtype=np.float32)
    obj[:, :3] = [1.0, 2.0, 3.0]
    out = orc.atmosphere_composite(p, r, cp, s, luts, 8, 6, depth=depth, object_luminance=obj, star_map=stars)
    np.testing.assert_allclose(out[:, :3], np.broadcast_to([1.0, 2.0, 3.0], (48, 3)), rtol=1e-6)


def test_oracle_lut_sky_close_to_raymarched_sky():
    """The sky-view LUT is the same integral tabulated: a coarse agreement."""
    p, s = W.earth_like_atmosphere(), W.plain_lut_sizes()
    cam = W.Camera(position=(0.0, 1.0, 0.0), yaw=90.0, pitch=20.0, width=16, height=9)
    r = W.render_parameters(cam, 45.0)
    luts = _luts(p, r, s)
    ray = orc.atmosphere_composite(p, r, composite_parameters(dither_sample_point=0), s, luts, 16, 9)
    lut = orc.atmosphere_composite(p, r, composite_parameters(use_sky_view_lut=1), s, luts, 16, 9)
    rel = np.abs(lut[:, :3] - ray[:, :3]).sum() / np.abs(ray[:, :3]).sum()
    assert rel < 0.05, rel
