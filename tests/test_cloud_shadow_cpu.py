"""CPU checks of the cloud shadow passes: the host-side light transform of the
library against the oracle's, argument checks, and known-answer tests that pin
the oracle's shadow passes (no GPU needed).

* light frame: the library builds the frustum section from NDC corners, the
  oracle from the Camera's vectors recovered from the matrix, as the
  reference does (GetLightProjection, VolumetricCloud.cpp:138-166); both
  agree to FP32 storage (1e-6 relative) for sun positions including the
  zenith (the lookAt up switches to +x) and the batched workload's views;
* reprojection: the identity for an unchanged frame without wind; a wind
  delta is a translation of the light NDC;
* oracle shadow map with a constant extinction: transmittance and depth in
  closed form (numpy restatement of VolumetricCloudShadowMap.comp:18-66);
  the temporal blend is 0.8 previous + 0.2 current;
* oracle blur of a constant map: the constant times (sum of weights)^2;
* oracle froxel of a constant map inside the light frustum: the map's
  transmittance in every texel.
"""
import ctypes as C
import math

import numpy as np
import pytest

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import cloud as CL
from skyrendering_gb300 import workloads as W

VIEWS = [(45.0, 60.0), (0.0, 0.0), (85.0, 200.0), (30.0, -40.0), (95.0, 10.0)]


def _mat_close(a, b, rel=1e-6):
    scale = max(np.abs(b).max(), 1.0)
    return np.abs(a - b).max() <= rel * scale


@pytest.mark.parametrize("zenith,azimuth", VIEWS)
def test_light_frame_matches_oracle(zenith, azimuth):
    atmo, cp = W.earth_like_atmosphere(), W.frame_cloud_parameters()
    v = W.frame_view(W.frame_camera(), zenith, azimuth)
    sizes = CL.shadow_sizes(v.viewport_width, v.viewport_height)
    f = CL.light_frame(atmo, cp, v, sizes)
    got = orc.frame_array(f)
    want, has = orc.light_frame(atmo, cp, v, 512, 512)
    assert not has and f.has_previous == 0
    for k in range(3):
        assert _mat_close(got[16 * k:16 * k + 16], want[16 * k:16 * k + 16]), k
    # the camera sits on the light's z = 0 plane at the light NDC of the map
    cam_l = np.array([0.0, 0.0, 1.0, 1.0])  # local frame: 1 km above the surface point below it
    lvp = want[:16].reshape(4, 4).T
    ndc = lvp @ cam_l
    assert abs(ndc[2]) < 1e-9 and abs(ndc[0]) <= 1 and abs(ndc[1]) <= 1


def test_light_frame_on_batched_views():
    params, renders, views, sov = W.batched_frame(8, 8, seed=0x5AD0)
    cp = W.frame_cloud_parameters()
    cp.shadow_map_max_distance = 48.266  # bin/config.json
    for i in range(8):
        v = views[i]
        sizes = CL.shadow_sizes(v.viewport_width, v.viewport_height)
        got = orc.frame_array(CL.light_frame(params[sov[i]], cp, v, sizes))
        want, _ = orc.light_frame(params[sov[i]], cp, v, 512, 512)
        for k in range(3):
            assert _mat_close(got[16 * k:16 * k + 16], want[16 * k:16 * k + 16]), (i, k)


def test_reprojection():
    atmo, cp = W.earth_like_atmosphere(), W.frame_cloud_parameters()
    v = W.frame_view(W.frame_camera(), 40.0, 30.0)
    sizes = CL.shadow_sizes(1920, 1080)
    f0 = CL.light_frame(atmo, cp, v, sizes)
    same = CL.light_frame(atmo, cp, v, sizes, previous=f0)
    assert same.has_previous == 1
    np.testing.assert_allclose(np.array(same.shadow_map_reproject[:]), np.eye(4).reshape(-1), atol=1e-6)
    # wind: the previous map's NDC of a point is shifted by the light VP of the wind vector
    wind = (0.3, -0.1)
    w = CL.light_frame(atmo, cp, v, sizes, previous=f0, wind_delta=wind)
    m = np.array(w.shadow_map_reproject[:]).reshape(4, 4).T
    lvp = np.array(f0.light_view_projection[:]).reshape(4, 4).T
    shift = lvp[:3, :3] @ np.array([wind[0], wind[1], 0.0])
    np.testing.assert_allclose(m[:3, :3], np.eye(3), atol=1e-6)
    np.testing.assert_allclose(m[:3, 3], shift, atol=1e-6)
    want, _ = orc.light_frame(atmo, cp, v, 512, 512, previous=orc.frame_array(f0), wind=wind)
    np.testing.assert_allclose(orc.frame_array(w)[48:], want[48:], atol=1e-6)
    # a moved camera and a turned sun: library and oracle agree
    v2 = W.frame_view(W.Camera(position=(0.4, 1.2, -0.3), yaw=95.0, pitch=12.0), 42.0, 33.0)
    w2 = CL.light_frame(atmo, cp, v2, sizes, previous=f0, wind_delta=wind)
    want2, _ = orc.light_frame(atmo, cp, v2, 512, 512, previous=orc.frame_array(f0), wind=wind)
    np.testing.assert_allclose(orc.frame_array(w2)[48:], want2[48:], atol=2e-6)


def test_sizes_and_invalid_arguments():
    s = CL.shadow_sizes(1920, 1080)
    assert (s.map_width, s.map_height, s.froxel_width, s.froxel_height, s.froxel_depth) == (512, 512, 160, 90, 128)
    with pytest.raises(_abi.SkyrError):
        CL.shadow_sizes(8, 8)
    atmo, cp = W.earth_like_atmosphere(), W.frame_cloud_parameters()
    v = W.frame_view(W.frame_camera(), 45.0)
    bad = _abi.CloudParameters.from_buffer_copy(cp)
    bad.shadow_map_max_distance = 0.0
    with pytest.raises(_abi.SkyrError):
        CL.light_frame(atmo, bad, v, s)
    sv = _abi.CloudView.from_buffer_copy(v)
    sv.view_projection[:] = [0.0] * 16
    with pytest.raises(_abi.SkyrError):
        CL.light_frame(atmo, cp, sv, s)
    bs = _abi.CloudShadowSizes.from_buffer_copy(s)
    bs.map_width = 0
    with pytest.raises(_abi.SkyrError):
        CL.light_frame(atmo, cp, v, bs)
    # the render entry point checks its arguments before touching a device
    lib = _abi.lib()
    f = CL.light_frame(atmo, cp, v, s)
    assert lib.skyr_cloud_shadow_render(None, C.byref(atmo), C.byref(cp), None, None, C.byref(v), C.byref(s),
                                        C.byref(f), None, None, None, None, None) == _abi.SKYR_EINVAL


# ---- oracle known answers ---------------------------------------------------
def _minimal(density=0.7):
    m = _abi.CloudMaterial()
    _abi.call("skyr_cloud_material_default", _abi.SKYR_MATERIAL_MINIMAL, C.byref(m))
    m.density = density
    return m


def _texel_closed_form(atmo, cp, frame, x, y, w, h, sun_local, density):
    """VolumetricCloudShadowMap.comp:37-66 with a constant SampleSigmaT."""
    ilvp = frame[16:32].reshape(4, 4).T
    u, v = (x + 0.5) / w, (y + 0.5) / h
    o = ilvp @ np.array([u * 2 - 1, v * 2 - 1, 0.0, 1.0])
    o = o[:3] / o[3]
    d = -sun_local
    R = atmo.bottom_radius
    up = np.array([o[0], o[1], o[2] + R])
    r = np.linalg.norm(up)
    mu = up @ d / r
    rb, rt = R + cp.bottom_altitude, R + cp.bottom_altitude + cp.thickness
    t1 = t2 = 0.0
    dt = r * r * (mu * mu - 1) + rt * rt
    if dt > 0:
        db = r * r * (mu * mu - 1) + rb * rb
        t1 = -r * mu - math.sqrt(dt)
        t2 = -r * mu + (-math.sqrt(db) if db >= 0 else math.sqrt(dt))
    dist = min(max(t2 - t1, 0.0), cp.thickness / math.cos(math.radians(85.0)))
    od = 0.0
    if dist > 0:
        steps = np.float32(12.0) + (np.float32(6.0) - np.float32(12.0)) * np.float32(abs(d[2]))
        od = density * int(steps) * (dist / float(steps))
    return 0.5 * (t1 + t2), math.exp(-od)


def _local_sun(atmo, view):
    """The sun in the local frame of VolumetricCloud::Update (VolumetricCloud.cpp:188-220)."""
    R = atmo.bottom_radius
    cam = np.array(view.camera_position[:], dtype=np.float64)
    up = cam - np.array([0.0, -R, 0.0])
    up /= np.linalg.norm(up)
    front = np.cross(up, [1.0, 0.0, 0.0])
    front /= np.linalg.norm(front)
    right = np.cross(up, front)
    right /= np.linalg.norm(right)
    th, ph = math.radians(view.sun_direction_theta), math.radians(view.sun_direction_phi)
    s = np.array([math.cos(ph) * math.sin(th), math.cos(th), math.sin(ph) * math.sin(th)])
    loc = np.array([front @ s, right @ s, up @ s])
    return loc / np.linalg.norm(loc)


@pytest.mark.parametrize("zenith", [30.0, 70.0])
def test_oracle_shadow_map_constant_density(zenith):
    atmo, cp = W.earth_like_atmosphere(), W.frame_cloud_parameters()
    v = W.frame_view(W.frame_camera(), zenith, 50.0, width=64, height=36)
    m = _minimal()
    frame, _ = orc.light_frame(atmo, cp, v, 32, 32)
    bn = np.random.default_rng(0).uniform(0, 1, 4096).astype(np.float32)
    got = orc.shadow_map(atmo, cp, m, {}, v, 32, 32, frame, False, bn).reshape(32, 32, 2)
    sun = _local_sun(atmo, v)
    for y in range(0, 32, 5):
        for x in range(0, 32, 3):
            d, t = _texel_closed_form(atmo, cp, frame, x, y, 32, 32, sun, m.density)
            assert got[y, x, 0] == pytest.approx(d, rel=1e-9, abs=1e-9)
            assert got[y, x, 1] == pytest.approx(t, rel=1e-9, abs=1e-12)
    assert (got[..., 1] < 1).all()
    # temporal blend with an unchanged frame: 0.8 of the previous map
    prev = np.stack([np.full((32, 32), 3.0), np.full((32, 32), 0.25)], axis=-1)
    same, _ = orc.light_frame(atmo, cp, v, 32, 32, previous=frame)
    blended = orc.shadow_map(atmo, cp, m, {}, v, 32, 32, same, True, bn, previous_map=prev).reshape(32, 32, 2)
    # (edge texels reproject onto the range check's bounds, where rounding decides)
    np.testing.assert_allclose(blended[1:-1, 1:-1], (0.8 * prev + 0.2 * got)[1:-1, 1:-1], rtol=1e-9, atol=1e-9)


def test_oracle_blur_constant_and_impulse():
    wgt = np.array([0.227027, 0.1945946, 0.1216216, 0.054054, 0.016216])
    total = wgt[0] + 2 * wgt[1:].sum()
    raw = np.stack([np.full((20, 24), 2.0), np.full((20, 24), 0.5)], axis=-1)
    out = orc.shadow_blur(raw)
    np.testing.assert_allclose(out, raw * total * total, rtol=1e-12)
    # an impulse away from the edges spreads as the outer product of the weights
    imp = np.zeros((20, 24, 2))
    imp[10, 12, 1] = 1.0
    out = orc.shadow_blur(imp)[..., 1]
    k = np.concatenate([wgt[:0:-1], wgt])
    want = np.zeros((20, 24))
    want[6:15, 8:17] = np.outer(k, k)
    np.testing.assert_allclose(out, want, atol=1e-15)


def test_oracle_froxel_of_constant_map():
    atmo, cp = W.earth_like_atmosphere(), W.frame_cloud_parameters()
    v = W.frame_view(W.frame_camera(), 45.0, 60.0)
    frame, _ = orc.light_frame(atmo, cp, v, 64, 64)
    t = 0.3125  # t * 65535 is not a tie
    m = np.stack([np.full((64, 64), -1e9), np.full((64, 64), t)], axis=-1)  # every sample behind the shadow
    fx, exact = orc.shadow_froxel(atmo, cp, _minimal(), {}, v, frame, m, (16, 9, 24))
    np.testing.assert_allclose(exact, t, rtol=1e-12)
    assert np.all(fx == 20480)
    # in front of the shadow's depth the visibility is 1
    m[..., 0] = 1e9
    fx, exact = orc.shadow_froxel(atmo, cp, _minimal(), {}, v, frame, m, (16, 9, 24))
    np.testing.assert_allclose(exact, 1.0, rtol=1e-12)
