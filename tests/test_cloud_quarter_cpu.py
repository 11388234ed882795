"""CPU checks of the quarter-resolution cloud pass: the host-side temporal
constants against a numpy restatement of VolumetricCloud::Update
(VolumetricCloud.cpp:188-239), argument checks, and known-answer tests of the
oracle's checkerboard, index, reconstruct and upscale passes (no GPU needed).
"""
import ctypes as C

import numpy as np
import pytest

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import cloud as CL
from skyrendering_gb300 import workloads as W

Z_NEAR, Z_FAR = 0.3, 50000.0  # the workload Camera's planes


def _model(R, cam):
    """The local z-up frame (VolumetricCloud.cpp:188-201) as a row-major 4x4."""
    cam = np.asarray(cam, dtype=np.float64)
    up = cam - np.array([0.0, -R, 0.0])
    up /= np.linalg.norm(up)
    origin = np.array([0.0, -R, 0.0]) + up * R
    front = np.cross(up, [1.0, 0.0, 0.0])
    front /= np.linalg.norm(front)
    right = np.cross(up, front)
    right /= np.linalg.norm(right)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = front, right, up, origin
    return m


def _vp(view):
    return np.array(view.view_projection[:], dtype=np.float64).reshape(4, 4).T


def test_temporal_frame_matches_numpy():
    atmo = W.earth_like_atmosphere()
    cam0 = W.Camera(position=(0.0, 1.0, 0.0), yaw=90.0, pitch=10.0)
    cam1 = W.Camera(position=(0.35, 1.05, -0.2), yaw=92.0, pitch=9.0)
    v0, v1 = W.frame_view(cam0, 45.0), W.frame_view(cam1, 45.0)
    f = CL.temporal_frame(atmo, v1, None, None, Z_NEAR, Z_FAR, 6)
    assert f.has_previous == 0 and f.base_shading_index == 2
    assert (f.z_near, f.z_far) == (pytest.approx(Z_NEAR), pytest.approx(Z_FAR))
    wind = (0.02, -0.01)
    f = CL.temporal_frame(atmo, v1, v0, wind, Z_NEAR, Z_FAR, 7)
    assert f.has_previous == 1 and f.base_shading_index == 3
    R = atmo.bottom_radius
    m1, m0 = _model(R, v1.camera_position[:]), _model(R, v0.camera_position[:])
    delta = np.linalg.inv(m1)[:3, :3] @ (np.array(v1.camera_position[:]) - np.array(v0.camera_position[:]))
    delta[:2] += wind
    dm = np.eye(4)
    dm[0, 3], dm[1, 3] = delta[0], delta[1]
    want = _vp(v0) @ m0 @ dm
    got = np.array(f.reproject[:]).reshape(4, 4).T
    np.testing.assert_allclose(got, want, rtol=2e-6, atol=1e-6 * np.abs(want).max())
    # an unchanged camera without wind reprojects every point onto itself
    same = CL.temporal_frame(atmo, v0, v0, None, Z_NEAR, Z_FAR, 0)
    p = np.array([3.0, 5.0, 2.0, 1.0])
    a = np.array(same.reproject[:]).reshape(4, 4).T @ p
    b = _vp(v0) @ _model(R, v0.camera_position[:]) @ p
    np.testing.assert_allclose(a[:3] / a[3], b[:3] / b[3], rtol=1e-5, atol=1e-6)


def test_temporal_frame_invalid_arguments():
    atmo = W.earth_like_atmosphere()
    v = W.frame_view(W.frame_camera(), 45.0)
    for zn, zf in ((0.0, 10.0), (5.0, 5.0), (-1.0, 10.0)):
        with pytest.raises(_abi.SkyrError):
            CL.temporal_frame(atmo, v, None, None, zn, zf, 0)
    sv = _abi.CloudView.from_buffer_copy(v)
    sv.view_projection[:] = [0.0] * 16
    with pytest.raises(_abi.SkyrError):
        CL.temporal_frame(atmo, v, sv, None, Z_NEAR, Z_FAR, 0)
    lib = _abi.lib()
    f = CL.temporal_frame(atmo, v, None, None, Z_NEAR, Z_FAR, 0)
    b = _abi.CloudQuarterBuffers()
    assert lib.skyr_cloud_render_quarter(None, C.byref(atmo), None, None, None, C.byref(v), None, None, None, None,
                                         None, None, C.byref(f), C.byref(b), None) == _abi.SKYR_EINVAL


# ---- oracle known answers ---------------------------------------------------
def _ld(d):
    zn, zf = float(np.float32(Z_NEAR)), float(np.float32(Z_FAR))  # the planes travel as float
    x, y = 1.0 / zn, (zf - zn) / (zf * zn)
    return 1.0 / (x - y * d)


def test_oracle_checkerboard():
    rng = np.random.default_rng(4)
    w, h = 40, 24
    d = rng.uniform(0.9, 1.0, (h, w)).astype(np.float32)
    cb = orc.checkerboard(d, w, h)
    blocks = d.reshape(h // 2, 2, w // 2, 2).transpose(0, 2, 1, 3).reshape(h // 2, w // 2, 4).astype(np.float64)
    yy, xx = np.mgrid[0:h // 2, 0:w // 2]
    want = np.where((xx & 1) == (yy & 1), blocks.max(-1), blocks.min(-1))
    np.testing.assert_array_equal(cb, want)
    np.testing.assert_array_equal(orc.checkerboard(None, w, h), np.ones((h // 2, w // 2)))


@pytest.mark.parametrize("base", [0, 1, 2, 3])
def test_oracle_index_on_flat_depth_rotates(base):
    w, h = 64, 40
    cb = np.full((h // 2, w // 2), 0.99)
    idx = orc.index_gen(cb, w, h, Z_NEAR, Z_FAR, base)
    yy, xx = np.mgrid[0:h // 4, 0:w // 4]
    # interior texels: every neighbour agrees, so the rotating PosToIndex choice
    want = (base + ((xx + yy) & 1)) & 3
    np.testing.assert_array_equal(idx[1:-1, 1:-1, 0], want[1:-1, 1:-1])
    np.testing.assert_allclose(idx[..., 1], _ld(0.99), rtol=1e-12)


def test_oracle_index_picks_a_lone_far_texel():
    w, h = 32, 32
    cb = np.full((16, 16), 0.9)
    cb[8, 9] = 1.0  # quarter texel (4, 4): its footprint is cb[8:10, 8:10]; (9, 8) is gather .z, index 2
    idx = orc.index_gen(cb, w, h, Z_NEAR, Z_FAR, 0)
    assert idx[4, 4, 0] == 2.0
    assert idx[4, 4, 1] == pytest.approx(_ld(1.0), rel=1e-12)


def test_oracle_upscale_constant():
    w, h = 36, 20
    rec = np.zeros((h // 2, w // 2, 4))
    rec[...] = [0.3, 0.2, 0.1, 0.5]
    hdr = np.random.default_rng(1).uniform(0, 2, (h, w, 4))
    out = orc.upscale(w, h, None, Z_NEAR, Z_FAR, np.ones((h // 2, w // 2)), rec, hdr)
    np.testing.assert_allclose(out[..., :3], hdr[..., :3] * 0.5 + [0.3, 0.2, 0.1], rtol=1e-12)
    np.testing.assert_array_equal(out[..., 3], hdr[..., 3])
    rec[..., 3] = 0.005  # below kMinTransmittance: the background is dropped
    out = orc.upscale(w, h, None, Z_NEAR, Z_FAR, np.ones((h // 2, w // 2)), rec, hdr)
    np.testing.assert_allclose(out[..., :3], np.broadcast_to([0.3, 0.2, 0.1], out[..., :3].shape), rtol=1e-12)


def test_oracle_reconstruct_without_history_takes_the_raymarch():
    atmo, cp = W.earth_like_atmosphere(), W.frame_cloud_parameters()
    m = _abi.CloudMaterial()
    _abi.call("skyr_cloud_material_default", _abi.SKYR_MATERIAL_MINIMAL, C.byref(m))
    v = W.frame_view(W.frame_camera(), 45.0, width=64, height=40)
    rng = np.random.default_rng(2)
    render = rng.uniform(0, 3, (10, 16, 4))
    render[..., 3] = rng.uniform(0, 1, (10, 16))
    index = np.zeros((10, 16, 2))
    index[..., 1] = _ld(1.0)
    f = CL.temporal_frame(atmo, v, None, None, Z_NEAR, Z_FAR, 0)
    out = orc.reconstruct(atmo, cp, m, {}, v, f, np.ones((20, 32)), index, render, np.full((10, 16), 5.0), None)
    want = np.repeat(np.repeat(render, 2, axis=0), 2, axis=1)
    np.testing.assert_allclose(out, want, rtol=1e-12)
