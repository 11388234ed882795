"""GPU parity of the full-screen atmosphere composite (include/skyr_composite.h)
against the FP64 oracle on the same LUTs, depth, noise, stars and froxel.

* the reference default (per-pixel raymarch, 40 dithered samples) over a
  480 x 270 viewport with the Earth's surface, a near occluder with an object
  luminance, the star map and a shadow froxel: mean relative error of the
  luminance <= 1e-3 (RGBA16F output);
* the same with the sky-view and aerial-perspective LUTs switched on;
* a camera in space (200 km): the raymarch starts at the atmosphere's top;
* the sun disc in view: its pixels within 1e-3;
* 1920 x 1080 default frame without objects, on sampled pixels;
* graph replay bit-identical; bad arguments refused.
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import batch as B
from skyrendering_gb300 import workloads as W
from skyrendering_gb300.atmosphere import Context, composite, composite_parameters, update_lut_set
from skyrendering_gb300.cloud import blue_noise_tile

pytestmark = pytest.mark.gpu


def mean_rel(got, want):
    return float(np.abs(got - want).sum() / max(np.abs(want).sum(), 1e-300))


class Scene:
    def __init__(self, ctx, cam, w, h, zenith=45.0, azimuth=60.0, depth=True, stars=True, froxel=True, fmt=0):
        self.p = W.earth_like_atmosphere()
        self.s = W.plain_lut_sizes(fmt)
        self.r = W.render_parameters(cam, zenith, azimuth)
        self.luts = update_lut_set(ctx, self.p, self.r, self.s)
        self.w, self.h = w, h
        self.bn = blue_noise_tile().cuda()
        rng = np.random.default_rng(21)
        self.depth_np = W.ground_depth(cam, w, h, self.p.bottom_radius) if depth else None
        self.obj_np = rng.uniform(0.0, 2.0, (h * w, 4)).astype(np.float32) if depth else None
        self.stars_np = W.star_map() if stars else None
        if froxel:
            fx = 0.3 + 0.7 * rng.uniform(0.0, 1.0, (16, 9, 20))
            self.froxel_np = np.round(fx * 65535).astype(np.uint16)
        else:
            self.froxel_np = None
        dev = lambda a: None if a is None else torch.from_numpy(a).cuda()
        self.depth, self.obj, self.stars = dev(self.depth_np), dev(self.obj_np), dev(self.stars_np)
        self.froxel = None if self.froxel_np is None else dev(self.froxel_np.view(np.int16))
        ctx.synchronize()

    def render(self, ctx, cp, out=None):
        o = composite(ctx, self.p, self.r, cp, self.s, self.luts, self.w, self.h, blue_noise=self.bn,
                      depth=self.depth, object_luminance=self.obj, star_map=self.stars, shadow_froxel=self.froxel,
                      shadow_froxel_max_distance=20.0, out=out)
        ctx.synchronize()
        return o

    def oracle(self, cp, pixels=None):
        L = self.luts
        luts = {k: getattr(L, k)[0].float().cpu().double().numpy() for k in
                ("transmittance", "multiscattering", "sky_view_luminance", "sky_view_transmittance",
                 "aerial_perspective_luminance", "aerial_perspective_transmittance")}
        return orc.atmosphere_composite(self.p, self.r, cp, self.s, luts, self.w, self.h,
                                        blue_noise=self.bn.cpu().numpy(), depth=self.depth_np,
                                        object_luminance=self.obj_np, star_map=self.stars_np, froxel=self.froxel_np,
                                        froxel_max_distance=20.0, pixels=pixels)


def _compare(sc, got, cp, pixels=None):
    want = sc.oracle(cp, pixels)
    g = got.float().cpu().numpy().reshape(-1, 4).astype(np.float64)
    if pixels is not None:
        g = g[pixels]
    assert np.all(g[:, 3] == 1.0)
    return mean_rel(g[:, :3], want[:, :3]), want


@pytest.mark.parametrize("luts,fmt", [(False, 0), (True, 0), (True, 1)])
def test_composite_matches_oracle(ctx, luts, fmt):
    cam = W.frame_camera()
    sc = Scene(ctx, cam, 480, 270, fmt=fmt)
    cp = composite_parameters(use_sky_view_lut=int(luts), use_aerial_perspective_lut=int(luts))
    got = sc.render(ctx, cp)
    err, want = _compare(sc, got, cp)
    obj = (sc.depth_np.reshape(-1) < 1).mean()
    print(f"luts={luts} fmt={fmt}: mean rel {err:.2e}; object pixels {obj:.2f}")
    assert obj > 0.2 and err <= 1e-3


def test_space_camera_and_sun_disc(ctx):
    # 200 km up, looking down at the limb
    cam = W.Camera(position=(0.0, 200.0, 0.0), yaw=90.0, pitch=-20.0, width=320, height=180)
    sc = Scene(ctx, cam, 320, 180, depth=False, froxel=False)
    cp = composite_parameters()
    err, _ = _compare(sc, sc.render(ctx, cp), cp)
    print(f"space camera: mean rel {err:.2e}")
    assert err <= 1e-3
    # the sun in the middle of a narrow view
    zen, az = 60.0, 30.0
    cam = W.Camera(position=(0.0, 1.0, 0.0), yaw=az, pitch=90.0 - zen, fovy=2.0, width=64, height=64)
    sc = Scene(ctx, cam, 64, 64, zenith=zen, azimuth=az, depth=False, froxel=False)
    got = sc.render(ctx, cp)
    err, want = _compare(sc, got, cp)
    sun = want[:, 0] > 100 * np.median(want[:, 0])
    print(f"sun disc: mean rel {err:.2e}; disc pixels {sun.sum()}")
    assert sun.sum() > 20 and err <= 1e-3


def test_1080p_default_frame(ctx):
    sc = Scene(ctx, W.frame_camera(), 1920, 1080, depth=False)
    cp = composite_parameters()
    got = sc.render(ctx, cp)
    px = np.sort(np.random.default_rng(5).choice(1920 * 1080, 40000, replace=False)).astype(np.int32)
    err, _ = _compare(sc, got, cp, px)
    print(f"1080p: mean rel {err:.2e}")
    assert err <= 1e-3


@pytest.fixture()
def sctx(cuda):
    s = torch.cuda.Stream()
    with torch.cuda.stream(s):
        c = Context(s)
        yield c
        c.close()


def test_graph_and_invalid_arguments(sctx):
    sc = Scene(sctx, W.frame_camera(), 320, 180)
    cp = composite_parameters()
    ref = sc.render(sctx, cp).clone()
    out = torch.zeros_like(ref)
    with B.capture(sctx) as cap:
        composite(sctx, sc.p, sc.r, cp, sc.s, sc.luts, sc.w, sc.h, blue_noise=sc.bn, depth=sc.depth,
                  object_luminance=sc.obj, star_map=sc.stars, shadow_froxel=sc.froxel, out=out)
    cap.graph.launch()
    sctx.synchronize()
    assert torch.equal(out, ref)
    cap.graph.close()
    for bad in (dict(raymarching_steps=0.0), dict(use_sky_view_lut=1)):
        bcp = composite_parameters(**bad)
        with pytest.raises(_abi.SkyrError):
            if "use_sky_view_lut" in bad:  # the switch without the LUTs
                inp = _abi.CompositeInputs()
                inp.width, inp.height, inp.blue_noise = 8, 8, sc.bn.data_ptr()
                _abi.call("skyr_atmosphere_composite", sctx.handle, C.byref(sc.p), C.byref(sc.r), C.byref(bcp),
                          C.byref(sc.s), C.c_void_p(sc.luts.transmittance.data_ptr()),
                          C.c_void_p(sc.luts.multiscattering.data_ptr()), None, None, None, None, C.byref(inp),
                          C.c_void_p(out.data_ptr()))
            else:
                composite(sctx, sc.p, sc.r, bcp, sc.s, sc.luts, sc.w, sc.h, blue_noise=sc.bn, out=out)
    with pytest.raises(_abi.SkyrError):  # dithering without blue noise
        composite(sctx, sc.p, sc.r, cp, sc.s, sc.luts, sc.w, sc.h, out=out)
