"""GPU parity and behaviour of the multiple-scattering surrogate
(include/skyr_surrogate.h) and the path tracer's point / pixel-list sources.

* lattice: node features and sun optical depth against FP64 grid lookups
  (oracle_grid_sigma): features within one BF16 rounding, optical depth 1e-4;
* records: trilinear interpolation of the lattice, within one BF16 rounding;
* point sources: per point and channel z = (mean_gpu - mean_oracle) /
  sqrt(2 var / N) with the RNG-matched FP64 oracle, |z| <= 4.5, mean z^2 <= 2;
* pixel list: the same paths as the region source (same seeds);
* render: the FP64 restatement of the raymarch over the GPU-built lattice and
  the committed network (BF16 rounding points mirrored): mean relative error
  of the luminance <= 1e-3, transmittance 1e-5;
* accuracy: on the 512x640x352 evaluation cloud at 128^2 the network image is
  within 2 % relative L1 of a 32768-spp path-traced reference while single
  scattering alone is >= 80 % off (what the trained network gains).
"""
import ctypes as C
import math

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from skyrendering_gb300 import _abi, mlp
from skyrendering_gb300 import surrogate as S
from skyrendering_gb300 import surrogate_train as T
from skyrendering_gb300 import workloads as W
from skyrendering_gb300.atmosphere import _ptr
from skyrendering_gb300.pathtrace import PathTracer

pytestmark = pytest.mark.gpu
SMALL = (64, 80, 44)


@pytest.fixture()
def small(ctx):
    sc = T.Scene(ctx, size=24, dims=SMALL)
    grid = sc.grid(0x5EED)
    fv = sc.lattice(grid)
    ctx.synchronize()
    return sc, grid, fv


def _luts_host(sc):
    L = sc.luts
    return {k: getattr(L, k).double().cpu().numpy() for k in
            ("transmittance", "sky_view_luminance", "sky_view_transmittance", "aerial_perspective_luminance",
             "aerial_perspective_transmittance")}


def _bf16(x):
    return torch.from_numpy(np.asarray(x, dtype=np.float32)).to(torch.bfloat16).float().numpy()


def _box_exit(lo, hi, x, d):
    with np.errstate(divide="ignore", invalid="ignore"):
        a, b = (lo - x) / d, (hi - x) / d
    t1 = np.min(np.maximum(a, b), axis=-1)
    return t1


def _view_neighbours(grid, x, v, sun, sigma_ref):
    """Features 33..40 (skyr_surrogate.h): extinction at the view-oriented cube corners."""
    g = grid.struct
    span = g.voxel_size * max(g.nx, g.ny, g.nz)
    r = 0.1 * span / math.sqrt(3.0)
    u = sun[None, :] - v * (v @ sun)[:, None]
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    w = np.cross(v, u)
    pts = [x + v * (r if j & 1 else -r) + u * (r if j & 2 else -r) + w * (r if j & 4 else -r) for j in range(8)]
    sig = orc.grid_sigma(g, grid.data.cpu().numpy(), np.concatenate(pts)).reshape(8, -1).T
    return sig / sigma_ref


REC = mlp.RECORD  # 112 bf16: features 0..102 (skyr_surrogate.h), then zeros
LAT = 80  # bf16 per lattice node: features 0..79 of the record, the per-sample slots zero


def _mips(data, levels=6):
    """The grid's mip chain in FP64: each texel the mean of the existing texels
    of the 2 x 2 x 2 block below it (ceil sizes), level 0 the grid."""
    out = [np.asarray(data, dtype=np.float64)]
    for _ in range(levels):
        a = out[-1]
        nz, ny, nx = a.shape
        p = np.full(((nz + 1) // 2 * 2, (ny + 1) // 2 * 2, (nx + 1) // 2 * 2), np.nan)
        p[:nz, :ny, :nx] = a
        b = p.reshape(p.shape[0] // 2, 2, p.shape[1] // 2, 2, p.shape[2] // 2, 2)
        out.append(np.nanmean(b, axis=(1, 3, 5)))
    return out


def _trilinear_zero(vol, origin, voxel, pts):
    """Trilinear between texel centres with a zero border (the grid lookups' convention)."""
    g = (pts - origin) / voxel - 0.5
    f0 = np.floor(g).astype(int)
    fr = g - f0
    nz, ny, nx = vol.shape
    out = np.zeros(len(pts))
    for c in range(8):
        d = np.array([c & 1, (c >> 1) & 1, c >> 2])
        i = f0 + d
        w = np.prod(np.where(d, fr, 1 - fr), 1)
        ok = (i[:, 0] >= 0) & (i[:, 0] < nx) & (i[:, 1] >= 0) & (i[:, 1] < ny) & (i[:, 2] >= 0) & (i[:, 2] < nz)
        v = np.zeros(len(pts))
        v[ok] = vol[i[ok, 2], i[ok, 1], i[ok, 0]]
        out += w * v
    return out


def _stencil(grid, x, sun, sigma_ref):
    """Features 44..78: the density stencil at mip levels 2..6, centre and +-2 texels
    of the level along the sun, its horizontal perpendicular (sun x z) and their cross."""
    g = grid.struct
    e1 = sun / np.linalg.norm(sun)
    e2 = np.array([e1[1], -e1[0], 0.0])
    if np.linalg.norm(e2) < 1e-3:
        e2 = np.array([0.0, e1[2], -e1[1]])
    e2 /= np.linalg.norm(e2)
    e3 = np.cross(e1, e2)
    axes = [e1, e2, e3]
    mips = _mips(grid.data.float().cpu().numpy())
    org = np.array(g.origin[:], dtype=np.float64)
    cols = []
    for lv in range(2, 7):
        h = g.voxel_size * 2 ** (lv + 1)
        for j in range(7):
            p = x if j == 0 else x + axes[(j - 1) >> 1] * (h if j & 1 else -h)
            cols.append(_trilinear_zero(mips[lv], org, g.voxel_size * 2 ** lv, p) * g.density / sigma_ref)
    return np.stack(cols, 1)


def test_lattice_matches_oracle(small):
    sc, grid, fv = small
    g = grid.struct
    raw = fv.buf.cpu().numpy()
    st = fv.struct
    nodes = st.nx * st.ny * st.nz
    rec = raw[: nodes * LAT * 2].view(np.uint16).reshape(nodes, LAT)
    tau = raw[nodes * LAT * 2: nodes * (LAT * 2 + 4)].view(np.float32)
    data = grid.data.cpu().numpy()
    rng = np.random.default_rng(1)
    idx = rng.choice(nodes, 48, replace=False)
    ix, iy, iz = idx % st.nx, (idx // st.nx) % st.ny, idx // (st.nx * st.ny)
    cell = g.voxel_size * st.stride
    org = np.array(g.origin[:], dtype=np.float64)
    x = org + np.stack([ix, iy, iz], 1) * cell
    sun = np.array(st.sun[:], dtype=np.float64)
    span = g.voxel_size * max(SMALL)
    pts = [x]
    for k in range(32):
        pts.append(x + sun * (span * 0.01 * 1000.0 ** (k / 31.0)))
    sig = orc.grid_sigma(g, data, np.concatenate(pts)).reshape(33, -1).T / st.sigma_ref
    hi = org + np.array(SMALL) * g.voxel_size
    alt = np.clip((x[:, 2] - org[2]) / (hi[2] - org[2]), 0, 1)
    # 33..40 depend on the view direction: zero in the lattice
    feat = np.concatenate([sig, np.zeros((len(x), 8)), alt[:, None]], 1)
    got = rec[idx, :42].astype(np.uint32) << 16
    got = got.view(np.float32)
    np.testing.assert_allclose(got, _bf16(feat), rtol=1e-2, atol=1e-3)
    # the per-sample slots (cos, far side) and the pad stay zero
    assert np.all(rec[idx, 42:44] == 0) and np.all(rec[idx, LAT - 1] == 0)
    # the stencil over the mip chain (the GPU's levels are FP16)
    got_s = (rec[idx, 44:79].astype(np.uint32) << 16).view(np.float32)
    np.testing.assert_allclose(got_s, _bf16(_stencil(grid, x, sun, st.sigma_ref)), rtol=1e-2, atol=2e-3)
    # optical depth to the sun: midpoint rule at half a voxel to the box exit
    t1 = _box_exit(org, hi, x, sun[None, :])
    for n, node in enumerate(idx):
        steps = max(int(math.ceil(t1[n] / (0.5 * g.voxel_size))), 1)
        h = t1[n] / steps
        s = orc.grid_sigma(g, data, x[n] + np.outer((np.arange(steps) + 0.5) * h, sun)).sum() * h
        assert tau[node] == pytest.approx(s, rel=1e-4, abs=1e-5)


def test_records_interpolate_lattice(ctx, small):
    sc, grid, fv = small
    pts = S.sample_points(ctx, grid, 256, 77, W.PT_SIGMA_MAX)
    rec = S.records(ctx, fv, pts)
    st = fv.struct
    nodes = st.nx * st.ny * st.nz
    raw = fv.buf.cpu().numpy()
    lat = (raw[: nodes * LAT * 2].view(np.uint16).reshape(nodes, LAT).astype(np.uint32) << 16).view(np.float32)
    p = pts.cpu().numpy().astype(np.float64)
    g = grid.struct
    q = (p[:, :3] - np.array(g.origin[:])) / (g.voxel_size * st.stride)
    n3 = np.array([st.nx, st.ny, st.nz])
    i0 = np.clip(np.floor(q).astype(int), 0, n3 - 2)
    fr = np.clip(q - i0, 0, 1)
    f = np.zeros((len(p), REC))
    fl = f[:, :LAT]
    for c in range(8):
        d = np.array([c & 1, (c >> 1) & 1, c >> 2])
        w = np.prod(np.where(d, fr, 1 - fr), 1)
        node = ((i0[:, 2] + d[2]) * st.ny + (i0[:, 1] + d[1])) * st.nx + (i0[:, 0] + d[0])
        fl += w[:, None] * lat[node]
    sun = np.array(st.sun[:], dtype=np.float64)
    f[:, 42] = p[:, 3:] @ sun
    f[:, 33:41] = _view_neighbours(grid, p[:, :3], p[:, 3:], sun, st.sigma_ref)
    # far side: transmittance along the view direction to the box's exit (midpoint, half-voxel steps)
    org = np.array(g.origin[:], dtype=np.float64)
    hi = org + np.array(SMALL) * g.voxel_size
    t1 = _box_exit(org, hi, p[:, :3], p[:, 3:])
    data = grid.data.cpu().numpy()
    for n in range(len(p)):
        steps = max(int(math.ceil(t1[n] / (0.5 * g.voxel_size))), 1)
        h = t1[n] / steps
        od = orc.grid_sigma(g, data, p[n, :3] + np.outer((np.arange(steps) + 0.5) * h, p[n, 3:])).sum() * h
        f[n, 43] = math.exp(-od)
    # 79..102: the view-oriented stencil, +-2^(l+1) voxels along v, u, w at mip levels 3..6
    v = p[:, 3:]
    u = sun[None, :] - v * (v @ sun)[:, None]
    u /= np.linalg.norm(u, axis=1, keepdims=True)
    w = np.cross(v, u)
    mips = _mips(grid.data.float().cpu().numpy())
    for s_ in range(24):
        lv, j = 3 + s_ // 6, s_ % 6
        ax = (v, u, w)[j >> 1]
        h = g.voxel_size * 2 ** (lv + 1) * (-1.0 if j & 1 else 1.0)
        f[:, 79 + s_] = _trilinear_zero(mips[lv], org, g.voxel_size * 2 ** lv, p[:, :3] + ax * h) * g.density / st.sigma_ref
    got = rec.float().cpu().numpy()
    np.testing.assert_allclose(got, _bf16(f), rtol=1e-2, atol=2e-3)


def test_point_radiance_matches_oracle(ctx, small):
    sc, grid, fv = small
    pts = S.sample_points(ctx, grid, 24, 5, W.PT_SIGMA_MAX)
    N = 2048
    m_gpu = S.point_radiance(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.env, sc.sizes, sc.luts, pts, N,
                             frame_begin=11).cpu().numpy()
    ctx.check_status()
    s, sq = orc.point_radiance(sc.atmo, sc.cloud, grid.struct, grid.data.cpu().numpy(), sc.pt, sc.view, sc.env,
                               sc.sizes, _luts_host(sc), 11, N, pts.cpu().numpy())
    m_o = s / N
    var = np.maximum(sq / N - m_o ** 2, 1e-30)
    z = (m_gpu - m_o) / np.sqrt(2 * var / N)
    print(f"point radiance: max|z|={np.max(np.abs(z)):.2f} mean z^2={np.mean(z ** 2):.2f} "
          f"mean gpu={m_gpu.mean():.4e} oracle={m_o.mean():.4e}")
    assert np.max(np.abs(z)) <= 4.5
    assert np.mean(z ** 2) <= 2.0


def test_pixel_list_matches_region(ctx, small):
    sc, grid, fv = small
    w, h = sc.view.width, sc.view.height
    tr = PathTracer(ctx, sc.pt, sc.cloud, sc.view, sc.env, sc.sizes, grid=grid)
    tr.frames = 41
    tr.render(sc.atmo, sc.luts, 4, region=(4, 6, 12, 14))
    pix = [y * w + x for y in range(6, 14) for x in range(4, 12)]
    lst = torch.tensor(pix + [-1, w * h, w * h + 5], dtype=torch.int32, device="cuda")  # last three are skipped
    acc = torch.zeros((h, w, 4), device="cuda")
    S.pathtrace_pixels(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.env, sc.sizes, sc.luts, lst, 4, acc,
                       frame_begin=42)
    ctx.check_status()
    torch.testing.assert_close(acc, tr.acc, rtol=1e-5, atol=1e-7)


@pytest.mark.parametrize("use_network,froxel", [(0, False), (1, False), (1, True)])
def test_render_matches_oracle(ctx, small, use_network, froxel):
    sc, grid, fv = small
    model = S.load_model(S.MODEL_PATH)
    net = model.packed(ctx)
    sp = S.parameters(use_network=use_network, network_error=0.1)
    view, syn = sc.view, None
    if froxel:  # a shadow froxel scaling the aerial-perspective luminance
        from .test_cloud_shadow_gpu import attach, device_froxel, synthetic_froxel

        syn = synthetic_froxel(seed=13)
        dev = device_froxel(syn)
        view = attach(_abi.CloudView.from_buffer_copy(sc.view), dev)
    img, err = S.render(ctx, sc.atmo, sc.cloud, grid, sc.pt, view, sc.sizes, sc.luts, fv, net, sp)
    ctx.synchronize()
    w, h = sc.view.width, sc.view.height
    pix = np.arange(w * h, dtype=np.int32)
    out, oerr = orc.surrogate_render(sc.atmo, sc.cloud, grid.struct, grid.data.cpu().numpy(), sc.pt, view,
                                     sc.sizes, _luts_host(sc), fv.buf.cpu().numpy(), fv.struct, model.params,
                                     model.label_scale, sp.steps, bool(use_network), sp.min_transmittance, 0.1, pix,
                                     froxel=syn)
    g = img.reshape(-1, 4).double().cpu().numpy()
    lum_g = g[:, :3] @ [0.2126, 0.7152, 0.0722]
    lum_o = out[:, :3] @ [0.2126, 0.7152, 0.0722]
    m = lum_o > 1e-4 * lum_o.max()
    assert m.sum() > 50
    rel = np.abs(lum_g[m] - lum_o[m]) / lum_o[m]
    print(f"render use_network={use_network}: mean rel {rel.mean():.2e} max rel {rel.max():.2e}")
    assert rel.mean() <= 1e-3
    assert rel.max() <= 2e-2
    np.testing.assert_allclose(g[:, 3], out[:, 3], atol=1e-5)
    e = err.reshape(-1).double().cpu().numpy()
    if use_network:
        np.testing.assert_allclose(e[m], oerr[m], rtol=2e-2, atol=1e-9)
    else:
        assert np.all(e == 0)


def test_surrogate_accuracy_and_network_gain(ctx):
    sc = T.Scene(ctx, size=128)
    grid = sc.grid(0x5EED)
    fv = sc.lattice(grid)
    model = S.load_model(S.MODEL_PATH)
    net = model.packed(ctx)
    with_net, _ = S.render(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.sizes, sc.luts, fv, net,
                           S.parameters(use_network=1))
    ss_only, _ = S.render(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.sizes, sc.luts, fv, None,
                          S.parameters(use_network=0))
    tr = PathTracer(ctx, sc.pt, sc.cloud, sc.view, sc.env, sc.sizes, grid=grid)
    for _ in range(8):
        tr.render(sc.atmo, sc.luts, 4096)
    ref = tr.acc / tr.frames
    ctx.check_status()
    e_net, e_ss = S.relative_l1(with_net, ref), S.relative_l1(ss_only, ref)
    print(f"relative L1 vs 32768 spp: network {e_net:.4f}, single scattering only {e_ss:.4f}")
    # the target: within 2% (measured 0.0179); the 32768-spp reference's own
    # noise (about 1.2% relative L1) is part of it
    assert e_net <= 0.02
    assert e_ss >= 0.8
    assert e_ss >= 15 * e_net
    # the view transmittance is the same with or without the network and matches the path tracer's alpha
    torch.testing.assert_close(with_net[..., 3], ss_only[..., 3])
    assert float((with_net[..., 3] - ref[..., 3]).abs().mean()) < 2e-3


def test_training_pipeline_reduces_error(ctx):
    sc = T.Scene(ctx, size=16, dims=SMALL)
    rec, lab = T.dataset(sc, range(1000, 1004), 4096, 16)
    vrec, vlab = T.dataset(sc, range(900, 901), 2048, 128)
    untrained = mlp.PackedMLP.from_params(ctx, mlp.init_params(7), float(lab.mean()))
    e0 = T.validation_error(untrained, vrec, vlab)
    params, scale, curve = T.train(ctx, rec, lab, vrec, vlab, epochs=24, batch=4096, log=lambda *a: None)
    e1 = T.validation_error(mlp.PackedMLP.from_params(ctx, params, scale), vrec, vlab)
    print(f"validation relative L1: untrained {e0:.3f} -> trained {e1:.3f}")
    assert e1 < 0.65 * e0  # measured 0.58 with the 103-input network


def test_fallback_replaces_flagged_pixels(ctx, small):
    sc, grid, fv = small
    model = S.load_model(S.MODEL_PATH)
    net = model.packed(ctx)
    table = torch.from_numpy(model.error_table).cuda()
    sp = S.parameters(error_table=table)
    base, err = S.render(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.sizes, sc.luts, fv, net, sp)
    none = S.render_with_fallback(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.env, sc.sizes, sc.luts, fv, net,
                                  sp, threshold=1e9, fallback_frames=16)
    assert none.flagged == 0
    torch.testing.assert_close(none.image, base)
    res = S.render_with_fallback(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.env, sc.sizes, sc.luts, fv, net,
                                 sp, threshold=0.0, fallback_frames=16)
    lum = S.luminance(base[..., :3])
    flagged = (err / lum.clamp_min(1e-3)) > 0.0
    assert res.flagged == int(flagged.sum())
    assert res.flagged > 0
    keep = ~flagged
    torch.testing.assert_close(res.image[keep], base[keep])


def test_copy_wait_bound_reports_timeout(ctx, small):
    """With a copy-wait bound of 0 every block of the surrogate raymarch gives
    up on the bulk copy of the network at once: it waits for the copy in
    flight (bounded), leaves without writing a pixel, and the call is reported
    as SKYR_ETIMEOUT; the default bound renders normally afterwards."""
    sc, grid, fv = small
    net = S.load_model(S.MODEL_PATH).packed(ctx)
    sp = S.parameters(use_network=1)
    default = ctx.limits
    tight = _abi.DeviceLimits.from_buffer_copy(default)
    tight.copy_wait_cycles = 0
    out = torch.full((sc.view.height, sc.view.width, 4), float("nan"), device="cuda")
    ctx.limits = tight
    S.render(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.sizes, sc.luts, fv, net, sp, out=out)
    with pytest.raises(_abi.SkyrError) as exc:
        ctx.check_status()
    assert exc.value.status == _abi.SKYR_ETIMEOUT
    assert bool(torch.isnan(out).all())
    ctx.limits = default
    S.render(ctx, sc.atmo, sc.cloud, grid, sc.pt, sc.view, sc.sizes, sc.luts, fv, net, sp, out=out)
    ctx.check_status()
    assert bool(torch.isfinite(out).all())


def test_invalid_arguments(ctx, small):
    sc, grid, fv = small
    lib = _abi.lib()
    sp = S.parameters(use_network=1)
    out = torch.empty((sc.view.height, sc.view.width, 4), device="cuda")
    L = sc.luts
    args = lambda fvs, pk, spp: (ctx.handle, C.byref(sc.atmo), C.byref(sc.cloud), C.byref(grid.struct),
                                 C.byref(sc.pt), C.byref(sc.view), C.byref(sc.sizes), _ptr(L.transmittance),
                                 _ptr(L.aerial_perspective_luminance), _ptr(L.aerial_perspective_transmittance),
                                 C.byref(fvs), pk, C.byref(spp), _ptr(out), None)
    assert lib.skyr_surrogate_render(*args(fv.struct, None, sp)) == _abi.SKYR_EINVAL  # network but none given
    bad = S.parameters(use_network=0, steps=0)
    assert lib.skyr_surrogate_render(*args(fv.struct, None, bad)) == _abi.SKYR_EINVAL
    other = _abi.FeatureVolume()
    C.memmove(C.byref(other), C.byref(fv.struct), C.sizeof(other))
    other.nx += 1  # a lattice of another grid
    assert lib.skyr_surrogate_render(*args(other, None, S.parameters(use_network=0))) == _abi.SKYR_EINVAL
    assert lib.skyr_surrogate_sample_points(ctx.handle, C.byref(grid.struct), C.c_float(float("nan")),
                                            C.c_float(0.0), C.c_uint64(1), 4, _ptr(out)) == _abi.SKYR_EINVAL
