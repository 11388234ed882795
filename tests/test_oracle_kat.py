"""Known-answer tests that pin the CPU oracle (the reference ships no golden
vectors).  CPU only."""
import ctypes as C
import math
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle as orc
from skyrendering_gb300 import workloads as W

GOLDEN = Path(__file__).with_name("golden") / "atmosphere_small.npz"


def exp_only(p, which):
    """Atmosphere with a single exponential (Rayleigh or Mie) constituent."""
    q = W.earth_like_atmosphere()
    C.memmove(C.byref(q), C.byref(p), C.sizeof(q))
    if which != "rayleigh":
        q.rayleigh_scattering_scale = 0.0
    if which != "mie":
        q.mie_scattering_scale = 0.0
        q.mie_absorption_scale = 0.0
    q.ozone_absorption_scale = 0.0
    return q


def test_vertical_transmittance_closed_form():
    # r = R, mu = 1: tau = sR HR (1 - e^{-L/HR}) + sM HM (1 - e^{-L/HM}) + sO * 15 (tent area)
    p = W.earth_like_atmosphere()
    p.transmittance_steps = 4000.0
    L = p.thickness
    sR = np.array(p.rayleigh_scattering, dtype=np.float64) * p.rayleigh_scattering_scale
    sM = (np.array(p.mie_scattering, dtype=np.float64) * p.mie_scattering_scale
          + np.array(p.mie_absorption, dtype=np.float64) * p.mie_absorption_scale)
    sO = np.array(p.ozone_absorption, dtype=np.float64) * p.ozone_absorption_scale
    HR, HM = p.rayleigh_exponential_distribution, p.mie_exponential_distribution
    tau = sR * HR * (1 - math.exp(-L / HR)) + sM * HM * (1 - math.exp(-L / HM)) + sO * p.ozone_width
    got = orc.transmittance_at(p, p.bottom_radius, 1.0)
    np.testing.assert_allclose(-np.log(got), tau, rtol=2e-6)


@pytest.mark.parametrize("which", ["rayleigh", "mie"])
def test_midpoint_sum_exact_geometric_series(which):
    # For one exponential constituent on the vertical ray the reference's
    # midpoint loop is a geometric series: sum_i s e^{-(i+1/2)dx/H} dx.
    p = exp_only(W.earth_like_atmosphere(), which)
    n = 40
    p.transmittance_steps = float(n)
    H = p.rayleigh_exponential_distribution if which == "rayleigh" else p.mie_exponential_distribution
    if which == "rayleigh":
        s = np.array(p.rayleigh_scattering, dtype=np.float64) * p.rayleigh_scattering_scale
    else:
        s = (np.array(p.mie_scattering, dtype=np.float64) * p.mie_scattering_scale
             + np.array(p.mie_absorption, dtype=np.float64) * p.mie_absorption_scale)
    dx = p.thickness / n
    q = math.exp(-dx / H)
    tau = s * dx * math.exp(-dx / (2 * H)) * (1 - q ** n) / (1 - q)
    got = orc.transmittance_at(p, p.bottom_radius, 1.0)
    np.testing.assert_allclose(-np.log(got), tau, rtol=1e-11)


def test_top_boundary_is_transparent():
    p = W.earth_like_atmosphere()
    top = p.bottom_radius + p.thickness
    for mu in (1.0, 0.5, 0.01):
        np.testing.assert_allclose(orc.transmittance_at(p, top, mu), 1.0, rtol=0, atol=1e-15)


def test_transmittance_lut_first_texel_is_vertical_ray():
    # texel (0, 0): x_mu = 0, x_r = 0 -> r = R, d = d_min -> mu = 1
    p = W.earth_like_atmosphere()
    s = W.plain_lut_sizes()
    o = orc.lut_set(p, None, s, 64, views=False)
    np.testing.assert_allclose(o["transmittance"][0, 0, :3], orc.transmittance_at(p, p.bottom_radius, 1.0),
                               rtol=1e-12)
    assert np.all(o["transmittance"][..., 3] == 1.0)
    # transmittance falls as the ray leans toward the horizon (x_mu grows)
    t = o["transmittance"][..., 2]
    assert np.all(np.diff(t, axis=1) <= 1e-15)


def test_multiscattering_mask_zero_removes_ms_term():
    from tests.golden.make_atmosphere_golden import small_sizes

    p = W.earth_like_atmosphere()
    p.multiscattering_mask = 0.0
    s = small_sizes()
    r = W.render_parameters(W.frame_camera(), 45.0)
    base = orc.lut_set(p, r, s, 64)
    zero_ms = orc.view_luts_from(p, r, s, base["transmittance"], np.zeros_like(base["multiscattering"]))
    np.testing.assert_array_equal(base["sky_view_luminance"], zero_ms["sky_view_luminance"])
    np.testing.assert_array_equal(base["aerial_perspective_luminance"], zero_ms["aerial_perspective_luminance"])


def test_fp32_mirror_tracks_fp64():
    # the like-for-like FP32 baseline is the same code; it must stay close
    from tests.golden.make_atmosphere_golden import small_sizes

    p = W.earth_like_atmosphere()
    s = small_sizes()
    r = W.render_parameters(W.frame_camera(), 45.0)
    a, b = orc.lut_set(p, r, s, 64), orc.lut_set(p, r, s, 32)
    for k in ("transmittance", "sky_view_luminance", "aerial_perspective_transmittance"):
        rel = np.abs(a[k] - b[k]) / np.maximum(np.abs(a[k]), 1e-6 * np.abs(a[k]).max())
        assert rel.max() < 5e-2, k


def test_oracle_matches_committed_golden():
    from tests.golden.make_atmosphere_golden import cases, small_sizes

    g = np.load(GOLDEN)
    s = small_sizes()
    for tag, p, r in cases():
        o = orc.lut_set(p, r, s, 64)
        for k, v in o.items():
            np.testing.assert_allclose(v, g[f"{tag}/{k}"], rtol=1e-10, atol=1e-300, err_msg=f"{tag}/{k}")
