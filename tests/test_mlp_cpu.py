"""CPU checks of the surrogate network's oracle (FP64) and host helpers.

The oracle's analytic gradient is pinned against central finite differences of
its own loss; the loss weights 1 / (y_sg^2 + eps) are frozen by the
stop-gradient, so the check uses a large eps, where they are constant to
O(y^2 / eps).
"""
import numpy as np
import pytest

from oracle import oracle as orc

IN = 103  # the network's inputs (include/skyr_mlp.h)
P = 19331


def _layer_slices():
    fan = [(IN, 64), (64, 64), (64, 64), (64, 64), (64, 3)]
    out, o = [], 0
    for fi, fo in fan:
        out.append(("W", o, o + fi * fo))
        o += fi * fo
        out.append(("b", o, o + fo))
        o += fo
    assert o == P
    return out


def _params(seed, scale=0.25):
    rng = np.random.default_rng(seed)
    return (rng.standard_normal(P) * scale).astype(np.float32)


def test_oracle_gradient_matches_finite_differences():
    """Directional central differences, one random direction inside each weight /
    bias block.  The network is piecewise smooth (ReLU); the step (1e-6 along a
    unit direction) is small enough that no pre-activation changes sign."""
    rng = np.random.default_rng(3)
    p = _params(1)
    x = rng.random((16, IN)).astype(np.float32)
    t = rng.random((16, 3)).astype(np.float32)
    eps = 1e8
    _, g = orc.mlp_gradient(p, x, t, loss_eps=eps, mirror=False)
    errs = []
    for kind, a, b in _layer_slices():
        v = np.zeros(P)
        v[a:b] = rng.standard_normal(b - a)
        v /= np.linalg.norm(v)
        h = 1e-6
        pp, pm = (p + h * v).astype(np.float32), (p - h * v).astype(np.float32)
        lp, _ = orc.mlp_gradient(pp, x, t, loss_eps=eps, mirror=False)
        lm, _ = orc.mlp_gradient(pm, x, t, loss_eps=eps, mirror=False)
        dv = pp.astype(np.float64) - pm.astype(np.float64)  # the perturbation actually applied
        an = float(np.dot(g, dv))
        errs.append(abs((lp - lm) - an) / abs(an))
    errs = np.array(errs)
    assert np.all(errs < 1e-4), errs


def test_oracle_loss_definition():
    rng = np.random.default_rng(4)
    p = _params(2)
    x = rng.random((5, IN)).astype(np.float32)
    t = rng.random((5, 3)).astype(np.float32)
    y = orc.mlp_predict(p, x, mirror=False)
    loss, _ = orc.mlp_gradient(p, x, t, label_scale=2.0, loss_eps=0.3, mirror=False)
    tt = t.astype(np.float64) / 2.0
    ref = np.mean((y - tt) ** 2 / (y ** 2 + 0.3))
    assert loss == pytest.approx(ref, rel=1e-12)


def test_oracle_bf16_mirror_is_close_to_fp64():
    rng = np.random.default_rng(5)
    p = _params(3, 0.15)
    x = rng.random((64, IN)).astype(np.float32)
    y64 = orc.mlp_predict(p, x, mirror=False)
    y16 = orc.mlp_predict(p, x, mirror=True)
    rms = np.sqrt(np.mean(y64 ** 2))
    assert np.max(np.abs(y16 - y64)) < 0.05 * rms


def test_oracle_adam_first_step_is_signed_learning_rate():
    g = np.array([3.0, -0.5, 1e-3, 0.0])
    p = np.zeros(4)
    m, v = np.zeros(4), np.zeros(4)
    orc.mlp_adam(p, m, v, g.copy(), lr=1e-3, step=1)
    expect = -1e-3 * g / (np.abs(g) + 1e-8)
    np.testing.assert_allclose(p, expect, rtol=1e-6, atol=1e-12)


def test_init_params_he_uniform():
    from skyrendering_gb300 import mlp

    p = mlp.init_params(7)
    q = mlp.init_params(7)
    np.testing.assert_array_equal(p, q)
    for kind, a, b in _layer_slices():
        seg = p[a:b]
        if kind == "b":
            assert np.all(seg == 0)
        else:
            fan_in = IN if a == 0 else 64
            bound = np.sqrt(6.0 / fan_in)
            assert np.max(np.abs(seg)) <= bound
            assert np.std(seg) == pytest.approx(bound / np.sqrt(3.0), rel=0.1)
    assert not np.array_equal(p, mlp.init_params(8))
