"""GPU parity of the surrogate network's tensor-core kernels against the FP64
oracle (oracle/oracle_mlp.hpp), through the C ABI.

The oracle mirrors the GPU's BF16 rounding points (weights, hidden activations,
back-propagated dZ); what remains is FP32 accumulation order and the rare
activation whose BF16 rounding flips because of it (one BF16 step, 0.4 %, of
one hidden unit, in a few samples per thousand).  Tolerances:
  * forward:  99 % of |y_gpu - y_oracle| <= 1e-5 x rms(y), all <= 2e-2 x rms(y);
  * gradient: ||g_gpu - g_oracle|| <= 2e-3 x ||g_oracle|| over the whole vector
              and per weight / bias block, loss within 1e-4 relative;
  * Adam:     the update from the GPU's own gradient matches the FP64 Adam step
              to 1e-6 absolute (parameters are O(0.1), steps O(1e-3)).
"""
import ctypes as C

import numpy as np
import pytest
import torch

from oracle import oracle as orc
from skyrendering_gb300 import _abi
from skyrendering_gb300 import mlp
from skyrendering_gb300.atmosphere import _ptr

pytestmark = pytest.mark.gpu
P = mlp.PARAMS
IN = mlp.INPUTS


def _blocks():
    fan = [(IN, 64), (64, 64), (64, 64), (64, 64), (64, 3)]
    out, o = [], 0
    for li, (fi, fo) in enumerate(fan):
        out.append((f"W{li + 1}", o, o + fi * fo))
        o += fi * fo
        out.append((f"b{li + 1}", o, o + fo))
        o += fo
    return out


def _data(n, seed):
    rng = np.random.default_rng(seed)
    x = rng.random((n, IN)).astype(np.float32)
    rec = mlp.to_records(torch.from_numpy(x))
    xb = mlp.records_to_numpy(rec)  # the bf16 values the GPU sees
    t = (0.5 + rng.random((n, 3))).astype(np.float32)
    return rec, xb, t


def _params(seed):
    p = mlp.init_params(seed)
    rng = np.random.default_rng(seed + 100)
    p += (0.01 * rng.standard_normal(P)).astype(np.float32)  # non-zero biases too
    return p


@pytest.mark.parametrize("n", [1, 100, 1000, 4096])
def test_forward_matches_oracle(ctx, n):
    p = _params(11)
    rec, xb, _ = _data(n, 12)
    net = mlp.PackedMLP.from_params(ctx, p, out_scale=1.0)
    y = net.infer(rec).cpu().numpy()
    yo = orc.mlp_predict(p, xb, mirror=True)
    rms = np.sqrt(np.mean(yo ** 2))
    err = np.abs(y - yo)
    assert np.quantile(err, 0.99) <= 1e-5 * rms
    assert np.max(err) <= 2e-2 * rms


def test_forward_output_scale(ctx):
    p = _params(13)
    rec, xb, _ = _data(256, 14)
    y1 = mlp.PackedMLP.from_params(ctx, p, out_scale=1.0).infer(rec)
    y3 = mlp.PackedMLP.from_params(ctx, p, out_scale=3.0).infer(rec)
    torch.testing.assert_close(y3, 3.0 * y1, rtol=1e-6, atol=0)


@pytest.mark.parametrize("n", [128, 1000, 16384])
def test_gradient_matches_oracle(ctx, n):
    p = _params(21)
    rec, xb, t = _data(n, 22)
    h = mlp.hparams(label_scale=1.5, loss_epsilon=1e-2)
    net = mlp.PackedMLP.from_params(ctx, p)
    g, loss = mlp.gradient(ctx, net, h, rec, torch.from_numpy(t).cuda())
    g = g.cpu().numpy().astype(np.float64)
    lo, go = orc.mlp_gradient(p, xb, t, label_scale=1.5, loss_eps=1e-2, mirror=True)
    assert float(loss.item()) == pytest.approx(lo, rel=1e-4)
    assert np.linalg.norm(g - go) <= 2e-3 * np.linalg.norm(go)
    for name, a, b in _blocks():
        ref = np.linalg.norm(go[a:b])
        assert np.linalg.norm(g[a:b] - go[a:b]) <= 2e-3 * ref + 1e-12, name


def test_gradient_is_deterministic(ctx):
    p = _params(31)
    rec, _, t = _data(3000, 32)
    h = mlp.hparams()
    net = mlp.PackedMLP.from_params(ctx, p)
    tt = torch.from_numpy(t).cuda()
    g1, l1 = mlp.gradient(ctx, net, h, rec, tt)
    g2, l2 = mlp.gradient(ctx, net, h, rec, tt)
    assert torch.equal(g1, g2) and torch.equal(l1, l2)


def test_trainer_checkpoint_resumes_bit_for_bit(ctx):
    """Save after k steps, go on for j more; a new trainer loaded from the save
    and stepped j times holds the same parameters, moments and step count, bit
    for bit (training is deterministic)."""
    p = _params(45)
    batches = []
    for i in range(6):
        rec, _, t = _data(4096, 46 + i)
        batches.append((rec, torch.from_numpy(t).cuda()))
    h = mlp.hparams(learning_rate=2e-3)
    a = mlp.Trainer(ctx, p, h)
    for rec, tt in batches[:3]:
        a.step(rec, tt)
    saved = {k: (v.cpu() if torch.is_tensor(v) else v) for k, v in a.state().items()}
    assert saved["steps"] == 3
    for rec, tt in batches[3:]:
        a.step(rec, tt)
    b = mlp.Trainer(ctx, _params(99), h)  # other parameters: all of them come from the checkpoint
    b.load_state(saved)
    assert b.steps == 3
    for rec, tt in batches[3:]:
        b.step(rec, tt)
    sa, sb = a.state(), b.state()
    ctx.synchronize()
    assert sa["steps"] == sb["steps"] == 6
    for k in ("params", "m", "v"):
        assert torch.equal(sa[k], sb[k]), k
    # the packed networks agree too
    na, nb = a.packed(), b.packed()
    ctx.synchronize()
    assert torch.equal(na.buf, nb.buf)
    a.close()
    b.close()


def test_epoch_gathers_batches_in_the_kernel(ctx):
    """skyr_mlp_train_epoch over a permutation equals one skyr_mlp_train_step per
    gathered batch, bit for bit; indices outside the data count as empty samples."""
    p = _params(51)
    rec, _, t = _data(3 * 2048 + 100, 52)
    tt = torch.from_numpy(t).cuda()
    perm = torch.randperm(rec.shape[0], device="cuda", generator=torch.Generator(device="cuda").manual_seed(3))
    h = mlp.hparams(learning_rate=2e-3)
    a, b = mlp.Trainer(ctx, p, h), mlp.Trainer(ctx, p, h)
    la, lb = torch.zeros(1, device="cuda"), torch.zeros(1, device="cuda")
    a.epoch(rec, tt, perm, 2048, la)
    for k in range(3):
        idx = perm[k * 2048:(k + 1) * 2048]
        b.step(rec[idx].contiguous(), tt[idx].contiguous(), lb)
    sa, sb = a.state(), b.state()
    ctx.synchronize()
    assert sa["steps"] == sb["steps"] == 3
    for k in ("params", "m", "v"):
        assert torch.equal(sa[k], sb[k]), k
    assert torch.equal(la, lb)
    # out-of-range indices are empty samples: the gradient equals the one of the valid samples alone
    c = mlp.Trainer(ctx, p, h)
    bad = perm[:2048].clone()
    bad[1000:] = -5
    c.epoch(rec, tt, bad, 2048)
    ctx.synchronize()
    assert torch.isfinite(c.params()).all()
    a.close()
    b.close()
    c.close()


def test_tensor_core_wait_bound_reports_timeout(ctx):
    """With a wait bound of 0 every CTA of the tcgen05 inference gives up on its
    first product: it lets the product land (bounded), frees its tensor memory
    and leaves without writing; the call reads SKYR_ETIMEOUT, the output stays
    untouched, and the default bound then infers normally."""
    p = _params(61)
    rec, _, _ = _data(1000, 62)
    net = mlp.PackedMLP.from_params(ctx, p)
    default = ctx.limits
    tight = _abi.DeviceLimits.from_buffer_copy(default)
    tight.copy_wait_cycles = 0
    y = torch.full((1000, 3), float("nan"), device="cuda")
    ctx.limits = tight
    net.infer(rec, out=y)
    with pytest.raises(_abi.SkyrError) as exc:
        ctx.check_status()
    assert exc.value.status == _abi.SKYR_ETIMEOUT
    assert bool(torch.isnan(y).all())
    ctx.limits = default
    net.infer(rec, out=y)
    ctx.check_status()
    assert bool(torch.isfinite(y).all())


def test_adam_step_matches_oracle(ctx):
    p = _params(41)
    rec, _, t = _data(2048, 42)
    tt = torch.from_numpy(t).cuda()
    h = mlp.hparams(learning_rate=1e-3)
    tr = mlp.Trainer(ctx, p, h)
    g_gpu = []
    pm = p.astype(np.float64).copy()
    m, v = np.zeros(P), np.zeros(P)
    for step in (1, 2, 3):
        # the gradient the trainer will use: same packed network, same batch
        g, _ = mlp.gradient(ctx, tr.packed(), h, rec, tt)
        g_gpu.append(g.cpu().numpy().astype(np.float64))
        tr.step(rec, tt)
        orc.mlp_adam(pm, m, v, g_gpu[-1].copy(), lr=1e-3, step=step)
        got = tr.params().cpu().numpy().astype(np.float64)
        assert np.max(np.abs(got - pm)) <= 1e-6, step
    assert tr.steps == 3
    tr.close()


def test_training_reduces_loss(ctx):
    rng = np.random.default_rng(51)
    n = 16384
    x = rng.random((n, IN)).astype(np.float32)
    # a smooth positive target of a few inputs
    t = np.stack([0.5 + x[:, 0] * x[:, 1], 1.0 + np.sin(3 * x[:, 2]) * 0.5, 0.2 + x[:, 3:8].mean(1)], 1)
    t = t.astype(np.float32)
    rec = mlp.to_records(torch.from_numpy(x))
    tt = torch.from_numpy(t).cuda()
    h = mlp.hparams(learning_rate=3e-3)
    tr = mlp.Trainer(ctx, mlp.init_params(52), h)
    loss = torch.zeros(1, device="cuda")
    tr.step(rec, tt, loss)
    first = float(loss.item())
    for _ in range(2000):
        tr.step(rec, tt)
    loss.zero_()
    tr.step(rec, tt, loss)
    last = float(loss.item())
    assert last < 0.05 * first, (first, last)
    y = tr.packed().infer(rec).cpu().numpy()
    assert np.mean(np.abs(y - t)) / np.mean(np.abs(t)) < 0.08


def test_invalid_arguments(ctx):
    p = _params(61)
    net = mlp.PackedMLP.from_params(ctx, p)
    rec, _, t = _data(64, 62)
    tt = torch.from_numpy(t).cuda()
    g = torch.empty(P, device="cuda")
    h = mlp.hparams()
    lib = _abi.lib()
    assert lib.skyr_mlp_gradient(ctx.handle, _ptr(net.buf), C.byref(h), _ptr(rec), _ptr(tt), 0, _ptr(g),
                                 None) == _abi.SKYR_EINVAL
    assert lib.skyr_mlp_gradient(ctx.handle, _ptr(net.buf), C.byref(h), _ptr(rec), _ptr(tt), 65537, _ptr(g),
                                 None) == _abi.SKYR_EINVAL
    bad = mlp.hparams(learning_rate=-1.0)
    assert lib.skyr_mlp_gradient(ctx.handle, _ptr(net.buf), C.byref(bad), _ptr(rec), _ptr(tt), 64, _ptr(g),
                                 None) == _abi.SKYR_EINVAL
    mis = C.c_void_p(rec.data_ptr() + 2)  # records must be 16-byte aligned
    assert lib.skyr_mlp_infer(ctx.handle, _ptr(net.buf), mis, 8, _ptr(g)) == _abi.SKYR_EINVAL
    assert lib.skyr_mlp_pack(ctx.handle, _ptr(torch.from_numpy(p).cuda()), C.c_float(0.0),
                             _ptr(net.buf)) == _abi.SKYR_EINVAL
