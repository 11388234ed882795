"""Host side of the surrogate network (include/skyr_mlp.h): parameter init,
feature records, the packed network, inference, gradients and the trainer.

The network (79 -> 64 -> 64 -> 64 -> 64 -> 3, ReLU, BF16 weights, FP32
accumulation) has no counterpart in the reference; it stands in for the
multiple-scattering heuristic of VolumetricCloudRender.comp:125-130.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _abi
from .atmosphere import Context, _ptr

PARAMS = _abi.SKYR_MLP_PARAMS
INPUTS = _abi.SKYR_MLP_INPUTS
RECORD = _abi.SKYR_MLP_RECORD


def packed_bytes() -> int:
    return int(_abi.lib().skyr_mlp_packed_bytes())


def init_params(seed: int) -> np.ndarray:
    """He-uniform weights, zero biases (FP32 parameter vector)."""
    p = np.zeros(PARAMS, dtype=np.float32)
    _abi.call("skyr_mlp_init_params", C.c_uint64(seed), p.ctypes.data)
    return p


def hparams(**kw) -> _abi.MlpHparams:
    h = _abi.MlpHparams()
    _abi.call("skyr_mlp_hparams_default", C.byref(h))
    for k, v in kw.items():
        setattr(h, k, v)
    return h


def to_records(x: torch.Tensor) -> torch.Tensor:
    """[n][INPUTS] features -> [n][RECORD] bf16 records on the GPU (zero pads)."""
    n = x.shape[0]
    r = torch.zeros((n, RECORD), dtype=torch.bfloat16, device="cuda")
    r[:, :INPUTS] = x.to(device="cuda", dtype=torch.bfloat16)
    return r


def records_to_numpy(rec: torch.Tensor) -> np.ndarray:
    """bf16 records -> the float32 [n][INPUTS] features they hold exactly."""
    return rec[:, :INPUTS].float().cpu().numpy()


def _check_records(rec: torch.Tensor):
    if rec.dtype != torch.bfloat16 or rec.dim() != 2 or rec.shape[1] != RECORD or not rec.is_contiguous():
        raise ValueError(f"records must be a contiguous [n][{RECORD}] bfloat16 CUDA tensor")


class PackedMLP:
    """The packed network an inference kernel reads (device bytes)."""

    def __init__(self, ctx: Context):
        self.ctx = ctx
        self.buf = torch.zeros(packed_bytes(), dtype=torch.uint8, device="cuda")

    @classmethod
    def from_params(cls, ctx: Context, params, out_scale: float = 1.0) -> "PackedMLP":
        m = cls(ctx)
        p = torch.as_tensor(np.asarray(params, dtype=np.float32)).cuda() if not torch.is_tensor(params) else params
        if p.dtype != torch.float32 or p.numel() != PARAMS or not p.is_cuda:
            raise ValueError(f"parameters must be {PARAMS} FP32 values on the GPU (got {p.numel()} {p.dtype})")
        m._params = p.contiguous()
        _abi.call("skyr_mlp_pack", ctx.handle, _ptr(m._params), C.c_float(out_scale), _ptr(m.buf))
        return m

    def infer(self, rec: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        _check_records(rec)
        y = out if out is not None else torch.empty((rec.shape[0], 3), dtype=torch.float32, device="cuda")
        _abi.call("skyr_mlp_infer", self.ctx.handle, _ptr(self.buf), _ptr(rec), rec.shape[0], _ptr(y))
        return y


def gradient(ctx: Context, packed: PackedMLP, h: _abi.MlpHparams, rec: torch.Tensor, targets: torch.Tensor):
    """(gradient[PARAMS] FP32, loss) of the mean relative-L2 loss on one batch."""
    _check_records(rec)
    t = targets.contiguous().float()
    g = torch.empty(PARAMS, dtype=torch.float32, device="cuda")
    loss = torch.zeros(1, dtype=torch.float32, device="cuda")
    _abi.call("skyr_mlp_gradient", ctx.handle, _ptr(packed.buf), C.byref(h), _ptr(rec), _ptr(t), rec.shape[0],
              _ptr(g), _ptr(loss))
    return g, loss


class Trainer:
    """FP32 master parameters + Adam moments; one call per batch."""

    def __init__(self, ctx: Context, params: np.ndarray, h: _abi.MlpHparams):
        self.ctx, self.h = ctx, h
        p = np.ascontiguousarray(params, dtype=np.float32)
        self._tr = C.c_void_p()
        _abi.call("skyr_mlp_trainer_create", ctx.handle, p.ctypes.data, C.byref(h), C.byref(self._tr))

    def step(self, rec: torch.Tensor, targets: torch.Tensor, loss_accum: torch.Tensor | None = None):
        _check_records(rec)
        _abi.call("skyr_mlp_train_step", self._tr, _ptr(rec), _ptr(targets), rec.shape[0], _ptr(loss_accum))

    def epoch(self, rec: torch.Tensor, targets: torch.Tensor, perm: torch.Tensor, batch: int,
              loss_accum: torch.Tensor | None = None):
        """The full batches of one epoch over the permutation `perm` (device int32 / int64
        indices into rec / targets), gathered by the gradient kernel itself."""
        _check_records(rec)
        idx = perm.to(torch.int32).contiguous()
        t = targets.contiguous().float()
        _abi.call("skyr_mlp_train_epoch", self._tr, _ptr(rec), _ptr(t), rec.shape[0], _ptr(idx), idx.shape[0], batch,
                  _ptr(loss_accum))

    def set_learning_rate(self, lr: float):
        _abi.call("skyr_mlp_trainer_set_learning_rate", self._tr, C.c_float(lr))

    @property
    def steps(self) -> int:
        return int(_abi.lib().skyr_mlp_trainer_steps(self._tr))

    def params(self) -> torch.Tensor:
        out = torch.empty(PARAMS, dtype=torch.float32, device="cuda")
        _abi.call("skyr_mlp_trainer_copy_params", self._tr, _ptr(out))
        return out

    def packed(self) -> PackedMLP:
        m = PackedMLP(self.ctx)
        _abi.call("skyr_mlp_trainer_copy_packed", self._tr, _ptr(m.buf))
        return m

    def state(self) -> dict:
        """Checkpoint: parameters, Adam moments (device FP32[PARAMS] each) and the step count."""
        out = {k: torch.empty(PARAMS, dtype=torch.float32, device="cuda") for k in ("params", "m", "v")}
        steps = C.c_int()
        _abi.call("skyr_mlp_trainer_save_state", self._tr, _ptr(out["params"]), _ptr(out["m"]), _ptr(out["v"]),
                  C.byref(steps))
        out["steps"] = steps.value
        return out

    def load_state(self, state: dict) -> None:
        """Resume from a checkpoint of state() (tensors on the device or host)."""
        dev = {k: state[k].to("cuda", torch.float32).contiguous() for k in ("params", "m", "v")}
        _abi.call("skyr_mlp_trainer_load_state", self._tr, _ptr(dev["params"]), _ptr(dev["m"]), _ptr(dev["v"]),
                  int(state["steps"]))
        self.ctx.synchronize()  # the sources may go away

    def close(self):
        if self._tr:
            _abi.call("skyr_mlp_trainer_destroy", self._tr)
            self._tr = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
