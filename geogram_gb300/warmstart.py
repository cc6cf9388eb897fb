"""Learned warm start for the optimal-transport solver.

A small MLP looks at every seed's position and the distances to its 16
nearest seeds (x, y, z, d_1 .. d_16 times n^(1/3)) and predicts the
cell-averaged Laplacian of the seed's optimal Kantorovich weight on the
cell graph at zero weights, t_i = (H0 w*)_i / vol_i(0).  By the
Monge-Ampere relation that is a function of the local density, which the
inputs see; the weights themselves are a global potential, which they do
not.  The solver turns the prediction into starting weights by solving
H0 w = t vol(0) and runs damped Newton from there
(gbv_ot_solve_learned_device).  The network
(19 -> 128 -> 128 -> 128 -> 1, GELU) runs forward and backward on the GPU's
tensor cores through libgbv.so (BF16 operands, FP32 accumulation, FP32
parameters trained with Adam); this module holds the parameters and drives
training and prediction.  The reference has no counterpart: its solver
starts from zero weights.

Device arrays are torch CUDA tensors (float32 unless stated).
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import _lib

HERE = os.path.dirname(os.path.abspath(__file__))
DEFAULT_MODEL = os.path.join(HERE, "data", "warmstart_mlp.npz")

H = 128
IN = _lib.MLP_INPUTS
IN_PAD = 32
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN_PAD
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + H * H
OFF_W4 = OFF_B3 + H
OFF_B4 = OFF_W4 + H
assert OFF_B4 + 1 == _lib.MLP_PARAMS


def init_params(seed: int = 0) -> np.ndarray:
    """He-style initialisation (biases zero, padded input columns zero)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(_lib.MLP_PARAMS, np.float32)
    w1 = np.zeros((H, IN_PAD), np.float32)
    w1[:, :IN] = rng.normal(0.0, np.sqrt(2.0 / IN), (H, IN))
    p[OFF_W1:OFF_B1] = w1.ravel()
    p[OFF_W2:OFF_B2] = rng.normal(0.0, np.sqrt(2.0 / H), H * H)
    p[OFF_W3:OFF_B3] = rng.normal(0.0, np.sqrt(2.0 / H), H * H)
    p[OFF_W4:OFF_B4] = rng.normal(0.0, np.sqrt(1.0 / H), H)
    return p


def unpack(p: np.ndarray) -> dict:
    """The parameter vector as named arrays (W1 without its padding)."""
    return dict(W1=p[OFF_W1:OFF_B1].reshape(H, IN_PAD)[:, :IN], b1=p[OFF_B1:OFF_W2],
                W2=p[OFF_W2:OFF_B2].reshape(H, H), b2=p[OFF_B2:OFF_W3],
                W3=p[OFF_W3:OFF_B3].reshape(H, H), b3=p[OFF_B3:OFF_W4],
                W4=p[OFF_W4:OFF_B4], b4=p[OFF_B4:OFF_B4 + 1])


class WarmStartModel:
    """Parameters (FP32) and normalisation of the warm-start network."""

    def __init__(self, params: np.ndarray | None = None, norm: np.ndarray | None = None,
                 seed: int = 0):
        self.params = (init_params(seed) if params is None
                       else np.asarray(params, np.float32).copy())
        if norm is None:
            norm = np.concatenate([np.zeros(IN), np.ones(IN), [0.0, 1.0]])
        self.norm = np.asarray(norm, np.float32).copy()
        assert self.params.shape == (_lib.MLP_PARAMS,) and self.norm.shape == (_lib.MLP_NORM,)
        self._dev = None

    # -- storage --------------------------------------------------------
    def save(self, path: str, **meta) -> None:
        os.makedirs(os.path.dirname(os.path.abspath(path)), exist_ok=True)
        np.savez_compressed(path, params=self.params, norm=self.norm,
                            **{k: np.asarray(v) for k, v in meta.items()})

    @classmethod
    def load(cls, path: str = DEFAULT_MODEL) -> "WarmStartModel":
        d = np.load(path)
        return cls(d["params"], d["norm"])

    def device(self):
        """(params, norm) as CUDA tensors (cached until the model changes)."""
        import torch
        if self._dev is None:
            self._dev = (torch.tensor(self.params, device="cuda"),
                         torch.tensor(self.norm, device="cuda"))
        return self._dev

    # -- normalisation ----------------------------------------------------
    def fit_normalisation(self, raw, target) -> None:
        """Per-feature mean and std of raw [N][19] and of the targets [N]."""
        import torch
        r = raw.double()
        t = target.double()
        mean = r.mean(0)
        std = r.std(0).clamp_min(1e-12)
        self.norm = np.concatenate([mean.cpu().numpy(), std.cpu().numpy(),
                                    [t.mean().item(), max(t.std().item(), 1e-12)]]).astype(
                                        np.float32)
        self._dev = None
        del torch

    # -- calls ----------------------------------------------------------------
    def forward(self, raw, ctx=None):
        """Standardised outputs of raw features [N][19] (CUDA float32)."""
        import torch
        from . import default_context
        ctx = ctx or default_context()
        p, nrm = self.device()
        raw = raw.contiguous()  # keeps the buffer alive across the call
        y = torch.empty(raw.shape[0], dtype=torch.float32, device="cuda")
        _lib.check(ctx._lib.gbv_mlp_forward(ctx.handle, _lib.ptr(p), _lib.ptr(nrm),
                                            _lib.ptr(raw), raw.shape[0], _lib.ptr(y), None))
        return y

    def loss_grad(self, raw, target, ctx=None):
        """(loss, gradient) of the mean squared error on one batch."""
        import torch
        from . import default_context
        ctx = ctx or default_context()
        p, nrm = self.device()
        raw = raw.contiguous()
        target = target.contiguous()
        g = torch.empty(_lib.MLP_PARAMS, dtype=torch.float32, device="cuda")
        loss = ctypes.c_double()
        _lib.check(ctx._lib.gbv_mlp_loss_grad(ctx.handle, _lib.ptr(p), _lib.ptr(nrm),
                                              _lib.ptr(raw), _lib.ptr(target), raw.shape[0],
                                              _lib.ptr(g), ctypes.byref(loss), None))
        return loss.value, g

    def train(self, raw, target, steps: int = 2000, batch: int = 8192, lr: float = 1e-3,
              seed: int = 0, ctx=None, log_every: int = 0) -> list[float]:
        """Adam on random batches of (raw, target); returns the losses."""
        import torch
        from . import default_context
        ctx = ctx or default_context()
        p, nrm = self.device()
        m = torch.zeros_like(p)
        v = torch.zeros_like(p)
        gen = torch.Generator(device="cuda")
        gen.manual_seed(seed)
        n = raw.shape[0]
        batch = min(batch, n, _lib.MLP_MAX_BATCH)
        losses = []
        for step in range(1, steps + 1):
            idx = torch.randint(0, n, (batch,), device="cuda", generator=gen)
            loss, g = self.loss_grad(raw[idx], target[idx], ctx)
            # cosine decay to 5% of the learning rate
            lr_t = lr * (0.05 + 0.95 * 0.5 * (1.0 + np.cos(np.pi * (step - 1) / steps)))
            _lib.check(ctx._lib.gbv_mlp_adam(ctx.handle, _lib.ptr(p), _lib.ptr(m), _lib.ptr(v),
                                             _lib.ptr(g), step, lr_t, 0.9, 0.999, 1e-8, None))
            losses.append(loss)
            if log_every and step % log_every == 0:
                print(f"step {step} loss {loss:.5f}", flush=True)
        torch.cuda.synchronize()
        self.params = p.cpu().numpy()
        return losses

    def predict_weights(self, xyz_dev, box=((0.0, 0.0, 0.0), (1.0, 1.0, 1.0)), ctx=None):
        """Starting weights (CUDA float64 [N]) for the seeds xyz_dev [N][3]."""
        import torch
        from . import default_context, ot_options
        ctx = ctx or default_context()
        p, nrm = self.device()
        xyz_dev = xyz_dev.contiguous()
        w = torch.empty(xyz_dev.shape[0], dtype=torch.float64, device="cuda")
        o = ot_options(box)
        _lib.check(ctx._lib.gbv_ot_warm_start(ctx.handle, _lib.ptr(xyz_dev), xyz_dev.shape[0],
                                              ctypes.byref(o), _lib.ptr(p), _lib.ptr(nrm),
                                              _lib.ptr(w), None))
        return w

    def solve(self, xyz_dev, w_out, nu_dev=None, ctx=None, **options) -> dict:
        """gbv_ot_solve_device from the learned start; weights into w_out
        (CUDA float64 [N]); options as for geogram_gb300.ot_options."""
        from . import default_context, ot_options
        from ._lib import OtReport
        ctx = ctx or default_context()
        p, nrm = self.device()
        xyz_dev = xyz_dev.contiguous()
        o = ot_options(**options)
        rep = OtReport()
        _lib.check(ctx._lib.gbv_ot_solve_learned_device(
            ctx.handle, _lib.ptr(xyz_dev), _lib.ptr(nu_dev), xyz_dev.shape[0], ctypes.byref(o),
            _lib.ptr(p), _lib.ptr(nrm), _lib.ptr(w_out), None, ctypes.byref(rep)))
        return rep.as_dict()


def laplacian_target(xyz: np.ndarray, w_opt: np.ndarray, ctx=None) -> np.ndarray:
    """Training target of the network: (H0 w*)_i / vol_i(0), with H0 the
    Hessian of the dual at zero weights (the cell graph's Laplacian), vol(0)
    the cell volumes there and w* the optimal weights (0 for empty cells)."""
    from . import ot_gradient_hessian
    n = len(xyz)
    grad, (rp, col, val, diag) = ot_gradient_hessian(xyz, np.zeros(n), ctx=ctx)
    vol0 = 1.0 / n - grad
    row = np.repeat(np.arange(n), np.diff(rp.astype(np.int64)))
    b = diag * w_opt
    np.add.at(b, row, val * w_opt[col])
    return np.where(vol0 > 0, b / np.where(vol0 > 0, vol0, 1.0), 0.0)


def features(xyz_dev, ctx=None):
    """Raw features [N][19] (CUDA float32) of the seeds xyz_dev [N][3] (float64)."""
    import torch
    from . import default_context
    ctx = ctx or default_context()
    xyz_dev = xyz_dev.contiguous()
    raw = torch.empty((xyz_dev.shape[0], IN), dtype=torch.float32, device="cuda")
    _lib.check(ctx._lib.gbv_mlp_features(ctx.handle, _lib.ptr(xyz_dev), xyz_dev.shape[0],
                                         _lib.ptr(raw), None))
    return raw


def gemm_nt(a_bf16, bt_bf16, ctx=None):
    """C = A Bt^T on the tensor cores (CUDA bfloat16 operands, float32 result)."""
    import torch
    from . import default_context
    ctx = ctx or default_context()
    a_bf16 = a_bf16.contiguous()
    bt_bf16 = bt_bf16.contiguous()
    M, K = a_bf16.shape
    N = bt_bf16.shape[0]
    c = torch.empty((M, N), dtype=torch.float32, device="cuda")
    _lib.check(ctx._lib.gbv_mlp_gemm_nt(ctx.handle, _lib.ptr(a_bf16), K, _lib.ptr(bt_bf16), K,
                                        _lib.ptr(c), N, M, N, K, None))
    return c
