"""CPU oracle of the learned preconditioner's network (test infrastructure only).

Restates in numpy the 3-layer MLP of the learned two-level preconditioner
(pdlsm-fem_mpi_gb300/csrc/k_learned.cu, Mlp::forward_backward): parameters in
one FP32 block (W1 [H x n], b1, W2 [H x H], b2, W3 [n x H], b3), tanh hidden
layers, loss sum_b w_b |y_b - t_b|^2.  With ``bf16=True`` every GEMM operand
is rounded to bfloat16 (round to nearest even) where the GPU kernels round
it, and products accumulate in float64; with ``bf16=False`` the computation
is plain float64, used to check the backward formulas against finite
differences.  The reference has no learned component, so this oracle is the
network's own specification; it is pinned by the finite-difference check.
"""
from __future__ import annotations

import numpy as np


def to_bf16(x: np.ndarray) -> np.ndarray:
    """Round to bfloat16 (nearest even) through float32; returned as float64."""
    f = np.ascontiguousarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def split(p: np.ndarray, n: int, H: int):
    i = 0
    W1 = p[i:i + H * n].reshape(H, n); i += H * n
    b1 = p[i:i + H]; i += H
    W2 = p[i:i + H * H].reshape(H, H); i += H * H
    b2 = p[i:i + H]; i += H
    W3 = p[i:i + n * H].reshape(n, H); i += n * H
    b3 = p[i:i + n]
    return W1, b1, W2, b2, W3, b3


def loss_grad(p: np.ndarray, n: int, H: int, X: np.ndarray, T: np.ndarray, w: np.ndarray, bf16: bool = True):
    """Loss and gradient (flat, same layout as p) for a batch X (B x n)."""
    p = np.asarray(p, dtype=np.float64)
    r = to_bf16 if bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    W1, b1, W2, b2, W3, b3 = split(p, n, H)
    Xr, W1r, W2r, W3r = r(X), r(W1), r(W2), r(W3)
    Z1 = Xr @ W1r.T + b1
    H1 = r(np.tanh(Z1))
    Z2 = H1 @ W2r.T + b2
    H2 = r(np.tanh(Z2))
    Y = H2 @ W3r.T + b3
    D = Y - T
    loss = float(np.sum(w[:, None] * D * D))
    dY = 2.0 * w[:, None] * D
    dYr = r(dY)
    gW3 = dYr.T @ H2
    gb3 = dY.sum(axis=0)
    dZ2 = (dYr @ W3r) * (1.0 - np.tanh(Z2) ** 2)
    dZ2r = r(dZ2)
    gW2 = dZ2r.T @ H1
    gb2 = dZ2.sum(axis=0)
    dZ1 = (dZ2r @ W2r) * (1.0 - np.tanh(Z1) ** 2)
    dZ1r = r(dZ1)
    gW1 = dZ1r.T @ Xr
    gb1 = dZ1.sum(axis=0)
    return loss, np.concatenate([gW1.ravel(), gb1, gW2.ravel(), gb2, gW3.ravel(), gb3])
