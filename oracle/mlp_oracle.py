"""CPU ORACLE -- test infrastructure only.

numpy restatement of the per-cell MLP's forward pass and gradients with the
same rounding points as the GPU kernels: GEMM operands rounded to BF16 (round
to nearest even), products summed in float64 here (FP32 on the GPU), bias and
ReLU on the FP32 output, next-layer input rounded to BF16; loss = mean squared
error.  Used to check the GPU gradients, and itself checked against finite
differences of its own loss."""
from __future__ import annotations

import numpy as np


def bf16(x):
    """Round float32 values to bfloat16 (nearest even), returned as float64."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    b = x.view(np.uint32).astype(np.uint64)
    b = (b + 0x7FFF + ((b >> 16) & 1)) & 0xFFFF0000
    return b.astype(np.uint32).view(np.float32).astype(np.float64)


def forward(Ws, bs, X):
    """Returns the list of FP32-level outputs z_l (post-ReLU except the last)."""
    h = bf16(X)
    outs = []
    for l, (W, b) in enumerate(zip(Ws, bs)):
        z = h @ bf16(W) + b
        if l < len(Ws) - 1:
            z = np.maximum(z, 0.0)
            h = bf16(z)
        outs.append(z)
    return outs


def loss_and_grads(Ws, bs, X, T):
    outs = forward(Ws, bs, X)
    Y = outs[-1]
    count = Y.size
    loss = float(np.sum((Y - T) ** 2) / count)
    dz = 2.0 * (Y - T) / count
    acts = [bf16(X)] + [bf16(z) for z in outs[:-1]]
    gW, gb = [None] * len(Ws), [None] * len(Ws)
    for l in reversed(range(len(Ws))):
        dzb = bf16(dz)
        gW[l] = acts[l].T @ dzb
        gb[l] = dz.sum(axis=0)
        if l > 0:
            dh = dzb @ bf16(Ws[l]).T
            dz = np.where(outs[l - 1] > 0.0, dh, 0.0)
    return loss, gW, gb


def loss_exact(Ws, bs, X, T):
    """The same network without any rounding (for finite-difference checks)."""
    h = X
    for l, (W, b) in enumerate(zip(Ws, bs)):
        h = h @ W + b
        if l < len(Ws) - 1:
            h = np.maximum(h, 0.0)
    return float(np.sum((h - T) ** 2) / h.size)


def grads_exact(Ws, bs, X, T):
    hs = [X]
    h = X
    zs = []
    for l, (W, b) in enumerate(zip(Ws, bs)):
        z = h @ W + b
        zs.append(z)
        h = np.maximum(z, 0.0) if l < len(Ws) - 1 else z
        hs.append(h)
    dz = 2.0 * (hs[-1] - T) / hs[-1].size
    gW, gb = [None] * len(Ws), [None] * len(Ws)
    for l in reversed(range(len(Ws))):
        gW[l] = hs[l].T @ dz
        gb[l] = dz.sum(axis=0)
        if l > 0:
            dz = (dz @ Ws[l].T) * (zs[l - 1] > 0.0)
    return gW, gb
