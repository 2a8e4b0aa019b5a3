"""CPU oracle of the warm-start MLP — TEST INFRASTRUCTURE ONLY.

Forward and backward of the BF16 network in numpy with the same rounding
points as the GPU kernels (spicier_gb300/csrc/mlp.cu): BF16 inputs, weights
and stored activations (round to nearest even), FP32 accumulation, GELU in
its tanh form evaluated on the FP32 pre-activation, GELU' on the stored
BF16 pre-activation, BF16 output-gradient.  `exact=True` disables every
rounding (FP64 throughout) for finite-difference checks of the formulas.
"""
from __future__ import annotations

import numpy as np


def f16(a: np.ndarray) -> np.ndarray:
    """Round to FP16 (nearest even) and back to FP32: the tcgen05 inference
    kernels' operands and stored activations."""
    return np.asarray(a, dtype=np.float32).astype(np.float16).astype(np.float32)


def bf16(a: np.ndarray) -> np.ndarray:
    a = np.ascontiguousarray(a, dtype=np.float32)
    b = a.view(np.uint32).astype(np.uint64)
    r = ((b >> 16) & 1) + 0x7FFF
    return ((b + r) & 0xFFFF0000).astype(np.uint32).view(np.float32)


_C, _A = np.sqrt(2.0 / np.pi), 0.044715


def gelu(z):
    """GELU in its tanh form (the kernels' activation, mlp_act.cuh)."""
    return 0.5 * z * (1.0 + np.tanh(_C * (z + _A * z ** 3)))


def gelu_grad(z):
    t = np.tanh(_C * (z + _A * z ** 3))
    return 0.5 * (1.0 + t) + 0.5 * z * (1.0 - t * t) * _C * (1.0 + 3.0 * _A * z * z)


def pad(a, cols):
    out = np.zeros((a.shape[0], cols), dtype=a.dtype)
    out[:, :a.shape[1]] = a
    return out


def forward_backward(layers, X, T, n_out, exact=False, rounding="bf16"):
    """layers: [(Wt[out_pad][in_pad], b[out_pad])] FP32 masters.
    rounding: "bf16" (the trainer and the mma.sync kernels) or "f16" (the
    tcgen05 inference kernels).  Returns (Y[rows][out_pad], loss, [(dWt, db)])."""
    dt = np.float64 if exact else np.float32
    rnd = (lambda a: np.asarray(a, dtype=np.float64)) if exact else (f16 if rounding == "f16" else bf16)
    rows = X.shape[0]
    kin = layers[0][0].shape[1]
    A = rnd(pad(X.astype(dt), kin))
    acts, zs = [A], []
    for Wt, b in layers[:-1]:
        Z = A.astype(dt) @ rnd(Wt).astype(dt).T + b.astype(dt)
        zs.append(rnd(Z))
        A = rnd(gelu(Z))
        acts.append(A)
    Wt, b = layers[-1]
    Y = A.astype(dt) @ rnd(Wt).astype(dt).T + b.astype(dt)
    kout = Wt.shape[0]
    Tp = pad(T.astype(dt), kout)
    diff = (Y - Tp)[:, :n_out]
    loss = float((diff.astype(np.float64) ** 2).mean())
    g = np.zeros_like(Y)
    g[:, :n_out] = 2.0 * diff / (rows * n_out)
    D = rnd(g)
    grads = [None] * len(layers)
    for l in range(len(layers) - 1, -1, -1):
        Wt, _ = layers[l]
        dWt = D.astype(dt).T @ acts[l].astype(dt)
        db = D.astype(dt).sum(0)
        grads[l] = (dWt, db)
        if l == 0:
            break
        dH = D.astype(dt) @ rnd(Wt).astype(dt)
        D = rnd(dH * gelu_grad(zs[l - 1].astype(dt)))
    return Y, loss, grads
