"""CPU oracle of the per-tet warm-start MLP (14 -> 64 -> 64 -> 64 -> 2, SiLU).

TEST INFRASTRUCTURE ONLY: the checker for the GPU forward/backward/Adam
kernels. The network has no reference counterpart (the reference has no
learned component); it follows the layer sizes, activation, precision and
optimiser stated for the learned warm start: BF16 weights and activations,
FP32 accumulation, Adam (lr 1e-3).

Precision model of the GPU kernels, reproduced here (rounding=True):
  * inputs, weights and hidden activations are rounded to BF16
    (round-to-nearest-even) before each matrix product;
  * products accumulate in FP32 (here FP64, compared with a tolerance);
  * biases, pre-activations and outputs stay in FP32;
  * backward: the error signals d_k of the hidden layers enter the tensor-core
    products (d_k W_k and d_k^T a_{k-1}) rounded to BF16 (round_grad=True);
    bias gradients and the 2-wide output layer use them unrounded.
rounding=False gives the plain FP64 network whose gradient the finite-
difference check verifies.
"""
from __future__ import annotations

import numpy as np

N_IN, N_IN_PAD, N_HID, N_OUT = 14, 16, 64, 2


def bf16(a: np.ndarray) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    rounding = 0x7FFF + ((u >> 16) & 1)
    r = ((u + rounding) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32)
    return np.where(np.isnan(a), a, out)


def silu(z):
    return z / (1.0 + np.exp(-z))


def dsilu(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init_params(seed: int = 0):
    """He-style init in FP32: W_k is (out, in), b_k is (out,). The padded input
    columns 14, 15 of W1 are zero."""
    rng = np.random.default_rng(seed)
    dims = [(N_HID, N_IN_PAD), (N_HID, N_HID), (N_HID, N_HID), (N_OUT, N_HID)]
    params = []
    for k, (o, i) in enumerate(dims):
        fan_in = N_IN if k == 0 else i
        W = (rng.standard_normal((o, i)) * np.sqrt(2.0 / fan_in)).astype(np.float32)
        if k == 0:
            W[:, N_IN:] = 0
        if k == 3:
            W *= 0.1
        params += [W, np.zeros(o, np.float32)]
    return params


def _r(a, on):
    """BF16 rounding when on (as FP64), identity otherwise."""
    a = np.asarray(a)
    return bf16(a.astype(np.float32)).astype(np.float64) if on else a.astype(np.float64)


def forward(params, X, rounding=True):
    """X: (B, 16) float32. Returns (out (B, 2), cache)."""
    W1, b1, W2, b2, W3, b3, W4, b4 = [np.asarray(p, np.float64) for p in params]
    a0 = _r(X, rounding)
    z1 = a0 @ _r(W1, rounding).T + b1
    a1 = _r(silu(z1), rounding)
    z2 = a1 @ _r(W2, rounding).T + b2
    a2 = _r(silu(z2), rounding)
    z3 = a2 @ _r(W3, rounding).T + b3
    a3 = _r(silu(z3), rounding)
    out = a3 @ _r(W4, rounding).T + b4
    return out, (a0, z1, a1, z2, a2, z3, a3)


def loss_and_grads(params, X, Y, rounding=True, round_grad=None):
    """Mean-squared error over the batch (sum over rows of ||out - y||^2 / B)
    and its gradients in FP64, through the forward pass's rounding."""
    if round_grad is None:
        round_grad = rounding
    W = [np.asarray(params[2 * k], np.float64) for k in range(4)]
    out, (a0, z1, a1, z2, a2, z3, a3) = forward(params, X, rounding)
    B = X.shape[0]
    diff = out - np.asarray(Y, np.float64)
    loss = float((diff ** 2).sum() / B)
    d4 = 2.0 * diff / B
    g = [None] * 8
    g[6] = d4.T @ a3
    g[7] = d4.sum(0)
    da3 = d4 @ _r(W[3], rounding)
    d3 = da3 * dsilu(z3)
    g[4] = _r(d3, round_grad).T @ a2
    g[5] = d3.sum(0)
    da2 = _r(d3, round_grad) @ _r(W[2], rounding)
    d2 = da2 * dsilu(z2)
    g[2] = _r(d2, round_grad).T @ a1
    g[3] = d2.sum(0)
    da1 = _r(d2, round_grad) @ _r(W[1], rounding)
    d1 = da1 * dsilu(z1)
    g[0] = _r(d1, round_grad).T @ a0
    g[1] = d1.sum(0)
    return loss, g


def flatten(params):
    """Parameter list -> the flat FP32 vector of the C ABI (W1, b1, ..., W4, b4)."""
    return np.concatenate([np.asarray(p, np.float32).ravel() for p in params])


def unflatten(v):
    """Flat vector -> [W1 (64x16), b1, W2, b2, W3, b3, W4 (2x64), b4]."""
    shapes = [(N_HID, N_IN_PAD), (N_HID,), (N_HID, N_HID), (N_HID,), (N_HID, N_HID), (N_HID,), (N_OUT, N_HID),
              (N_OUT,)]
    out, o = [], 0
    for sh in shapes:
        n = int(np.prod(sh))
        out.append(np.asarray(v[o:o + n], np.float32).reshape(sh))
        o += n
    assert o == len(v)
    return out


def adam_step(params, grads, m, v, t, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (FP32 master weights, step t >= 1); returns new lists."""
    out_p, out_m, out_v = [], [], []
    c1 = 1.0 - b1 ** t
    c2 = 1.0 - b2 ** t
    for p, gr, mm, vv in zip(params, grads, m, v):
        gr = np.asarray(gr, np.float64)
        mm = b1 * mm + (1 - b1) * gr
        vv = b2 * vv + (1 - b2) * gr * gr
        p = p - lr * (mm / c1) / (np.sqrt(vv / c2) + eps)
        out_p.append(p.astype(np.float32))
        out_m.append(mm)
        out_v.append(vv)
    return out_p, out_m, out_v
