"""FP64 reference of the b_kappa surrogate network (TEST INFRASTRUCTURE ONLY).

The surrogate maps 8 features (log l1, log l2, log l3, Omega_m, sigma_8, h, w,
n_s; scaled to [-1, 1] over the training box) to the scaled log b_kappa with a
multilayer perceptron 8 -> 256 -> 256 -> 256 -> 256 -> 1, SiLU after each
hidden layer and a linear output; the loss is the mean squared error. The GPU
product (threepoint_gb300/csrc/tp_mlp.cu) trains and evaluates it with BF16
operands and FP32 accumulation; this module restates the same forward and
backward passes in FP64 numpy so that the GPU activations and gradients can be
checked, with an optional BF16 rounding of the operands exactly where the GPU
rounds them.
"""
from __future__ import annotations

import numpy as np

WIDTHS = (8, 256, 256, 256, 256, 1)


def bf16(a):
    """Round to the nearest BF16 value (ties to even), returned as float64."""
    a32 = np.ascontiguousarray(a, dtype=np.float32)
    u = a32.view(np.uint32).astype(np.uint64)
    lsb = (u >> 16) & 1
    r = ((u + 0x7FFF + lsb) >> 16) << 16
    out = r.astype(np.uint32).view(np.float32).astype(np.float64)
    nan = np.isnan(a32)
    out[nan] = np.nan
    return out


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def init_params(seed=0, widths=WIDTHS):
    """He-style initial weights [(W [out, in], b [out])] (the GPU trainer's
    initialisation draws from the same distribution with its own generator)."""
    rng = np.random.default_rng(seed)
    ps = []
    for i in range(len(widths) - 1):
        fan_in, fan_out = widths[i], widths[i + 1]
        ps.append((rng.normal(0.0, np.sqrt(2.0 / fan_in), (fan_out, fan_in)), np.zeros(fan_out)))
    return ps


def forward(params, x, round_bf16=False):
    """y [n] and the per-layer caches (input h, pre-activation z).

    round_bf16: round the GEMM operands (weights and layer inputs) to BF16 as
    the GPU does; accumulation, bias, activation and the last layer in FP64."""
    r = bf16 if round_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    h = np.asarray(x, dtype=np.float64)
    caches = []
    n = len(params)
    for i, (W, b) in enumerate(params):
        last = i == n - 1
        hin = h if last else r(h)
        Wm = W if last else r(W)
        z = hin @ Wm.T + b
        caches.append((hin, z))
        h = z if last else silu(z)
    return h[:, 0], caches


def loss_and_grads(params, x, t, round_bf16=False):
    """Mean squared error and its gradients [(dW, db)] by the chain rule."""
    y, caches = forward(params, x, round_bf16)
    n = len(y)
    diff = y - t
    loss = float(np.mean(diff * diff))
    dz = (2.0 / n) * diff[:, None]
    grads = [None] * len(params)
    for i in range(len(params) - 1, -1, -1):
        hin, z = caches[i]
        W, _ = params[i]
        grads[i] = (dz.T @ hin, dz.sum(0))
        if i > 0:
            Wm = W if i == len(params) - 1 else (bf16(W) if round_bf16 else W)
            dh = dz @ Wm
            _, zprev = caches[i - 1]
            dz = dh * silu_grad(zprev)
    return loss, grads


def adam_step(params, grads, state, lr=1e-3, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (Kingma & Ba 2015, bias-corrected), in place; state is
    a dict with 't' and the first/second moments."""
    state["t"] = state.get("t", 0) + 1
    t = state["t"]
    if "m" not in state:
        state["m"] = [(np.zeros_like(W), np.zeros_like(b)) for W, b in params]
        state["v"] = [(np.zeros_like(W), np.zeros_like(b)) for W, b in params]
    out = []
    for i, ((W, b), (gW, gb)) in enumerate(zip(params, grads)):
        new = []
        for j, (p, g) in enumerate(((W, gW), (b, gb))):
            m = state["m"][i][j]
            v = state["v"][i][j]
            m[...] = b1 * m + (1 - b1) * g
            v[...] = b2 * v + (1 - b2) * g * g
            mh = m / (1 - b1 ** t)
            vh = v / (1 - b2 ** t)
            new.append(p - lr * mh / (np.sqrt(vh) + eps))
        out.append(tuple(new))
    return out
