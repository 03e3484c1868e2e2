"""CPU oracle of the residual CNN coarse propagator (test infrastructure only).

Imported by ``tests/`` as the checker of the GPU forward/backward kernels
(``pararealml_gb300/csrc/prml_cnn.cu``); the product never imports it.

The network maps a 2-component state u (c, mu) on an H x W grid to
``u + s_out * net(s_in * u)`` where net is six 3x3 "same" convolutions with
zero padding: 2 -> 32, four 32 -> 32, 32 -> 2, ReLU after the first five.
The GPU keeps hidden activations (and their gradients) in bfloat16 and
accumulates in float32; this oracle computes in float64 and rounds to
bfloat16 at exactly the points where the GPU stores bfloat16, so the two
agree up to accumulation order.

This is the reference's ``SupervisedMLOperator`` contract
(``pararealml/operators/ml/supervised/supervised_ml_operator.py:16-128``:
an autoregressive operator trained on trajectories of an oracle solver)
with a convolutional model in place of the reference's per-point dense
regressors.
"""

from __future__ import annotations

from typing import Dict, List

import numpy as np

TAPS = [(dy, dx) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
HIDDEN = 32
N_MID = 4


def bf16(x: np.ndarray) -> np.ndarray:
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    f = np.asarray(x, dtype=np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    rounding = ((u >> 16) & 1) + 0x7FFF
    r = ((u + rounding) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def shift(x: np.ndarray, dy: int, dx: int) -> np.ndarray:
    """out[.., y, x, :] = x[.., y + dy, x + dx, :] with zero outside (NHWC)."""
    out = np.zeros_like(x)
    h, w = x.shape[-3], x.shape[-2]
    ys = slice(max(0, -dy), min(h, h - dy))
    xs = slice(max(0, -dx), min(w, w - dx))
    yd = slice(max(0, dy), min(h, h + dy))
    xd = slice(max(0, dx), min(w, w + dx))
    out[..., ys, xs, :] = x[..., yd, xd, :]
    return out


def conv(x: np.ndarray, w: np.ndarray, b: np.ndarray) -> np.ndarray:
    """x: (B, H, W, Ci); w: (9, Ci, Co) indexed by TAPS; b: (Co,)."""
    out = np.zeros(x.shape[:-1] + (w.shape[-1],))
    for t, (dy, dx) in enumerate(TAPS):
        out += shift(x, dy, dx) @ w[t]
    return out + b


def init_params(seed: int = 0) -> Dict[str, np.ndarray]:
    rng = np.random.default_rng(seed)
    p = {}
    chans = [2] + [HIDDEN] * (N_MID + 1) + [2]
    for layer in range(len(chans) - 1):
        ci, co = chans[layer], chans[layer + 1]
        scale = np.sqrt(2.0 / (9 * ci))
        if layer == len(chans) - 2:
            scale *= 0.1
        p[f"w{layer}"] = rng.normal(0.0, scale, (9, ci, co))
        p[f"b{layer}"] = np.zeros(co)
    return p


def forward(p: Dict[str, np.ndarray], u: np.ndarray, s_in: np.ndarray, s_out: np.ndarray):
    """u: (B, H, W, 2).  Returns (y, cache) with bf16 points emulated."""
    n_layers = N_MID + 2
    acts: List[np.ndarray] = []
    x = u * s_in
    for layer in range(n_layers - 1):
        w = p[f"w{layer}"]
        if layer > 0:
            w = bf16(w)
        x = bf16(np.maximum(conv(x, w, p[f"b{layer}"]), 0.0))
        acts.append(x)
    z = conv(x, p[f"w{n_layers - 1}"], p[f"b{n_layers - 1}"])
    return u + s_out * z, {"u": u, "acts": acts}


def backward(p, cache, dy: np.ndarray, s_in: np.ndarray, s_out: np.ndarray) -> Dict[str, np.ndarray]:
    """Gradients of sum(dy * y) w.r.t. all weights and biases."""
    n_layers = N_MID + 2
    acts = cache["acts"]
    grads = {}
    g = dy * s_out  # dL/dz
    last = n_layers - 1
    grads[f"w{last}"] = np.stack([np.einsum("bhwi,bhwo->io", shift(acts[-1], *t), g) for t in TAPS])
    grads[f"b{last}"] = g.sum(axis=(0, 1, 2))
    w = p[f"w{last}"]
    gx = np.zeros_like(acts[-1])
    for t, (dy_, dx_) in enumerate(TAPS):
        gx += shift(g @ w[t].T, -dy_, -dx_)
    g = bf16(gx * (acts[-1] > 0))
    for layer in range(n_layers - 2, -1, -1):
        x_in = acts[layer - 1] if layer > 0 else cache["u"] * s_in
        grads[f"w{layer}"] = np.stack([np.einsum("bhwi,bhwo->io", shift(x_in, *t), g) for t in TAPS])
        grads[f"b{layer}"] = g.sum(axis=(0, 1, 2))
        if layer == 0:
            break
        w = bf16(p[f"w{layer}"])
        gx = np.zeros_like(x_in)
        for t, (dy_, dx_) in enumerate(TAPS):
            gx += shift(g @ w[t].T, -dy_, -dx_)
        g = bf16(gx * (x_in > 0))
    return grads


def mse_and_grad(y: np.ndarray, target: np.ndarray):
    d = y - target
    return float(np.mean(d * d)), 2.0 * d / d.size
