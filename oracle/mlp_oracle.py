"""CPU oracle of the learned-MV network (TEST INFRASTRUCTURE ONLY).

The network has no counterpart in the reference, so this numpy restatement
is its checker: a fully connected ReLU net, parameters laid out per layer as
W_l [din, dout] row-major then b_l [dout], mean-squared-error loss
sum(mask * (y - t)^2) / (rows * n_out), and one Adam step.

`forward`/`backward` with quantize=True round to BF16 (round to nearest even)
at exactly the points where the device kernels do: the input, every weight
matrix, every hidden activation (after bias and ReLU), the output gradient and
every back-propagated activation gradient; products accumulate in float64
here and in FP32 on the device, so the two differ by accumulation rounding
only. With quantize=False everything is float64 (checked against finite
differences).
"""

from __future__ import annotations

import numpy as np


def bf16(x) -> np.ndarray:
    """Round float32 values to the nearest BF16 (ties to even), as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u >> 16) & 1) + 0x7FFF
    out = ((u + r) & 0xFFFF0000).astype(np.uint32)
    return out.view(np.float32).reshape(a.shape)


def layers(params, dims):
    out, o = [], 0
    for din, dout in zip(dims[:-1], dims[1:]):
        w = params[o:o + din * dout].reshape(din, dout)
        o += din * dout
        out.append((w, params[o:o + dout]))
        o += dout
    return out


def forward(params, dims, x, quantize=True):
    """Returns (output float64 [rows, n_out], activations [a_0 .. a_{L-1}])."""
    q = bf16 if quantize else (lambda v: np.asarray(v, np.float64))
    a = q(x).astype(np.float64)
    acts = [a]
    ls = layers(np.asarray(params, np.float32 if quantize else np.float64), dims)
    for l, (w, b) in enumerate(ls):
        h = a @ q(w).astype(np.float64) + np.asarray(b, np.float64)
        if l == len(ls) - 1:
            return h, acts
        a = q(np.maximum(h, 0.0)).astype(np.float64)
        acts.append(a)
    raise AssertionError("unreachable")


def loss(params, dims, x, t, mask=None, quantize=False) -> float:
    y, _ = forward(params, dims, x, quantize)
    m = 1.0 if mask is None else mask
    d = (y - t) * m
    return float((d * d).sum() / d.size)


def backward(params, dims, x, t, mask=None, quantize=True):
    """(loss, gradient vector float64) of the masked mean squared error."""
    q = bf16 if quantize else (lambda v: np.asarray(v, np.float64))
    y, acts = forward(params, dims, x, quantize)
    m = 1.0 if mask is None else mask
    d = (y - t) * m
    n = d.size
    lval = float((d * d).sum() / n)
    g = q(2.0 * d / n).astype(np.float64)
    ls = layers(np.asarray(params, np.float32 if quantize else np.float64), dims)
    grads = []
    for l in range(len(ls) - 1, -1, -1):
        w, _ = ls[l]
        a = acts[l]
        grads.append((a.T @ g, g.sum(0)))
        if l > 0:
            da = g @ q(w).astype(np.float64).T
            da = np.where(a > 0, da, 0.0)
            g = q(da).astype(np.float64)
    grads.reverse()
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return lval, flat


def adam_step(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (bias-corrected); returns (params, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    p = params - lr * (m / c1) / (np.sqrt(v / c2) + eps)
    return p, m, v
