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


def lmv_output_loss(y, t, mask, x, beta):
    """Learned-MV output loss and its gradient with respect to y (float64).

    y, t, mask: [rows, 128] (64 complex weights interleaved); x: [rows, 256]
    features whose entries 128..255 are the normalised averaged snapshot a.
    Per row: o = sum conj(w) a / conj(sum w) over the masked weights, o_ref the
    same with t, loss = |o - o_ref|^2 + |sum w / L - 1|^2 + beta * sum mask
    |w - t|^2, averaged over rows (L = the number of masked weights)."""
    y = np.asarray(y, np.float64)
    t = np.asarray(t, np.float64)
    m = np.asarray(mask, np.float64)[:, 0::2]
    a = np.asarray(x, np.float64)[:, 128::2] + 1j * np.asarray(x, np.float64)[:, 129::2]
    w = y[:, 0::2] + 1j * y[:, 1::2]
    tw = t[:, 0::2] + 1j * t[:, 1::2]
    rows = y.shape[0]
    D = np.conj((m * w).sum(1))
    small = np.abs(D) ** 2 < 1e-6
    D = np.where(small, 1e-3, D)
    o = (m * np.conj(w) * a).sum(1) / D
    o_ref = (m * np.conj(tw) * a).sum(1) / np.conj((m * tw).sum(1))
    e = o - o_ref
    Lr = np.maximum(m.sum(1), 1.0)
    sd = (m * w).sum(1) / Lr - 1.0
    loss = float((np.abs(e) ** 2 + np.abs(sd) ** 2 + beta * (m * np.abs(w - tw) ** 2).sum(1)).sum() / rows)
    g = ((2 * np.conj(e) / D)[:, None] * (a - o[:, None]) + (2 * sd / Lr)[:, None]) * m + 2 * beta * m * (w - tw)
    g /= rows
    out = np.empty_like(y)
    out[:, 0::2] = g.real
    out[:, 1::2] = g.imag
    return loss, out


def _beam_basis(L):
    """Columns u_b[i] = e^{j 2 pi b i / L} / sqrt(L), b = 0, 1, -1, 2, -2 (first min(5, L))."""
    i = np.arange(L)
    bs = [0, 1, -1, 2, -2][:min(5, L)]
    return np.stack([np.exp(2j * np.pi * b * i / L) / np.sqrt(L) for b in bs], 1)


def lmv_subspace_loss(y, t, mask, beta):
    """Learned-subspace loss and its gradient with respect to y (float64).

    Per row, with L the masked count, w / tt the predicted / target complex
    weights i < L and P the projector onto the complement of the first
    min(5, L) DFT beams: u = P w, v = P tt,
    loss = 1 - |u^H v|^2 / (|u|^2 |v|^2) (0 where |v|^2 <= 1e-8 |tt|^2)
           + beta * sum |w - tt|^2 / L, averaged over rows."""
    y = np.asarray(y, np.float64)
    t = np.asarray(t, np.float64)
    m = np.asarray(mask, np.float64)[:, 0::2]
    rows = y.shape[0]
    total = 0.0
    out = np.zeros_like(y)
    for r in range(rows):
        L = int(round(m[r].sum()))
        if L == 0:
            continue
        w = y[r, 0:2 * L:2] + 1j * y[r, 1:2 * L:2]
        tt = t[r, 0:2 * L:2] + 1j * t[r, 1:2 * L:2]
        U = _beam_basis(L)
        P = np.eye(L) - U @ U.conj().T
        u, v = P @ w, P @ tt
        a, b = np.vdot(u, u).real, np.vdot(v, v).real
        c = np.vdot(u, v)
        g = np.zeros(L, complex)
        lr = beta * np.sum(np.abs(w - tt) ** 2) / L
        if b > 1e-8 * np.vdot(tt, tt).real and a > 1e-30:
            lr += 1.0 - abs(c) ** 2 / (a * b)
            g = P @ (-2.0 * (v * np.conj(c) / (a * b) - abs(c) ** 2 * u / (a * a * b)))
        g = g + 2.0 * beta * (w - tt) / L
        total += lr
        out[r, 0:2 * L:2] = g.real / rows
        out[r, 1:2 * L:2] = g.imag / rows
    return total / rows, out


def backward_from(params, dims, x, g_out, quantize=True):
    """Gradient vector for a given output gradient g_out = dLoss/dy."""
    q = bf16 if quantize else (lambda v: np.asarray(v, np.float64))
    _, acts = forward(params, dims, x, quantize)
    g = q(g_out).astype(np.float64)
    ls = layers(np.asarray(params, np.float32 if quantize else np.float64), dims)
    grads = []
    for l in range(len(ls) - 1, -1, -1):
        w, _ = ls[l]
        a = acts[l]
        grads.append((a.T @ g, g.sum(0)))
        if l > 0:
            da = g @ q(w).astype(np.float64).T
            g = q(np.where(a > 0, da, 0.0)).astype(np.float64)
    grads.reverse()
    return np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])


def adam_step(params, grad, m, v, step, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam update (bias-corrected); returns (params, m, v)."""
    m = b1 * m + (1 - b1) * grad
    v = b2 * v + (1 - b2) * grad * grad
    c1, c2 = 1 - b1 ** step, 1 - b2 ** step
    p = params - lr * (m / c1) / (np.sqrt(v / c2) + eps)
    return p, m, v
