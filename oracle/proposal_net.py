"""CPU oracle of the learned proposal network (test infrastructure only).

The reference has no network: its candidates beyond the neighbours'
continuations are uniform random draws (lib/synthesize.h:583-603).  The GPU
engine adds a small convolutional network that proposes candidate sources;
this module restates that network's forward pass, loss and gradients in
numpy float64 so the CUDA kernels can be checked against it.  Only tests,
the smoke check and the bench's CPU leg use it.

Network (all convolutions 3x3, stride 1, no padding, 32 output channels):
  input   11 x 11 x 16   context around the target pixel (channel layout in
                         ``CONTEXT_CHANNELS``), bf16
  layer 1 11 -> 9,  ReLU   K = 9 * 16
  layer 2  9 -> 7,  ReLU   K = 9 * 32
  layer 3  7 -> 5,  ReLU   K = 9 * 32
  layer 4  5 -> 3,  ReLU   K = 9 * 32
  head     3 -> 1,  linear K = 9 * 32 -> 32 = 16 offsets x (dx, dy)
The kernels compute in bf16 with fp32 accumulation: weights, activations and
the back-propagated activation gradients are rounded to bf16 at the same
points here (``rounding=True``), everything else is float64.

Loss: relaxed multiple-choice loss over the K = 16 offsets, label y = (source -
target) / LABEL_SCALE clipped to +-LABEL_CLIP: the nearest offset k* gets weight
1 - EPS, every other EPS / (K - 1); loss = mean over samples of
sum_k w_k |o_k - y|^2.
"""
from __future__ import annotations

import numpy as np

CTX = 11
CIN0 = 16
COUT = 32
K_OFFSETS = 16
EPS = 0.05
LABEL_SCALE = 64.0
LABEL_CLIP = 16.0
LAYERS = [(16, 11), (32, 9), (32, 7), (32, 5), (32, 3)]   # (input channels, input width)
CONTEXT_CHANNELS = ("colour 0", "colour 1", "colour 2", "has value", "map 0")


def bf16(x, rounding=True):
    """Round to the nearest even bfloat16 (as float64); identity if not rounding."""
    if not rounding:
        return np.asarray(x, np.float64)
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def param_count():
    return sum(COUT * 9 * cin + COUT for cin, _ in LAYERS)


def unflatten(theta):
    """Flat parameter vector -> [(W [32 x 9 cin], b [32]), ...] (views)."""
    out, o = [], 0
    for cin, _ in LAYERS:
        k = 9 * cin
        W = theta[o:o + COUT * k].reshape(COUT, k)
        o += COUT * k
        b = theta[o:o + COUT]
        o += COUT
        out.append((W, b))
    return out


def init_params(seed):
    """He-normal weights, zero biases (the library draws its own; this is for tests)."""
    rng = np.random.default_rng(seed)
    theta = np.zeros(param_count(), np.float64)
    for (W, b), (cin, _) in zip(unflatten(theta), LAYERS):
        W[...] = rng.standard_normal(W.shape) * np.sqrt(2.0 / (9 * cin))
    return theta.astype(np.float32)


def im2col(a):
    """a [n, w, w, c] -> [n * (w-2)^2, 9 c], column (ky * 3 + kx) * c + ci."""
    n, w, _, c = a.shape
    wo = w - 2
    cols = np.empty((n, wo, wo, 9, c), a.dtype)
    for ky in range(3):
        for kx in range(3):
            cols[:, :, :, ky * 3 + kx, :] = a[:, ky:ky + wo, kx:kx + wo, :]
    return cols.reshape(n * wo * wo, 9 * c)


def col2im(d, n, w, c):
    """Adjoint of im2col: [n * (w-2)^2, 9 c] -> [n, w, w, c]."""
    wo = w - 2
    d = d.reshape(n, wo, wo, 9, c)
    out = np.zeros((n, w, w, c), np.float64)
    for ky in range(3):
        for kx in range(3):
            out[:, ky:ky + wo, kx:kx + wo, :] += d[:, :, :, ky * 3 + kx, :]
    return out


def forward(theta, x0, rounding=True):
    """x0 [n, 11, 11, 16] -> (out [n, 32] float64, cache)."""
    layers = [(bf16(W, rounding), np.asarray(b, np.float64)) for W, b in unflatten(np.asarray(theta, np.float64))]
    a = bf16(x0, rounding)
    n = a.shape[0]
    cols, acts = [], [a]
    for i, ((W, b), (cin, w)) in enumerate(zip(layers, LAYERS)):
        col = im2col(a)
        z = col @ W.T + b
        cols.append(col)
        if i < len(LAYERS) - 1:
            a = bf16(np.maximum(z, 0.0), rounding).reshape(n, w - 2, w - 2, COUT)
            acts.append(a)
        else:
            out = z.reshape(n, COUT)
    return out, (layers, cols, acts)


def mcl_loss(out, labels):
    """Relaxed multiple-choice loss and its gradient w.r.t. out (float64)."""
    n = out.shape[0]
    o = out.reshape(n, K_OFFSETS, 2)
    y = np.clip(np.asarray(labels, np.float64), -LABEL_CLIP, LABEL_CLIP)[:, None, :]
    d = ((o - y) ** 2).sum(-1)
    win = np.argmin(d, axis=1)
    w = np.full((n, K_OFFSETS), EPS / (K_OFFSETS - 1))
    w[np.arange(n), win] = 1.0 - EPS
    loss = float((w * d).sum() / n)
    grad = (2.0 / n) * w[:, :, None] * (o - y)
    return loss, grad.reshape(n, COUT)


def loss_and_grad(theta, x0, labels, rounding=True):
    """(loss, flat gradient float64) of the mean relaxed MCL loss."""
    out, (layers, cols, acts) = forward(theta, x0, rounding)
    loss, dy = mcl_loss(out, labels)
    n = out.shape[0]
    grads = [None] * len(LAYERS)
    for i in range(len(LAYERS) - 1, -1, -1):
        W, _ = layers[i]
        cin, w = LAYERS[i]
        g = bf16(dy, rounding)
        grads[i] = (g.T @ cols[i], dy.sum(0))
        if i == 0:
            break
        dcol = g @ W
        dx = col2im(dcol, n, w, cin)
        dy = (dx * (acts[i] > 0)).reshape(-1, cin)
    flat = np.concatenate([np.concatenate([gw.ravel(), gb]) for gw, gb in grads])
    return loss, flat


def decode(out, tx, ty):
    """Proposed source points of targets at (tx, ty): [n, 16, 2] int (x, y)."""
    o = np.asarray(out, np.float64).reshape(-1, K_OFFSETS, 2) * LABEL_SCALE
    return np.stack([np.asarray(tx)[:, None] + np.rint(o[..., 0]),
                     np.asarray(ty)[:, None] + np.rint(o[..., 1])], -1).astype(np.int64)


def bf16_bits(x):
    """float -> bfloat16 bits (uint16), round to nearest even."""
    f = np.ascontiguousarray(x, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) & 0xFFFF).astype(np.uint16)


def bits_to_float(b):
    return (np.asarray(b, np.uint32) << 16).view(np.float32)


def context(colors, valued, mapc, x, y):
    """The 11 x 11 x 16 context (bf16 bits) of the target at (x, y).

    colors [H, W, C] uint8 (C = 1..3 matched colour channels), valued [H, W]
    bool, mapc [H, W] uint8 first map channel or None."""
    h, w, nc = colors.shape
    out = np.zeros((CTX, CTX, CIN0), np.float32)
    for dy in range(-5, 6):
        for dx in range(-5, 6):
            qx, qy = x + dx, y + dy
            if not (0 <= qx < w and 0 <= qy < h):
                continue
            o = out[dy + 5, dx + 5]
            if valued[qy, qx]:
                for j in range(3):
                    o[j] = np.float32(colors[qy, qx, min(j, nc - 1)]) / np.float32(255) - np.float32(0.5)
                o[3] = 1.0
            if mapc is not None:
                o[4] = np.float32(mapc[qy, qx]) / np.float32(255) - np.float32(0.5)
    return bf16_bits(out)
