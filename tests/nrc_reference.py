"""NumPy reference of the radiance-cache MLP (test infrastructure).

Mirrors the kernels' arithmetic contract: fp16 weights and activations,
fp32 accumulation, ReLU hidden layers, no biases, relative L2 loss
(p - y)^2 / (sg(p)^2 + 0.01) averaged over samples and the 3 channels, and
the loss scale applied to the fp16 output gradients.
"""
import math

import numpy as np

LAYER_SHAPES = [(64, 64)] * 4 + [(64, 16)]
SH_C = [0.28209479, 0.48860251, 1.09254843, 0.31539157, 0.54627422, 0.59004359, 2.89061144, 0.45704580,
        0.37317633, 1.44530572]


def layers(w):
    out, off = [], 0
    for i, o in LAYER_SHAPES:
        out.append(np.asarray(w[off:off + i * o]).reshape(i, o))
        off += 64 * 64
    return out


def encode(q, box_min, box_max):
    """q: (n, 12) -> (n, 64) float32 (before the fp16 rounding)."""
    q = np.asarray(q, np.float64)
    n = q.shape[0]
    p = (q[:, 0:3] - box_min) / (np.asarray(box_max) - np.asarray(box_min))
    cols = []
    for d in range(3):
        f = math.pi * p[:, d]
        for o in range(6):
            cols += [np.sin(f), np.cos(f)]
            f = f * 2
    x, y, z = q[:, 3], q[:, 4], q[:, 5]
    xx, yy, zz = x * x, y * y, z * z
    c = SH_C
    cols += [np.full(n, c[0]), -c[1] * y, c[1] * z, -c[1] * x, c[2] * x * y, -c[2] * y * z, c[3] * (3 * zz - 1),
             -c[2] * x * z, c[4] * (xx - yy), c[5] * y * (-3 * xx + yy), c[6] * x * y * z, c[7] * y * (1 - 5 * zz),
             c[8] * z * (5 * zz - 3), c[7] * x * (1 - 5 * zz), c[9] * z * (xx - yy), c[5] * x * (-xx + 3 * yy)]
    for k in range(6, 12):
        cols.append(q[:, k])
    cols.append(np.ones(n))
    while len(cols) < 64:
        cols.append(np.zeros(n))
    return np.stack(cols, 1).astype(np.float32)


def forward(x0_half, w, fp16=True):
    """x0_half: (n, 64) encoded inputs. Returns (layer inputs, raw output (n, 16))."""
    W = [l.astype(np.float16).astype(np.float32) if fp16 else l.astype(np.float64) for l in layers(w)]
    h = x0_half.astype(np.float32 if fp16 else np.float64)
    acts = [h]
    for l in range(4):
        h = np.maximum(h @ W[l], 0)
        if fp16:
            h = h.astype(np.float16).astype(np.float32)
        acts.append(h)
    return acts, h @ W[4]


def loss_and_grad(x0_half, w, target, loss_scale=128.0, fp16=True):
    """Mean relative L2 loss and d loss / d weights (flat, like the master array)."""
    n = x0_half.shape[0]
    W = [l.astype(np.float16).astype(np.float32) if fp16 else l.astype(np.float64) for l in layers(w)]
    acts, out = forward(x0_half, w, fp16)
    p = out[:, :3]
    den = p * p + 0.01
    loss = float(((p - target) ** 2 / den).mean())
    dy = np.zeros_like(out)
    dy[:, :3] = 2 * (p - target) / den / (3 * n) * (loss_scale if fp16 else 1.0)
    if fp16:
        dy = dy.astype(np.float16).astype(np.float32)
    grads = [None] * 5
    for l in range(4, -1, -1):
        grads[l] = acts[l].T @ dy
        if l == 0:
            break
        dx = dy @ W[l].T
        dy = dx * (acts[l] > 0)
        if fp16:
            dy = dy.astype(np.float16).astype(np.float32)
    flat = np.zeros(17408, np.float64)
    off = 0
    for l, (i, o) in enumerate(LAYER_SHAPES):
        flat[off:off + i * o] = grads[l].reshape(-1) / (loss_scale if fp16 else 1.0)
        off += 64 * 64
    return loss, p, flat
