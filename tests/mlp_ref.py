"""Float64 CPU restatement of the learned mode's network (test
infrastructure): 48 -> 128 -> 128 -> 128 -> 8, GELU (tanh form), masked MSE on
outputs 0..5. Operands are rounded to BF16 where the GPU kernels keep BF16
(inputs, weights, hidden activations, output and hidden gradients), so the
comparison isolates the kernels' arithmetic from the storage format."""
from __future__ import annotations

import numpy as np

DIMS = [(48, 128), (128, 128), (128, 128), (128, 8)]
N_PARAMS = sum(i * o + o for i, o in DIMS)


def bf16(x):
    x = np.asarray(x, np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unflatten(flat):
    out, o = [], 0
    for i, n in DIMS:
        W = flat[o:o + i * n].reshape(i, n)
        o += i * n
        b = flat[o:o + n]
        o += n
        out.append((W, b))
    return out


A, B = np.sqrt(2.0 / np.pi), 0.044715


def gelu(z):  # tanh form (Hendrycks and Gimpel)
    return 0.5 * z * (1.0 + np.tanh(A * (z + B * z ** 3)))


def gelu_grad(z):
    th = np.tanh(A * (z + B * z ** 3))
    return 0.5 * (1.0 + th) + 0.5 * z * (1.0 - th * th) * A * (1.0 + 3.0 * B * z * z)


def forward(flat, X):
    layers = unflatten(np.asarray(flat, np.float64))
    h = bf16(X)
    for l, (W, b) in enumerate(layers):
        z = h @ bf16(W) + b
        h = bf16(gelu(z)) if l < 3 else z
    return h


def loss_and_grads(flat, X, T, valid):
    layers = unflatten(np.asarray(flat, np.float64))
    hs, zs = [bf16(X)], []
    for l, (W, b) in enumerate(layers):
        z = hs[-1] @ bf16(W) + b
        zs.append(z)
        if l < 3:
            hs.append(bf16(gelu(z)))
    Y = zs[-1]
    nv = max(1, int(valid.sum()))
    mask = np.zeros_like(Y)
    mask[valid.astype(bool), :6] = 1.0
    d = (Y - T) * mask
    loss = float((d * d).sum() / nv)
    dz = 2.0 * d / nv
    grads = [None] * 4
    for l in range(3, -1, -1):
        W, b = layers[l]
        dzb = bf16(dz)
        grads[l] = (hs[l].T @ dzb, dz.sum(0))
        if l > 0:
            dh = dzb @ bf16(W).T
            dz = dh * gelu_grad(zs[l - 1])
    flat_g = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat_g
