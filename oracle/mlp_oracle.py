"""FP64 CPU oracle of the MLP surrogate's forward and backward passes.

TEST INFRASTRUCTURE ONLY (imported by tests/).  It restates the network the
library's nz_mlp_* kernels compute -- fully connected layers, GELU (erf form)
on hidden layers, linear output, weighted squared-error loss -- in float64,
rounding to BF16 (round-to-nearest-even) exactly where the kernels round the
operands of their products, so the only remaining difference is FP32 versus
FP64 accumulation.  The network has no counterpart in the reference.
"""
import math

import numpy as np


def bf16(x):
    """Round float32 values to bfloat16 (nearest, ties to even), as float64."""
    a = np.asarray(x, dtype=np.float32).copy()
    u = a.view(np.uint32).astype(np.uint64)
    rounded = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return rounded.astype(np.uint32).view(np.float32).astype(np.float64)


_erf = np.vectorize(math.erf)


def gelu(z):
    return 0.5 * z * (1.0 + _erf(z / math.sqrt(2.0)))


def gelu_grad(z):
    return 0.5 * (1.0 + _erf(z / math.sqrt(2.0))) + z * np.exp(-0.5 * z * z) / math.sqrt(2 * math.pi)


def unpack(params, widths):
    out, o = [], 0
    for i in range(len(widths) - 1):
        k, n = widths[i], widths[i + 1]
        W = np.asarray(params[o:o + k * n], dtype=np.float64).reshape(k, n)
        o += k * n
        b = np.asarray(params[o:o + n], dtype=np.float64)
        o += n
        out.append((W, b))
    return out


def forward(params, widths, x):
    """Returns (y, zs, hs) with zs[l] pre-activations and hs[l] layer outputs."""
    layers = unpack(params, widths)
    h = np.asarray(x, dtype=np.float64)
    zs, hs = [], []
    for i, (W, b) in enumerate(layers):
        z = bf16(h) @ bf16(W) + b
        zs.append(z)
        h = z if i == len(layers) - 1 else gelu(z)
        # the kernels keep activations in float32 between layers
        h = h.astype(np.float32).astype(np.float64)
        hs.append(h)
    return hs[-1], zs, hs


def loss_and_grads(params, widths, x, t, w=None):
    """Weighted squared error sum w (y-t)^2 / B and the flat gradient."""
    y, zs, hs = forward(params, widths, x)
    B = y.shape[0]
    w = np.ones_like(y) if w is None else np.asarray(w, dtype=np.float64)
    loss = float(np.sum(w * (y - t) ** 2) / B)
    dz = (2.0 * w * (y - t) / B).astype(np.float32).astype(np.float64)
    layers = unpack(params, widths)
    grads = [None] * len(layers)
    for i in range(len(layers) - 1, -1, -1):
        W, _ = layers[i]
        a = np.asarray(x, dtype=np.float64) if i == 0 else hs[i - 1]
        gW = bf16(a).T @ bf16(dz)
        gb = dz.sum(axis=0)
        grads[i] = (gW, gb)
        if i == 0:
            break
        da = (bf16(dz) @ bf16(W).T).astype(np.float32).astype(np.float64)
        dz = (da * gelu_grad(zs[i - 1])).astype(np.float32).astype(np.float64)
    flat = np.concatenate([np.concatenate([gW.ravel(), gb]) for gW, gb in grads])
    return loss, flat
