"""CPU restatement of the warm-start network (test infrastructure only: the checker of the GPU
kernels, never part of the product path).

Forward and backward of the 12 -> 128 -> 128 -> 128 -> 3 GELU network in float64, rounding to
bfloat16 exactly where the GPU kernels keep bfloat16 values (normalised inputs, weights,
activations, output gradients and pre-activation gradients), so the only remaining differences
are float32-vs-float64 accumulation and the float32 erf/exp of the GPU epilogues.  The loss is
the mean squared error over the 3 outputs in normalised target units; the parameter and
normalisation layouts are those of include/b3g_capi.h (B3G_MLP_PARAMS, B3G_MLP_NORM).
"""
from __future__ import annotations

import math

import numpy as np

F, H, O = 12, 128, 3
N_PARAMS = F * H + H + 2 * (H * H + H) + H * O + O
N_NORM = 2 * F + 2 * O

_erf = np.vectorize(math.erf, otypes=[np.float64])


def bf16(x):
    """Round to the nearest bfloat16 (ties to even), returned as float64."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(p):
    p = np.asarray(p, np.float64)
    k = 0
    out = []
    for shape in ((F, H), (H,), (H, H), (H,), (H, H), (H,), (H, O), (O,)):
        n = int(np.prod(shape))
        out.append(p[k:k + n].reshape(shape))
        k += n
    assert k == N_PARAMS
    return out


def pack(parts):
    return np.concatenate([np.asarray(a, np.float64).ravel() for a in parts]).astype(np.float32)


def gelu(x):
    return 0.5 * x * (1.0 + _erf(x / math.sqrt(2.0)))


def gelu_grad(x):
    return 0.5 * (1.0 + _erf(x / math.sqrt(2.0))) + x * np.exp(-0.5 * x * x) / math.sqrt(2.0 * math.pi)


def init_params(seed=0):
    rng = np.random.Generator(np.random.PCG64(seed))
    parts = [rng.standard_normal((F, H)) * math.sqrt(2 / F), np.zeros(H),
             rng.standard_normal((H, H)) * math.sqrt(2 / H), np.zeros(H),
             rng.standard_normal((H, H)) * math.sqrt(2 / H), np.zeros(H),
             rng.standard_normal((H, O)) * math.sqrt(2 / H), np.zeros(O)]
    return pack(parts)


def identity_norm():
    n = np.zeros(N_NORM, np.float32)
    n[F:2 * F] = 1.0
    n[2 * F + O:] = 1.0
    return n


def forward(params, norm, x):
    """Returns (predictions in impulse units, cache for backward)."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(params)
    norm = np.asarray(norm, np.float64)
    xn = bf16((np.asarray(x, np.float64) - norm[:F]) * norm[F:2 * F])
    pres, hs = [], [xn]
    h = xn
    for W, b in ((W1, b1), (W2, b2), (W3, b3)):
        pre = h @ bf16(W) + b
        pres.append(pre)
        h = bf16(gelu(pre))
        hs.append(h)
    y = h @ bf16(W4) + b4
    tm, ts = norm[2 * F:2 * F + O], norm[2 * F + O:]
    return y / ts + tm, (pres, hs, y)


def gradients(params, norm, x, t):
    """Gradients (public layout, float64) and loss of the batch mean squared error."""
    W1, b1, W2, b2, W3, b3, W4, b4 = unpack(params)
    norm = np.asarray(norm, np.float64)
    _, (pres, hs, y) = forward(params, norm, x)
    n = len(x)
    tm, ts = norm[2 * F:2 * F + O], norm[2 * F + O:]
    e = y - (np.asarray(t, np.float64) - tm) * ts
    loss = float((e * e).sum() / (3 * n))
    dp = bf16(2.0 * e / (3.0 * n))          # dY as the GPU keeps it
    g = [None] * 8
    g[7] = dp.sum(0)
    g[6] = hs[3].T @ dp
    Ws = [W1, W2, W3, W4]
    for l in (2, 1, 0):
        dh = dp @ bf16(Ws[l + 1]).T
        dp = bf16(dh * gelu_grad(pres[l]))
        g[2 * l + 1] = dp.sum(0)
        g[2 * l] = hs[l].T @ dp
    return np.concatenate([a.ravel() for a in g]), loss
