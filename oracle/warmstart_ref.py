"""CPU restatement of the warm-start network (libwlc wlc_net_*) -- TEST
INFRASTRUCTURE ONLY (the oracle of the GPU forward / backward kernels;
imported by tests/ alone).  The network has no counterpart in the
reference.

Same architecture, parameter layout and rounding points as the device
code: BF16 weights, BF16 input and post-ReLU activations, BF16 output
gradients of each layer (dz), FP32 (here FP64) accumulation, FP32 output
layer.  Convolutions are 3x3x3, periodic, stride 1 or 2, channel-last
[point][channel], point = x + g (y + g z), neighbour kk = (dx, dy, dz) =
(kk % 3 - 1, (kk / 3) % 3 - 1, kk / 9 - 1).
"""
import numpy as np


ROUND = True  # False: exact float64 arithmetic (used to check the restatement by finite differences)


def bf16(a):
    """Round float32 values to bfloat16 (nearest, ties to even), as float32;
    the identity in float64 when ROUND is False."""
    if not ROUND:
        return np.asarray(a, dtype=np.float64)
    a = np.ascontiguousarray(a, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def neighbours(gi, go, stride):
    """nb[m, kk]: input point of output point m for neighbour kk."""
    m = np.arange(go ** 3)
    x, y, z = m % go, (m // go) % go, m // (go * go)
    kk = np.arange(27)
    dx, dy, dz = kk % 3 - 1, (kk // 3) % 3 - 1, kk // 9 - 1
    xi = (stride * x[:, None] + dx[None, :]) % gi
    yi = (stride * y[:, None] + dy[None, :]) % gi
    zi = (stride * z[:, None] + dz[None, :]) % gi
    return xi + gi * (yi + gi * zi)


def layers(G, C):
    """(ci, co, stride, gin, relu) of e1..e6, d1..d3, out."""
    return [(16, C, 1, G, 1), (C, 2 * C, 2, G, 1), (2 * C, 2 * C, 1, G // 2, 1), (2 * C, 4 * C, 2, G // 2, 1),
            (4 * C, 4 * C, 1, G // 4, 1), (4 * C, 4 * C, 2, G // 4, 1), (8 * C, 4 * C, 1, G // 4, 1),
            (6 * C, 2 * C, 1, G // 2, 1), (3 * C, C, 1, G, 1), (C, 16, 1, G, 0)]


def unpack(params, G, C):
    out, off = [], 0
    for ci, co, s, gi, relu in layers(G, C):
        w = params[off:off + 27 * ci * co].reshape(27, ci, co)
        off += 27 * ci * co
        b = params[off:off + co]
        off += co
        out.append((w, b, ci, co, s, gi, relu))
    return out


def up(x, gc):
    """nearest x2 upsampling, channel-last"""
    gf = 2 * gc
    p = np.arange(gf ** 3)
    X, Y, Z = p % gf, (p // gf) % gf, p // (gf * gf)
    return x[(X // 2) + gc * ((Y // 2) + gc * (Z // 2))], (X // 2) + gc * ((Y // 2) + gc * (Z // 2))


def _f32(a):
    return np.asarray(a, dtype=np.float32) if ROUND else np.asarray(a, dtype=np.float64)


def loss_grad(params, x_in, target, G, C):
    """Loss and gradient (FP32 vector in the device's parameter layout) of
    one sample: x_in (6, G^3), target (3, G^3)."""
    P = G ** 3
    L = unpack(_f32(params), G, C)
    x0 = np.zeros((P, 16))
    x0[:, :6] = _f32(x_in).T
    x0 = bf16(x0)
    cache = []

    def conv(li, x):
        w, b, ci, co, s, gi, relu = L[li]
        go = gi // s
        nb = neighbours(gi, go, s)
        wb = bf16(w).astype(np.float64)
        y = np.einsum("mkc,kcd->md", x.astype(np.float64)[nb], wb) + b.astype(np.float64)
        if li == 9:
            out = _f32(y)
        else:
            out = bf16(_f32(np.maximum(y, 0.0))) if relu else bf16(_f32(y))
        cache.append((li, x, out, nb))
        return out

    e = [None] * 7
    e[1] = conv(0, x0)
    for k in range(2, 7):
        e[k] = conv(k - 1, e[k - 1])
    u, _ = up(e[6], G // 8)
    d1 = conv(6, np.concatenate([u, e[5]], axis=1))
    u, _ = up(d1, G // 4)
    d2 = conv(7, np.concatenate([u, e[3]], axis=1))
    u, _ = up(d2, G // 2)
    d3 = conv(8, np.concatenate([u, e[1]], axis=1))
    out = conv(9, d3)
    diff = out[:, :3].astype(np.float64) - np.asarray(target, dtype=np.float64).T
    loss = float((diff ** 2).sum() / (3 * P))
    gout = np.zeros((P, 16))
    gout[:, :3] = _f32(2.0 / (3 * P)) * _f32(diff)
    grads = [None] * 10
    byli = {c[0]: c for c in cache}

    def back(li, dy):
        w, b, ci, co, s, gi, relu = L[li]
        _, x, y, nb = byli[li]
        dz = dy * (y > 0) if relu else dy
        dz = bf16(_f32(dz)).astype(np.float64)
        dw = np.einsum("mkc,md->kcd", x.astype(np.float64)[nb], dz)
        db = dz.sum(axis=0)
        grads[li] = (dw, db)
        dx = np.zeros((gi ** 3, ci))
        contrib = np.einsum("md,kcd->mkc", dz, bf16(w).astype(np.float64))
        np.add.at(dx, nb.reshape(-1), contrib.reshape(-1, ci))
        return dx

    def up_back(dcat, gc, c):
        _, idx = up(np.zeros((gc ** 3, 1)), gc)
        g = np.zeros((gc ** 3, c))
        np.add.at(g, idx, dcat)
        return g

    dd3 = back(9, gout)
    dc3 = back(8, dd3)
    dd2 = up_back(dc3[:, :2 * C], G // 2, 2 * C)
    de1 = dc3[:, 2 * C:].copy()
    dc2 = back(7, dd2)
    dd1 = up_back(dc2[:, :4 * C], G // 4, 4 * C)
    de3 = dc2[:, 4 * C:].copy()
    dc1 = back(6, dd1)
    de6 = up_back(dc1[:, :4 * C], G // 8, 4 * C)
    de5 = dc1[:, 4 * C:].copy()
    de5 += back(5, de6)
    de4 = back(4, de5)
    de3 += back(3, de4)
    de2 = back(2, de3)
    de1 += back(1, de2)
    back(0, de1)
    flat = _f32(np.concatenate([np.concatenate([g[0].reshape(-1), g[1]]) for g in grads]))
    return loss, flat
