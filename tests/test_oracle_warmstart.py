"""The CPU restatement of the warm-start network checked by central finite
differences in exact float64 arithmetic (no BF16 rounding)."""
import numpy as np

import warmstart_ref as ref


def test_restatement_gradient_by_finite_differences():
    G, C = 8, 16
    n = sum(27 * ci * co + co for ci, co, *_ in ref.layers(G, C))
    rng = np.random.default_rng(0)
    p = rng.normal(0.0, 0.08, size=n)
    x = rng.normal(size=(6, G ** 3))
    t = rng.normal(size=(3, G ** 3))
    old = ref.ROUND
    ref.ROUND = False
    try:
        _, g = ref.loss_grad(p, x, t, G, C)
        offs, off = [], 0
        for ci, co, *_ in ref.layers(G, C):
            offs.append((off, 27 * ci * co + co))
            off += 27 * ci * co + co
        for li in (0, 3, 6, 9):  # first, stride-2, decoder and output layers
            o, m = offs[li]
            for idx in (o + 5, o + m // 2, o + m - 1):  # weights and the last bias
                h = 1e-5
                pp, pm = p.copy(), p.copy()
                pp[idx] += h
                pm[idx] -= h
                fd = (ref.loss_grad(pp, x, t, G, C)[0] - ref.loss_grad(pm, x, t, G, C)[0]) / (2 * h)
                assert abs(fd - g[idx]) <= 1e-6 + 1e-5 * abs(fd), (li, idx, fd, g[idx])
    finally:
        ref.ROUND = old
