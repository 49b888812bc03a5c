"""Learned warm start network (wlc_net_*): the device forward / backward
kernels (BF16 tensor-core implicit GEMMs, FP32 accumulation) against the
CPU restatement in oracle/warmstart_ref.py with the same rounding points,
and a training run that fits a fixed target."""
import numpy as np
import pytest

import warmstart_ref as ref
import wlc

pytestmark = pytest.mark.gpu

G, C = 8, 16


def _sample(seed):
    rng = np.random.default_rng(seed)
    x = np.concatenate([rng.normal(size=(1, G ** 3)), np.repeat(rng.uniform(-1, 1, size=(5, 1)), G ** 3, axis=1)])
    t = rng.normal(0.0, 0.5, size=(3, G ** 3))
    return x.astype(np.float32), t.astype(np.float32)


def test_gradient_matches_cpu_restatement():
    net = wlc.WarmStartNet(G, C, seed=3)
    p = net.params()
    assert p.size == net.np == sum(27 * ci * co + co for ci, co, *_ in ref.layers(G, C))
    for seed in (1, 2):
        x, t = _sample(seed)
        loss, g = net.loss_grad(x, t)
        rloss, rg = ref.loss_grad(p, x, t, G, C)
        assert abs(loss - rloss) <= 1e-4 * rloss, (loss, rloss)
        off = 0
        for li, (ci, co, *_r) in enumerate(ref.layers(G, C)):
            n = 27 * ci * co + co
            a, b = g[off:off + n], rg[off:off + n]
            err = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-30)
            assert err < 2e-2, "layer %d gradient rel err %.3e" % (li, err)
            off += n


def test_forward_matches_cpu_restatement_and_training_fits():
    net = wlc.WarmStartNet(G, C, seed=5)
    x, t = _sample(4)
    out = net.forward(x)
    # the output of the restatement: loss at target = out gives zero
    l0, _ = ref.loss_grad(net.params(), x, out, G, C)
    assert l0 < 1e-8
    xs = np.stack([_sample(10 + k)[0] for k in range(4)])
    ts = 0.3 * np.tanh(xs[:, :1, :].repeat(3, axis=1))  # a learnable map of the noise channel
    hist = net.train(xs, ts, batch=2, epochs=60, lr=3e-3)
    assert hist[-1] < 0.2 * hist[0], hist
