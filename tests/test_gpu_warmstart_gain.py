"""What the learned warm start gains over the method without it, end to end
on the device at a small size: the batched solver generates converged
fields (16^3, L=2, Ns=20, the warm-start parameter ranges), a small network
is trained on them with the library's own kernels, and on held-out draws
its prediction starts the same iteration that a cold start does.  The
training fields are converged to 1e-3 (the morphology has settled; at this
size few draws reach 1e-4 within a few hundred iterations).  The test
asserts that the warm starts end closer to convergence: a lower median
residual after the same number of iterations."""
import numpy as np
import pytest

import wlc
from wlc import warmstart as ws

pytestmark = pytest.mark.gpu

G, L, NMAX = 16, 2, 20


def test_trained_network_beats_cold_start_on_held_out_draws():
    train = ws.draw_params(144, 4242)
    res = []
    for c0 in range(0, len(train), 48):
        part = train[c0:c0 + 48]
        res += ws.solve_batch(part, [ws.cold_start(d, G) for d in part], 500, 1e-3, grid=G, lmax=L, nmax=NMAX)
    kept = [(d, r) for d, r in zip(train, res) if r["iterations"] is not None]
    assert len(kept) >= 12, "too few converged training fields: %d" % len(kept)
    X = np.stack([ws.net_input(d, G) for d, _ in kept]).astype(np.float32)
    T = np.stack([ws.to_target(r["fields"], d["chi"]) for d, r in kept]).astype(np.float32)
    net = wlc.WarmStartNet(G, 16, seed=3)
    hist = net.train(X, T, batch=8, epochs=80, lr=1e-3, seed=5)
    assert hist[-1] < hist[0]
    test = ws.draw_params(48, 777)
    iters = 150
    cold = ws.solve_batch(test, [ws.cold_start(d, G) for d in test], iters, 1e-4, grid=G, lmax=L, nmax=NMAX)
    warm = ws.solve_batch(test, ws.predict(net, test), iters, 1e-4, grid=G, lmax=L, nmax=NMAX)
    net.close()
    rc = np.array([r["residual"] if np.isfinite(r["residual"]) else 1.0 for r in cold])
    rw = np.array([r["residual"] if np.isfinite(r["residual"]) else 1.0 for r in warm])
    nc = sum(r["iterations"] is not None for r in cold)
    nw = sum(r["iterations"] is not None for r in warm)
    print("training fields %d; after %d iterations median residual cold %.2e warm %.2e; converged cold %d warm %d"
          % (len(kept), iters, np.median(rc), np.median(rw), nc, nw))
    assert np.median(rw) < np.median(rc)
