"""CPU checks of the field-update restatement (oracle/mixing.py)."""
import numpy as np

import oracle
from oracle_mixing import Mixer, anderson_index


def test_anderson_index_table():
    # the index table written in the comment of Anderson_index
    # (SCFT_iterate.f90:7-13) for n_r = 5
    table = {0: [-6, 0, 6, 12], 1: [-5, 1, 7, 13], 2: [-4, 2, 8, 14], 3: [-3, 3, 9, 15], 4: [-2, 4, 10, 16],
             5: [-1, 5, 11, 17]}
    for want, idx in table.items():
        for i in idx:
            assert anderson_index(i, 5) == want, (i, want)


def _small(chi=(8.0, 8.0, 8.0), ns=(4, 2, 4)):
    n, L = 8, 2
    nmax = sum(ns)
    dx = 2.0 / n
    return oracle.Oracle((n, n, n), L, nmax, ns, (dx, dx, dx), 1.0, (0.5, 0.5, 0.5), chi), ns, nmax


def test_fixed_point_is_kept():
    """At a self-consistent point (dW = 0) neither mixing form moves w
    (symmetric melt: the two residual forms share the homogeneous point)."""
    o, ns, nmax = _small(ns=(4, 4, 4))
    mx = Mixer(o, (8.0, 8.0, 8.0), ns, nmax, depth=3, num_simple=2)
    f = np.array(ns, dtype=float) / nmax
    phi = np.repeat(f[:, None], o.nr, axis=1)
    w = np.full((3, o.nr), 0.25)
    for it in range(8):
        wn, err, _ = mx.step(w, phi)
        assert np.abs(wn - w).max() < 1e-12, it
        assert err[:3].max() < 1e-12
        w = wn


def test_oracle_scft_loop_converges():
    """Simple then Anderson mixing on the oracle drives the block errors
    down by orders of magnitude (three-block melt, weak segregation)."""
    o, ns, nmax = _small()
    mx = Mixer(o, (8.0, 8.0, 8.0), ns, nmax, depth=5, num_simple=20, tol=1e-6)
    n = 8
    x = (np.arange(n ** 3) % n) * (2.0 / n)
    w = np.stack([np.cos(2 * np.pi * x / 2.0), -np.cos(2 * np.pi * x / 2.0), np.zeros(n ** 3)])
    errs = []
    for it in range(120):
        o.set_fields(w)
        o.propagate(1)
        o.propagate(-1)
        d = o.density(want_s=False)
        w, err, conv = mx.step(w, d["phi"])
        errs.append(err[:3].max())
        if conv:
            break
    assert conv, errs[-5:]
    assert errs[-1] < 1e-6 < errs[0]
