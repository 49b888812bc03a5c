"""Overlapped sweeps: with every slice stored, the backward propagator does
not read the forward one, so wlc_propagate(-1) runs on a second stream
(its own k-space buffer) and overlaps the forward sweep.  The kernels and
their inputs are the same as in the sequential order (which timing mode
keeps), so the results must be bit-identical; a field change between the
two sweeps must reach the backward sweep."""
import numpy as np
import pytest

import wlc

pytestmark = pytest.mark.gpu


def _run(g, w, timing):
    g.enable_timing(timing)
    g.set_fields(w)
    g.MDE_q()
    g.MDE_qstar()
    d = g.density(want_s=True)
    return d, g.get_q(1, g.nmax), g.get_q(-1, 0), g.free_energy()


@pytest.mark.parametrize("precision", [wlc.WLC_FP64, wlc.WLC_FP32])
def test_overlapped_sweeps_bit_identical(precision):
    n, L, nmax, ns = 16, 4, 12, (4, 4, 4)
    g = wlc.Instance(n, L, nmax, ns, 1.2 / n, 1.3, (0.5, 0.6, 0.7), (15.0, 12.0, 18.0), precision=precision)
    w = np.random.default_rng(3).normal(0.0, 0.5, size=(3, n ** 3))
    a = _run(g, w, False)  # overlapped
    b = _run(g, w, True)   # sequential (timing mode)
    c = _run(g, w, False)  # overlapped again, after the sequential run
    for x, y in ((a, b), (a, c)):
        assert x[0]["lnQ"] == y[0]["lnQ"]
        assert np.array_equal(x[0]["phi"], y[0]["phi"]) and np.array_equal(x[0]["S"], y[0]["S"])
        assert np.array_equal(x[1], y[1]) and np.array_equal(x[2], y[2]) and x[3] == y[3]
    g.close()


def test_field_change_between_sweeps_reaches_backward_sweep():
    n, L, nmax, ns = 16, 4, 12, (4, 4, 4)
    args = (n, L, nmax, ns, 1.2 / n, 1.3, (0.5, 0.6, 0.7), (15.0, 12.0, 18.0))
    rng = np.random.default_rng(4)
    w1, w2 = rng.normal(0.0, 0.5, size=(3, n ** 3)), rng.normal(0.0, 0.5, size=(3, n ** 3))
    g = wlc.Instance(*args)
    g.set_fields(w1)
    g.MDE_q()
    g.set_fields(w2)
    g.MDE_qstar()
    qb = g.get_q(-1, 0)
    qf = g.get_q(1, nmax)
    h = wlc.Instance(*args)
    h.enable_timing(True)
    h.set_fields(w2)
    h.MDE_qstar()
    h.set_fields(w1)
    h.MDE_q()
    assert np.array_equal(qb, h.get_q(-1, 0))
    assert np.array_equal(qf, h.get_q(1, nmax))
    g.close()
    h.close()
