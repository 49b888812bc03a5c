"""wlc_set_precision: switching the propagator precision of a live context
gives the same results as a context created in that precision (FP32: bit
for bit; FP64: the oracle at 1e-10)."""
import numpy as np
import pytest

import oracle
import wlc

pytestmark = pytest.mark.gpu

N, L, NMAX, NS = 12, 3, 12, (4, 4, 4)
DX = 1.2 / N
KAPPA = (0.5, 0.6, 0.7)
CHI = (15.0, 12.0, 18.0)


def _inst(prec):
    return wlc.Instance(N, L, NMAX, NS, DX, 1.3, KAPPA, CHI, precision=prec)


def _run(g, w):
    g.set_fields(w)
    g.MDE_q()
    g.MDE_qstar()
    d = g.density(want_s=True)
    return d, g.free_energy()


def _fields(seed=3):
    return np.random.default_rng(seed).normal(0.0, 0.5, size=(3, N ** 3))


def test_fp64_to_fp32_matches_fp32_context():
    w = _fields()
    a = _inst(wlc.WLC_FP64)
    _run(a, w)
    a.set_precision(wlc.WLC_FP32)
    da, fa = _run(a, w)
    b = _inst(wlc.WLC_FP32)
    db, fb = _run(b, w)
    assert da["lnQ"] == db["lnQ"] and fa == fb
    assert np.array_equal(da["phi"], db["phi"]) and np.array_equal(da["S"], db["S"])


def test_fp32_to_fp64_matches_oracle_after_box_change():
    w = _fields(4)
    g = _inst(wlc.WLC_FP32)
    _run(g, w)
    dx2 = 1.5 / N
    g.init_inverse_sparse_GAB(dx2)  # box change while FP32 is active
    _run(g, w)
    g.set_precision(wlc.WLC_FP64)  # widens the propagator storage, rebuilds FP64 pivots
    d, fe = _run(g, w)
    o = oracle.Oracle((N, N, N), L, NMAX, NS, (dx2,) * 3, 1.3, KAPPA, CHI)
    o.set_fields(w)
    o.propagate(1)
    o.propagate(-1)
    od = o.density(want_s=True)
    ofe = o.free_energy(od["lnQ"], od["phi"])
    assert abs(d["lnQ"] - od["lnQ"]) <= 1e-10 * abs(od["lnQ"])
    assert np.abs(d["phi"] - od["phi"]).max() <= 1e-10 * np.abs(od["phi"]).max()
    assert abs(fe - ofe) <= 1e-10 * abs(ofe)


def test_switch_keeps_fields_and_mixing():
    """A precision switch between field updates keeps the fields and the
    Anderson history: the FP64 iterates after the switch match a context
    that ran FP64 throughout to FP32 accuracy."""
    w = _fields(5)
    mp = wlc.mix_params(anderson_depth=3, num_simple=3)
    a, b = _inst(wlc.WLC_FP64), _inst(wlc.WLC_FP64)
    a.set_fields(w)
    b.set_fields(w)
    for it in range(8):
        if it == 2:
            a.set_precision(wlc.WLC_FP32)
        if it == 5:
            a.set_precision(wlc.WLC_FP64)
        for g in (a, b):
            g.MDE_q()
            g.MDE_qstar()
            g.density(want_junction=False)
            g.iterate(mp)
    wa, wb = a.get_fields(), b.get_fields()
    assert np.abs(wa - wb).max() < 1e-4 * np.abs(wb).max()
    assert not np.array_equal(wa, wb)  # the FP32 iterations did run
