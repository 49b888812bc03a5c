"""Propagator storage modes: streamed densities (store_qstar 0 / 2: a ring
of four q* slices, the density integrals accumulated during the backward
sweep) and contour checkpointing (q_checkpoint K: the BDF3 history at every
K-th slice, segments of q recomputed during the backward sweep).  Every mode
must give the stored-mode results to rounding (the integrals are summed in
the opposite order) and the oracle to 1e-10."""
import numpy as np
import pytest

import oracle
import wlc

pytestmark = pytest.mark.gpu

CASES = [
    dict(n=8, L=3, nmax=14, ns=(4, 4, 6), mode=0, K=0),
    dict(n=8, L=3, nmax=14, ns=(4, 4, 6), mode=2, K=0),
    dict(n=8, L=3, nmax=14, ns=(4, 4, 6), mode=2, K=3),   # K does not divide nmax
    dict(n=8, L=3, nmax=14, ns=(4, 4, 6), mode=0, K=7),   # K divides nmax
    dict(n=12, L=2, nmax=16, ns=(6, 0, 10), mode=2, K=4),  # empty middle block
    dict(n=8, L=4, nmax=12, ns=(4, 4, 4), mode=2, K=12),  # a single segment
]


def _rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def _run(case, mode, K, w, mop=None, nmu=0.0):
    n = case["n"]
    g = wlc.Instance(n, case["L"], case["nmax"], case["ns"], 1.3 / n, 1.2, (0.5, 0.6, 0.7), (15.0, 12.0, 18.0),
                     nmu=nmu, store_qstar=mode, q_checkpoint=K)
    g.set_fields(w, mop)
    g.MDE_q()
    g.MDE_qstar()
    d = g.density(want_s=(mode != 0))
    fe = g.free_energy()
    g.close()
    return d, fe


@pytest.mark.parametrize("case", CASES, ids=lambda c: "n%d_L%d_mode%d_K%d" % (c["n"], c["L"], c["mode"], c["K"]))
def test_storage_mode_matches_stored_and_oracle(case):
    n = case["n"]
    w = np.random.default_rng(31).normal(0.0, 0.5, size=(3, n ** 3))
    ref, fref = _run(case, 1, 0, w)
    d, fe = _run(case, case["mode"], case["K"], w)
    assert abs(d["lnQ"] - ref["lnQ"]) <= 1e-13 * max(1.0, abs(ref["lnQ"]))
    assert _rel(d["phi"], ref["phi"]) < 1e-13
    assert _rel(d["junction"], ref["junction"]) < 1e-13
    assert abs(fe - fref) <= 1e-13 * abs(fref)
    if case["mode"] == 2:
        assert _rel(d["S"], ref["S"]) < 1e-12
    o = oracle.Oracle((n, n, n), case["L"], case["nmax"], case["ns"], (1.3 / n,) * 3, 1.2, (0.5, 0.6, 0.7),
                      (15.0, 12.0, 18.0))
    o.set_fields(w)
    o.propagate(1)
    o.propagate(-1)
    od = o.density(want_s=False)
    assert abs(d["lnQ"] - od["lnQ"]) <= 1e-10 * max(1.0, abs(od["lnQ"]))
    assert _rel(d["phi"], od["phi"]) < 1e-10
    assert abs(fe - o.free_energy(od["lnQ"], od["phi"])) <= 1e-10 * abs(fe)


def test_checkpointing_with_maier_saupe_term():
    """The recomputed segments include the Theta(r) term of the right-hand side."""
    case = dict(n=8, L=4, nmax=12, ns=(4, 4, 4))
    n = 8
    rng = np.random.default_rng(8)
    w = rng.normal(0.0, 0.5, size=(3, n ** 3))
    a = rng.normal(0.0, 0.3, size=(3, 3, n ** 3))
    mop = 0.5 * (a + a.transpose(1, 0, 2))
    tr = (mop[0, 0] + mop[1, 1] + mop[2, 2]) / 3.0
    for k in range(3):
        mop[k, k] -= tr
    ref, fref = _run(case, 1, 0, w, mop, nmu=5.0)
    d, fe = _run(case, 2, 5, w, mop, nmu=5.0)
    assert abs(d["lnQ"] - ref["lnQ"]) <= 1e-13 * max(1.0, abs(ref["lnQ"]))
    assert _rel(d["phi"], ref["phi"]) < 1e-13 and _rel(d["S"], ref["S"]) < 1e-12
    assert abs(fe - fref) <= 1e-13 * abs(fref)


def test_unstored_slices_are_refused():
    n = 8
    g = wlc.Instance(n, 2, 10, (4, 2, 4), 0.15, 1.0, (0.5, 0.5, 0.5), (15.0,) * 3, store_qstar=0, q_checkpoint=4,
                     literals=wlc.WLC_LIT_REAL8)
    g.set_fields(np.zeros((3, n ** 3)))
    with pytest.raises(wlc.WlcError) as e:
        g.MDE_qstar()  # the forward sweep must come first
    assert e.value.code == -4
    g.MDE_q()
    g.MDE_qstar()
    for call in (lambda: g.get_q(-1, 3), lambda: g.get_q(1, 3), lambda: g.init_pr(-1, 3),
                 lambda: g.density(want_s=True)):
        with pytest.raises(wlc.WlcError) as e:
            call()
        assert e.value.code == -4
    d = g.density(want_s=False)
    assert abs(d["lnQ"]) < 1e-12  # w = 0: Q = 1 (double-precision BDF coefficients sum to c0)
