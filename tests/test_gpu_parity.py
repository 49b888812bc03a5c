"""GPU parity: libwlc (CUDA sm_103a, called through the C ABI) against the
CPU FP64 oracle on the same seeded inputs.

Tolerance: 1e-10 relative for the FP64 drop-in (the target stated for Q,
block densities and free energy), applied here to every intermediate as
well; FP32 propagators are checked against looser bounds and their error
is reported.
"""
import numpy as np
import pytest

import oracle
import wlc

pytestmark = pytest.mark.gpu

TOL64 = 1e-10

CASES = [
    dict(n=8, L=2, nmax=10, ns=(4, 2, 4), lit=wlc.WLC_LIT_REAL4, kappa=(0.5, 0.7, 0.9), seed=1),
    dict(n=12, L=3, nmax=12, ns=(4, 4, 4), lit=wlc.WLC_LIT_REAL8, kappa=(0.5, 0.5, 0.5), seed=2),
    dict(n=16, L=4, nmax=8, ns=(2, 4, 2), lit=wlc.WLC_LIT_REAL4, kappa=(0.5, 0.5, 0.5), seed=3),
    dict(n=8, L=6, nmax=6, ns=(2, 2, 2), lit=wlc.WLC_LIT_REAL4, kappa=(0.5, 0.5, 0.5), seed=4),
]


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def make(case, precision=wlc.WLC_FP64, dx=None):
    n = case["n"]
    dx = dx if dx is not None else 1.1 / n
    chi = (15.0, 12.0, 18.0)
    loa = 1.3
    g = wlc.Instance(n, case["L"], case["nmax"], case["ns"], dx, loa, case["kappa"], chi,
                     precision=precision, literals=case["lit"])
    o = oracle.Oracle((n, n, n), case["L"], case["nmax"], case["ns"], (dx, dx, dx), loa, case["kappa"], chi,
                      real4=1 if case["lit"] == wlc.WLC_LIT_REAL4 else 0)
    rng = np.random.default_rng(case["seed"])
    w = rng.normal(0.0, 0.5, size=(3, n ** 3))
    g.set_fields(w)
    o.set_fields(w)
    return g, o, w


@pytest.mark.parametrize("case", CASES, ids=lambda c: "n%d_L%d_lit%d" % (c["n"], c["L"], c["lit"]))
def test_one_step_all_g_indices(case):
    g, o, _ = make(case)
    rng = np.random.default_rng(100 + case["seed"])
    table = {1: (1, 1, 0), 2: (2, 1, 0), 3: (3, 1, 0), 4: (3, 1, 1), 5: (3, 1, 2),
             6: (3, -1, 0), 7: (3, -1, 1), 8: (3, -1, 2), 9: (2, -1, 2), 10: (1, -1, 2)}
    for gi, (order, sigma, blk) in table.items():
        pr = rng.standard_normal((g.M, g.nr))
        ref = o.one_step(order, sigma, blk, pr)
        out = g.mde_one_step(gi, pr.T.copy())
        assert rel(out.T, ref) < TOL64, "G_index %d rel err %.3e" % (gi, rel(out.T, ref))


@pytest.mark.parametrize("case", CASES, ids=lambda c: "n%d_L%d_lit%d" % (c["n"], c["L"], c["lit"]))
def test_sweeps_density_free_energy(case):
    g, o, _ = make(case)
    g.MDE_q()
    g.MDE_qstar()
    o.propagate(1)
    o.propagate(-1)
    for s in (1, 2, 3, case["ns"][0] + 1, case["nmax"]):
        assert rel(g.get_q(1, s).T, o.get_q(1, s)) < TOL64, "q(s=%d)" % s
    for s in (case["nmax"] - 1, case["nmax"] - 3, 0):
        assert rel(g.get_q(-1, s).T, o.get_q(-1, s)) < TOL64, "q*(s=%d)" % s
    d = g.density(want_s=True)
    od = o.density(want_s=True)
    assert abs(d["lnQ"] - od["lnQ"]) <= TOL64 * abs(od["lnQ"])
    assert rel(d["phi"], od["phi"]) < TOL64
    assert rel(d["junction"], od["junction"]) < TOL64
    # S: device [blk][b][a][r], oracle [blk][a*3+b][r] (symmetric)
    S = d["S"].reshape(3, 9, -1)
    assert rel(S, od["S"]) < TOL64
    fe = g.free_energy()
    ofe = o.free_energy(od["lnQ"], od["phi"])
    assert abs(fe - ofe) <= TOL64 * abs(ofe)


@pytest.mark.parametrize("case", CASES[:2], ids=lambda c: "n%d_L%d" % (c["n"], c["L"]))
def test_init_pr(case):
    g, o, _ = make(case)
    g.MDE_q()
    g.MDE_qstar()
    o.propagate(1)
    o.propagate(-1)
    for d, s in ((1, 1), (1, 2), (1, 5), (-1, case["nmax"] - 1), (-1, case["nmax"] - 2), (-1, 0)):
        assert rel(g.init_pr(d, s).T, o.init_pr(d, s)) < TOL64


def test_fp32_error_against_fp64_oracle():
    case = CASES[2]
    g, o, _ = make(case, precision=wlc.WLC_FP32)
    g.MDE_q()
    g.MDE_qstar()
    o.propagate(1)
    o.propagate(-1)
    d = g.density()
    od = o.density(want_s=False)
    fe = g.free_energy()
    ofe = o.free_energy(od["lnQ"], od["phi"])
    eq = abs(d["lnQ"] - od["lnQ"])  # = relative error of Q
    ep = rel(d["phi"], od["phi"])
    ef = abs(fe - ofe) / abs(ofe)
    print("fp32 vs fp64 oracle: lnQ %.2e phi %.2e F %.2e" % (eq, ep, ef))
    assert eq < 1e-4 and ep < 1e-4 and ef < 1e-4


def test_box_change_rebuilds_operator():
    case = CASES[0]
    g, o, w = make(case)
    dx2 = 1.4 / case["n"]
    g.init_inverse_sparse_GAB(dx2)
    o.set_box((dx2, dx2, dx2))
    g.set_fields(w)
    o.set_fields(w)
    rng = np.random.default_rng(5)
    pr = rng.standard_normal((g.M, g.nr))
    assert rel(g.mde_one_step(3, pr.T.copy()).T, o.one_step(3, 1, 0, pr)) < TOL64


def _symmetric_traceless_mop(rng, nr, amp=0.3):
    a = rng.normal(0.0, amp, size=(3, 3, nr))
    m = 0.5 * (a + a.transpose(1, 0, 2))
    tr = (m[0, 0] + m[1, 1] + m[2, 2]) / 3.0
    for k in range(3):
        m[k, k] -= tr
    return m


@pytest.mark.parametrize("lit", [wlc.WLC_LIT_REAL4, wlc.WLC_LIT_REAL8])
def test_maier_saupe_sweeps(lit):
    """Theta(r) coupling (calc_THETAij + the Theta term of init_pr) with a
    seeded symmetric traceless M_OP, NMu != 0."""
    n, L, nmax, ns = 8, 4, 8, (2, 4, 2)
    dx = 1.0 / n
    nmu = 5.0
    g = wlc.Instance(n, L, nmax, ns, dx, 1.1, (0.5, 0.5, 0.5), (15.0, 15.0, 15.0), nmu=nmu, literals=lit)
    o = oracle.Oracle((n, n, n), L, nmax, ns, (dx, dx, dx), 1.1, (0.5, 0.5, 0.5), (15.0, 15.0, 15.0), nmu=nmu,
                      real4=1 if lit == wlc.WLC_LIT_REAL4 else 0)
    rng = np.random.default_rng(21)
    w = rng.normal(0.0, 0.5, size=(3, n ** 3))
    mop = _symmetric_traceless_mop(rng, n ** 3)
    g.set_fields(w, mop)
    o.set_fields(w, mop.reshape(9, -1))
    g.MDE_q()
    g.MDE_qstar()
    o.propagate(1)
    o.propagate(-1)
    for s in (1, 2, 5, nmax):
        assert rel(g.get_q(1, s).T, o.get_q(1, s)) < TOL64
    assert rel(g.init_pr(-1, 3).T, o.init_pr(-1, 3)) < TOL64
    d = g.density(want_s=True)
    od = o.density(want_s=True)
    assert abs(d["lnQ"] - od["lnQ"]) <= TOL64 * max(1.0, abs(od["lnQ"]))
    assert rel(d["phi"], od["phi"]) < TOL64
    assert rel(d["S"].reshape(3, 9, -1), od["S"]) < TOL64
    fe = g.free_energy()
    ofe = o.free_energy(od["lnQ"], od["phi"])
    assert abs(fe - ofe) <= TOL64 * abs(ofe)
