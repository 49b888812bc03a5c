"""GPU parity of the operator-split contour step (WLC_SCHEME_SPLIT):
libwlc through the C ABI against the CPU oracle's split scheme on the same
seeded inputs.

The scheme has no counterpart in the reference's harmonic-basis solver
(its field half steps follow split_operator_MDE_mod.f90:163-166), so its
parity with the reference is unpinned; the oracle's split step is pinned
by tests/test_oracle_split.py (numpy restatement, exact homogeneous
answer, second order in ds).

Tolerance: 1e-10 relative (FP64); storage modes bit-for-bit equivalent to
1e-13; FP32 against the FP64 oracle 1e-4 with the error printed.
"""
import numpy as np
import pytest

import oracle
import wlc

pytestmark = pytest.mark.gpu

TOL64 = 1e-10
R4, R8 = wlc.WLC_LIT_REAL4, wlc.WLC_LIT_REAL8


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def make(n, L, nmax, ns, lit=R4, seed=1, precision=wlc.WLC_FP64, store_qstar=1, q_checkpoint=0, oracle_too=True):
    dx = 1.1 / n
    kappa, chi, loa = (0.5, 0.6, 0.8), (15.0, 12.0, 18.0), 1.3
    g = wlc.Instance(n, L, nmax, ns, dx, loa, kappa, chi, precision=precision, literals=lit,
                     store_qstar=store_qstar, q_checkpoint=q_checkpoint, scheme=wlc.WLC_SCHEME_SPLIT)
    o = None
    if oracle_too:
        o = oracle.Oracle((n, n, n), L, nmax, ns, (dx, dx, dx), loa, kappa, chi, real4=1 if lit == R4 else 0,
                          scheme=1)
    w = np.random.default_rng(seed).normal(0.0, 0.5, size=(3, n ** 3))
    g.set_fields(w)
    if o is not None:
        o.set_fields(w)
    return g, o, w


CASES = [(8, 2, 10, (4, 2, 4), R4), (12, 4, 12, (4, 4, 4), R8), (8, 10, 8, (2, 4, 2), R4), (16, 6, 8, (2, 4, 2), R8)]


@pytest.mark.parametrize("n,L,nmax,ns,lit", CASES, ids=lambda v: str(v))
def test_split_sweeps_density_free_energy(n, L, nmax, ns, lit):
    g, o, _ = make(n, L, nmax, ns, lit, seed=n + L)
    g.MDE_q()
    g.MDE_qstar()
    o.propagate(1)
    o.propagate(-1)
    for s in (1, 2, ns[0] + 1, nmax):
        assert rel(g.get_q(1, s).T, o.get_q(1, s)) < TOL64, "q(s=%d)" % s
    for s in (nmax - 1, ns[0], 0):
        assert rel(g.get_q(-1, s).T, o.get_q(-1, s)) < TOL64, "q*(s=%d)" % s
    d = g.density(want_s=True)
    od = o.density(want_s=True)
    assert abs(d["lnQ"] - od["lnQ"]) <= TOL64 * max(1.0, abs(od["lnQ"]))
    assert rel(d["phi"], od["phi"]) < TOL64
    assert rel(d["junction"], od["junction"]) < TOL64
    assert rel(d["S"].reshape(3, 9, -1), od["S"]) < TOL64
    fe = g.free_energy()
    ofe = o.free_energy(od["lnQ"], od["phi"])
    assert abs(fe - ofe) <= TOL64 * abs(ofe)
    g.close()
    o.close()


def test_split_homogeneous_fields_exact():
    n, nmax, ns = 16, 12, (4, 4, 4)
    g = wlc.Instance(n, 4, nmax, ns, 1.2 / n, 1.3, (0.5, 0.6, 0.7), (15.0,) * 3, scheme=wlc.WLC_SCHEME_SPLIT)
    wv = np.array([0.7, -0.3, 1.1])
    g.set_fields(wv[:, None] * np.ones((3, n ** 3)))
    g.MDE_q()
    g.MDE_qstar()
    d = g.density()
    assert abs(d["lnQ"] + float((wv * np.array(ns) / nmax).sum())) < 1e-13
    g.close()


def test_split_storage_modes_agree():
    """Streamed densities and contour checkpointing give the stored mode's
    results (same kernels, recomputed segments)."""
    n, L, nmax, ns = 12, 4, 16, (4, 8, 4)
    ref, _, w = make(n, L, nmax, ns, seed=9, oracle_too=False)
    ref.MDE_q()
    ref.MDE_qstar()
    dr = ref.density(want_s=True)
    fr = ref.free_energy()
    for sq, K in ((0, 0), (2, 0), (2, 5)):
        g, _, _ = make(n, L, nmax, ns, seed=9, store_qstar=sq, q_checkpoint=K, oracle_too=False)
        g.MDE_q()
        g.MDE_qstar()
        d = g.density(want_s=(sq == 2))
        assert abs(d["lnQ"] - dr["lnQ"]) < 1e-13
        assert rel(d["phi"], dr["phi"]) < 1e-13
        if sq == 2:
            assert rel(d["S"], dr["S"]) < 1e-13
        assert abs(g.free_energy() - fr) < 1e-13 * abs(fr)
        g.close()
    ref.close()


def test_split_fp32_error_and_launch_variants():
    n, L, nmax, ns = 16, 6, 12, (4, 4, 4)
    g, o, w = make(n, L, nmax, ns, seed=13, precision=wlc.WLC_FP32)
    g.MDE_q()
    q_default = g.get_q(1, nmax)
    # every pass-A variant (generic / staged) and solve split gives the same slice
    for av, th in ((1, n), (2, 4 * n), (1, 16 * n)):
        g.set_launch_config(av, th, 256, 0)
        g.MDE_q()
        assert np.array_equal(g.get_q(1, nmax), q_default), (av, th)
    g.set_launch_config(0, 0, 0, 0)
    g.MDE_q()
    g.MDE_qstar()
    o.propagate(1)
    o.propagate(-1)
    d = g.density()
    od = o.density(want_s=False)
    fe = g.free_energy()
    ofe = o.free_energy(od["lnQ"], od["phi"])
    eq, ep, ef = abs(d["lnQ"] - od["lnQ"]), rel(d["phi"], od["phi"]), abs(fe - ofe) / abs(ofe)
    print("split fp32 vs fp64 oracle: lnQ %.2e phi %.2e F %.2e" % (eq, ep, ef))
    assert eq < 1e-4 and ep < 1e-4 and ef < 1e-4
    g.close()
    o.close()


def test_split_rejects_maier_saupe_and_batches():
    with pytest.raises(wlc.WlcError) as e:
        wlc.Instance(8, 2, 6, (2, 2, 2), 0.1, 1.0, (0.5,) * 3, (15.0,) * 3, nmu=5.0, scheme=wlc.WLC_SCHEME_SPLIT)
    assert e.value.code == -6
