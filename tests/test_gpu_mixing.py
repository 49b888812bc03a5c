"""GPU parity of the SCFT field update (wlc_iterate: simple mixing, then
Anderson mixing on the device) against the CPU restatement of AB_iterate
(SCFT_iterate.f90:27-334, three-block form) driven by the FP64 oracle.

Tolerance: 1e-9 relative on the fields and the free energy after every
iteration of a free-running loop (the Anderson solve amplifies the 1e-13
differences of the propagators by the conditioning of U), 1e-10 on a
single update from identical inputs.
"""
import numpy as np
import pytest

import oracle
from oracle_mixing import Mixer
import wlc

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def _pair(n=8, L=2, nmax=10, ns=(4, 2, 4), chi=(15.0, 12.0, 18.0), lit=wlc.WLC_LIT_REAL4, seed=7):
    dx = 1.6 / n
    kappa = (0.5, 0.6, 0.7)
    g = wlc.Instance(n, L, nmax, ns, dx, 1.2, kappa, chi, literals=lit)
    o = oracle.Oracle((n, n, n), L, nmax, ns, (dx, dx, dx), 1.2, kappa, chi,
                      real4=1 if lit == wlc.WLC_LIT_REAL4 else 0)
    rng = np.random.default_rng(seed)
    w = rng.normal(0.0, 1.0, size=(3, n ** 3))
    return g, o, w


def _oracle_density(o, w):
    o.set_fields(w)
    o.propagate(1)
    o.propagate(-1)
    d = o.density(want_s=False)
    return d, o.free_energy(d["lnQ"], d["phi"])


@pytest.mark.parametrize("depth,num_simple", [(3, 4), (5, 20)])
def test_iterate_free_running(depth, num_simple):
    g, o, w = _pair()
    mp = wlc.mix_params(anderson_depth=depth, num_simple=num_simple, tol=1e-12, min_iter=20)
    mx = Mixer(o, (15.0, 12.0, 18.0), (4, 2, 4), 10, depth=depth, num_simple=num_simple, tol=1e-12, min_iter=20)
    g.set_fields(w)
    wo = w.copy()
    iters = num_simple + 3 * (depth + 1) + 2  # wraps the history ring three times
    for it in range(iters):
        g.MDE_q()
        g.MDE_qstar()
        d = g.density(want_junction=False)
        fe = g.free_energy()
        od, ofe = _oracle_density(o, wo)
        assert abs(fe - ofe) <= 1e-9 * abs(ofe), "iteration %d: F %.15g vs %.15g" % (it + 1, fe, ofe)
        err, conv = g.iterate(mp)
        wo, oerr, oconv = mx.step(wo, od["phi"])
        wg = g.get_fields()
        assert rel(wg, wo) < 1e-9, "iteration %d: fields rel err %.3e" % (it + 1, rel(wg, wo))
        assert np.allclose(err, oerr, rtol=1e-8, atol=1e-14), (it + 1, err, oerr)
        assert conv == oconv
    # the loop made progress
    assert err[:3].max() < 1.0


def test_iterate_single_update_identical_inputs():
    """Each Anderson update from identical (w, phi): the oracle's w is loaded
    into the device before every iteration, so only one update's rounding is
    compared."""
    g, o, w = _pair(seed=9, lit=wlc.WLC_LIT_REAL8)
    depth, ns = 4, 3
    mp = wlc.mix_params(anderson_depth=depth, num_simple=ns)
    mx = Mixer(o, (15.0, 12.0, 18.0), (4, 2, 4), 10, depth=depth, num_simple=ns)
    wo = w.copy()
    for it in range(ns + 2 * (depth + 1)):
        g.set_fields(wo)
        g.MDE_q()
        g.MDE_qstar()
        g.density(want_junction=False)
        od, _ = _oracle_density(o, wo)
        g.iterate(mp)
        wo, _, _ = mx.step(wo, od["phi"])
        assert rel(g.get_fields(), wo) < 1e-10, it + 1


def test_cal_scft_converges_and_matches_driver_loop():
    """Instance.cal_scft (the driver loop of SCFT_control.f90:237-273) to a
    loose tolerance; the reported F equals a fresh evaluation at the final
    fields' predecessor and the errors fall by orders of magnitude."""
    n, L, nmax, ns = 8, 2, 10, (4, 2, 4)
    dx = 2.0 / n
    g = wlc.Instance(n, L, nmax, ns, dx, 1.0, (0.5, 0.5, 0.5), (8.0, 8.0, 8.0))
    x = np.arange(n) * dx
    X = np.broadcast_to(x[None, None, :], (n, n, n)).reshape(-1)
    w = np.stack([np.cos(2 * np.pi * X / (n * dx)), -np.cos(2 * np.pi * X / (n * dx)), np.zeros(n ** 3)])
    g.set_fields(w)
    out = g.cal_scft(max_iter=400, anderson_depth=5, num_simple=20, tol=1e-6)
    errs = np.array([h[1][:3].max() for h in out["history"]])
    assert out["converged"], (out["n_iter"], errs[-5:])
    assert errs[-1] < 1e-6 and errs[0] > 1e-3
    assert np.isfinite(out["F"])


def test_iterate_maier_saupe_tensor():
    """With NMu != 0 the field update also mixes the Maier-Saupe tensor
    towards NMu S (simple mixing, lanbtM) and reports its error in err[4];
    the next sweeps use the updated tensor."""
    n, L, nmax, ns = 8, 4, 8, (2, 4, 2)
    nmu, chi = 5.0, (15.0, 15.0, 15.0)
    dx = 1.0 / n
    g = wlc.Instance(n, L, nmax, ns, dx, 1.1, (0.5, 0.5, 0.5), chi, nmu=nmu)
    o = oracle.Oracle((n, n, n), L, nmax, ns, (dx,) * 3, 1.1, (0.5, 0.5, 0.5), chi, nmu=nmu)
    rng = np.random.default_rng(17)
    w = rng.normal(0.0, 0.5, size=(3, n ** 3))
    a = rng.normal(0.0, 0.3, size=(3, 3, n ** 3))
    m = 0.5 * (a + a.transpose(1, 0, 2))
    tr = (m[0, 0] + m[1, 1] + m[2, 2]) / 3.0
    for k in range(3):
        m[k, k] -= tr
    g.set_fields(w, m)
    mp = wlc.mix_params(anderson_depth=2, num_simple=3)
    mx = Mixer(o, chi, ns, nmax, depth=2, num_simple=3, nmu=nmu)
    wo, mo = w.copy(), m.reshape(9, -1).copy()
    for it in range(7):
        g.MDE_q()
        g.MDE_qstar()
        g.density(want_junction=False)
        err, conv = g.iterate(mp)
        o.set_fields(wo, mo)
        o.propagate(1)
        o.propagate(-1)
        od = o.density(want_s=True)
        wo, oerr, oconv = mx.step(wo, od["phi"], od["S"], mo)
        mo = mx.mop
        assert rel(g.get_fields(), wo) < 1e-9, it + 1
        assert rel(g.get_mop().reshape(9, -1), mo) < 1e-9, it + 1
        assert np.allclose(err, oerr, rtol=1e-8, atol=1e-14), (it + 1, err, oerr)
        assert conv == oconv
    assert err[4] > 0.0


def test_w_dump_and_readw_round_trip(tmp_path):
    """W_dump / readW through the reference's file formats restore the
    fields and the Maier-Saupe tensor exactly."""
    n = 8
    g = wlc.Instance(n, 2, 6, (2, 2, 2), 0.12, 1.0, (0.5, 0.5, 0.5), (15.0,) * 3, nmu=3.0)
    rng = np.random.default_rng(4)
    w = rng.normal(size=(3, n ** 3))
    a = rng.normal(size=(3, 3, n ** 3))
    m = 0.5 * (a + a.transpose(1, 0, 2))
    g.set_fields(w, m)
    g.W_dump(tmp_path, rank=0)
    h = wlc.Instance(n, 2, 6, (2, 2, 2), 0.12, 1.0, (0.5, 0.5, 0.5), (15.0,) * 3, nmu=3.0)
    h.readW(tmp_path, rank=0)
    assert np.array_equal(h.get_fields(), w) and np.array_equal(h.get_mop(), m)
