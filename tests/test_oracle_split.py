"""Oracle pins of the operator-split contour step (scheme 1):
  q(s) = e^{-w ds/2} C2R[ G_CN(k) R2C[ e^{-w ds/2} q(s-1) ] ] / N^3,
  G_CN = (I + ds/2 A)^-1 (I - ds/2 A),  A = Loa l(l+1)/(2 kappa) + i sigma k.R.
The scheme has no counterpart in the reference's harmonic-basis solver
(its field half steps follow split_operator_MDE_mod.f90:163-166), so these
pins are what the oracle of the GPU split step rests on:
  * an independent numpy restatement of one step (numpy.fft and a dense
    matrix inverse of I + ds/2 A, G_CN applied as written, not as
    2 (I + ds/2 A)^-1 - I);
  * homogeneous fields: the l = 0, k = 0 mode is propagated exactly,
    ln Q = -sum_K f_K w_K;
  * second-order convergence in ds of ln Q (Strang splitting around a
    Crank-Nicolson step).
"""
import numpy as np
import pytest

import oracle


def _fold(i, n):
    return i if i <= n // 2 else i - n


def numpy_split_step(o, sigma, kappa, w, q, real4=1):
    n, M = o.n, o.M
    R = [o.matrix("RX"), o.matrix("RY"), o.matrix("RZ")]
    twopi = float(np.float32(2.0) * np.float32(np.pi)) if real4 else 2 * np.pi
    kf = [twopi / (n[a] * o.dx[a]) for a in range(3)]
    ds = 1.0 / o.nmax
    l = np.array([int(np.floor(np.sqrt(i) + 1e-9)) for i in range(M)])
    eh = np.exp(-0.5 * ds * w)
    P = np.stack([np.fft.rfftn((eh * q[i]).reshape(n[2], n[1], n[0])) for i in range(M)])
    out = np.empty_like(P)
    for iz in range(n[2]):
        for iy in range(n[1]):
            for ix in range(n[0] // 2 + 1):
                k = (_fold(ix, n[0]) * kf[0], _fold(iy, n[1]) * kf[1], _fold(iz, n[2]) * kf[2])
                A = np.diag(o._loa * l * (l + 1) / (2.0 * kappa)).astype(complex) + \
                    1j * sigma * (k[0] * R[0] + k[1] * R[1] + k[2] * R[2])
                Gcn = np.linalg.inv(np.eye(M) + 0.5 * ds * A) @ (np.eye(M) - 0.5 * ds * A)
                out[:, iz, iy, ix] = Gcn @ P[:, iz, iy, ix]
    qn = np.stack([np.fft.irfftn(out[i], s=(n[2], n[1], n[0]), axes=(0, 1, 2)).reshape(-1) for i in range(M)])
    return eh * qn


@pytest.mark.parametrize("real4", [1, 0])
@pytest.mark.parametrize("sigma,blk,L", [(1, 0, 2), (-1, 2, 2), (1, 1, 10)])
def test_split_step_matches_numpy_restatement(sigma, blk, L, real4):
    n = (6, 4, 8)
    kappa = (0.5, 0.7, 0.9)
    o = oracle.Oracle(n, L, 10, (4, 2, 4), (0.2, 0.25, 0.15), 1.3, kappa, (15, 15, 15), real4=real4, scheme=1)
    rng = np.random.default_rng(5 + blk)
    w = rng.normal(0.0, 0.7, size=(3, o.nr))
    o.set_fields(w)
    q = rng.standard_normal((o.M, o.nr))
    a = o.split_step(sigma, blk, q)
    b = numpy_split_step(o, sigma, kappa[blk], w[blk], q, real4)
    assert np.abs(a - b).max() < 1e-12 * np.abs(b).max()


def test_split_homogeneous_fields_exact():
    n, nmax, ns = 8, 12, (4, 4, 4)
    o = oracle.Oracle((n,) * 3, 4, nmax, ns, (1.2 / n,) * 3, 1.3, (0.5, 0.6, 0.7), (15.0,) * 3, scheme=1)
    wv = np.array([0.7, -0.3, 1.1])
    o.set_fields(wv[:, None] * np.ones((3, n ** 3)))
    o.propagate(1)
    o.propagate(-1)
    d = o.density(want_s=False)
    expect = -float((wv * np.array(ns) / nmax).sum())
    assert abs(d["lnQ"] - expect) < 1e-13
    # every block density is its composition, every point
    for b in range(3):
        assert np.abs(d["phi"][b] - ns[b] / nmax).max() < 1e-12


def test_split_second_order_in_ds():
    n, L = 8, 2
    x = np.arange(n) / n
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    base = (np.cos(2 * np.pi * X) + 0.5 * np.sin(2 * np.pi * Y) * np.cos(2 * np.pi * Z)).transpose(2, 1, 0).reshape(-1)
    w = np.stack([0.8 * base, -0.5 * base, 0.3 * base + 0.2])

    def lnq(nmax):
        ns = (nmax // 4, nmax // 2, nmax - nmax // 4 - nmax // 2)
        o = oracle.Oracle((n,) * 3, L, nmax, ns, (1.2 / n,) * 3, 1.3, (0.5, 0.6, 0.7), (15.0,) * 3, scheme=1)
        o.set_fields(w)
        o.propagate(1)
        o.propagate(-1)
        v = o.density(want_s=False)["lnQ"]
        o.close()
        return v

    ref = lnq(512)
    e = [abs(lnq(m) - ref) for m in (16, 32, 64)]
    r1, r2 = e[0] / e[1], e[1] / e[2]
    assert 3.5 < r1 < 4.8 and 3.5 < r2 < 4.8, (e, r1, r2)
