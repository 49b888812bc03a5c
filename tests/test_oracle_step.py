"""Oracle step pins: an independent numpy restatement of one contour step
(numpy.fft + numpy.linalg.solve of the same dense G(k)), analytic known
answers for homogeneous fields, and the density normalisation."""
import numpy as np
import pytest

import oracle


def _fold(i, n):
    return i if i <= n // 2 else i - n


def numpy_step(o, order, sigma, kappa, pr, real4=1):
    """q = C2R(G^-1 R2C(Pr)) / N^3 with dense per-k solves (numpy)."""
    n = o.n
    M = o.M
    R = [o.matrix("RX"), o.matrix("RY"), o.matrix("RZ")]
    c0 = {1: 1.0, 2: 1.5, 3: float(np.float32(11.0) / np.float32(6.0)) if real4 else 11.0 / 6.0}[order]
    twopi = float(np.float32(2.0) * np.float32(np.pi)) if real4 else 2 * np.pi
    kf = [twopi / (n[a] * o.dx[a]) for a in range(3)]
    ds = 1.0 / o.nmax
    l = np.array([int(np.floor(np.sqrt(i) + 1e-9)) for i in range(M)])
    diag = c0 + ds * o._loa * l * (l + 1) / (2.0 * kappa)
    P = np.stack([np.fft.rfftn(pr[i].reshape(n[2], n[1], n[0])) for i in range(M)])
    out = np.empty_like(P)
    for iz in range(n[2]):
        for iy in range(n[1]):
            for ix in range(n[0] // 2 + 1):
                k = (_fold(ix, n[0]) * kf[0], _fold(iy, n[1]) * kf[1], _fold(iz, n[2]) * kf[2])
                G = np.diag(diag).astype(complex) + 1j * sigma * ds * (k[0] * R[0] + k[1] * R[1] + k[2] * R[2])
                out[:, iz, iy, ix] = np.linalg.solve(G, P[:, iz, iy, ix])
    q = np.stack([np.fft.irfftn(out[i], s=(n[2], n[1], n[0]), axes=(0, 1, 2)) for i in range(M)])
    return q.reshape(M, -1)


@pytest.mark.parametrize("real4", [1, 0])
@pytest.mark.parametrize("order,sigma,blk", [(1, 1, 0), (2, 1, 0), (3, 1, 1), (3, -1, 2), (1, -1, 2)])
def test_one_step_matches_numpy_restatement(order, sigma, blk, real4):
    n = (6, 4, 8)
    kappa = (0.5, 0.7, 0.9)
    o = oracle.Oracle(n, 2, 10, (4, 2, 4), (0.2, 0.25, 0.15), 1.3, kappa, (15, 15, 15), real4=real4)
    o._loa = 1.3
    pr = np.random.default_rng(order + 10 * blk).standard_normal((o.M, o.nr))
    a = o.one_step(order, sigma, blk, pr)
    b = numpy_step(o, order, sigma, kappa[blk], pr, real4)
    assert np.abs(a - b).max() < 1e-12 * np.abs(b).max()


def _bdf_scalar(w_of_step, nmax, real4=1):
    """q_0(s) for spatially constant fields: the l=0, k=0 mode obeys the
    BDF1/2/3 recurrence c0 q_s = sum_j a_j q_{s-j} - ds w sum_j b_j q_{s-j}."""
    ds = 1.0 / nmax
    third = float(np.float32(1.0) / np.float32(3.0)) if real4 else 1.0 / 3.0
    c03 = float(np.float32(11.0) / np.float32(6.0)) if real4 else 11.0 / 6.0
    q = [1.0]
    for s in range(1, nmax + 1):
        W = w_of_step(s)
        o = min(s, 3)
        if o == 1:
            q.append((1.0 - ds * W) * q[-1])
        elif o == 2:
            q.append((2 * q[-1] - 0.5 * q[-2] - ds * W * (2 * q[-1] - q[-2])) / 1.5)
        else:
            q.append((3 * q[-1] - 1.5 * q[-2] + third * q[-3] - ds * W * (3 * q[-1] - 3 * q[-2] + q[-3])) / c03)
    return np.array(q)


def test_homogeneous_fields_known_answer():
    n, L, nmax, ns = (4, 4, 4), 3, 12, (4, 4, 4)
    wv = (0.3, -0.2, 0.5)
    o = oracle.Oracle(n, L, nmax, ns, (0.25,) * 3, 1.0, (0.5,) * 3, (15, 15, 15))
    o.set_fields(np.repeat(np.array(wv)[:, None], o.nr, axis=1))
    o.propagate(1)
    def blk(s):
        return 0 if s <= ns[0] else (1 if s <= ns[0] + ns[1] else 2)
    ref = _bdf_scalar(lambda s: wv[blk(s)], nmax)
    for s in range(nmax + 1):
        q = o.get_q(1, s)
        assert np.abs(q[0] - ref[s]).max() < 1e-14
        assert np.abs(q[1:]).max() < 1e-14
    o.propagate(-1)
    d = o.density(want_s=False)
    assert abs(d["lnQ"] - np.log(ref[-1])) < 1e-13


def test_densities_are_normalised_and_q_consistent():
    n, L, nmax, ns = (8, 8, 8), 2, 10, (4, 2, 4)
    o = oracle.Oracle(n, L, nmax, ns, (0.15,) * 3, 1.0, (0.5,) * 3, (15, 12, 18))
    rng = np.random.default_rng(3)
    o.set_fields(rng.normal(0, 0.5, (3, o.nr)))
    o.propagate(1)
    o.propagate(-1)
    d = o.density(want_s=True)
    tot = o.simpson3(d["phi"].sum(axis=0)) / o.volume
    assert abs(tot - 1.0) < 1e-12
    # Q from the forward end equals Q from the backward start (same chain)
    qb0 = o.get_q(-1, 0)[0]
    lnq_b = np.log(o.simpson3(qb0) / o.volume)
    assert abs(lnq_b - d["lnQ"]) < 5e-3  # equal up to the O(ds^3) scheme error
    S = d["S"].reshape(3, 3, 3, -1)
    assert np.abs(S[:, 0, 0] + S[:, 1, 1] + S[:, 2, 2]).max() < 1e-12  # traceless
    F = o.free_energy(d["lnQ"], d["phi"])
    assert np.isfinite(F)
