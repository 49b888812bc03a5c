"""Oracle pins for the harmonic algebra (SPH_mod.f90:11-233,
init_array_2dcomp_mod.f90:142-375) against sympy's exact Wigner 3j symbols
and real Gaunt coefficients."""
import itertools
import math

import numpy as np
import pytest

import oracle

sympy = pytest.importorskip("sympy")
from sympy.physics.wigner import real_gaunt, wigner_3j  # noqa: E402


def test_three_j_matches_sympy():
    worst = 0.0
    for l1, l2, l3 in itertools.product(range(5), range(5), range(5)):
        for m1 in range(-l1, l1 + 1):
            for m2 in range(-l2, l2 + 1):
                m3 = -m1 - m2
                if abs(m3) > l3:
                    continue
                worst = max(worst, abs(oracle.three_j(l1, l2, l3, m1, m2, m3) - float(wigner_3j(l1, l2, l3, m1, m2, m3))))
    assert worst < 1e-14


def test_three_j_factorial_split_large_l():
    # (l1+l2+l3+1) > 20 takes the reference's split 20! * 21*...*(n) path
    for (l1, l2, l3, m1, m2) in [(8, 8, 6, 2, -1), (10, 9, 2, 3, -3), (12, 11, 2, 0, 0)]:
        m3 = -m1 - m2
        assert abs(oracle.three_j(l1, l2, l3, m1, m2, m3) - float(wigner_3j(l1, l2, l3, m1, m2, m3))) < 1e-14


def test_triple_product_is_real_gaunt_in_double_literals():
    worst = 0.0
    for l1, l2, l3 in itertools.product(range(4), range(4), range(3)):
        for m1, m2, m3 in itertools.product(range(-l1, l1 + 1), range(-l2, l2 + 1), range(-l3, l3 + 1)):
            v = oracle.triple_product(l1, l2, l3, m1, m2, m3, 0)
            e = float(real_gaunt(l1, l2, l3, m1, m2, m3) * sympy.sqrt(4 * sympy.pi))
            worst = max(worst, abs(v - e))
    assert worst < 1e-14


def test_single_precision_literals_deviate_at_float_rounding():
    worst = 0.0
    for l1, l2 in itertools.product(range(5), range(5)):
        for m1, m2 in itertools.product(range(-l1, l1 + 1), range(-l2, l2 + 1)):
            for m3 in (-1, 0, 1):
                a = oracle.triple_product(l1, l2, 1, m1, m2, m3, 1)
                b = oracle.triple_product(l1, l2, 1, m1, m2, m3, 0)
                if b != 0:
                    worst = max(worst, abs(a - b) / abs(b))
    assert 1e-9 < worst < 1e-7


_W3J = {}


def _w3j(l1, l2, l3, m1, m2, m3):
    key = (l1, l2, l3, m1, m2, m3)
    if key not in _W3J:
        _W3J[key] = float(wigner_3j(l1, l2, l3, m1, m2, m3))
    return _W3J[key]


def test_three_j_matches_sympy_through_l12():
    """Every 3j symbol the couplings use up to L = 12 (l3 = 1 for Rx/Ry/Rz,
    l3 = 2 for Theta and J, and l3 = 0), across the FACTVALUE = 20 split of
    (l1+l2+l3+1)! (SPH_mod.f90:104,116-122): l1+l2+l3+1 reaches 27."""
    worst, split = 0.0, 0
    for l1 in range(13):
        for l3 in (0, 1, 2):
            for l2 in range(max(0, l1 - l3), min(12, l1 + l3) + 1):
                for m1 in range(-l1, l1 + 1):
                    for m2 in range(-l2, l2 + 1):
                        m3 = -m1 - m2
                        if abs(m3) > l3:
                            continue
                        split += (l1 + l2 + l3 + 1) > 20
                        worst = max(worst, abs(oracle.three_j(l1, l2, l3, m1, m2, m3) - _w3j(l1, l2, l3, m1, m2, m3)))
    assert split > 1000  # the split path is exercised
    assert worst < 1e-14


def _real_sh_transform(l):
    """Rows: real harmonics of degree l (m = -l..l) in terms of the complex
    Y_l^mu, in the convention of sympy's real_gaunt (m < 0:
    i/sqrt2 (Y^m - (-1)^m Y^-m); m > 0: 1/sqrt2 (Y^-m + (-1)^m Y^m))."""
    u = np.zeros((2 * l + 1, 2 * l + 1), complex)
    s = 1.0 / math.sqrt(2.0)
    for m in range(-l, l + 1):
        if m < 0:
            u[m + l, m + l] = 1j * s
            u[m + l, -m + l] = -1j * s * (-1) ** m
        elif m == 0:
            u[l, l] = 1.0
        else:
            u[m + l, -m + l] = s
            u[m + l, m + l] = s * (-1) ** m
    return u


def _real_gaunt_exact(l1, l2, l3):
    """Real Gaunt coefficients of one (l1, l2, l3) for all m, from sympy's
    exact 3j symbols and the unitary map from complex to real harmonics."""
    G = np.zeros((2 * l1 + 1, 2 * l2 + 1, 2 * l3 + 1), complex)
    pre = math.sqrt((2 * l1 + 1) * (2 * l2 + 1) * (2 * l3 + 1) / (4 * math.pi)) * _w3j(l1, l2, l3, 0, 0, 0)
    if pre != 0.0:
        for a in range(-l1, l1 + 1):
            for b in range(-l2, l2 + 1):
                c = -a - b
                if abs(c) <= l3:
                    G[a + l1, b + l2, c + l3] = pre * _w3j(l1, l2, l3, a, b, c)
    R = np.einsum("ia,jb,kc,abc->ijk", _real_sh_transform(l1), _real_sh_transform(l2), _real_sh_transform(l3), G)
    assert np.abs(R.imag).max() < 1e-13
    return R.real


def test_exact_real_gaunt_restatement_matches_sympy():
    """The 3j-based real Gaunt used below agrees with sympy's real_gaunt
    (spot checks, including l = 12; real_gaunt itself is too slow for the
    full sweep)."""
    worst = 0.0
    rng = np.random.default_rng(3)
    for (l1, l2, l3) in [(2, 1, 1), (3, 3, 2), (12, 11, 1), (12, 12, 2), (10, 8, 2)]:
        R = _real_gaunt_exact(l1, l2, l3)
        for _ in range(3):
            m1, m2 = int(rng.integers(-l1, l1 + 1)), int(rng.integers(-l2, l2 + 1))
            for m3 in range(-l3, l3 + 1):
                worst = max(worst, abs(R[m1 + l1, m2 + l2, m3 + l3] - float(real_gaunt(l1, l2, l3, m1, m2, m3))))
    assert worst < 1e-15


def test_triple_product_is_real_gaunt_through_l12():
    """triple_product (double literals) equals sqrt(4 pi) times the real
    Gaunt coefficient for every (l1, m1, l2, m2) up to L = 12 with l3 = 1
    (Rx, Ry, Rz) and l3 = 2 (Theta, J) -- the whole coupling algebra of the
    L = 8, 10, 12 workloads."""
    worst, count = 0.0, 0
    for l1 in range(13):
        for l3 in (1, 2):
            for l2 in range(max(0, l1 - l3), min(12, l1 + l3) + 1):
                R = _real_gaunt_exact(l1, l2, l3) * math.sqrt(4 * math.pi)
                for m1, m2, m3 in itertools.product(range(-l1, l1 + 1), range(-l2, l2 + 1), range(-l3, l3 + 1)):
                    v = oracle.triple_product(l1, l2, l3, m1, m2, m3, 0)
                    worst = max(worst, abs(v - R[m1 + l1, m2 + l2, m3 + l3]))
                    count += 1
    assert count > 80000
    assert worst < 1e-14


def _R(L, real4):
    o = oracle.Oracle((4, 4, 4), L, 6, (2, 2, 2), (0.1,) * 3, 1.0, (0.5,) * 3, (15,) * 3, real4=real4)
    return [o.matrix("RX"), o.matrix("RY"), o.matrix("RZ")], o


def test_coupling_is_rotation_covariant_in_double_literals():
    R, _ = _R(6, 0)
    ev0 = np.sort(np.linalg.eigvalsh(R[2]))
    rng = np.random.default_rng(1)
    for _ in range(4):
        k = rng.standard_normal(3)
        k /= np.linalg.norm(k)
        K = k[0] * R[0] + k[1] * R[1] + k[2] * R[2]
        assert np.abs(np.sort(np.linalg.eigvalsh(0.5 * (K + K.T))) - ev0).max() < 1e-13
    for a in range(3):
        assert np.abs(R[a] - R[a].T).max() < 1e-15


def test_single_literals_break_covariance_at_1e8():
    R, _ = _R(6, 1)
    ev0 = np.sort(np.linalg.eigvalsh(R[2]))
    k = np.array([0.3, -0.5, 0.8])
    k /= np.linalg.norm(k)
    K = k[0] * R[0] + k[1] * R[1] + k[2] * R[2]
    d = np.abs(np.sort(np.linalg.eigvalsh(0.5 * (K + K.T))) - ev0).max()
    assert 1e-10 < d < 1e-7


def test_rz_is_multiplication_by_cos_theta():
    # Rz couples (l, m) only to (l +- 1, m) with sqrt(((l+1)^2 - m^2)/((2l+1)(2l+3)))
    R, _ = _R(5, 0)
    Rz = R[2]
    for l in range(5):
        for m in range(-l, l + 1):
            i = l * l + l + m
            j = (l + 1) ** 2 + (l + 1) + m
            expect = math.sqrt(((l + 1) ** 2 - m * m) / ((2 * l + 1) * (2 * l + 3)))
            assert abs(Rz[i, j] - expect) < 1e-14
