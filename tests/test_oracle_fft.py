"""Oracle FFT pins against numpy (FFTW conventions, 2DECOMP order)."""
import numpy as np

import oracle


def _o(n):
    return oracle.Oracle(n, 1, 6, (2, 2, 2), (0.1, 0.12, 0.09), 1.0, (0.5,) * 3, (15,) * 3)


def test_r2c_matches_numpy():
    for n in [(8, 6, 10), (12, 12, 12), (16, 8, 4)]:
        o = _o(n)
        a = np.random.default_rng(0).standard_normal((n[2], n[1], n[0]))
        A = o.fft_r2c(a)
        assert np.abs(A - np.fft.rfftn(a)).max() < 1e-12 * np.abs(A).max()


def test_c2r_matches_numpy_on_non_hermitian_input():
    """Imaginary parts at kx = 0 and N/2 are discarded, as a c2r does."""
    n = (8, 6, 10)
    o = _o(n)
    rng = np.random.default_rng(1)
    X = rng.standard_normal((n[2], n[1], n[0] // 2 + 1)) + 1j * rng.standard_normal((n[2], n[1], n[0] // 2 + 1))
    b = o.fft_c2r(X)
    ref = np.fft.irfftn(X, s=(n[2], n[1], n[0]), axes=(0, 1, 2)) * (n[0] * n[1] * n[2])
    assert np.abs(b - ref).max() < 1e-12 * np.abs(ref).max()


def test_round_trip():
    n = (12, 12, 12)
    o = _o(n)
    a = np.random.default_rng(2).standard_normal((12, 12, 12))
    b = o.fft_c2r(o.fft_r2c(a)) / a.size
    assert np.abs(a - b).max() < 1e-13
