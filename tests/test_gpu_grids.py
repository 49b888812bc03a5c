"""GPU parity at every compiled grid edge that the other parity tests do not
cover (FFT radices 3 and 5, N = 96 and 128): one sweep in each direction,
densities and F against the FP64 oracle at 1e-10, small L and chain."""
import numpy as np
import pytest

import oracle
import wlc

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,L,nmax,ns", [(24, 2, 6, (2, 2, 2)), (32, 2, 4, (2, 0, 2)), (40, 2, 4, (2, 2, 0)),
                                        (48, 1, 4, (2, 2, 0)), (64, 1, 4, (0, 2, 2)), (96, 1, 4, (2, 2, 0)),
                                        (128, 0, 4, (2, 0, 2))])
def test_grid_edge_parity(n, L, nmax, ns):
    dx = 1.5 / n
    chi, kappa = (14.0, 12.0, 16.0), (0.5, 0.6, 0.7)
    # one FP64 xy plane of N = 128 does not fit in shared memory: FP64 stops at
    # N = 96 and is refused above; N = 128 runs the FP32 form
    fp32 = n == 128
    tol = 1e-4 if fp32 else 1e-10
    if fp32:
        with pytest.raises(wlc.WlcError) as e:
            wlc.Instance(n, L, nmax, ns, dx, 1.2, kappa, chi)
        assert e.value.code == -6
    g = wlc.Instance(n, L, nmax, ns, dx, 1.2, kappa, chi, precision=wlc.WLC_FP32 if fp32 else wlc.WLC_FP64)
    o = oracle.Oracle((n, n, n), L, nmax, ns, (dx,) * 3, 1.2, kappa, chi)
    w = np.random.default_rng(n).normal(0.0, 0.5, size=(3, n ** 3))
    g.set_fields(w)
    o.set_fields(w)
    g.MDE_q()
    g.MDE_qstar()
    o.propagate(1)
    o.propagate(-1)
    for s in (1, nmax):
        a, b = g.get_q(1, s).T, o.get_q(1, s)
        assert np.abs(a - b).max() <= tol * np.abs(b).max(), s
    d = g.density()
    od = o.density(want_s=False)
    assert abs(d["lnQ"] - od["lnQ"]) <= tol * max(1.0, abs(od["lnQ"]))
    assert np.abs(d["phi"] - od["phi"]).max() <= tol * np.abs(od["phi"]).max()
    fe = g.free_energy()
    assert abs(fe - o.free_energy(od["lnQ"], od["phi"])) <= tol * abs(fe)


@pytest.mark.parametrize("precision", [wlc.WLC_FP64, wlc.WLC_FP32], ids=["fp64", "fp32"])
@pytest.mark.parametrize("n", [12, 24, 40, 48, 96])
def test_launch_variants_every_grid(n, precision):
    """Every pass-A/C variant (default, half planes, batched x-FFTs, both; 256
    or 512 threads) and pass-A kind gives bit-identical results at each grid
    edge with an FFT radix other than 2, and those results match the oracle
    (the shared-memory layout of the line FFTs depends on N and the variant)."""
    L, nmax, ns = 2, 4, (2, 0, 2)
    dx = 1.5 / n
    chi, kappa = (14.0, 12.0, 16.0), (0.5, 0.6, 0.7)
    g = wlc.Instance(n, L, nmax, ns, dx, 1.2, kappa, chi, precision=precision)
    w = np.random.default_rng(500 + n).normal(0.0, 0.5, size=(3, n ** 3))
    g.set_fields(w)
    s2 = 2 * n if 2 * n <= 256 else n
    configs = [(1, n, 256, 0), (1, n, 512, 1), (1, s2, 256, 2), (1, s2, 512, 3), (2, n, 256, 1), (0, 0, 0, 0)]
    ref = None
    for cfg in configs:
        g.set_launch_config(*cfg)
        g.MDE_q()
        g.MDE_qstar()
        d = g.density()
        if ref is None:
            ref = d
        else:
            assert d["lnQ"] == ref["lnQ"] and np.array_equal(d["phi"], ref["phi"]), cfg
    o = oracle.Oracle((n, n, n), L, nmax, ns, (dx,) * 3, 1.2, kappa, chi)
    o.set_fields(w)
    o.propagate(1)
    o.propagate(-1)
    od = o.density(want_s=False)
    tol = 1e-10 if precision == wlc.WLC_FP64 else 1e-4
    assert abs(ref["lnQ"] - od["lnQ"]) <= tol * max(1.0, abs(od["lnQ"]))
    assert np.abs(ref["phi"] - od["phi"]).max() <= tol * np.abs(od["phi"]).max()
