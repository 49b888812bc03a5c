"""Golden fixtures (tests/golden/, made by make_golden.py from the oracle):
the oracle still reproduces them (CPU) and the GPU path matches them."""
import os

import numpy as np
import pytest

import oracle

from golden.make_golden import CASES, inputs  # noqa: E402

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def rel(a, b):
    return float(np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(np.asarray(b)).max(), 1e-300))


def load(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_reproduces_golden(name):
    from golden.make_golden import run
    g = load(name)
    out = run(name, CASES[name])
    for k in ("qf", "qb", "phi", "junction", "S"):
        assert rel(out[k], g[k]) < 1e-13, k
    assert abs(out["lnQ"] - g["lnQ"]) < 1e-13 * max(1, abs(g["lnQ"]))
    assert abs(out["F"] - g["F"]) < 1e-13 * abs(g["F"])


@pytest.mark.gpu
@pytest.mark.parametrize("name", sorted(CASES))
def test_gpu_matches_golden(name):
    import wlc
    c = CASES[name]
    g = load(name)
    inst = wlc.Instance(c["n"], c["L"], c["nmax"], c["ns"], c["dx"], c["loa"], c["kappa"], c["chi"], nmu=c["nmu"],
                        literals=wlc.WLC_LIT_REAL4 if c["real4"] else wlc.WLC_LIT_REAL8)
    w, mop = inputs(c)
    inst.set_fields(w, mop)
    inst.MDE_q()
    inst.MDE_qstar()
    for j, s in enumerate(g["qf_s"]):
        assert rel(inst.get_q(1, int(s)).T, g["qf"][j]) < 1e-10
    for j, s in enumerate(g["qb_s"]):
        assert rel(inst.get_q(-1, int(s)).T, g["qb"][j]) < 1e-10
    d = inst.density(want_s=True)
    assert abs(d["lnQ"] - g["lnQ"]) < 1e-10 * max(1, abs(g["lnQ"]))
    assert rel(d["phi"], g["phi"]) < 1e-10
    assert rel(d["junction"], g["junction"]) < 1e-10
    assert rel(d["S"].reshape(3, 9, -1), g["S"]) < 1e-10
    assert abs(inst.free_energy() - g["F"]) < 1e-10 * abs(g["F"])
