"""Generate the golden fixtures of tests/golden/ from the CPU oracle.

The reference (Fortran/MPI/FFTW/MKL) cannot be built here and ships no
golden vectors, so these fixtures freeze the oracle's answers on seeded
inputs: forward/backward propagator slices, Q, block and junction
densities, the orientation tensor and the free energy.  The tests check
that the oracle still reproduces them and that the GPU path matches them.

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(HERE)), "oracle"))
import oracle  # noqa: E402

CASES = {
    "abc_n8_L2_real4": dict(n=8, L=2, nmax=10, ns=(4, 2, 4), dx=0.15, loa=1.0, kappa=(0.5, 0.6, 0.7),
                            chi=(15.0, 12.0, 18.0), nmu=0.0, real4=1, seed=101),
    "abc_n12_L3_real8": dict(n=12, L=3, nmax=12, ns=(4, 4, 4), dx=0.1, loa=1.3, kappa=(0.5, 0.5, 0.5),
                             chi=(18.0, 18.0, 18.0), nmu=0.0, real4=0, seed=102),
    "abc_n8_L4_ms_real4": dict(n=8, L=4, nmax=8, ns=(2, 4, 2), dx=0.125, loa=1.1, kappa=(0.5, 0.5, 0.5),
                               chi=(15.0, 15.0, 15.0), nmu=5.0, real4=1, seed=103),
}


def inputs(c):
    rng = np.random.default_rng(c["seed"])
    nr = c["n"] ** 3
    w = rng.normal(0.0, 0.5, size=(3, nr))
    mop = None
    if c["nmu"]:
        a = rng.normal(0.0, 0.3, size=(3, 3, nr))
        mop = 0.5 * (a + a.transpose(1, 0, 2))
        tr = (mop[0, 0] + mop[1, 1] + mop[2, 2]) / 3.0
        for k in range(3):
            mop[k, k] -= tr
    return w, mop


def run(name, c):
    n = c["n"]
    o = oracle.Oracle((n, n, n), c["L"], c["nmax"], c["ns"], (c["dx"],) * 3, c["loa"], c["kappa"], c["chi"],
                      nmu=c["nmu"], real4=c["real4"])
    w, mop = inputs(c)
    o.set_fields(w, None if mop is None else mop.reshape(9, -1))
    o.propagate(1)
    o.propagate(-1)
    d = o.density(want_s=True)
    fe = o.free_energy(d["lnQ"], d["phi"])
    s_list = [1, c["ns"][0] + 1, c["nmax"]]
    out = dict(qf=np.stack([o.get_q(1, s) for s in s_list]), qf_s=np.array(s_list),
               qb=np.stack([o.get_q(-1, s) for s in (0,)]), qb_s=np.array([0]),
               lnQ=d["lnQ"], phi=d["phi"], junction=d["junction"], S=d["S"], F=fe)
    return out


def main():
    for name, c in CASES.items():
        out = run(name, c)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
        print(name, "lnQ %.15f F %.15f" % (out["lnQ"], out["F"]))


if __name__ == "__main__":
    main()
