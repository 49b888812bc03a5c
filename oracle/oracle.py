"""ctypes handle on the CPU FP64 oracle (oracle/wlc_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's cpu_baseline / reference leg, always to test against.  The product
library never imports it.

The oracle restates the reference's arithmetic (file:line citations live in
wlc_oracle.c).  Parity with the Fortran reference itself is unpinned (the
reference cannot be built); the restatement is pinned against sympy's exact
Wigner 3j symbols, numpy.fft, numpy.linalg.solve, analytic known answers and
an independent numpy restatement (tests/test_oracle_*.py).

Array layouts (C order): real-space r = (z*ny + y)*nx + x; propagator slices
[i][r]; fields [blk][r]; Maier-Saupe tensor [a*3+b][r].
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libwlc_oracle.so")
_lib = None

MATS = ["RX", "RY", "RZ", "T1122", "T33", "T12", "T13", "T23",
        "J11", "J22", "J12", "J13", "J23"]


def build(force=False):
    """Compile the oracle with its Makefile (gcc + OpenMP)."""
    src = os.path.join(_HERE, "wlc_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _load():
    global _lib
    if _lib is not None:
        return _lib
    build()
    lib = ctypes.CDLL(_LIB_PATH)
    P = ctypes.c_void_p
    D = ctypes.c_double
    Ip = ctypes.POINTER(ctypes.c_int)
    Dp = ctypes.POINTER(ctypes.c_double)
    Int = ctypes.c_int
    lib.orc_create.restype = P
    lib.orc_create.argtypes = [Ip, Int, Int, Ip, Dp, D, Dp, Dp, D, Int, Int]
    lib.orc_destroy.argtypes = [P]
    lib.orc_M.argtypes = [P]
    lib.orc_M.restype = Int
    lib.orc_nk.argtypes = [P]
    lib.orc_nk.restype = Int
    lib.orc_get_matrix.argtypes = [P, Int, Dp]
    lib.orc_set_box.argtypes = [P, Dp]
    lib.orc_set_fields.argtypes = [P, Dp, Dp]
    lib.orc_init_pr.argtypes = [P, Int, Int, Dp]
    lib.orc_one_step.argtypes = [P, Int, Int, Int, Dp, Dp]
    lib.orc_propagate.argtypes = [P, Int]
    lib.orc_get_q.argtypes = [P, Int, Int, Dp]
    lib.orc_set_q.argtypes = [P, Int, Int, Dp]
    lib.orc_density.argtypes = [P, Dp, Dp, Dp, Dp]
    lib.orc_density.restype = D
    lib.orc_free_energy.argtypes = [P, D, Dp]
    lib.orc_free_energy.restype = D
    lib.orc_simpson3.argtypes = [P, Dp]
    lib.orc_simpson3.restype = D
    lib.orc_fft_r2c.argtypes = [P, Dp, Dp]
    lib.orc_fft_c2r.argtypes = [P, Dp, Dp]
    lib.orc_bench_step.argtypes = [P, Int, Dp]
    lib.orc_set_scheme.argtypes = [P, Int]
    lib.orc_bench_steps.argtypes = [P, Int, Dp]
    lib.orc_split_step.argtypes = [P, Int, Int, Dp, Dp]
    lib.orc_three_j.argtypes = [Int] * 6
    lib.orc_three_j.restype = D
    lib.orc_triple_product.argtypes = [Int] * 7
    lib.orc_triple_product.restype = D
    _lib = lib
    return lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def three_j(l1, l2, l3, m1, m2, m3):
    return _load().orc_three_j(l1, l2, l3, m1, m2, m3)


def triple_product(l1, l2, l3, m1, m2, m3, real4=1):
    return _load().orc_triple_product(l1, l2, l3, m1, m2, m3, int(real4))


class Oracle:
    """One SCFT instance on the CPU (ABC triblock, one L for all blocks)."""

    def __init__(self, n, L, nmax, ns, dx, loa, kappa, chi, nmu=0.0, real4=1, nthreads=None, scheme=0):
        lib = _load()
        self.lib = lib
        self.n = tuple(int(v) for v in n)
        self.L = int(L)
        self.M = (self.L + 1) ** 2
        self.nmax = int(nmax)
        self.ns = tuple(int(v) for v in ns)
        self.nr = self.n[0] * self.n[1] * self.n[2]
        self.nkx = self.n[0] // 2 + 1
        self.nk = self.nkx * self.n[1] * self.n[2]
        if nthreads is None:
            nthreads = os.cpu_count() or 1
        self.nthreads = int(nthreads)
        n3 = (ctypes.c_int * 3)(*self.n)
        ns3 = (ctypes.c_int * 3)(*self.ns)
        dx3 = (ctypes.c_double * 3)(*[float(v) for v in dx])
        k3 = (ctypes.c_double * 3)(*[float(v) for v in kappa])
        c3 = (ctypes.c_double * 3)(*[float(v) for v in chi])
        self.h = lib.orc_create(n3, self.L, self.nmax, ns3, dx3, float(loa), k3, c3, float(nmu),
                                int(real4), self.nthreads)
        self.dx = tuple(float(v) for v in dx)
        self._loa = float(loa)
        self.scheme = int(scheme)
        lib.orc_set_scheme(self.h, self.scheme)

    def close(self):
        if self.h:
            self.lib.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def volume(self):
        return self.dx[0] * self.dx[1] * self.dx[2] * self.nr

    def matrix(self, name):
        out = np.empty((self.M, self.M))
        self.lib.orc_get_matrix(self.h, MATS.index(name), _dp(out))
        return out

    def set_box(self, dx):
        self.dx = tuple(float(v) for v in dx)
        self.lib.orc_set_box(self.h, (ctypes.c_double * 3)(*self.dx))

    def set_fields(self, w, mop=None):
        w = np.ascontiguousarray(w, dtype=np.float64).reshape(3, self.nr)
        self._w = w
        if mop is None:
            self.lib.orc_set_fields(self.h, _dp(w), None)
        else:
            mop = np.ascontiguousarray(mop, dtype=np.float64).reshape(9, self.nr)
            self._mop = mop
            self.lib.orc_set_fields(self.h, _dp(w), _dp(mop))

    def init_pr(self, direction, s):
        out = np.empty((self.M, self.nr))
        self.lib.orc_init_pr(self.h, int(direction), int(s), _dp(out))
        return out

    def one_step(self, order, sigma, blk, pr):
        pr = np.ascontiguousarray(pr, dtype=np.float64).reshape(self.M, self.nr)
        out = np.empty((self.M, self.nr))
        self.lib.orc_one_step(self.h, int(order), int(sigma), int(blk), _dp(pr), _dp(out))
        return out

    def split_step(self, sigma, blk, q):
        """One step of the operator-split scheme from slice q ([M][nr])."""
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.M, self.nr)
        out = np.empty((self.M, self.nr))
        self.lib.orc_split_step(self.h, int(sigma), int(blk), _dp(q), _dp(out))
        return out

    def propagate(self, direction):
        self.lib.orc_propagate(self.h, int(direction))

    def get_q(self, direction, s):
        out = np.empty((self.M, self.nr))
        self.lib.orc_get_q(self.h, int(direction), int(s), _dp(out))
        return out

    def set_q(self, direction, s, q):
        q = np.ascontiguousarray(q, dtype=np.float64).reshape(self.M, self.nr)
        self.lib.orc_set_q(self.h, int(direction), int(s), _dp(q))

    def density(self, want_s=True):
        lnq = np.zeros(1)
        phi = np.empty((3, self.nr))
        junc = np.empty((3, self.nr))
        sop = np.empty((3, 9, self.nr)) if want_s else None
        totden = self.lib.orc_density(self.h, _dp(lnq), _dp(phi), _dp(junc),
                                      _dp(sop) if want_s else None)
        return dict(lnQ=float(lnq[0]), phi=phi, junction=junc, S=sop, totden=totden)

    def free_energy(self, lnq, phi):
        phi = np.ascontiguousarray(phi, dtype=np.float64).reshape(3, self.nr)
        return self.lib.orc_free_energy(self.h, float(lnq), _dp(phi))

    def simpson3(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        if a.size != self.nr:  # several stacked fields: integrate their sum
            a = a.reshape(-1, self.nr).sum(axis=0)
        a = np.ascontiguousarray(a.reshape(self.nr))
        return self.lib.orc_simpson3(self.h, _dp(a))

    def bench_step(self, nk_sample):
        """Timed BDF3 step with the per-k solve sampled on nk_sample
        wavevectors; returns (stage seconds[4], full-step estimate)."""
        t = np.zeros(4)
        self.lib.orc_bench_step(self.h, int(nk_sample), _dp(t))
        est = t[0] + t[1] + t[2] * self.nk / max(1, min(nk_sample, self.nk)) + t[3]
        return t, est

    def bench_steps(self, nsteps):
        """Timed whole BDF3 contour steps (every wavevector, plus the slice's
        density contribution); returns (set-up s, timed s, s per step)."""
        t = np.zeros(3)
        self.lib.orc_bench_steps(self.h, int(nsteps), _dp(t))
        return float(t[0]), float(t[1]), float(t[2])

    def fft_r2c(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64).reshape(self.nr)
        out = np.empty(self.nk, dtype=np.complex128)
        self.lib.orc_fft_r2c(self.h, _dp(a), out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)))
        return out.reshape(self.n[2], self.n[1], self.nkx)

    def fft_c2r(self, a):
        a = np.ascontiguousarray(a, dtype=np.complex128).reshape(self.nk)
        out = np.empty(self.nr)
        self.lib.orc_fft_c2r(self.h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), _dp(out))
        return out.reshape(self.n[2], self.n[1], self.n[0])
