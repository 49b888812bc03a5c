"""CPU restatement of the SCFT field update -- TEST INFRASTRUCTURE ONLY
(the oracle of libwlc's wlc_iterate; imported by tests/ alone).
Parity unpinned: the reference has no two- or three-block golden vectors
for the iteration.

Follows AB_iterate (SCFT_iterate.f90:27-334) with the reference's two-block
formulas written for three blocks (f_J = N_J/Nmax, chi_KJ the block
interaction matrix):
  * simple mixing while n_iter <= Num_simple_mixing_AB (:141-197):
      dW_K = sum_J chi_KJ (phi_J - f_J) + (1/3) sum_J w_J - w_K,
      w_K += lambda_s dW_K, error max |dW_K|;
    the last simple iteration also stores history slot 0 (:167-173);
  * Anderson output field and residual (:206-209)
      w_K^out = sum_J chi_KJ phi_J + (1/3)(sum_J w_J - sum_KJ chi_KJ f_J),
      dW_K = w_K^out - w_K, error sqrt(|<dW_K,dW_K>/<w_K^out,w_K^out>|);
  * U_mn = <dW_k - dW_km, dW_k - dW_kn>, V_m = <dW_k - dW_km, dW_k> summed
    over the blocks (:237-276), U c = V by LU (dgetrf/dgetrs,
    matrix_inverse_mod.f90:167-199), new w from :307-331;
  * Maier-Saupe tensor (nmu != 0) by simple mixing (:351-372),
    M += lanbtM (NMu S - M), S summed over the blocks;
  * convergence (:1124-1160): every block error < CC (and the M error
    < 5 CC when nmu != 0), or (nmu == 0,
    n_iter >= 150) every error < 5e-4; never while n_iter < 20
    (SCFT_control.f90:270-272);
  * <a, b> = S3(a b)/V (dot_product_mpi, :1193-1237).
"""
import numpy as np


def anderson_index(i, nr):
    """Anderson_index (SCFT_iterate.f90:1-25) with Fortran MOD semantics."""
    a = int(np.fmod(i, nr + 1))
    if i < 0:
        a = nr + 1 + a
        if a == nr + 1:
            a = 0
    return a


def lu_solve(U, V):
    """U c = V by Gaussian elimination with partial pivoting (first maximal
    pivot, as dgetrf); a zero pivot gives a zero coefficient instead of a
    division by zero."""
    U = np.array(U, dtype=np.float64)
    V = np.array(V, dtype=np.float64)
    n = len(V)
    for c in range(n):
        p = c
        for r in range(c + 1, n):
            if abs(U[r, c]) > abs(U[p, c]):
                p = r
        if p != c:
            U[[c, p]] = U[[p, c]]
            V[[c, p]] = V[[p, c]]
        piv = U[c, c]
        for r in range(c + 1, n):
            f = U[r, c] / piv if piv != 0.0 else 0.0
            U[r, c:] -= f * U[c, c:]
            V[r] -= f * V[c]
    x = np.zeros(n)
    for r in range(n - 1, -1, -1):
        s = V[r] - np.dot(U[r, r + 1:], x[r + 1:])
        x[r] = s / U[r, r] if U[r, r] != 0.0 else 0.0
    return x


class Mixer:
    def __init__(self, oracle_instance, chi, ns, nmax, depth=5, num_simple=20, lambda_simple=0.1,
                 lambda_anderson=0.1, tol=1e-4, min_iter=20, relax_iter=150, relax_tol=5e-4, nmu=0.0,
                 lambda_m=0.08):
        self.o = oracle_instance
        self.C = np.array([[0.0, chi[0], chi[1]], [chi[0], 0.0, chi[2]], [chi[1], chi[2], 0.0]])
        self.f = np.array(ns, dtype=np.float64) / float(nmax)
        self.cf = self.C @ self.f
        self.fsum = self.cf.sum()
        self.depth, self.ns = depth, num_simple
        self.ls, self.la, self.tol, self.min_iter = lambda_simple, lambda_anderson, tol, min_iter
        self.relax_iter, self.relax_tol, self.nmu = relax_iter, relax_tol, nmu
        self.lambda_m = lambda_m
        self.mop = None  # Maier-Saupe tensor after the last step (nmu != 0)
        self.n = 0
        nr = oracle_instance.nr
        self.wout = np.zeros((depth + 1, 3, nr))
        self.dw = np.zeros((depth + 1, 3, nr))

    def dot(self, a, b):
        return self.o.simpson3(np.asarray(a) * np.asarray(b)) / self.o.volume

    def step(self, w, phi, S=None, mop=None):
        """One iterate(converge) call; returns (new w, err[5], converged).
        With nmu != 0, S (the oracle's [blk][a*3+b][r] orientation tensor)
        and mop ([a*3+b][r]) give the Maier-Saupe update
        M += lambda_m (NMu sum_blk S - M) (SCFT_iterate.f90:351-372); the new
        tensor is left in self.mop and err[4] = max |NMu S - M|."""
        w = np.asarray(w, dtype=np.float64).reshape(3, -1)
        phi = np.asarray(phi, dtype=np.float64).reshape(3, -1)
        self.n += 1
        n, ns, d = self.n, self.ns, self.depth
        cp = self.C @ phi
        sw = w.sum(axis=0)
        k = 0 if n <= ns else (n - ns) % (d + 1)
        err = np.zeros(5)
        err[3] = np.abs(phi.sum(axis=0) - 1.0).max()
        if n >= ns:  # the last simple iteration fills history slot 0
            wout = cp + (sw - self.fsum) / 3.0
            self.wout[k] = wout
            self.dw[k] = wout - w
        if n <= ns:
            dws = (self.C @ (phi - self.f[:, None])) + sw / 3.0 - w
            wn = w + self.ls * dws
            err[:3] = np.abs(dws).max(axis=1)
        else:
            nrt = min(n - ns, d)
            km = [anderson_index(k - m, d) for m in range(1, nrt + 1)]
            dk = self.dw[k]
            e = [dk - self.dw[a] for a in km]
            U = np.array([[self.dot(e[m], e[q]) for q in range(nrt)] for m in range(nrt)])
            V = np.array([self.dot(e[m], dk) for m in range(nrt)])
            c = lu_solve(U, V)
            wi = np.zeros_like(w)
            di = np.zeros_like(w)
            for m, a in enumerate(km):
                wi += c[m] * (self.wout[a] - self.wout[k])
                di += c[m] * (self.dw[a] - dk)
            wn = (wi + self.wout[k]) + self.la * (di + dk)
            for K in range(3):
                num = self.dot(dk[K], dk[K])
                den = self.dot(self.wout[k][K], self.wout[k][K])
                err[K] = np.sqrt(abs(num / den)) if den != 0 else 0.0
        ms = abs(self.nmu) >= 1e-5
        if ms:
            d = self.nmu * np.asarray(S).reshape(3, 9, -1).sum(axis=0) - np.asarray(mop).reshape(9, -1)
            self.mop = np.asarray(mop).reshape(9, -1) + self.lambda_m * d
            err[4] = np.abs(d).max()
        strict = bool((err[:3] < self.tol).all()) and (not ms or err[4] < 5 * self.tol)
        relaxed = bool(self.nmu == 0.0 and self.relax_iter > 0 and n >= self.relax_iter
                       and (err[:3] < self.relax_tol).all())
        conv = (strict or relaxed) and n >= self.min_iter
        return wn, err, conv
