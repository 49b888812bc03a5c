"""Generate wlc_rot_gen.cuh: register codelets for the constant rotation
blocks of the factorised G(k) solve.

For each degree l the real-harmonic coefficients of block l transform under
the rotation by +pi/2 about x with a fixed (2l+1)x(2l+1) orthogonal matrix
X_l (about a quarter of its entries are nonzero); X_l^T undoes it.  The
factorised solve applies X_l and X_l^T four times per wavevector, so the
codelets unroll them into straight-line FMAs on register arrays (no table
loads).  The entries are computed here by exact Gauss-Legendre x uniform
quadrature of products of real harmonics, with the harmonic convention the
reference uses (checked against its triple products in the tests).

    python gen_rotation.py [LMAX]      # writes wlc_rot_gen.cuh next to this file
"""
import math
import os
import sys

import mpmath as mp
import numpy as np

LMAX_DEFAULT = 12
mp.mp.dps = 40


def assoc_legendre(L, x):
    """P_l^m(x), Condon-Shortley phase, for one point (mpmath)."""
    P = [[mp.mpf(0)] * (L + 1) for _ in range(L + 1)]
    P[0][0] = mp.mpf(1)
    s = mp.sqrt(max(mp.mpf(0), 1 - x * x))
    for m in range(1, L + 1):
        P[m][m] = -(2 * m - 1) * s * P[m - 1][m - 1]
    for m in range(0, L):
        P[m + 1][m] = (2 * m + 1) * x * P[m][m]
    for m in range(0, L + 1):
        for l in range(m + 2, L + 1):
            P[l][m] = ((2 * l - 1) * x * P[l - 1][m] - (l + m - 1) * P[l - 2][m]) / (l - m)
    return P


def real_harmonics_block(l, ct, phi):
    """Y_{l,m}(u) for m = -l..l at one point (mpmath)."""
    P = assoc_legendre(l, ct)
    out = []
    for m in range(-l, l + 1):
        am = abs(m)
        N = mp.sqrt(mp.mpf(2 * l + 1) / (4 * mp.pi) * mp.factorial(l - am) / mp.factorial(l + am))
        if m == 0:
            out.append(N * P[l][0])
        elif m > 0:
            out.append(mp.sqrt(2) * N * P[l][am] * mp.cos(am * phi))
        else:
            out.append(mp.sqrt(2) * N * P[l][am] * mp.sin(am * phi))
    return out


def gauss_legendre(n):
    xs, ws = [], []
    for i in range(n):
        z = mp.cos(mp.pi * (i + mp.mpf(3) / 4) / (n + mp.mpf(1) / 2))
        for _ in range(100):
            p0, p1 = mp.mpf(1), z
            for k in range(2, n + 1):
                p0, p1 = p1, ((2 * k - 1) * z * p1 - (k - 1) * p0) / k
            dp = n * (z * p1 - p0) / (z * z - 1)
            dz = p1 / dp
            z -= dz
            if abs(dz) < mp.mpf(10) ** (-35):
                break
        p0, p1 = mp.mpf(1), z
        for k in range(2, n + 1):
            p0, p1 = p1, ((2 * k - 1) * z * p1 - (k - 1) * p0) / k
        dp = n * (z * p1 - p0) / (z * z - 1)
        xs.append(z)
        ws.append(2 / ((1 - z * z) * dp * dp))
    return xs, ws


def rotation_x90(l):
    """X_l[i][j] = int Y_i(u) Y_j(Q^T u) du, Q = Rx(+pi/2), exact quadrature."""
    nt, nph = l + 2, 2 * l + 3
    xs, ws = gauss_legendre(nt)
    n = 2 * l + 1
    X = [[mp.mpf(0)] * n for _ in range(n)]
    for a in range(nt):
        for b in range(nph):
            ct, phi = xs[a], 2 * mp.pi * b / nph
            wq = ws[a] * 2 * mp.pi / nph
            st = mp.sqrt(max(mp.mpf(0), 1 - ct * ct))
            ux, uy, uz = st * mp.cos(phi), st * mp.sin(phi), ct
            vx, vy, vz = ux, uz, -uy  # Q^T u
            Y = real_harmonics_block(l, ct, phi)
            Y2 = real_harmonics_block(l, vz, mp.atan2(vy, vx))
            for i in range(n):
                for j in range(n):
                    X[i][j] += wq * Y[i] * Y2[j]
    Xd = np.array([[float(X[i][j]) if abs(X[i][j]) > mp.mpf(10) ** (-25) else 0.0 for j in range(n)]
                   for i in range(n)])
    return Xd


def emit_apply(name, X, l):
    n = 2 * l + 1
    lines = ["    template <typename T, typename C> __device__ __forceinline__ static void %s(const C* v, C* u) {" % name]
    # X maps each x-parity class onto itself: emit one class after the
    # other so the inputs of the first class die early (register pressure)
    order = sorted(range(n), key=lambda j: (min([m for m in range(n) if X[j, m] != 0.0] or [0]) % 2, j))
    cls = {}
    for j in range(n):
        nz = [m for m in range(n) if X[j, m] != 0.0]
        cls[j] = ((nz[0] - l) % 2 if nz else 0, (j - l) % 2)
    order = sorted(range(n), key=lambda j: (cls[j], j))
    for j in order:
        terms = [(X[j, m], m) for m in range(n) if X[j, m] != 0.0]
        if not terms:
            lines.append("        u[%d] = cmk<C>((T)0, (T)0);" % j)
            continue
        c, m = terms[0]
        ex = "(T)%.17g * v[%d].x" % (c, m)
        ey = "(T)%.17g * v[%d].y" % (c, m)
        for c, m in terms[1:]:
            ex = "fma((T)%.17g, v[%d].x, %s)" % (c, m, ex)
            ey = "fma((T)%.17g, v[%d].y, %s)" % (c, m, ey)
        lines.append("        u[%d] = cmk<C>(%s, %s);" % (j, ex, ey))
    lines.append("    }")
    return lines


def main():
    lmax = int(sys.argv[1]) if len(sys.argv) > 1 else LMAX_DEFAULT
    here = os.path.dirname(os.path.abspath(__file__))
    out = [
        "// wlc_rot_gen.cuh -- GENERATED by gen_rotation.py; do not edit.",
        "// Rotation by +pi/2 about x of the real-harmonic block l (XRot<l>::p,",
        "// u = X_l v) and its transpose (XRot<l>::m, u = X_l^T v), l = 0..%d," % lmax,
        "// as straight-line FMAs on register arrays v[2l+1], u[2l+1] (index m+l).",
        "#pragma once",
        '#include "wlc_fft.cuh"',
        "",
        "namespace wlc {",
        "",
        "template <int l> struct XRot;",
        "",
    ]
    total = 0
    for l in range(lmax + 1):
        X = rotation_x90(l)
        assert np.abs(X @ X.T - np.eye(2 * l + 1)).max() < 1e-13
        total += int((X != 0).sum())
        out.append("template <> struct XRot<%d> {" % l)
        out += emit_apply("p", X, l)
        out += emit_apply("m", X.T.copy(), l)
        out.append("};")
        out.append("")
    out.append("constexpr int kRotLmax = %d;" % lmax)
    out.append("")
    out.append("}  // namespace wlc")
    path = os.path.join(here, "wlc_rot_gen.cuh")
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    print("wrote", path, "nonzeros", total)


if __name__ == "__main__":
    main()
