// wlc_host.cpp -- host-side set-up of the harmonic algebra and of the
// factorised k-space operator.
//
// Reference (file:line, tjz2026/wormlike-chain-triblock):
//   three_j / triple_product / basis      SPH_mod.f90:11-233
//   Rx, Ry, Rz, Theta and J tensors        init_array_2dcomp_mod.f90:142-375
//   G(k) = c0 + ds*Loa*l(l+1)/(2 kappa) + i sigma ds (k . R)
//                                          Gmatrix_2dcomp_mod.f90:384-500
//
// The reference inverts G(k) densely per wavevector (zgetrf/zgetri,
// matrix_inverse_mod.f90:85-124) and stores the inverse.  Here G(k) is
// factorised instead: k . R is the Galerkin matrix of multiplication by
// k . u in the real-harmonic basis, so with D(k) the real-harmonic rotation
// taking z to k,
//     k . R = |k| D Rz D^T,   G^-1 = D (A + i sigma ds |k| Rz)^-1 D^T,
// and A + i sigma ds |k| Rz splits into one tridiagonal system per m.
// D = Dz(alpha) Xm Dz(beta) Xp with Dz a rotation about z (2x2 blocks on
// the (m, -m) pairs) and Xp = X(+pi/2 about x), Xm = Xp^T.
//
// Under single-precision literal semantics the reference's Rx/Ry carry
// float-rounded sqrt factors that break exact rotation covariance at the
// 1e-8 level; dR holds that difference and the device applies a
// first-order correction with it (error O(|dR|^2) ~ 1e-16).
#include <cmath>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <random>

#include "wlc_internal.h"

namespace wlc {

// ---------------------------------------------------------------- literals
double lit_c0(int order, int real4) {  // Gmatrix_2dcomp_mod.f90:307-317
    if (order == 1) return 1.0;
    if (order == 2) return 1.5;
    return real4 ? (double)(11.0f / 6.0f) : 11.0 / 6.0;
}
double lit_third(int real4) { return real4 ? (double)(1.0f / 3.0f) : 1.0 / 3.0; }  // MDE_ABC.f90:290
double lit_thresh(int real4) { return real4 ? (double)1.0e-10f : 1.0e-10; }        // global_parameters.f90:60
double lit_kfactor(int n, double d, int real4) {  // Gmatrix_2dcomp_mod.f90:298-300, PI is REAL(SP)
    double twopi = real4 ? (double)(2.0f * 3.14159265358979323846f) : 2.0 * M_PI;
    return twopi / ((double)n * d);
}

// ------------------------------------------------------------ 3j symbols
static int sgn(int i) { return (i % 2 == 0) ? 1 : -1; }
static double factd(int l) {
    double f = 1.0;
    for (int i = 2; i <= l; ++i) f *= (double)i;
    return f;
}
static double fact_range(int a, int b) {
    double f = 1.0;
    for (int i = a; i <= b; ++i) f *= (double)i;
    return f;
}

// Racah formula with the (l1+l2+l3+1)! split at 20! used by the reference.
static double three_j(int l1, int l2, int l3, int m1, int m2, int m3) {
    if ((m1 + m2 + m3) != 0 || (l1 + l2 - l3) < 0 || (l1 - l2 + l3) < 0 || (l2 + l3 - l1) < 0 ||
        std::abs(l1) < std::abs(m1) || std::abs(l2) < std::abs(m2) || std::abs(l3) < std::abs(m3))
        return 0.0;
    const int kSplit = 20;
    double inv_big, inv_rest;
    if (l1 + l2 + l3 + 1 > kSplit) {
        inv_big = 1.0 / factd(kSplit);
        inv_rest = 1.0 / fact_range(kSplit + 1, l1 + l2 + l3 + 1);
    } else {
        inv_big = 1.0 / factd(l1 + l2 + l3 + 1);
        inv_rest = 1.0;
    }
    double pre = factd(l1 + l2 - l3) * factd(l1 - l2 + l3) * factd(l2 + l3 - l1) * inv_big;
    pre = pre * factd(l1 - m1) * factd(l1 + m1) * factd(l2 - m2) * factd(m2 + l2) * factd(l3 - m3) *
          factd(l3 + m3) * inv_rest;
    pre = sgn(l1 - l2 - m3) * std::sqrt(pre);
    int kmin = std::max(0, std::max(l2 - l3 - m1, l1 - l3 + m2));
    int kmax = std::min(l1 + l2 - l3, std::min(l1 - m1, l2 + m2));
    double acc = 0.0;
    for (int k = kmin; k <= kmax; ++k) {
        double t = pre / factd(k);
        t = t / factd(l1 + l2 - l3 - k);
        t = t / factd(l1 - m1 - k);
        t = t / factd(l2 + m2 - k);
        t = t / factd(l3 - l2 + m1 + k);
        t = t / factd(l3 - l1 - m2 + k);
        acc += sgn(k) * t;
    }
    return acc;
}

static double fsqrt_lit(double p, int real4) { return real4 ? (double)std::sqrt((float)p) : std::sqrt(p); }

// Integral of three real harmonics times sqrt(4 pi), with the reference's
// eleven sign cases and its literal-precision sqrt factors.
static double triple(int l1, int l2, int l3, int m1, int m2, int m3, int real4) {
    if (sgn(l1 + l2 + l3) == -1) return 0.0;
    const double P = (double)((2 * l1 + 1) * (2 * l2 + 1) * (2 * l3 + 1));
    const double s1 = fsqrt_lit(P, real4);
    const double s2 = s1 / (real4 ? (double)std::sqrt(2.0f) : std::sqrt(2.0));
    const double j0 = three_j(l1, l2, l3, 0, 0, 0);
    if (m1 == 0 && m2 == 0 && m3 == 0) return s1 * j0 * j0;
    if (m1 > 0 && m2 > 0 && m3 > 0) {
        double h = real4 ? (double)std::sqrt((float)P / 2.0f) : std::sqrt(P / 2.0);
        return (h * j0) * (sgn(m1) * three_j(l1, l2, l3, -m1, m2, m3) + sgn(m2) * three_j(l1, l2, l3, m1, -m2, m3) +
                           sgn(m3) * three_j(l1, l2, l3, m1, m2, -m3));
    }
    if (m1 == 0 && m2 > 0 && m3 > 0) return sgn(m2) * s1 * j0 * three_j(l1, l2, l3, 0, -m2, m3);
    if (m1 > 0 && m2 == 0 && m3 > 0) return sgn(m1) * s1 * j0 * three_j(l1, l2, l3, -m1, 0, m3);
    if (m1 > 0 && m2 > 0 && m3 == 0) return sgn(m1) * s1 * j0 * three_j(l1, l2, l3, -m1, m2, 0);
    if (m1 == 0 && m2 < 0 && m3 < 0) return sgn(m2) * s1 * j0 * three_j(l1, l2, l3, 0, m2, -m3);
    if (m1 < 0 && m2 == 0 && m3 < 0) return sgn(m1) * s1 * j0 * three_j(l1, l2, l3, m1, 0, -m3);
    if (m1 < 0 && m2 < 0 && m3 == 0) return sgn(m1) * s1 * j0 * three_j(l1, l2, l3, m1, -m2, 0);
    if (m1 > 0 && m2 < 0 && m3 < 0)
        return (s2 * j0) * (sgn(m2) * three_j(l1, l2, l3, m1, m2, -m3) + sgn(m3) * three_j(l1, l2, l3, m1, -m2, m3) -
                            sgn(m1) * three_j(l1, l2, l3, m1, m2, m3));
    if (m1 < 0 && m2 > 0 && m3 < 0)
        return (s2 * j0) * (sgn(m1) * three_j(l1, l2, l3, m1, m2, -m3) - sgn(m2) * three_j(l1, l2, l3, m1, m2, m3) +
                            sgn(m3) * three_j(l1, l2, l3, -m1, m2, m3));
    if (m1 < 0 && m2 < 0 && m3 > 0)
        return (s2 * j0) * (sgn(m1) * three_j(l1, l2, l3, m1, -m2, m3) + sgn(m2) * three_j(l1, l2, l3, -m1, m2, m3) -
                            sgn(m3) * three_j(l1, l2, l3, m1, m2, m3));
    return 0.0;
}

static double lit_ratio(double a, double b, int real4) {
    return real4 ? (double)((float)a / std::sqrt((float)b)) : a / std::sqrt(b);
}

static void build_coupling(int L, int real4, std::vector<double> R[3], std::vector<double> T[5],
                           std::vector<double> J[5]) {
    const int M = (L + 1) * (L + 1);
    const double cR = lit_ratio(1.0, 3.0, real4);
    const double c15 = lit_ratio(1.0, 15.0, real4);
    const double c5 = lit_ratio(1.0, 5.0, real4);
    const double c2_15 = lit_ratio(2.0, 15.0, real4);
    const double cJ2 = real4 ? (double)(-1.0f / (3.0f * std::sqrt(5.0f))) : -1.0 / (3.0 * std::sqrt(5.0));
    for (int a = 0; a < 3; ++a) R[a].assign((size_t)M * M, 0.0);
    for (int a = 0; a < 5; ++a) {
        T[a].assign((size_t)M * M, 0.0);
        J[a].assign((size_t)M * M, 0.0);
    }
    for (int i = 0; i < M; ++i) {
        const int li = basis_l(i), mi = basis_m(i);
        for (int j = 0; j < M; ++j) {
            const int lj = basis_l(j), mj = basis_m(j);
            const size_t o = (size_t)i * M + j;
            R[0][o] = -cR * triple(li, lj, 1, mi, mj, 1, real4);
            R[1][o] = -cR * triple(li, lj, 1, mi, mj, -1, real4);
            R[2][o] = cR * triple(li, lj, 1, mi, mj, 0, real4);
            const double t22 = triple(li, lj, 2, mi, mj, 2, real4), t20 = triple(li, lj, 2, mi, mj, 0, real4);
            const double t2m2 = triple(li, lj, 2, mi, mj, -2, real4), t21 = triple(li, lj, 2, mi, mj, 1, real4);
            const double t2m1 = triple(li, lj, 2, mi, mj, -1, real4);
            T[0][o] = c15 * t22;
            T[1][o] = c5 * t20;
            T[2][o] = c2_15 * t2m2;
            T[3][o] = -c2_15 * t21;
            T[4][o] = -c2_15 * t2m1;
            J[0][o] = c15 * t22 + cJ2 * t20;
            J[1][o] = -c15 * t22 + cJ2 * t20;
            J[2][o] = c15 * t2m2;
            J[3][o] = -c15 * t21;
            J[4][o] = -c15 * t2m1;
        }
    }
}

// ------------------------------------------------- real harmonics / rotation
// Real harmonics with the reference's convention (checked against its
// triple products): Y_l0 = N P_l^0, Y_l,m>0 = sqrt2 N P_l^m cos(m phi),
// Y_l,m<0 = sqrt2 N P_l^|m| sin(|m| phi), Condon-Shortley phase in P_l^m.
static void real_harmonics(int L, double ct, double phi, double* Y) {
    const double st = std::sqrt(std::max(0.0, 1.0 - ct * ct));
    std::vector<double> P((size_t)(L + 1) * (L + 1), 0.0);
    auto p = [&](int l, int m) -> double& { return P[(size_t)l * (L + 1) + m]; };
    p(0, 0) = 1.0;
    for (int m = 1; m <= L; ++m) p(m, m) = -(2 * m - 1) * st * p(m - 1, m - 1);
    for (int m = 0; m < L; ++m) p(m + 1, m) = (2 * m + 1) * ct * p(m, m);
    for (int m = 0; m <= L; ++m)
        for (int l = m + 2; l <= L; ++l) p(l, m) = ((2 * l - 1) * ct * p(l - 1, m) - (l + m - 1) * p(l - 2, m)) / (l - m);
    for (int l = 0; l <= L; ++l)
        for (int m = -l; m <= l; ++m) {
            const int am = std::abs(m);
            const double N = std::sqrt((2 * l + 1) / (4.0 * M_PI) * factd(l - am) / factd(l + am));
            const int i = l * l + l + m;
            if (m == 0)
                Y[i] = N * p(l, 0);
            else if (m > 0)
                Y[i] = std::sqrt(2.0) * N * p(l, am) * std::cos(am * phi);
            else
                Y[i] = std::sqrt(2.0) * N * p(l, am) * std::sin(am * phi);
        }
}

static void gauss_legendre(int n, std::vector<double>& x, std::vector<double>& w) {
    x.resize(n);
    w.resize(n);
    for (int i = 0; i < n; ++i) {
        double z = std::cos(M_PI * (i + 0.75) / (n + 0.5));
        for (int it = 0; it < 100; ++it) {
            double p0 = 1.0, p1 = z;
            for (int k = 2; k <= n; ++k) {
                double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
                p0 = p1;
                p1 = p2;
            }
            // p1 = P_n(z), p0 = P_{n-1}(z)
            double dp = n * (z * p1 - p0) / (z * z - 1.0);
            double dz = p1 / dp;
            z -= dz;
            if (std::fabs(dz) < 1e-16) break;
        }
        double p0 = 1.0, p1 = z;
        for (int k = 2; k <= n; ++k) {
            double p2 = ((2 * k - 1) * z * p1 - (k - 1) * p0) / k;
            p0 = p1;
            p1 = p2;
        }
        double dp = n * (z * p1 - p0) / (z * z - 1.0);
        x[i] = z;
        w[i] = 2.0 / ((1.0 - z * z) * dp * dp);
    }
}

// Matrix of the rotation by +pi/2 about x acting on harmonic coefficients:
// Xp_ij = int Y_i(u) Y_j(Q^T u) du, Q = Rx(pi/2), by exact quadrature.
static void rotation_x90(int L, std::vector<double>& X) {
    const int M = (L + 1) * (L + 1);
    const int nt = L + 2, np = 2 * L + 3;
    std::vector<double> gx, gw;
    gauss_legendre(nt, gx, gw);
    X.assign((size_t)M * M, 0.0);
    std::vector<double> Y(M), Y2(M);
    for (int a = 0; a < nt; ++a)
        for (int b = 0; b < np; ++b) {
            const double ct = gx[a], phi = 2.0 * M_PI * b / np, wq = gw[a] * 2.0 * M_PI / np;
            const double st = std::sqrt(std::max(0.0, 1.0 - ct * ct));
            const double ux = st * std::cos(phi), uy = st * std::sin(phi), uz = ct;
            // Q^T u = (ux, uz, -uy)
            const double vx = ux, vy = uz, vz = -uy;
            real_harmonics(L, ct, phi, Y.data());
            real_harmonics(L, vz, std::atan2(vy, vx), Y2.data());
            for (int i = 0; i < M; ++i)
                for (int j = 0; j < M; ++j) X[(size_t)i * M + j] += wq * Y[i] * Y2[j];
        }
    for (auto& v : X)
        if (std::fabs(v) < 1e-12) v = 0.0;
}

static void to_csr(const std::vector<double>& A, int M, bool transpose, std::vector<int>& ptr,
                   std::vector<int>& col, std::vector<double>& val) {
    ptr.assign(M + 1, 0);
    col.clear();
    val.clear();
    for (int i = 0; i < M; ++i) {
        for (int j = 0; j < M; ++j) {
            double v = transpose ? A[(size_t)j * M + i] : A[(size_t)i * M + j];
            if (v != 0.0) {
                col.push_back(j);
                val.push_back(v);
            }
        }
        ptr[i + 1] = (int)val.size();
    }
}

// ----------------------------------------------------- host factored solve
using cd = std::complex<double>;

static void dz_apply(int L, double gamma, std::vector<cd>& v) {
    for (int l = 1; l <= L; ++l)
        for (int m = 1; m <= l; ++m) {
            const int ic = l * l + l + m, is = l * l + l - m;
            const double c = std::cos(m * gamma), s = std::sin(m * gamma);
            const cd a = v[ic], b = v[is];
            v[ic] = c * a - s * b;
            v[is] = s * a + c * b;
        }
}

static void csr_apply(const std::vector<int>& ptr, const std::vector<int>& col, const std::vector<double>& val,
                      const std::vector<cd>& in, std::vector<cd>& out) {
    const int M = (int)ptr.size() - 1;
    out.assign(M, cd(0, 0));
    for (int i = 0; i < M; ++i) {
        cd acc(0, 0);
        for (int e = ptr[i]; e < ptr[i + 1]; ++e) acc += val[e] * in[col[e]];
        out[i] = acc;
    }
}

static void tridiag_solve(const BasisTables& t, double c0, double diag_coef, double tk, std::vector<cd>& v) {
    const int L = t.L;
    for (int m = -L; m <= L; ++m) {
        const int am = std::abs(m);
        const int n = L - am + 1;
        std::vector<double> d(n), g(n);
        std::vector<cd> y(n);
        for (int j = 0; j < n; ++j) {
            const int l = am + j;
            const double A = c0 + diag_coef * l * (l + 1);
            const int idx = l * l + l + m;
            if (j == 0) {
                d[0] = A;
                y[0] = v[idx];
            } else {
                const int prev = (l - 1) * (l - 1) + (l - 1) + m;
                const double e = tk * t.zoff[prev];
                g[j] = e / d[j - 1];
                d[j] = A + e * g[j];
                y[j] = v[idx] - cd(0, g[j]) * y[j - 1];
            }
        }
        std::vector<cd> x(n);
        x[n - 1] = y[n - 1] / d[n - 1];
        for (int j = n - 2; j >= 0; --j) {
            const int l = am + j;
            const int idx = l * l + l + m;
            const double e = tk * t.zoff[idx];
            x[j] = (y[j] - cd(0, e) * x[j + 1]) / d[j];
        }
        for (int j = 0; j < n; ++j) {
            const int l = am + j;
            v[l * l + l + m] = x[j];
        }
    }
}

static void cov_solve(const BasisTables& t, double c0, double diag_coef, const double k[3], double ds, int sigma,
                      std::vector<cd>& v) {
    const double rho = std::sqrt(k[0] * k[0] + k[1] * k[1]);
    const double kn = std::sqrt(rho * rho + k[2] * k[2]);
    const double alpha = rho > 0 ? std::atan2(k[1], k[0]) : 0.0;
    const double beta = kn > 0 ? std::atan2(rho, k[2]) : 0.0;
    std::vector<cd> w;
    dz_apply(t.L, -alpha, v);
    csr_apply(t.xp_ptr, t.xp_col, t.xp_val, v, w);
    dz_apply(t.L, -beta, w);
    csr_apply(t.xm_ptr, t.xm_col, t.xm_val, w, v);
    tridiag_solve(t, c0, diag_coef, sigma * ds * kn, v);
    csr_apply(t.xp_ptr, t.xp_col, t.xp_val, v, w);
    dz_apply(t.L, beta, w);
    csr_apply(t.xm_ptr, t.xm_col, t.xm_val, w, v);
    dz_apply(t.L, alpha, v);
}

void host_factored_solve(const BasisTables& t, double c0, double diag_coef, const double k[3], double ds, int sigma,
                         const double* bre, const double* bim, double* xre, double* xim, bool correct) {
    const int M = t.M;
    std::vector<cd> v(M);
    for (int i = 0; i < M; ++i) v[i] = cd(bre[i], bim[i]);
    cov_solve(t, c0, diag_coef, k, ds, sigma, v);
    if (correct) {
        std::vector<cd> r(M, cd(0, 0));
        for (int a = 0; a < 3; ++a)
            for (size_t e = 0; e < t.dR[a].size(); ++e)
                r[t.dR[a].row[e]] += cd(0, sigma * ds * k[a] * t.dR[a].val[e]) * v[t.dR[a].col[e]];
        cov_solve(t, c0, diag_coef, k, ds, sigma, r);
        for (int i = 0; i < M; ++i) v[i] -= r[i];
    }
    for (int i = 0; i < M; ++i) {
        xre[i] = v[i].real();
        xim[i] = v[i].imag();
    }
}

void host_dense_G(const BasisTables& t, double c0, double diag_coef, const double k[3], double ds,
                  std::vector<double>& gre, std::vector<double>& gim) {
    const int M = t.M;
    gre.assign((size_t)M * M, 0.0);
    gim.assign((size_t)M * M, 0.0);
    for (int i = 0; i < M; ++i)
        for (int j = 0; j < M; ++j) {
            const size_t o = (size_t)i * M + j;
            gim[o] = ds * (t.R[0][o] * k[0] + t.R[1][o] * k[1] + t.R[2][o] * k[2]);
        }
    for (int j = 0; j < M; ++j) {
        const int l = basis_l(j);
        gre[(size_t)j * M + j] = c0 + diag_coef * l * (l + 1);
    }
}

static void dense_solve(int M, std::vector<cd> A, std::vector<cd>& b) {
    for (int k = 0; k < M; ++k) {
        int p = k;
        for (int i = k + 1; i < M; ++i)
            if (std::abs(A[(size_t)i * M + k]) > std::abs(A[(size_t)p * M + k])) p = i;
        if (p != k) {
            for (int j = 0; j < M; ++j) std::swap(A[(size_t)k * M + j], A[(size_t)p * M + j]);
            std::swap(b[k], b[p]);
        }
        for (int i = k + 1; i < M; ++i) {
            cd f = A[(size_t)i * M + k] / A[(size_t)k * M + k];
            for (int j = k; j < M; ++j) A[(size_t)i * M + j] -= f * A[(size_t)k * M + j];
            b[i] -= f * b[k];
        }
    }
    for (int i = M - 1; i >= 0; --i) {
        cd s = b[i];
        for (int j = i + 1; j < M; ++j) s -= A[(size_t)i * M + j] * b[j];
        b[i] = s / A[(size_t)i * M + i];
    }
}

bool build_basis_tables(int L, int real4, BasisTables& t, std::string& err) {
    t.L = L;
    t.M = (L + 1) * (L + 1);
    t.real4 = real4;
    const int M = t.M;
    build_coupling(L, real4, t.R, t.T, t.J);
    std::vector<double> Rex[3], Tex[5], Jex[5];
    build_coupling(L, 0, Rex, Tex, Jex);

    // rotation tables
    std::vector<double> X;
    rotation_x90(L, X);
    to_csr(X, M, false, t.xp_ptr, t.xp_col, t.xp_val);
    to_csr(X, M, true, t.xm_ptr, t.xm_col, t.xm_val);

    // per-(l, l+1) scale that maps the exact couplings onto the reference's Rz
    std::vector<double> rho(L + 1, 1.0);
    for (int l = 0; l < L; ++l) {
        const size_t o = (size_t)(l * l + l) * M + (size_t)((l + 1) * (l + 1) + (l + 1));
        rho[l] = t.R[2][o] / Rex[2][o];
    }
    t.zoff.assign(M, 0.0);
    for (int i = 0; i < M; ++i) {
        const int l = basis_l(i), m = basis_m(i);
        if (l < L) t.zoff[i] = t.R[2][(size_t)i * M + (size_t)((l + 1) * (l + 1) + (l + 1) + m)];
    }
    double rmax = 0.0;
    for (int a = 0; a < 3; ++a)
        for (double v : t.R[a]) rmax = std::max(rmax, std::fabs(v));
    t.max_dR = 0.0;
    for (int a = 0; a < 3; ++a) {
        t.dR[a] = Triplets();
        for (int i = 0; i < M; ++i)
            for (int j = 0; j < M; ++j) {
                const int li = basis_l(i), lj = basis_l(j);
                const size_t o = (size_t)i * M + j;
                double s = 1.0;
                if (lj == li + 1) s = rho[li];
                if (li == lj + 1) s = rho[lj];
                const double d = t.R[a][o] - s * Rex[a][o];
                if (std::fabs(d) > 1e-15 * rmax) {
                    t.dR[a].row.push_back(i);
                    t.dR[a].col.push_back(j);
                    t.dR[a].val.push_back(d);
                    t.max_dR = std::max(t.max_dR, std::fabs(d));
                }
            }
    }
    const double thr = lit_thresh(real4);
    for (int a = 0; a < 5; ++a) {
        t.Tsp[a] = Triplets();
        t.Jsp[a] = Triplets();
        for (int i = 0; i < M; ++i)
            for (int j = 0; j < M; ++j) {
                const size_t o = (size_t)i * M + j;
                if (t.T[a][o] != 0.0) {
                    t.Tsp[a].row.push_back(i);
                    t.Tsp[a].col.push_back(j);
                    t.Tsp[a].val.push_back(t.T[a][o]);
                }
                if (std::fabs(t.J[a][o]) >= thr) {
                    t.Jsp[a].row.push_back(i);
                    t.Jsp[a].col.push_back(j);
                    t.Jsp[a].val.push_back(t.J[a][o]);
                }
            }
    }

    // self-check: factorised solve (with the correction when dR != 0)
    // against a dense LU solve of the reference G(k)
    std::mt19937_64 rng(12345);
    std::normal_distribution<double> nd(0.0, 1.0);
    const bool correct = !t.dR[0].val.empty() || !t.dR[1].val.empty() || !t.dR[2].val.empty();
    double worst = 0.0;
    for (int trial = 0; trial < 6; ++trial) {
        double k[3] = {nd(rng) * 60.0, nd(rng) * 60.0, nd(rng) * 60.0};
        if (trial == 0) k[0] = k[1] = 0.0;  // k along z
        if (trial == 1) k[0] = k[1] = k[2] = 0.0;
        const double ds = 0.005, c0 = lit_c0(1 + trial % 3, real4), dc = 0.005 * 1.3 / 1.0;
        const int sigma = (trial % 2) ? -1 : 1;
        std::vector<double> gre, gim;
        host_dense_G(t, c0, dc, k, ds, gre, gim);
        std::vector<cd> A((size_t)M * M);
        for (size_t o = 0; o < A.size(); ++o) A[o] = cd(gre[o], sigma * gim[o]);
        std::vector<double> bre(M), bim(M), xre(M), xim(M);
        std::vector<cd> b(M);
        for (int i = 0; i < M; ++i) {
            bre[i] = nd(rng);
            bim[i] = nd(rng);
            b[i] = cd(bre[i], bim[i]);
        }
        dense_solve(M, A, b);
        host_factored_solve(t, c0, dc, k, ds, sigma, bre.data(), bim.data(), xre.data(), xim.data(), correct);
        double num = 0.0, den = 0.0;
        for (int i = 0; i < M; ++i) {
            num = std::max(num, std::abs(cd(xre[i], xim[i]) - b[i]));
            den = std::max(den, std::abs(b[i]));
        }
        worst = std::max(worst, num / den);
    }
    if (!(worst < 1e-11)) {
        char buf[160];
        std::snprintf(buf, sizeof buf, "factorised G(k)^-1 self-check failed: rel err %.3e (L=%d)", worst, L);
        err = buf;
        return false;
    }
    return true;
}

}  // namespace wlc
