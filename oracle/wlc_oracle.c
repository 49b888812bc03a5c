/*
 * wlc_oracle.c -- CPU FP64 restatement of the wormlike-chain MDE hot path of
 * tjz2026/wormlike-chain-triblock (Fortran 90, MPI/FFTW/MKL).
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the oracle: only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference leg load it.
 * The product (libwlc, CUDA sm_103a) never links or calls it.
 *
 * Parity status: the reference cannot be compiled or run (no Fortran compiler,
 * MPI, FFTW or MKL; undefined routines iterate / w_init_or_not /
 * AB_melt_driver; MDE_ABC.f90 does not parse).  Parity with the reference
 * itself is therefore UNPINNED.  This restatement is pinned instead against
 * (a) exact Wigner-3j / real Gaunt coefficients (sympy), (b) numpy.fft,
 * (c) numpy.linalg.solve, (d) analytic known answers (homogeneous fields),
 * and (e) an independent numpy restatement -- see tests/.
 *
 * What it follows (file:line in the reference):
 *   three_j / triple_product / basis      SPH_mod.f90:11-233
 *   Rx/Ry/Rz, Theta and J tensors          init_array_2dcomp_mod.f90:142-375
 *   G(k) = c0 + ds*Loa*l(l+1)/(2kappa) + i*sigma*ds*(k.R)
 *                                          Gmatrix_2dcomp_mod.f90:384-500,
 *                                          Gmatrix_mod.f90:765-908,
 *                                          Gmatrix_mod-old.f90:446-518 (ABC table)
 *   k folding n -> n or n-N                Gmatrix_2dcomp_mod.f90:450-467
 *   BDF1/2/3 right-hand side (init_pr)     MDE_ABC.f90:223-383,
 *                                          wormlike_MDE_2dcomp_mod.f90:323-343,484-502
 *   R2C forward FFT, G^-1 apply, C2R / N^3 wormlike_MDE_2dcomp_mod.f90:357-455
 *   ABC sweep driver (block order, BDF ramp) MDE_ABC.f90:8-88
 *   Maier-Saupe Theta(r)                   wormlike_MDE_2dcomp_mod.f90:5-110
 *   Q, block densities, junctions, S       SCFT_Density_FE_ABC.f90:3-271,
 *                                          SCFT_Density_FE.f90:48-220
 *   Simpson integrators                    utility_mod.f90:195-374
 *   Sum_sparse_2D (q^T J q*)               utility_mod.f90:376-407
 *   free energy                            SCFT_Density_FE.f90:273-342 (AB form,
 *                                          generalised to three blocks)
 *
 * Second contour-step scheme (scheme = 1, orc_set_scheme), which has no
 * counterpart in the reference's harmonic-basis solver: the operator split
 *   q(s) = e^{-w ds/2} C2R[ G_CN(k) R2C[ e^{-w ds/2} q(s-1) ] ] / N^3,
 *   G_CN = (I + ds/2 A)^-1 (I - ds/2 A) = 2 (I + ds/2 A)^-1 - I,
 *   A = Loa l(l+1)/(2 kappa) + i sigma (k.R),
 * i.e. Strang splitting of the field term around a Crank-Nicolson step of
 * the orientation and streaming terms.  Its real-space half steps follow the
 * reference's angular-grid split-operator solver
 * (split_operator_MDE_mod.f90:163-166,290-420); (I + ds/2 A) is the
 * reference's G with c0 = 1 and ds/2.  Parity with the reference is
 * unpinned for this scheme by construction.
 *
 * Literal semantics.  The reference writes constants such as 11.0/6.0,
 * 1.0/3.0, 1.0/sqrt(3.0), sqrt(1.0*(2l1+1)...) and PI (declared REAL(SP)) as
 * default-kind reals, so a standard build evaluates them in single precision
 * and stores them into REAL(8) variables.  A build with a default-real-8 flag
 * evaluates them in double.  `real4 = 1` reproduces the former (the standard
 * semantics), `real4 = 0` the latter.
 *
 * Layouts (C order, last index fastest):
 *   real-space grid index r = (z*ny + y)*nx + x   (the reference's x-pencil k
 *     index on one rank, grid_mod.f90:356-379)
 *   k-space (R2C) index kk = (kz*ny + ky)*(nx/2+1) + kx
 *   propagators q[s][i][r]; fields w[blk][r]; M_OP mop[a*3+b][r]
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef double complex cplx;

/* ------------------------------------------------------------------ */
/* Basis algebra: SPH_mod.f90                                           */
/* ------------------------------------------------------------------ */

static int sign_ov(int i) { return (i % 2 == 0) ? 1 : -1; } /* SPH_mod.f90:145-156 */

static double fact(int l) { /* SPH_mod.f90:158-171 */
    double f = 1.0;
    for (int i = 2; i <= l; ++i) f *= (double)i;
    return f;
}

static double fact_con(int m1, int m2) { /* SPH_mod.f90:174-189 */
    double f = 1.0;
    for (int i = m1; i <= m2; ++i) f *= (double)i;
    return f;
}

/* Wigner 3j symbol, evaluated with the reference's formula and its
 * FACTVALUE=20 split of (l1+l2+l3+1)!  (SPH_mod.f90:101-142). */
double orc_three_j(int l1, int l2, int l3, int m1, int m2, int m3) {
    const int FACTVALUE = 20;
    if ((m1 + m2 + m3) != 0 || (l1 + l2 - l3) < 0 || (l1 - l2 + l3) < 0 ||
        (l2 + l3 - l1) < 0 || abs(l1) < abs(m1) || abs(l2) < abs(m2) || abs(l3) < abs(m3))
        return 0.0;
    double temp1, temp2;
    if ((l1 + l2 + l3 + 1) > FACTVALUE) {
        temp1 = 1.0 / fact(FACTVALUE);
        temp2 = 1.0 / fact_con(FACTVALUE + 1, l1 + l2 + l3 + 1);
    } else {
        temp1 = 1.0 / fact(l1 + l2 + l3 + 1);
        temp2 = 1.0;
    }
    double temp = fact(l1 + l2 - l3) * fact(l1 - l2 + l3) * fact(l2 + l3 - l1) * temp1;
    temp = temp * fact(l1 - m1) * fact(l1 + m1) * fact(l2 - m2) * fact(m2 + l2) * fact(l3 - m3) *
           fact(l3 + m3) * temp2;
    temp = sign_ov(l1 - l2 - m3) * sqrt(temp);
    int kmin = 0, kmax;
    if (l2 - l3 - m1 > kmin) kmin = l2 - l3 - m1;
    if (l1 - l3 + m2 > kmin) kmin = l1 - l3 + m2;
    kmax = l1 + l2 - l3;
    if (l1 - m1 < kmax) kmax = l1 - m1;
    if (l2 + m2 < kmax) kmax = l2 + m2;
    double suma = 0.0;
    for (int k = kmin; k <= kmax; ++k) {
        double tk = temp / fact(k);
        tk = tk / fact(l1 + l2 - l3 - k);
        tk = tk / fact(l1 - m1 - k);
        tk = tk / fact(l2 + m2 - k);
        tk = tk / fact(l3 - l2 + m1 + k);
        tk = tk / fact(l3 - l1 - m2 + k);
        suma += sign_ov(k) * tk;
    }
    return suma;
}

/* sqrt of a small integer product written as sqrt(1.0*...) in the reference:
 * single precision under the default-kind literal semantics. */
static double lit_sqrt(double p, int real4) {
    return real4 ? (double)sqrtf((float)p) : sqrt(p);
}

/* Real-spherical-harmonic triple product integral (SPH_mod.f90:11-98), with
 * the same 11 sign cases and the same single-precision sqrt factors. */
double orc_triple_product(int l1, int l2, int l3, int m1, int m2, int m3, int real4) {
    double P = (double)((2 * l1 + 1) * (2 * l2 + 1) * (2 * l3 + 1));
    double sqrt1 = lit_sqrt(P, real4);
    double sqrt2 = sqrt1 / (real4 ? (double)sqrtf(2.0f) : sqrt(2.0));
    double trpd = 0.0, temp, suma;
    if (sign_ov(l1 + l2 + l3) == -1) return 0.0;
    if (m1 == 0 && m2 == 0 && m3 == 0) { /* 1 */
        temp = orc_three_j(l1, l2, l3, 0, 0, 0);
        trpd = lit_sqrt(P, real4) * temp * temp;
    } else if (m1 > 0 && m2 > 0 && m3 > 0) { /* 2 */
        temp = real4 ? (double)sqrtf((float)P / 2.0f) : sqrt(P / 2.0);
        temp = temp * orc_three_j(l1, l2, l3, 0, 0, 0);
        suma = sign_ov(m1) * orc_three_j(l1, l2, l3, -m1, m2, m3) +
               sign_ov(m2) * orc_three_j(l1, l2, l3, m1, -m2, m3) +
               sign_ov(m3) * orc_three_j(l1, l2, l3, m1, m2, -m3);
        trpd = temp * suma;
    } else if (m1 == 0 && m2 > 0 && m3 > 0) { /* 3 */
        temp = sign_ov(m2) * lit_sqrt(P, real4);
        trpd = temp * orc_three_j(l1, l2, l3, 0, 0, 0) * orc_three_j(l1, l2, l3, 0, -m2, m3);
    } else if (m1 > 0 && m2 == 0 && m3 > 0) { /* 4 */
        temp = sign_ov(m1) * lit_sqrt(P, real4);
        trpd = temp * orc_three_j(l1, l2, l3, 0, 0, 0) * orc_three_j(l1, l2, l3, -m1, 0, m3);
    } else if (m1 > 0 && m2 > 0 && m3 == 0) { /* 5 */
        temp = sign_ov(m1) * lit_sqrt(P, real4);
        trpd = temp * orc_three_j(l1, l2, l3, 0, 0, 0) * orc_three_j(l1, l2, l3, -m1, m2, 0);
    } else if (m1 == 0 && m2 < 0 && m3 < 0) { /* 6 */
        temp = sign_ov(m2) * sqrt1;
        trpd = temp * orc_three_j(l1, l2, l3, 0, 0, 0) * orc_three_j(l1, l2, l3, 0, m2, -m3);
    } else if (m1 < 0 && m2 == 0 && m3 < 0) { /* 7 */
        temp = sign_ov(m1) * sqrt1;
        trpd = temp * orc_three_j(l1, l2, l3, 0, 0, 0) * orc_three_j(l1, l2, l3, m1, 0, -m3);
    } else if (m1 < 0 && m2 < 0 && m3 == 0) { /* 8 */
        temp = sign_ov(m1) * sqrt1;
        trpd = temp * orc_three_j(l1, l2, l3, 0, 0, 0) * orc_three_j(l1, l2, l3, m1, -m2, 0);
    } else if (m1 > 0 && m2 < 0 && m3 < 0) { /* 9 */
        temp = sqrt2 * orc_three_j(l1, l2, l3, 0, 0, 0);
        suma = sign_ov(m2) * orc_three_j(l1, l2, l3, m1, m2, -m3) +
               sign_ov(m3) * orc_three_j(l1, l2, l3, m1, -m2, m3) -
               sign_ov(m1) * orc_three_j(l1, l2, l3, m1, m2, m3);
        trpd = temp * suma;
    } else if (m1 < 0 && m2 > 0 && m3 < 0) { /* 10 */
        temp = sqrt2 * orc_three_j(l1, l2, l3, 0, 0, 0);
        suma = sign_ov(m1) * orc_three_j(l1, l2, l3, m1, m2, -m3) -
               sign_ov(m2) * orc_three_j(l1, l2, l3, m1, m2, m3) +
               sign_ov(m3) * orc_three_j(l1, l2, l3, -m1, m2, m3);
        trpd = temp * suma;
    } else if (m1 < 0 && m2 < 0 && m3 > 0) { /* 11 */
        temp = sqrt2 * orc_three_j(l1, l2, l3, 0, 0, 0);
        suma = sign_ov(m1) * orc_three_j(l1, l2, l3, m1, -m2, m3) +
               sign_ov(m2) * orc_three_j(l1, l2, l3, -m1, m2, m3) -
               sign_ov(m3) * orc_three_j(l1, l2, l3, m1, m2, m3);
        trpd = temp * suma;
    } else {
        trpd = 0.0;
    }
    return trpd;
}

/* basis index i <-> (l, m), l = 0..L, m = -l..l  (SPH_mod.f90:192-233) */
static void basis_lm(int i, int* l, int* m) {
    int ll = (int)floor(sqrt((double)i) + 1e-9);
    while ((ll + 1) * (ll + 1) <= i) ++ll;
    while (ll * ll > i) --ll;
    *l = ll;
    *m = i - ll * ll - ll;
}

/* literal a/sqrt(b) constant: single precision under real4 */
static double lit_ratio(double a, double b, int real4) {
    return real4 ? (double)((float)a / sqrtf((float)b)) : a / sqrt(b);
}

enum {
    ORC_RX = 0, ORC_RY, ORC_RZ, ORC_T1122, ORC_T33, ORC_T12, ORC_T13, ORC_T23,
    ORC_J11, ORC_J22, ORC_J12, ORC_J13, ORC_J23, ORC_NMAT
};

/* Coupling matrices of init_array_2dcomp_mod.f90:166-375 (M x M, row-major
 * [i*M + j] = matrix(i, j)). */
static void build_basis(int L, int real4, double** mats) {
    int M = (L + 1) * (L + 1);
    double cR = lit_ratio(1.0, 3.0, real4);                      /* 1/sqrt(3)   :166,177 */
    double c15 = lit_ratio(1.0, 15.0, real4);                    /* 1/sqrt(15)  :188     */
    double c5 = lit_ratio(1.0, 5.0, real4);                      /* 1/sqrt(5)   :196     */
    double c2_15 = lit_ratio(2.0, 15.0, real4);                  /* 2/sqrt(15)  :204     */
    double cJ2 = real4 ? (double)(-1.0f / (3.0f * sqrtf(5.0f))) : -1.0 / (3.0 * sqrt(5.0)); /* :277 */
    for (int t = 0; t < ORC_NMAT; ++t) memset(mats[t], 0, sizeof(double) * M * M);
    for (int i = 0; i < M; ++i) {
        int li, mi;
        basis_lm(i, &li, &mi);
        for (int j = 0; j < M; ++j) {
            int lj, mj;
            basis_lm(j, &lj, &mj);
            size_t o = (size_t)i * M + j;
            mats[ORC_RX][o] = -cR * orc_triple_product(li, lj, 1, mi, mj, 1, real4);
            mats[ORC_RY][o] = -cR * orc_triple_product(li, lj, 1, mi, mj, -1, real4);
            mats[ORC_RZ][o] = cR * orc_triple_product(li, lj, 1, mi, mj, 0, real4);
            double t22 = orc_triple_product(li, lj, 2, mi, mj, 2, real4);
            double t20 = orc_triple_product(li, lj, 2, mi, mj, 0, real4);
            double t2m2 = orc_triple_product(li, lj, 2, mi, mj, -2, real4);
            double t21 = orc_triple_product(li, lj, 2, mi, mj, 1, real4);
            double t2m1 = orc_triple_product(li, lj, 2, mi, mj, -1, real4);
            mats[ORC_T1122][o] = c15 * t22;
            mats[ORC_T33][o] = c5 * t20;
            mats[ORC_T12][o] = c2_15 * t2m2;
            mats[ORC_T13][o] = -c2_15 * t21;
            mats[ORC_T23][o] = -c2_15 * t2m1;
            mats[ORC_J11][o] = c15 * t22 + cJ2 * t20;
            mats[ORC_J22][o] = -c15 * t22 + cJ2 * t20;
            mats[ORC_J12][o] = c15 * t2m2;
            mats[ORC_J13][o] = -c15 * t21;
            mats[ORC_J23][o] = -c15 * t2m1;
        }
    }
}

/* ------------------------------------------------------------------ */
/* FFT (own mixed-radix, FFTW sign conventions: forward e^{-i}, backward
 * e^{+i}, both unnormalised)                                           */
/* ------------------------------------------------------------------ */

typedef struct {
    int n;
    cplx* tw_f; /* exp(-2 pi i j / n) */
    cplx* tw_b; /* exp(+2 pi i j / n) */
} fft_plan;

static void plan_init(fft_plan* p, int n) {
    p->n = n;
    p->tw_f = (cplx*)malloc(sizeof(cplx) * n);
    p->tw_b = (cplx*)malloc(sizeof(cplx) * n);
    for (int j = 0; j < n; ++j) {
        double a = 2.0 * M_PI * (double)j / (double)n;
        p->tw_f[j] = cos(a) - I * sin(a);
        p->tw_b[j] = cos(a) + I * sin(a);
    }
}

static void plan_free(fft_plan* p) {
    free(p->tw_f);
    free(p->tw_b);
}

static int smallest_factor(int n) {
    if (n % 4 == 0 && n > 4) return 4;
    for (int p = 2; p * p <= n; ++p)
        if (n % p == 0) return p;
    return n;
}

/* recursive decimation-in-time; `twstride` = top_n / n */
static void fft_rec(const cplx* in, int istride, cplx* out, int n, const cplx* tw, int twstride,
                    int topn) {
    if (n == 1) {
        out[0] = in[0];
        return;
    }
    int p = smallest_factor(n);
    int m = n / p;
    for (int r = 0; r < p; ++r) fft_rec(in + (size_t)r * istride, istride * p, out + r * m, m, tw, twstride * p, topn);
    cplx tmp[128];
    for (int k = 0; k < m; ++k) {
        for (int q = 0; q < p; ++q) {
            cplx acc = 0.0;
            int kk = k + q * m;
            for (int r = 0; r < p; ++r) {
                long e = ((long)r * kk) % n;
                acc += tw[(size_t)e * twstride % topn] * out[r * m + k];
            }
            tmp[q] = acc;
        }
        for (int q = 0; q < p; ++q) out[k + q * m] = tmp[q];
    }
}

/* in-place 1D transform of `n` points spaced `stride` apart */
static void fft1d(cplx* data, int stride, const fft_plan* p, int backward, cplx* work) {
    int n = p->n;
    cplx* in = work;
    cplx* out = work + n;
    for (int j = 0; j < n; ++j) in[j] = data[(size_t)j * stride];
    fft_rec(in, 1, out, n, backward ? p->tw_b : p->tw_f, 1, n);
    for (int j = 0; j < n; ++j) data[(size_t)j * stride] = out[j];
}

/* ------------------------------------------------------------------ */
/* Context                                                             */
/* ------------------------------------------------------------------ */

#define ORC_MAXVAR 12

typedef struct {
    int order;    /* 1, 2, 3 (BDF); 4: I + ds/2 A of the split scheme */
    double kappa; /* block kappa */
    cplx* lu;     /* [nk][M][M] LU factors of G(sigma=+1) */
    int* piv;     /* [nk][M] */
} g_variant;

typedef struct {
    int n[3], nkx, nr, nk;
    int L, M, nmax, ns[3], nstart[3];
    double dx[3], ds, loa, kappa[3], chi[3], nmu, vol;
    int real4;
    double* mats[ORC_NMAT];
    double* w;   /* [3][nr] */
    double* mop; /* [9][nr] */
    int have_mop;
    double* qf;  /* [(nmax+1)][M][nr] */
    double* qb;
    fft_plan plan[3];
    g_variant var[ORC_MAXVAR];
    int nvar;
    int nthreads;
    int scheme; /* 0: the reference's BDF steps; 1: the operator split */
} orc_ctx;

static double lit_c0(int order, int real4) { /* Gmatrix_2dcomp_mod.f90:307-317 */
    if (order == 1) return 1.0;
    if (order == 2) return 1.5;
    return real4 ? (double)(11.0f / 6.0f) : 11.0 / 6.0;
}

static double lit_third(int real4) { /* temp=1.0/3.0, MDE_ABC.f90:290 */
    return real4 ? (double)(1.0f / 3.0f) : 1.0 / 3.0;
}

static double lit_thresh(int real4) { /* Thresh_sprase_matrix=1.0e-10, global_parameters.f90:60 */
    return real4 ? (double)1.0e-10f : 1.0e-10;
}

/* 2*PI/(SIDE*d) with PI declared REAL(SP) in nrtype (nr_files.f90:10) */
static double kfactor(int n, double d, int real4) {
    double twopi = real4 ? (double)(2.0f * 3.141592653589793238462643383279502884197f) : 2.0 * M_PI;
    return twopi / ((double)n * d);
}

static int fold(int i, int n) { return (i <= n / 2) ? i : i - n; } /* Gmatrix_2dcomp_mod.f90:450-467 */

orc_ctx* orc_create(const int* n3, int L, int nmax, const int* ns3, const double* dx3, double loa,
                    const double* kappa3, const double* chi3, double nmu, int real4, int nthreads) {
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    for (int a = 0; a < 3; ++a) {
        c->n[a] = n3[a];
        c->dx[a] = dx3[a];
        c->ns[a] = ns3[a];
        c->kappa[a] = kappa3[a];
        c->chi[a] = chi3[a];
    }
    c->nstart[0] = 0;
    c->nstart[1] = ns3[0];
    c->nstart[2] = ns3[0] + ns3[1];
    c->nkx = n3[0] / 2 + 1;
    c->nr = n3[0] * n3[1] * n3[2];
    c->nk = c->nkx * n3[1] * n3[2];
    c->L = L;
    c->M = (L + 1) * (L + 1);
    c->nmax = nmax;
    c->ds = 1.0 / nmax; /* initialize_mod.f90:140 */
    c->loa = loa;
    c->nmu = nmu;
    c->real4 = real4;
    c->vol = dx3[0] * dx3[1] * dx3[2] * c->nr; /* SCFT_control.f90:180 */
    c->nthreads = nthreads > 0 ? nthreads : 1;
    for (int t = 0; t < ORC_NMAT; ++t) c->mats[t] = (double*)malloc(sizeof(double) * c->M * c->M);
    build_basis(L, real4, c->mats);
    c->w = (double*)calloc((size_t)3 * c->nr, sizeof(double));
    c->mop = (double*)calloc((size_t)9 * c->nr, sizeof(double));
    size_t qsz = (size_t)(nmax + 1) * c->M * c->nr;
    c->qf = (double*)calloc(qsz, sizeof(double));
    c->qb = (double*)calloc(qsz, sizeof(double));
    for (int a = 0; a < 3; ++a) plan_init(&c->plan[a], n3[a]);
    return c;
}

static void clear_variants(orc_ctx* c) {
    for (int v = 0; v < c->nvar; ++v) {
        free(c->var[v].lu);
        free(c->var[v].piv);
    }
    c->nvar = 0;
}

void orc_destroy(orc_ctx* c) {
    if (!c) return;
    clear_variants(c);
    for (int t = 0; t < ORC_NMAT; ++t) free(c->mats[t]);
    free(c->w);
    free(c->mop);
    free(c->qf);
    free(c->qb);
    for (int a = 0; a < 3; ++a) plan_free(&c->plan[a]);
    free(c);
}

int orc_M(orc_ctx* c) { return c->M; }
int orc_nk(orc_ctx* c) { return c->nk; }

void orc_get_matrix(orc_ctx* c, int which, double* out) {
    memcpy(out, c->mats[which], sizeof(double) * c->M * c->M);
}

void orc_set_box(orc_ctx* c, const double* dx3) {
    for (int a = 0; a < 3; ++a) c->dx[a] = dx3[a];
    c->vol = dx3[0] * dx3[1] * dx3[2] * c->nr;
    clear_variants(c); /* G must be rebuilt when the box changes (Gmatrix_2dcomp_mod.f90:223-224) */
}

void orc_set_fields(orc_ctx* c, const double* w, const double* mop) {
    memcpy(c->w, w, sizeof(double) * 3 * c->nr);
    if (mop) {
        memcpy(c->mop, mop, sizeof(double) * 9 * c->nr);
        c->have_mop = 1;
    } else {
        memset(c->mop, 0, sizeof(double) * 9 * c->nr);
        c->have_mop = 0;
    }
}

/* ------------------------------------------------------------------ */
/* G(k): build, LU (zgetrf-style partial pivoting), solve               */
/* ------------------------------------------------------------------ */

static void k_components(const orc_ctx* c, int kk, double* kx, double* ky, double* kz) {
    int ix = kk % c->nkx;
    int iy = (kk / c->nkx) % c->n[1];
    int iz = kk / (c->nkx * c->n[1]);
    *kx = fold(ix, c->n[0]) * kfactor(c->n[0], c->dx[0], c->real4);
    *ky = fold(iy, c->n[1]) * kfactor(c->n[1], c->dx[1], c->real4);
    *kz = fold(iz, c->n[2]) * kfactor(c->n[2], c->dx[2], c->real4);
}

/* Dense G(k) for sigma = +1, row-major G[i*M+j] = G(i,j)  (init_G_mat,
 * Gmatrix_mod.f90:765-908) */
static void build_G(const orc_ctx* c, int kk, int order, double kappa, cplx* G) {
    int M = c->M;
    double kx, ky, kz;
    k_components(c, kk, &kx, &ky, &kz);
    /* order 4: the split scheme's I + ds/2 A (c0 = 1, step ds/2) */
    double c0 = order == 4 ? 1.0 : lit_c0(order, c->real4);
    double dse = order == 4 ? 0.5 * c->ds : c->ds;
    const double *Rx = c->mats[ORC_RX], *Ry = c->mats[ORC_RY], *Rz = c->mats[ORC_RZ];
    for (int i = 0; i < M; ++i)
        for (int j = 0; j < M; ++j) {
            size_t o = (size_t)i * M + j;
            double gi = 1.0 * dse * (Rx[o] * kx + Ry[o] * ky + Rz[o] * kz);
            G[o] = 0.0 + I * gi;
        }
    for (int j = 0; j < M; ++j) {
        int l, m;
        basis_lm(j, &l, &m);
        double gr = c0 + dse * c->loa * l * (l + 1) / (2.0 * kappa);
        G[(size_t)j * M + j] = gr + I * cimag(G[(size_t)j * M + j]);
    }
}

static double cabs1(cplx z) { return fabs(creal(z)) + fabs(cimag(z)); }

static void lu_factor(cplx* A, int* piv, int M) {
    for (int k = 0; k < M; ++k) {
        int p = k;
        double best = cabs1(A[(size_t)k * M + k]);
        for (int i = k + 1; i < M; ++i) {
            double v = cabs1(A[(size_t)i * M + k]);
            if (v > best) {
                best = v;
                p = i;
            }
        }
        piv[k] = p;
        if (p != k)
            for (int j = 0; j < M; ++j) {
                cplx t = A[(size_t)k * M + j];
                A[(size_t)k * M + j] = A[(size_t)p * M + j];
                A[(size_t)p * M + j] = t;
            }
        cplx inv = 1.0 / A[(size_t)k * M + k];
        for (int i = k + 1; i < M; ++i) {
            cplx f = A[(size_t)i * M + k] * inv;
            A[(size_t)i * M + k] = f;
            for (int j = k + 1; j < M; ++j) A[(size_t)i * M + j] -= f * A[(size_t)k * M + j];
        }
    }
}

static void lu_solve(const cplx* A, const int* piv, int M, cplx* b) {
    for (int k = 0; k < M; ++k) {
        int p = piv[k];
        if (p != k) {
            cplx t = b[k];
            b[k] = b[p];
            b[p] = t;
        }
    }
    for (int i = 0; i < M; ++i) {
        cplx s = b[i];
        for (int j = 0; j < i; ++j) s -= A[(size_t)i * M + j] * b[j];
        b[i] = s;
    }
    for (int i = M - 1; i >= 0; --i) {
        cplx s = b[i];
        for (int j = i + 1; j < M; ++j) s -= A[(size_t)i * M + j] * b[j];
        b[i] = s / A[(size_t)i * M + i];
    }
}

static g_variant* get_variant(orc_ctx* c, int order, double kappa) {
    for (int v = 0; v < c->nvar; ++v)
        if (c->var[v].order == order && c->var[v].kappa == kappa) return &c->var[v];
    if (c->nvar >= ORC_MAXVAR) clear_variants(c);
    g_variant* g = &c->var[c->nvar++];
    int M = c->M;
    g->order = order;
    g->kappa = kappa;
    g->lu = (cplx*)malloc(sizeof(cplx) * (size_t)c->nk * M * M);
    g->piv = (int*)malloc(sizeof(int) * (size_t)c->nk * M);
#pragma omp parallel for num_threads(c->nthreads) schedule(dynamic, 16)
    for (int kk = 0; kk < c->nk; ++kk) {
        cplx* A = g->lu + (size_t)kk * M * M;
        build_G(c, kk, order, kappa, A);
        lu_factor(A, g->piv + (size_t)kk * M, M);
    }
    return g;
}

/* ------------------------------------------------------------------ */
/* 3D R2C / C2R (2DECOMP order: x r2c, y c2c, z c2c; inverse z, y, x c2r) */
/* ------------------------------------------------------------------ */

static void r2c3(const orc_ctx* c, const double* in, cplx* out, cplx* work) {
    int nx = c->n[0], ny = c->n[1], nz = c->n[2], nkx = c->nkx;
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            cplx* row = work + 2 * 256;
            for (int x = 0; x < nx; ++x) row[x] = in[((size_t)z * ny + y) * nx + x];
            fft1d(row, 1, &c->plan[0], 0, work);
            for (int kx = 0; kx < nkx; ++kx) out[((size_t)z * ny + y) * nkx + kx] = row[kx];
        }
    for (int z = 0; z < nz; ++z)
        for (int kx = 0; kx < nkx; ++kx) fft1d(out + (size_t)z * ny * nkx + kx, nkx, &c->plan[1], 0, work);
    for (int ky = 0; ky < ny; ++ky)
        for (int kx = 0; kx < nkx; ++kx) fft1d(out + (size_t)ky * nkx + kx, nkx * ny, &c->plan[2], 0, work);
}

/* destroys `in` */
static void c2r3(const orc_ctx* c, cplx* in, double* out, cplx* work) {
    int nx = c->n[0], ny = c->n[1], nz = c->n[2], nkx = c->nkx;
    for (int ky = 0; ky < ny; ++ky)
        for (int kx = 0; kx < nkx; ++kx) fft1d(in + (size_t)ky * nkx + kx, nkx * ny, &c->plan[2], 1, work);
    for (int z = 0; z < nz; ++z)
        for (int kx = 0; kx < nkx; ++kx) fft1d(in + (size_t)z * ny * nkx + kx, nkx, &c->plan[1], 1, work);
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            const cplx* h = in + ((size_t)z * ny + y) * nkx;
            cplx* row = work + 2 * 256;
            /* Hermitian extension; the DC and Nyquist imaginary parts are
             * discarded, as a c2r transform does */
            for (int kx = 0; kx < nx; ++kx) {
                if (kx == 0 || (kx == nx / 2))
                    row[kx] = creal(h[kx]);
                else if (kx < nx / 2)
                    row[kx] = h[kx];
                else
                    row[kx] = conj(h[nx - kx]);
            }
            fft1d(row, 1, &c->plan[0], 1, work);
            for (int x = 0; x < nx; ++x) out[((size_t)z * ny + y) * nx + x] = creal(row[x]);
        }
}

void orc_fft_r2c(orc_ctx* c, const double* in, double* out_interleaved) {
    cplx* work = (cplx*)malloc(sizeof(cplx) * 1024);
    r2c3(c, in, (cplx*)out_interleaved, work);
    free(work);
}

void orc_fft_c2r(orc_ctx* c, const double* in_interleaved, double* out) {
    cplx* work = (cplx*)malloc(sizeof(cplx) * 1024);
    cplx* tmp = (cplx*)malloc(sizeof(cplx) * c->nk);
    memcpy(tmp, in_interleaved, sizeof(cplx) * c->nk);
    c2r3(c, tmp, out, work);
    free(tmp);
    free(work);
}

/* ------------------------------------------------------------------ */
/* One contour step                                                     */
/* ------------------------------------------------------------------ */

/* Maier-Saupe coupling Theta_ij(r) (calc_THETAij, wormlike_MDE_2dcomp_mod.f90:5-110) */
static double theta_ij(const orc_ctx* c, size_t o, size_t r) {
    const double* m = c->mop;
    size_t nr = c->nr;
    double v = (m[0 * nr + r] - m[4 * nr + r]) * c->mats[ORC_T1122][o] + m[8 * nr + r] * c->mats[ORC_T33][o] +
               m[1 * nr + r] * c->mats[ORC_T12][o] + m[2 * nr + r] * c->mats[ORC_T13][o] +
               m[5 * nr + r] * c->mats[ORC_T23][o];
    return v;
}

/* BDF right-hand side (init_pr, MDE_ABC.f90:223-383).  `h1,h2,h3` are the
 * previous slices q(s-1), q(s-2), q(s-3) (forward) or q(s+1).. (backward),
 * each [M][nr]; `order` is the BDF order; `wb` the block field. */
static void rhs(const orc_ctx* c, int order, const double* h1, const double* h2, const double* h3,
                const double* wb, double* pr) {
    int M = c->M;
    size_t nr = c->nr;
    double ds = c->ds, third = lit_third(c->real4), thresh = lit_thresh(c->real4);
    int ms = fabs(c->nmu) >= 1.0e-5 && c->have_mop;
#pragma omp parallel for num_threads(c->nthreads)
    for (long r = 0; r < (long)nr; ++r) {
        double W = wb[r];
        for (int i = 0; i < M; ++i) {
            double acc = 0.0;
            if (ms) {
                /* sum over nonzero Theta_ij(r) (|Theta| >= Thresh) */
                for (int j = 0; j < M; ++j) {
                    double th = theta_ij(c, (size_t)i * M + j, r);
                    if (fabs(th) < thresh) continue;
                    double hj;
                    if (order == 1)
                        hj = h1[(size_t)j * nr + r];
                    else if (order == 2)
                        hj = 2.0 * h1[(size_t)j * nr + r] - h2[(size_t)j * nr + r];
                    else
                        hj = 3.0 * h1[(size_t)j * nr + r] - 3.0 * h2[(size_t)j * nr + r] + h3[(size_t)j * nr + r];
                    acc = acc + ds * th * hj;
                }
            }
            size_t o = (size_t)i * nr + r;
            if (order == 1)
                acc = acc + (1.0 - ds * W) * h1[o];
            else if (order == 2)
                acc = acc + 2.0 * h1[o] - 0.5 * h2[o] - ds * W * (2.0 * h1[o] - h2[o]);
            else
                acc = acc + 3.0 * h1[o] - 1.5 * h2[o] + third * h3[o] - ds * W * (3.0 * h1[o] - 3.0 * h2[o] + h3[o]);
            pr[o] = acc;
        }
    }
}

/* mde_one_step (MDE_ABC.f90:90-221; wormlike_MDE_2dcomp_mod.f90:357-455):
 * q = C2R( G(order, sigma, kappa_blk)^-1 . R2C(Pr) ) / N^3 */
void orc_one_step(orc_ctx* c, int order, int sigma, int blk, const double* pr, double* qout) {
    int M = c->M;
    size_t nr = c->nr, nk = c->nk;
    g_variant* g = get_variant(c, order, c->kappa[blk]);
    cplx* P = (cplx*)malloc(sizeof(cplx) * nk * M);
    double minv = 1.0 / (double)nr;
#pragma omp parallel num_threads(c->nthreads)
    {
        cplx* work = (cplx*)malloc(sizeof(cplx) * 1024);
#pragma omp for
        for (int i = 0; i < M; ++i) r2c3(c, pr + (size_t)i * nr, P + (size_t)i * nk, work);
#pragma omp for
        for (long kk = 0; kk < (long)nk; ++kk) {
            cplx b[512];
            for (int i = 0; i < M; ++i) b[i] = P[(size_t)i * nk + kk];
            const cplx* A = g->lu + (size_t)kk * M * M;
            const int* piv = g->piv + (size_t)kk * M;
            if (sigma > 0) {
                lu_solve(A, piv, M, b);
            } else {
                /* G(sigma=-1) = conj(G(sigma=+1)): solve G x* = b* */
                for (int i = 0; i < M; ++i) b[i] = conj(b[i]);
                lu_solve(A, piv, M, b);
                for (int i = 0; i < M; ++i) b[i] = conj(b[i]);
            }
            if (order == 4) /* Crank-Nicolson: (2 (I + ds/2 A)^-1 - I) b */
                for (int i = 0; i < M; ++i) b[i] = 2.0 * b[i] - P[(size_t)i * nk + kk];
            for (int i = 0; i < M; ++i) P[(size_t)i * nk + kk] = b[i];
        }
#pragma omp for
        for (int i = 0; i < M; ++i) {
            double* q = qout + (size_t)i * nr;
            c2r3(c, P + (size_t)i * nk, q, work);
            for (size_t r = 0; r < nr; ++r) q[r] = q[r] * minv;
        }
        free(work);
    }
    free(P);
}

void orc_set_scheme(orc_ctx* c, int scheme) { c->scheme = scheme; }

/* One step of the split scheme (block blk, direction sigma) from slice qin
 * to qout: e^{-w ds/2} . C2R[ G_CN . R2C[ e^{-w ds/2} qin ] ] / N^3.  The
 * field half steps follow split_operator_MDE_mod.f90:163-166. */
void orc_split_step(orc_ctx* c, int sigma, int blk, const double* qin, double* qout) {
    int M = c->M;
    size_t nr = c->nr, sl = (size_t)M * nr;
    const double* wb = c->w + (size_t)blk * nr;
    double* eh = (double*)malloc(sizeof(double) * nr);
    double* pr = (double*)calloc(sl, sizeof(double));
    for (size_t r = 0; r < nr; ++r) eh[r] = exp(-0.5 * c->ds * wb[r]);
    for (int i = 0; i < M; ++i)
        for (size_t r = 0; r < nr; ++r) pr[(size_t)i * nr + r] = eh[r] * qin[(size_t)i * nr + r];
    orc_one_step(c, 4, sigma, blk, pr, qout);
    for (int i = 0; i < M; ++i)
        for (size_t r = 0; r < nr; ++r) qout[(size_t)i * nr + r] *= eh[r];
    free(pr);
    free(eh);
}

/* block containing the forward step s-1 -> s (MDE_ABC.f90:44-57) */
static int blk_fwd(const orc_ctx* c, int s) {
    if (s <= c->nstart[1]) return 0;
    if (s <= c->nstart[2]) return 1;
    return 2;
}

/* block containing the backward step s+1 -> s (MDE_ABC.f90:69-83) */
static int blk_bwd(const orc_ctx* c, int s) {
    if (s >= c->nstart[2]) return 2;
    if (s >= c->nstart[1]) return 1;
    return 0;
}

/* Right-hand side for contour index s in direction dir (+1 forward, -1
 * backward) from the stored slices. */
void orc_init_pr(orc_ctx* c, int dir, int s, double* pr) {
    size_t sl = (size_t)c->M * c->nr;
    if (dir > 0) {
        int order = s < 3 ? s : 3;
        int b = blk_fwd(c, s);
        const double* q = c->qf;
        rhs(c, order, q + (size_t)(s - 1) * sl, order >= 2 ? q + (size_t)(s - 2) * sl : NULL,
            order >= 3 ? q + (size_t)(s - 3) * sl : NULL, c->w + (size_t)b * c->nr, pr);
    } else {
        int d = c->nmax - s;
        int order = d < 3 ? d : 3;
        int b = blk_bwd(c, s);
        const double* q = c->qb;
        rhs(c, order, q + (size_t)(s + 1) * sl, order >= 2 ? q + (size_t)(s + 2) * sl : NULL,
            order >= 3 ? q + (size_t)(s + 3) * sl : NULL, c->w + (size_t)b * c->nr, pr);
    }
}

/* ABC_melt_driver (MDE_ABC.f90:8-88): dir=+1 forward q, dir=-1 backward q* */
void orc_propagate(orc_ctx* c, int dir) {
    int M = c->M;
    size_t nr = c->nr, sl = (size_t)M * nr;
    double* pr = (double*)malloc(sizeof(double) * sl);
    if (dir > 0) {
        memset(c->qf, 0, sizeof(double) * sl);
        for (size_t r = 0; r < nr; ++r) c->qf[r] = 1.0; /* q(0) = delta_i0 */
        for (int s = 1; s <= c->nmax; ++s) {
            if (c->scheme == 1) {
                orc_split_step(c, +1, blk_fwd(c, s), c->qf + (size_t)(s - 1) * sl, c->qf + (size_t)s * sl);
                continue;
            }
            orc_init_pr(c, +1, s, pr);
            int order = s < 3 ? s : 3;
            orc_one_step(c, order, +1, blk_fwd(c, s), pr, c->qf + (size_t)s * sl);
        }
    } else {
        double* top = c->qb + (size_t)c->nmax * sl;
        memset(top, 0, sizeof(double) * sl);
        for (size_t r = 0; r < nr; ++r) top[r] = 1.0; /* q*(Nmax) = delta_i0 */
        for (int s = c->nmax - 1; s >= 0; --s) {
            if (c->scheme == 1) {
                orc_split_step(c, -1, blk_bwd(c, s), c->qb + (size_t)(s + 1) * sl, c->qb + (size_t)s * sl);
                continue;
            }
            orc_init_pr(c, -1, s, pr);
            int d = c->nmax - s;
            int order = d < 3 ? d : 3;
            orc_one_step(c, order, -1, blk_bwd(c, s), pr, c->qb + (size_t)s * sl);
        }
    }
    free(pr);
}

void orc_get_q(orc_ctx* c, int dir, int s, double* out) {
    size_t sl = (size_t)c->M * c->nr;
    memcpy(out, (dir > 0 ? c->qf : c->qb) + (size_t)s * sl, sizeof(double) * sl);
}

void orc_set_q(orc_ctx* c, int dir, int s, const double* in) {
    size_t sl = (size_t)c->M * c->nr;
    memcpy((dir > 0 ? c->qf : c->qb) + (size_t)s * sl, in, sizeof(double) * sl);
}

/* ------------------------------------------------------------------ */
/* Integrators (utility_mod.f90:195-374) and densities                  */
/* ------------------------------------------------------------------ */

/* periodic 3D Simpson: weight (h/3)*(2 if index even else 4) per axis */
double orc_simpson3(const orc_ctx* c, const double* a) {
    int nx = c->n[0], ny = c->n[1], nz = c->n[2];
    double* a2 = (double*)malloc(sizeof(double) * (size_t)ny * nz);
    /* innermost axis first, as simposon_3D_mpi does (FUN_A+FUN_B = 2*a(0)) */
    for (int z = 0; z < nz; ++z)
        for (int y = 0; y < ny; ++y) {
            const double* row = a + ((size_t)z * ny + y) * nx;
            double fa = row[0], fb = row[0], f2 = 0.0, f4 = row[1];
            int s1 = 1;
            for (int f = 1; f <= nx / 2 - 1; ++f) {
                s1++;
                f2 += row[s1];
                s1++;
                f4 += row[s1];
            }
            a2[(size_t)z * ny + y] = (c->dx[0] / 3.0) * (fa + fb + 4.0 * f4 + 2.0 * f2);
        }
    double* a1 = (double*)malloc(sizeof(double) * nz);
    for (int z = 0; z < nz; ++z) {
        const double* row = a2 + (size_t)z * ny;
        double fa = row[0], fb = row[0], f2 = 0.0, f4 = row[1];
        int s1 = 1;
        for (int f = 1; f <= ny / 2 - 1; ++f) {
            s1++;
            f2 += row[s1];
            s1++;
            f4 += row[s1];
        }
        a1[z] = (c->dx[1] / 3.0) * (fa + fb + 4.0 * f4 + 2.0 * f2);
    }
    double f2 = 0.0, f4 = 0.0;
    for (int s1 = 0; s1 < nz; s1 += 2) {
        f2 += a1[s1];
        f4 += a1[s1 + 1];
    }
    free(a1);
    free(a2);
    return (c->dx[2] / 3.0) * (4.0 * f4 + 2.0 * f2);
}

/* composite Simpson over a[n0..n1] (simposon_1D_NR, utility_mod.f90:346-374) */
static double simpson1(const double* a, int n0, int n1, double h) {
    double fa = a[n0], fb = a[n1], f2 = 0.0, f4 = a[n0 + 1];
    int s1 = n0 + 1;
    for (int f = 1; f <= (n1 - n0) / 2 - 1; ++f) {
        s1++;
        f2 += a[s1];
        s1++;
        f4 += a[s1];
    }
    return (h / 3.0) * (fa + fb + 4.0 * f4 + 2.0 * f2);
}

/* density (SCFT_Density_FE_ABC.f90:3-271, per-block restatement):
 *   lnq            ln[(1/V) S3(q_0(r, Nmax))]
 *   phi[3][nr]     block densities  V * sum_i S1_{s in K}(q_i q*_i) / totden
 *   junc[3][nr]    V*sum_i q_i q*_i/totden at s = NA, NA+NB, Nmax
 *   sop[3][9][nr]  orientation tensors per block (a*3+b), S_zz = -S_xx-S_yy
 * any output pointer may be NULL. Returns totden. */
double orc_density(orc_ctx* c, double* lnq, double* phi, double* junc, double* sop) {
    int M = c->M;
    size_t nr = c->nr, sl = (size_t)M * nr;
    double ds = c->ds, V = c->vol, thresh = lit_thresh(c->real4);
    double* ar = (double*)malloc(sizeof(double) * nr);
    const double* qend = c->qf + (size_t)c->nmax * sl;
    for (size_t r = 0; r < nr; ++r) ar[r] = qend[r];
    double pff = orc_simpson3(c, ar) / V;
    if (lnq) *lnq = log(pff);
    double* rb = (double*)malloc(sizeof(double) * 3 * nr);
    double* denz = (double*)malloc(sizeof(double) * nr);
#pragma omp parallel num_threads(c->nthreads)
    {
        double* cc = (double*)malloc(sizeof(double) * (c->nmax + 1));
#pragma omp for
        for (long r = 0; r < (long)nr; ++r) {
            double tot = 0.0;
            for (int b = 0; b < 3; ++b) {
                double sum_i = 0.0;
                int s0 = c->nstart[b], s1 = c->nstart[b] + c->ns[b];
                if (c->ns[b] > 0) {
                    for (int i = 0; i < M; ++i) {
                        for (int s = s0; s <= s1; ++s)
                            cc[s] = c->qf[(size_t)s * sl + (size_t)i * nr + r] * c->qb[(size_t)s * sl + (size_t)i * nr + r];
                        sum_i += simpson1(cc, s0, s1, ds);
                    }
                }
                rb[(size_t)b * nr + r] = sum_i;
                tot += sum_i;
            }
            denz[r] = tot;
        }
        free(cc);
    }
    double totden = orc_simpson3(c, denz);
    if (phi)
        for (int b = 0; b < 3; ++b)
            for (size_t r = 0; r < nr; ++r) phi[(size_t)b * nr + r] = V * rb[(size_t)b * nr + r] / totden;
    if (junc) {
        int sj[3] = {c->nstart[1], c->nstart[2], c->nmax};
        for (int j = 0; j < 3; ++j)
            for (size_t r = 0; r < nr; ++r) {
                double sum = 0.0;
                for (int i = 0; i < M; ++i)
                    sum += c->qf[(size_t)sj[j] * sl + (size_t)i * nr + r] * c->qb[(size_t)sj[j] * sl + (size_t)i * nr + r];
                junc[(size_t)j * nr + r] = V * sum / totden;
            }
    }
    if (sop) {
        const int jm[5] = {ORC_J11, ORC_J22, ORC_J12, ORC_J13, ORC_J23};
        double nor = V / totden;
#pragma omp parallel num_threads(c->nthreads)
        {
            double* cc = (double*)malloc(sizeof(double) * 5 * (c->nmax + 1));
            double* tmp = (double*)malloc(sizeof(double) * M);
#pragma omp for
            for (long r = 0; r < (long)nr; ++r) {
                for (int b = 0; b < 3; ++b) {
                    int s0 = c->nstart[b], s1 = c->nstart[b] + c->ns[b];
                    double S[9] = {0};
                    if (c->ns[b] > 0) {
                        for (int t = 0; t < 5; ++t) {
                            const double* J = c->mats[jm[t]];
                            for (int s = s0; s <= s1; ++s) {
                                const double* qa = c->qf + (size_t)s * sl + r;
                                const double* qs = c->qb + (size_t)s * sl + r;
                                /* Sum_sparse_2D: temp_i(i) += J_ij q*_j ; sum += temp_i(i) q_i */
                                for (int i = 0; i < M; ++i) tmp[i] = 0.0;
                                for (int i = 0; i < M; ++i)
                                    for (int j = 0; j < M; ++j) {
                                        double v = J[(size_t)i * M + j];
                                        if (fabs(v) >= thresh) tmp[i] += v * qs[(size_t)j * nr];
                                    }
                                double sum = 0.0;
                                for (int i = 0; i < M; ++i) sum += tmp[i] * qa[(size_t)i * nr];
                                cc[t * (c->nmax + 1) + s] = sum;
                            }
                        }
                        double s11 = simpson1(cc + 0 * (c->nmax + 1), s0, s1, ds) * nor;
                        double s22 = simpson1(cc + 1 * (c->nmax + 1), s0, s1, ds) * nor;
                        double s12 = simpson1(cc + 2 * (c->nmax + 1), s0, s1, ds) * nor;
                        double s13 = simpson1(cc + 3 * (c->nmax + 1), s0, s1, ds) * nor;
                        double s23 = simpson1(cc + 4 * (c->nmax + 1), s0, s1, ds) * nor;
                        S[0] = s11;
                        S[4] = s22;
                        S[8] = -(s11 + s22);
                        S[1] = S[3] = s12;
                        S[2] = S[6] = s13;
                        S[5] = S[7] = s23;
                    }
                    for (int t = 0; t < 9; ++t) sop[((size_t)b * 9 + t) * nr + r] = S[t];
                }
            }
            free(tmp);
            free(cc);
        }
    }
    free(ar);
    free(rb);
    free(denz);
    return totden;
}

/* free energy (SCFT_Density_FE.f90:273-342) generalised to three blocks:
 * F = -lnQ + (1/V) S3( sum_{K<J} chi_KJ phi_K phi_J - sum_K w_K phi_K
 *                      + xi (sum_K phi_K - 1) [+ M:M/(2 NMu)] ),
 * xi = (wA+wB+wC)/3 (the AB form uses xi = (wA+wB)/2). chi = {AB, AC, BC}. */
double orc_free_energy(orc_ctx* c, double lnq, const double* phi) {
    size_t nr = c->nr;
    double* ar = (double*)malloc(sizeof(double) * nr);
    const double* w = c->w;
    for (size_t r = 0; r < nr; ++r) {
        double pa = phi[r], pb = phi[nr + r], pc = phi[2 * nr + r];
        double wa = w[r], wb = w[nr + r], wc = w[2 * nr + r];
        double v = c->chi[0] * pa * pb + c->chi[1] * pa * pc + c->chi[2] * pb * pc - wa * pa - wb * pb - wc * pc +
                   (wa + wb + wc) / 3.0 * (pa + pb + pc - 1.0);
        if (fabs(c->nmu) >= 1.0e-5 && c->have_mop) {
            double dd = 0.0;
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) dd += c->mop[(a * 3 + b) * nr + r] * c->mop[(b * 3 + a) * nr + r];
            v += 0.5 * (dd / c->nmu);
        }
        ar[r] = v;
    }
    double e = orc_simpson3(c, ar) / c->vol;
    free(ar);
    return -lnq + e;
}

/* ------------------------------------------------------------------ */
/* Bounded timing sample of one BDF3 contour step (CPU baseline)         */
/* ------------------------------------------------------------------ */

static double now_s(void) {
#ifdef _OPENMP
    return omp_get_wtime();
#else
    return 0.0;
#endif
}

/* One BDF3 forward step at slice s=3 from slices 0..2 with every stage run
 * on the full grid except the per-k solve, which runs for the first
 * `nk_sample` wavevectors only (their LU factors, which the reference
 * precomputes once per box, are built outside the timed stages).
 * t[0] rhs, t[1] forward FFTs, t[2] sampled solve, t[3] inverse FFTs
 * (seconds).  The full-step estimate is t0 + t1 + t2*nk/nk_sample + t3. */
void orc_bench_step(orc_ctx* c, int nk_sample, double* t) {
    int M = c->M;
    size_t nr = c->nr, nk = c->nk, sl = (size_t)M * nr;
    if (nk_sample > (int)nk) nk_sample = (int)nk;
    double* pr = (double*)malloc(sizeof(double) * sl);
    cplx* P = (cplx*)malloc(sizeof(cplx) * nk * M);
    cplx* lu = (cplx*)malloc(sizeof(cplx) * (size_t)nk_sample * M * M);
    int* piv = (int*)malloc(sizeof(int) * (size_t)nk_sample * M);
#pragma omp parallel for num_threads(c->nthreads)
    for (int kk = 0; kk < nk_sample; ++kk) {
        build_G(c, kk, 3, c->kappa[0], lu + (size_t)kk * M * M);
        lu_factor(lu + (size_t)kk * M * M, piv + (size_t)kk * M, M);
    }
    double t0 = now_s();
    rhs(c, 3, c->qf + 2 * sl, c->qf + 1 * sl, c->qf, c->w, pr);
    double t1 = now_s();
#pragma omp parallel num_threads(c->nthreads)
    {
        cplx* work = (cplx*)malloc(sizeof(cplx) * 1024);
#pragma omp for
        for (int i = 0; i < M; ++i) r2c3(c, pr + (size_t)i * nr, P + (size_t)i * nk, work);
        free(work);
    }
    double t2 = now_s();
#pragma omp parallel for num_threads(c->nthreads)
    for (int kk = 0; kk < nk_sample; ++kk) {
        cplx b[512];
        for (int i = 0; i < M; ++i) b[i] = P[(size_t)i * nk + kk];
        lu_solve(lu + (size_t)kk * M * M, piv + (size_t)kk * M, M, b);
        for (int i = 0; i < M; ++i) P[(size_t)i * nk + kk] = b[i];
    }
    double t3 = now_s();
#pragma omp parallel num_threads(c->nthreads)
    {
        cplx* work = (cplx*)malloc(sizeof(cplx) * 1024);
#pragma omp for
        for (int i = 0; i < M; ++i) c2r3(c, P + (size_t)i * nk, c->qf + 3 * sl + (size_t)i * nr, work);
        free(work);
    }
    double t4 = now_s();
    t[0] = t1 - t0;
    t[1] = t2 - t1;
    t[2] = t3 - t2;
    t[3] = t4 - t3;
    free(pr);
    free(P);
    free(lu);
    free(piv);
}

/* Timed sample of whole BDF3 contour steps (the CPU baseline of the
 * contour-step throughput): `nsteps` forward steps of block A, each the
 * right-hand side from the last three slices (init_pr, MDE_ABC.f90:245-309),
 * the R2C FFTs, the per-k solve at EVERY wavevector, the C2R FFTs
 * (mde_one_step, wormlike_MDE_2dcomp_mod.f90:357-455), and the slice's
 * Simpson-weighted q . q* contribution to a block density accumulator
 * (SCFT_Density_FE_ABC.f90:102-117).  The slices live in a ring of four
 * (the context needs nmax >= 4); q* is the stored slice q_star(0).  The LU
 * factors of G(k), which the reference precomputes once per box
 * (init_inverse_sparse_GAB, Gmatrix_2dcomp_mod.f90:222-652), are built
 * before the clock starts.  t[0]: set-up seconds (LU factors), t[1]: timed
 * seconds for the nsteps steps, t[2]: seconds per step. */
void orc_bench_steps(orc_ctx* c, int nsteps, double* t) {
    int M = c->M;
    size_t nr = c->nr, sl = (size_t)M * nr;
    double ts = now_s();
    get_variant(c, 3, c->kappa[0]);
    double t0 = now_s();
    double* pr = (double*)malloc(sizeof(double) * sl);
    double* acc = (double*)calloc(nr, sizeof(double));
    const double* qs = c->qb;
    for (int s = 3; s < 3 + nsteps; ++s) {
        double* q1 = c->qf + (size_t)((s - 1) & 3) * sl;
        double* q2 = c->qf + (size_t)((s - 2) & 3) * sl;
        double* q3 = c->qf + (size_t)((s - 3) & 3) * sl;
        double* out = c->qf + (size_t)(s & 3) * sl;
        rhs(c, 3, q1, q2, q3, c->w, pr);
        orc_one_step(c, 3, +1, 0, pr, out);
        const double wgt = (s & 1) ? 4.0 : 2.0; /* interior Simpson weights (times ds/3) */
#pragma omp parallel for num_threads(c->nthreads)
        for (long r = 0; r < (long)nr; ++r) {
            double v = 0.0;
            for (int i = 0; i < M; ++i) v += out[(size_t)i * nr + r] * qs[(size_t)i * nr + r];
            acc[r] += wgt * c->ds / 3.0 * v;
        }
    }
    double t1 = now_s();
    t[0] = t0 - ts;
    t[1] = t1 - t0;
    t[2] = (t1 - t0) / (nsteps > 0 ? nsteps : 1);
    free(pr);
    free(acc);
}
