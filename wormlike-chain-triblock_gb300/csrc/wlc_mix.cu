// wlc_mix.cu -- SCFT field update on the device: simple mixing, then
// Anderson mixing, three blocks (the reference's AB_iterate,
// SCFT_iterate.f90:27-334, generalised from two to three blocks).
//
// With f_J = N_J/N and chi_KJ N the block interaction parameters:
//  * simple-mixing residual (SCFT_iterate.f90:146-148)
//      dW_K = sum_J chi_KJ (phi_J - f_J) + (1/3) sum_J w_J - w_K,
//    w_K += lambda_s dW_K, block error max |dW_K|;
//  * Anderson output field and residual (SCFT_iterate.f90:170-173, 206-209)
//      w_K^out = sum_J chi_KJ phi_J + (1/3)(sum_J w_J - sum_KJ chi_KJ f_J),
//      dW_K = w_K^out - w_K.
// For two blocks both reduce term by term to the reference's formulas
// (chiN (phi_B - f_B) + (w_A + w_B)/2 - w_A and chiN phi_B + (w_A + w_B - chiN)/2).
// Inner products <a, b> = S3(a b)/V with the periodic Simpson weights
// (dot_product_mpi, SCFT_iterate.f90:1193-1237).  Every reduction is
// deterministic: fixed CTA partition, fixed-order trees.
#include <cstdint>

#include "wlc_mix.h"

namespace wlc {

__device__ __forceinline__ double simpson_weight(int64_t r, const MixGrid& g) {
    const int x = (int)(r % g.n[0]);
    const int y = (int)((r / g.n[0]) % g.n[1]);
    const int z = (int)(r / ((int64_t)g.n[0] * g.n[1]));
    const double wx = (x & 1) ? 4.0 : 2.0, wy = (y & 1) ? 4.0 : 2.0, wz = (z & 1) ? 4.0 : 2.0;
    return (g.d[0] / 3.0 * wx) * (g.d[1] / 3.0 * wy) * (g.d[2] / 3.0 * wz);
}

// residuals, optional store of (w_out, dW) into the current history slot,
// optional simple-mixing update; max |residual_K| and max |sum_K phi_K - 1|
// partials per CTA
__global__ void mix_out(const double* __restrict__ phi, double* __restrict__ w, MixChi chi, int64_t nr, int mode,
                        double lambda, double* __restrict__ wout, double* __restrict__ dw,
                        double* __restrict__ maxpart) {
    __shared__ double sm[4][256];
    double mx[4] = {0, 0, 0, 0};
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        const double p[3] = {phi[r], phi[nr + r], phi[2 * nr + r]};
        const double ww[3] = {w[r], w[nr + r], w[2 * nr + r]};
        const double sw = ww[0] + ww[1] + ww[2];
        if (mode != kMixSimple) {
            const double xi = (sw - chi.fsum) / 3.0;
            for (int K = 0; K < 3; ++K) {
                const double o = (chi.c[K][0] * p[0] + chi.c[K][1] * p[1] + chi.c[K][2] * p[2]) + xi;
                wout[K * nr + r] = o;
                const double d = o - ww[K];
                dw[K * nr + r] = d;
                if (mode == kMixStore) mx[K] = fmax(mx[K], fabs(d));
            }
        }
        if (mode != kMixStore) {
            const double pc = sw / 3.0;
            for (int K = 0; K < 3; ++K) {
                const double d = (chi.c[K][0] * (p[0] - chi.f[0]) + chi.c[K][1] * (p[1] - chi.f[1]) +
                                  chi.c[K][2] * (p[2] - chi.f[2])) + pc - ww[K];
                w[K * nr + r] = ww[K] + lambda * d;
                mx[K] = fmax(mx[K], fabs(d));
            }
        }
        mx[3] = fmax(mx[3], fabs(p[0] + p[1] + p[2] - 1.0));
    }
    for (int q = 0; q < 4; ++q) sm[q][threadIdx.x] = mx[q];
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s)
            for (int q = 0; q < 4; ++q) sm[q][threadIdx.x] = fmax(sm[q][threadIdx.x], sm[q][threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0)
        for (int q = 0; q < 4; ++q) maxpart[q * gridDim.x + blockIdx.x] = sm[q][0];
}

__global__ void max_final(const double* __restrict__ part, int nblk, int nq, double* __restrict__ out) {
    __shared__ double sm[256];
    for (int q = 0; q < nq; ++q) {
        double m = 0.0;
        for (int k = threadIdx.x; k < nblk; k += blockDim.x) m = fmax(m, part[q * nblk + k]);
        sm[threadIdx.x] = m;
        __syncthreads();
        for (int s = 128; s > 0; s >>= 1) {
            if (threadIdx.x < s) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + s]);
            __syncthreads();
        }
        if (threadIdx.x == 0) out[q] = sm[0];
        __syncthreads();
    }
}

__global__ void mix_m(double* __restrict__ mop, const double* __restrict__ srs, double nmu, double lambda, int64_t nr,
                      double* __restrict__ maxpart) {
    __shared__ double sm[256];
    double mx = 0.0;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        double t[5] = {0, 0, 0, 0, 0};
        for (int b = 0; b < 3; ++b)
            for (int q = 0; q < 5; ++q) t[q] += srs[((int64_t)b * 5 + q) * nr + r];
        const double S[9] = {t[0], t[2], t[3], t[2], t[1], t[4], t[3], t[4], -(t[0] + t[1])};  // [a + 3b]
        for (int q = 0; q < 9; ++q) {
            const double m = mop[(int64_t)q * nr + r];
            const double d = nmu * S[q] - m;
            mop[(int64_t)q * nr + r] = m + lambda * d;
            mx = fmax(mx, fabs(d));
        }
    }
    sm[threadIdx.x] = mx;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) maxpart[blockIdx.x] = sm[0];
}

constexpr int kDotThreads = 128;

// Anderson inner products in one pass over the history (SCFT_iterate.f90:237-276):
// per grid point, with e_m = dW_k - dW_km summed over the blocks,
// U_mn += w3 e_m e_n (n >= m), V_m += w3 e_m dW_k, plus the per-block norms.
template <int NRT>
__global__ void __launch_bounds__(kDotThreads) anderson_dots(AndersonSlots s, MixGrid g, int64_t nr,
                                                             double* __restrict__ part) {
    constexpr int NU = NRT * (NRT + 1) / 2;
    constexpr int NACC = NU + NRT + 6;
    __shared__ double sm[kDotThreads / 32][NACC];
    double acc[NACC];
#pragma unroll
    for (int q = 0; q < NACC; ++q) acc[q] = 0.0;
    const int64_t chunk = (nr + gridDim.x - 1) / gridDim.x;
    const int64_t beg = blockIdx.x * chunk, end = min(nr, beg + chunk);
    for (int64_t r = beg + threadIdx.x; r < end; r += kDotThreads) {
        const double wr = simpson_weight(r, g);
        double u[NU], v[NRT], nrm[6];
#pragma unroll
        for (int q = 0; q < NU; ++q) u[q] = 0.0;
#pragma unroll
        for (int m = 0; m < NRT; ++m) v[m] = 0.0;
#pragma unroll
        for (int K = 0; K < 3; ++K) {
            const int64_t e0 = K * nr + r;
            const double dk = s.dwk[e0], ok = s.woutk[e0];
            double e[NRT];
#pragma unroll
            for (int m = 0; m < NRT; ++m) e[m] = dk - s.dwm[m][e0];
            int q = 0;
#pragma unroll
            for (int m = 0; m < NRT; ++m) {
#pragma unroll
                for (int n = m; n < NRT; ++n) u[q++] += e[m] * e[n];
                v[m] += e[m] * dk;
            }
            nrm[2 * K] = dk * dk;
            nrm[2 * K + 1] = ok * ok;
        }
#pragma unroll
        for (int q = 0; q < NU; ++q) acc[q] += wr * u[q];
#pragma unroll
        for (int m = 0; m < NRT; ++m) acc[NU + m] += wr * v[m];
#pragma unroll
        for (int q = 0; q < 6; ++q) acc[NU + NRT + q] += wr * nrm[q];
    }
    // fixed-order reduction: butterfly within each warp, then warps in order
#pragma unroll
    for (int q = 0; q < NACC; ++q) {
        double a = acc[q];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
        acc[q] = a;
    }
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) {
#pragma unroll
        for (int q = 0; q < NACC; ++q) sm[warp][q] = acc[q];
    }
    __syncthreads();
    for (int q = threadIdx.x; q < NACC; q += kDotThreads) {
        double t = 0.0;
        for (int wi = 0; wi < kDotThreads / 32; ++wi) t += sm[wi][q];
        part[q * gridDim.x + blockIdx.x] = t;
    }
}

__global__ void dots_final(const double* __restrict__ part, int nblk, int nq, double vol, double* __restrict__ out) {
    __shared__ double sm[256];
    for (int q = 0; q < nq; ++q) {
        double s = 0.0;
        for (int k = threadIdx.x; k < nblk; k += blockDim.x) s += part[q * nblk + k];
        sm[threadIdx.x] = s;
        __syncthreads();
        for (int st = 128; st > 0; st >>= 1) {
            if (threadIdx.x < st) sm[threadIdx.x] += sm[threadIdx.x + st];
            __syncthreads();
        }
        if (threadIdx.x == 0) out[q] = sm[0] / vol;
        __syncthreads();
    }
}

// Anderson least squares (one thread, FP64): U c = V by LU with partial
// pivoting (first maximal pivot, as dgetrf; the reference's lapacksolver,
// matrix_inverse_mod.f90:129-199), U from the packed upper triangle.
__global__ void anderson_solve(const double* __restrict__ acc, int nrt, double* __restrict__ coef) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double U[kMaxAnderson][kMaxAnderson], V[kMaxAnderson];
    int q = 0;
    for (int m = 0; m < nrt; ++m)
        for (int n = m; n < nrt; ++n) {
            U[m][n] = acc[q];
            U[n][m] = acc[q];
            ++q;
        }
    for (int m = 0; m < nrt; ++m) V[m] = acc[q + m];
    for (int c = 0; c < nrt; ++c) {
        int p = c;
        for (int r = c + 1; r < nrt; ++r)
            if (fabs(U[r][c]) > fabs(U[p][c])) p = r;
        if (p != c) {
            for (int j = 0; j < nrt; ++j) {
                const double t = U[c][j];
                U[c][j] = U[p][j];
                U[p][j] = t;
            }
            const double t = V[c];
            V[c] = V[p];
            V[p] = t;
        }
        const double piv = U[c][c];
        for (int r = c + 1; r < nrt; ++r) {
            const double f = piv != 0.0 ? U[r][c] / piv : 0.0;
            for (int j = c; j < nrt; ++j) U[r][j] -= f * U[c][j];
            V[r] -= f * V[c];
        }
    }
    for (int r = nrt - 1; r >= 0; --r) {
        double s = V[r];
        for (int j = r + 1; j < nrt; ++j) s -= U[r][j] * coef[j];
        coef[r] = U[r][r] != 0.0 ? s / U[r][r] : 0.0;
    }
}

struct KmList {
    int k[kMaxAnderson];
};

// w = (w_out^k + sum_m c_m (w_out^km - w_out^k)) + lambda (dW^k + sum_m c_m (dW^km - dW^k))
// (SCFT_iterate.f90:307-331)
__global__ void anderson_apply(double* __restrict__ w, const double* __restrict__ wout, const double* __restrict__ dw,
                               int64_t slot_stride, int k, KmList km, int nrt, const double* __restrict__ coef,
                               double lambda, int64_t n) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const double ok = wout[k * slot_stride + e], dk = dw[k * slot_stride + e];
        double wi = 0.0, di = 0.0;
        for (int m = 0; m < nrt; ++m) {
            const double c = coef[m];
            wi += c * (wout[km.k[m] * slot_stride + e] - ok);
            di += c * (dw[km.k[m] * slot_stride + e] - dk);
        }
        w[e] = (wi + ok) + lambda * (di + dk);
    }
}

static int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    return (int)(g > 2048 ? 2048 : (g < 1 ? 1 : g));
}

void launch_mix_out(const double* phi, double* w, const MixChi& chi, int64_t nr, int mode, double lambda, double* wout,
                    double* dw, double* maxpart, double* maxout, cudaStream_t st) {
    mix_out<<<kMixBlocks, 256, 0, st>>>(phi, w, chi, nr, mode, lambda, wout, dw, maxpart);
    max_final<<<1, 256, 0, st>>>(maxpart, kMixBlocks, 4, maxout);
}

void launch_mix_m(double* mop, const double* srs, double nmu, double lambda, int64_t nr, double* maxpart,
                  double* maxout, cudaStream_t st) {
    mix_m<<<kMixBlocks, 256, 0, st>>>(mop, srs, nmu, lambda, nr, maxpart);
    max_final<<<1, 256, 0, st>>>(maxpart, kMixBlocks, 1, maxout);
}

int anderson_acc_count(int nrt) { return nrt * (nrt + 1) / 2 + nrt + 6; }

template <int NRT>
static void dots_n(const AndersonSlots& s, const MixGrid& g, int64_t nr, double* part, cudaStream_t st) {
    anderson_dots<NRT><<<kMixBlocks, kDotThreads, 0, st>>>(s, g, nr, part);
}

void launch_anderson_dots(const AndersonSlots& s, int nrt, const MixGrid& g, int64_t nr, double vol, double* part,
                          double* out, cudaStream_t st) {
    switch (nrt) {
        case 1: dots_n<1>(s, g, nr, part, st); break;
        case 2: dots_n<2>(s, g, nr, part, st); break;
        case 3: dots_n<3>(s, g, nr, part, st); break;
        case 4: dots_n<4>(s, g, nr, part, st); break;
        case 5: dots_n<5>(s, g, nr, part, st); break;
        case 6: dots_n<6>(s, g, nr, part, st); break;
        case 7: dots_n<7>(s, g, nr, part, st); break;
        case 8: dots_n<8>(s, g, nr, part, st); break;
        case 9: dots_n<9>(s, g, nr, part, st); break;
        case 10: dots_n<10>(s, g, nr, part, st); break;
        default: return;
    }
    static_assert(kMaxAnderson == 10, "extend the switch");
    dots_final<<<1, 256, 0, st>>>(part, kMixBlocks, anderson_acc_count(nrt), vol, out);
}

void launch_anderson(const double* acc, int nrt, double* coef, double* w, const double* wout_hist,
                     const double* dw_hist, int64_t slot_stride, int k, const int* km, double lambda, int64_t n,
                     cudaStream_t st) {
    KmList kl;
    for (int m = 0; m < kMaxAnderson; ++m) kl.k[m] = m < nrt ? km[m] : 0;
    anderson_solve<<<1, 32, 0, st>>>(acc, nrt, coef);
    anderson_apply<<<grid_for(n), 256, 0, st>>>(w, wout_hist, dw_hist, slot_stride, k, kl, nrt, coef, lambda, n);
}

}  // namespace wlc
