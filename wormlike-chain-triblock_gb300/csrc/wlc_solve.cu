// wlc_solve.cu -- pass B of a contour step: for one (kx, ky) column, the
// z-FFT of every harmonic coefficient, the per-wavevector solve of G(k)
// (replacing the stored dense G^-1 of Gmatrix_2dcomp_mod.f90:384-600 and
// its apply, wormlike_MDE_2dcomp_mod.f90:395-409) and the inverse z-FFT.
//
// Factorised solve (see wlc_host.cpp): G^-1 = D T^-1 D^T with
// D = Dz(alpha) Xm Dz(beta) Xp and T = A + i sigma ds |k| Rz, one
// tridiagonal system per m.  One warp owns one kz at a time and runs the
// whole solve warp-synchronously (no CTA barrier); the column lives in
// shared memory with line stride N+1 so that the per-k strided accesses are
// bank-conflict free.  Operator tables are staged in shared memory.
// Tridiagonal pivots come from a per-(order, block) table keyed by
// ix^2+iy^2+iz^2 when the grid spacing is isotropic.
#include <cstdio>

#include "wlc_kernels.cuh"
#include "wlc_step.h"

namespace wlc {

__device__ __forceinline__ int fold_n(int i, int n) { return i <= n / 2 ? i : i - n; }

// shared-memory views of the tables for one solve type TS
template <typename TS> struct WTab {
    int L, M, npairs;
    const int16_t* pairs;
    const int* xp_ptr;
    const int16_t* xp_col;
    const TS* xp_val;
    const int* xm_ptr;
    const int16_t* xm_col;
    const TS* xm_val;
    const TS* zoff;
};

template <typename TS, typename CS>
__device__ __forceinline__ void w_dz(CS* v, int vs, const TS* cs, int sgn, const WTab<TS>& t, int lane) {
    for (int q = lane; q < t.npairs; q += 32) {
        const int ic = t.pairs[3 * q], is = t.pairs[3 * q + 1], m = t.pairs[3 * q + 2];
        const TS cm = cs[2 * m], sm = sgn > 0 ? cs[2 * m + 1] : -cs[2 * m + 1];
        const CS x = v[ic * vs], y = v[is * vs];
        v[ic * vs] = cmk<CS>(cm * x.x - sm * y.x, cm * x.y - sm * y.y);
        v[is * vs] = cmk<CS>(sm * x.x + cm * y.x, sm * x.y + cm * y.y);
    }
}

template <typename TS, typename CS>
__device__ __forceinline__ void w_csr(const int* ptr, const int16_t* col, const TS* val, const CS* in, int is, CS* out,
                                      int os, int M, int lane) {
    for (int i = lane; i < M; i += 32) {
        TS ax = 0, ay = 0;
        const int e1 = ptr[i + 1];
        for (int e = ptr[i]; e < e1; ++e) {
            const TS g = val[e];
            const CS x = in[col[e] * is];
            ax = fma(g, x.x, ax);
            ay = fma(g, x.y, ay);
        }
        out[i * os] = cmk<CS>(ax, ay);
    }
}

// Both systems +m and -m of one m share their real pivots d_j:
// d_0 = A_m, d_j = A_l + e^2/d_{j-1}, e = t z_{l-1}; forward
// y_l = b_l - i (e/d_{j-1}) y_{l-1}; back x_l = (y_l - i t z_l x_{l+1})/d_l.
template <typename TS, typename CS>
__device__ __forceinline__ void w_tridiag(CS* v, int vs, TS t, TS c0, TS dcoef, const WTab<TS>& tb, const TS* pivrow,
                                          int lane) {
    const int L = tb.L;
    for (int m = lane; m <= L; m += 32) {
        const int n = L - m + 1;
        TS dinv[16];
        if (pivrow) {
            const TS* pr = pivrow + m * (L + 1) - (m * (m - 1)) / 2;
            for (int j = 0; j < n; ++j) dinv[j] = pr[j];
        } else {
            TS d = c0 + dcoef * (TS)(m * (m + 1));
            dinv[0] = (TS)1 / d;
            for (int j = 1; j < n; ++j) {
                const int l = m + j;
                const TS e = t * tb.zoff[(l - 1) * (l - 1) + (l - 1) + m];
                d = (c0 + dcoef * (TS)(l * (l + 1))) + e * (e * dinv[j - 1]);
                dinv[j] = (TS)1 / d;
            }
        }
        for (int sgn = 1; sgn >= -1; sgn -= 2) {
            if (sgn < 0 && m == 0) break;
            const int mm = sgn * m;
            int idx = m * m + m + mm;
            CS yp = v[idx * vs];
            for (int j = 1; j < n; ++j) {
                const int l = m + j;
                const int prev = idx;
                idx = l * l + l + mm;
                const TS g = t * tb.zoff[prev] * dinv[j - 1];
                CS y = v[idx * vs];
                y = cmk<CS>(fma(g, yp.y, y.x), fma(-g, yp.x, y.y));
                v[idx * vs] = y;
                yp = y;
            }
            CS xn = cmk<CS>(yp.x * dinv[n - 1], yp.y * dinv[n - 1]);
            v[idx * vs] = xn;
            for (int j = n - 2; j >= 0; --j) {
                const int l = m + j;
                idx = l * l + l + mm;
                const TS e = t * tb.zoff[idx];
                const CS y = v[idx * vs];
                xn = cmk<CS>(fma(e, xn.y, y.x) * dinv[j], fma(-e, xn.x, y.y) * dinv[j]);
                v[idx * vs] = xn;
            }
        }
    }
}

template <typename TS, typename CS>
__device__ __forceinline__ void w_cov_solve(CS* v, int vs, CS* tmp, const WTab<TS>& tb, const TS* csa, const TS* csb,
                                            TS t, TS c0, TS dcoef, const TS* pivrow, int lane) {
    w_dz<TS, CS>(v, vs, csa, -1, tb, lane);
    __syncwarp();
    w_csr<TS, CS>(tb.xp_ptr, tb.xp_col, tb.xp_val, v, vs, tmp, 1, tb.M, lane);
    __syncwarp();
    w_dz<TS, CS>(tmp, 1, csb, -1, tb, lane);
    __syncwarp();
    w_csr<TS, CS>(tb.xm_ptr, tb.xm_col, tb.xm_val, tmp, 1, v, vs, tb.M, lane);
    __syncwarp();
    w_tridiag<TS, CS>(v, vs, t, c0, dcoef, tb, pivrow, lane);
    __syncwarp();
    w_csr<TS, CS>(tb.xp_ptr, tb.xp_col, tb.xp_val, v, vs, tmp, 1, tb.M, lane);
    __syncwarp();
    w_dz<TS, CS>(tmp, 1, csb, +1, tb, lane);
    __syncwarp();
    w_csr<TS, CS>(tb.xm_ptr, tb.xm_col, tb.xm_val, tmp, 1, v, vs, tb.M, lane);
    __syncwarp();
    w_dz<TS, CS>(v, vs, csa, +1, tb, lane);
    __syncwarp();
}

template <typename X> __device__ __forceinline__ void stage(X* dst, const X* src, int n) {
    for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = src[e];
}

template <typename T, int N>
__global__ void __launch_bounds__(kSolveWarpsMax * 32) zfft_solve(SolveArgs<T> a) {
    using C = typename cvec<T>::t;
    constexpr int NP = N + 1;
    const SolveTablesT<T>& g = a.tab;
    const int M = g.M, L = g.L;
    const int nw = blockDim.x / 32, warp = threadIdx.x / 32, lane = threadIdx.x % 32;
    const int correct = a.correct;
    const SolveSmem sm = solve_smem(N, M, L, nw, g.npairs, g.nnz, g.ndr, sizeof(T), correct);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* col = reinterpret_cast<C*>(smem_raw + sm.col);
    C* tw = reinterpret_cast<C*>(smem_raw + sm.tw);
    T* csa = reinterpret_cast<T*>(smem_raw + sm.csa);
    float* csaf = reinterpret_cast<float*>(smem_raw + sm.csaf);
    WTab<T> tb;
    tb.L = L;
    tb.M = M;
    tb.npairs = g.npairs;
    int16_t* s_pairs = reinterpret_cast<int16_t*>(smem_raw + sm.pairs);
    int* s_xpp = reinterpret_cast<int*>(smem_raw + sm.xp_ptr);
    int16_t* s_xpc = reinterpret_cast<int16_t*>(smem_raw + sm.xp_col);
    T* s_xpv = reinterpret_cast<T*>(smem_raw + sm.xp_val);
    int* s_xmp = reinterpret_cast<int*>(smem_raw + sm.xm_ptr);
    int16_t* s_xmc = reinterpret_cast<int16_t*>(smem_raw + sm.xm_col);
    T* s_xmv = reinterpret_cast<T*>(smem_raw + sm.xm_val);
    T* s_zoff = reinterpret_cast<T*>(smem_raw + sm.zoff);
    stage(s_pairs, g.pairs, 3 * g.npairs);
    stage(s_xpp, g.xp_ptr, M + 1);
    stage(s_xpc, g.xp_col, g.nnz);
    stage(s_xpv, g.xp_val, g.nnz);
    stage(s_xmp, g.xm_ptr, M + 1);
    stage(s_xmc, g.xm_col, g.nnz);
    stage(s_xmv, g.xm_val, g.nnz);
    stage(s_zoff, g.zoff, M);
    tb.pairs = s_pairs;
    tb.xp_ptr = s_xpp;
    tb.xp_col = s_xpc;
    tb.xp_val = s_xpv;
    tb.xm_ptr = s_xmp;
    tb.xm_col = s_xmc;
    tb.xm_val = s_xmv;
    tb.zoff = s_zoff;
    WTab<float> tf;
    int* s_drp = nullptr;
    int16_t* s_drc = nullptr;
    int8_t* s_dra = nullptr;
    float* s_drv = nullptr;
    if (correct) {
        float* s_xpvf = reinterpret_cast<float*>(smem_raw + sm.xp_valf);
        float* s_xmvf = reinterpret_cast<float*>(smem_raw + sm.xm_valf);
        float* s_zofff = reinterpret_cast<float*>(smem_raw + sm.zofff);
        s_drp = reinterpret_cast<int*>(smem_raw + sm.dr_ptr);
        s_drc = reinterpret_cast<int16_t*>(smem_raw + sm.dr_col);
        s_dra = reinterpret_cast<int8_t*>(smem_raw + sm.dr_axis);
        s_drv = reinterpret_cast<float*>(smem_raw + sm.dr_valf);
        stage(s_xpvf, g.xp_valf, g.nnz);
        stage(s_xmvf, g.xm_valf, g.nnz);
        stage(s_zofff, g.zofff, M);
        stage(s_drp, g.dr_ptr, M + 1);
        stage(s_drc, g.dr_col, g.ndr);
        stage(s_dra, g.dr_axis, g.ndr);
        stage(s_drv, g.dr_valf, g.ndr);
        tf.L = L;
        tf.M = M;
        tf.npairs = g.npairs;
        tf.pairs = s_pairs;
        tf.xp_ptr = s_xpp;
        tf.xp_col = s_xpc;
        tf.xp_val = s_xpvf;
        tf.xm_ptr = s_xmp;
        tf.xm_col = s_xmc;
        tf.xm_val = s_xmvf;
        tf.zoff = s_zofff;
    }

    const int colid = blockIdx.x;
    const int kyi = colid / a.nkx, kxi = colid % a.nkx;
    const int ix = fold_n(kxi, N), iy = fold_n(kyi, N);
    const double kx = ix * a.kf[0], ky = iy * a.kf[1];
    const double rho = sqrt(kx * kx + ky * ky);
    C* gcol = a.phat + (size_t)colid * M * N;
    for (int e = threadIdx.x; e < M * N; e += blockDim.x) col[(e / N) * NP + (e % N)] = gcol[e];
    for (int e = threadIdx.x; e < N; e += blockDim.x) tw[e] = a.twg[e];
    if (threadIdx.x == 0) {
        const double ca = rho > 0 ? kx / rho : 1.0, sa = rho > 0 ? ky / rho : 0.0;
        double cm = 1.0, sm2 = 0.0;
        for (int m = 0; m <= L; ++m) {
            csa[2 * m] = (T)cm;
            csa[2 * m + 1] = (T)sm2;
            if (correct) {
                csaf[2 * m] = (float)cm;
                csaf[2 * m + 1] = (float)sm2;
            }
            const double cn = cm * ca - sm2 * sa, sn = sm2 * ca + cm * sa;
            cm = cn;
            sm2 = sn;
        }
    }
    __syncthreads();
    fft_nat2perm<N, -1>(col, M, 1, NP, tw);

    C* wtmp = reinterpret_cast<C*>(smem_raw + sm.wtmp) + (size_t)warp * M;
    float2* wrf = reinterpret_cast<float2*>(smem_raw + sm.wrf) + (size_t)warp * M;
    float2* wtmf = reinterpret_cast<float2*>(smem_raw + sm.wtmf) + (size_t)warp * M;
    // per-kz geometry of this column, computed once: cos/sin(m beta) for
    // m = 0..L and t = sigma ds |k| (stride 2(L+1)+1), FP32 copies + kz
    const int gs = 2 * (L + 1) + 1, gsf = 2 * (L + 1) + 2;
    T* geo = reinterpret_cast<T*>(smem_raw + sm.wcsb);
    float* geof = reinterpret_cast<float*>(smem_raw + sm.wcsbf);
    for (int p = threadIdx.x; p < N; p += blockDim.x) {
        const int iz = fold_n(perm_index<N>(p), N);
        const double kz = iz * a.kf[2];
        const double kn = sqrt(rho * rho + kz * kz);
        const double cb = kn > 0 ? kz / kn : 1.0, sb = kn > 0 ? rho / kn : 0.0;
        T* gp = geo + (size_t)p * gs;
        float* gf = geof + (size_t)p * gsf;
        double cm = 1.0, sm2 = 0.0;
        for (int m = 0; m <= L; ++m) {
            gp[2 * m] = (T)cm;
            gp[2 * m + 1] = (T)sm2;
            if (correct) {
                gf[2 * m] = (float)cm;
                gf[2 * m + 1] = (float)sm2;
            }
            const double cn = cm * cb - sm2 * sb, sn = sm2 * cb + cm * sb;
            cm = cn;
            sm2 = sn;
        }
        gp[2 * (L + 1)] = (T)(a.sigma * a.ds * kn);
        if (correct) {
            gf[2 * (L + 1)] = (float)(a.sigma * a.ds * kn);
            gf[2 * (L + 1) + 1] = (float)kz;
        }
    }
    __syncthreads();
    const T c0 = (T)a.c0, dcoef = (T)a.dcoef;
    const float kxf = (float)kx, kyf = (float)ky;
    for (int p = warp; p < N; p += nw) {
        const int iz = fold_n(perm_index<N>(p), N);
        const T* wcsb = geo + (size_t)p * gs;
        const T t = wcsb[2 * (L + 1)];
        const T* pivrow = a.pivtab ? a.pivtab + (size_t)(ix * ix + iy * iy + iz * iz) * a.npiv : nullptr;
        C* v = col + p;
        w_cov_solve<T, C>(v, NP, wtmp, tb, csa, wcsb, t, c0, dcoef, pivrow, lane);
        if (correct) {
            // x -= G_cov^-1 (i sigma ds (k . dR) x), in FP32: the vector is
            // rounded to FP32 once, the matvec and the solve run in FP32
            const float* wcsbf = geof + (size_t)p * gsf;
            const float sds = (float)(a.sigma * a.ds);
            const float kk[3] = {kxf, kyf, wcsbf[2 * (L + 1) + 1]};
            for (int i = lane; i < M; i += 32) {
                const C x = v[i * NP];
                wtmf[i] = make_float2((float)x.x, (float)x.y);
            }
            __syncwarp();
            for (int i = lane; i < M; i += 32) {
                float ax = 0.f, ay = 0.f;
                for (int e = s_drp[i]; e < s_drp[i + 1]; ++e) {
                    const float gv = kk[s_dra[e]] * s_drv[e];
                    const float2 x = wtmf[s_drc[e]];
                    ax = fmaf(gv, x.x, ax);
                    ay = fmaf(gv, x.y, ay);
                }
                wrf[i] = make_float2(-sds * ay, sds * ax);
            }
            __syncwarp();
            w_cov_solve<float, float2>(wrf, 1, wtmf, tf, csaf, wcsbf, wcsbf[2 * (L + 1)], (float)a.c0, (float)a.dcoef,
                                       nullptr, lane);
            for (int i = lane; i < M; i += 32) {
                const float2 r = wrf[i];
                C x = v[i * NP];
                x.x -= (T)r.x;
                x.y -= (T)r.y;
                v[i * NP] = x;
            }
            __syncwarp();
        }
    }
    __syncthreads();
    fft_perm2nat<N, +1>(col, M, 1, NP, tw);
    for (int e = threadIdx.x; e < M * N; e += blockDim.x) gcol[e] = col[(e / N) * NP + (e % N)];
}

// inverse pivots 1/d_j of the tridiagonal systems for every key
// ix^2+iy^2+iz^2 <= nkeys-1 (isotropic spacing), one (order, block)
template <typename T>
__global__ void pivot_table(T* out, int nkeys, int L, double c0, double dcoef, double ds, double kf,
                            const T* __restrict__ zoff) {
    const int npiv = (L + 1) * (L + 2) / 2;
    for (int key = blockIdx.x * blockDim.x + threadIdx.x; key < nkeys; key += gridDim.x * blockDim.x) {
        const T t = (T)(ds * kf * sqrt((double)key));
        T* row = out + (size_t)key * npiv;
        for (int m = 0; m <= L; ++m) {
            T* pr = row + m * (L + 1) - (m * (m - 1)) / 2;
            T d = (T)c0 + (T)dcoef * (T)(m * (m + 1));
            T dinv = (T)1 / d;
            pr[0] = dinv;
            for (int j = 1; j <= L - m; ++j) {
                const int l = m + j;
                const T e = t * zoff[(l - 1) * (l - 1) + (l - 1) + m];
                d = ((T)c0 + (T)dcoef * (T)(l * (l + 1))) + e * (e * dinv);
                dinv = (T)1 / d;
                pr[j] = dinv;
            }
        }
    }
}

// warps per CTA: 16 when their per-warp buffers fit next to the column,
// else 8
template <typename T> int solve_warps(const SolveArgs<T>& a) {
    const int N = 2 * (a.nkx - 1);
    for (int nw = kSolveWarpsMax; nw >= 8; nw /= 2)
        if (solve_smem(N, a.tab.M, a.tab.L, nw, a.tab.npairs, a.tab.nnz, a.tab.ndr, sizeof(T), a.correct).total <=
            227 * 1024)
            return nw;
    return 8;
}

template <typename T> size_t solve_smem_bytes(const SolveArgs<T>& a) {
    const int N = 2 * (a.nkx - 1);
    return solve_smem(N, a.tab.M, a.tab.L, solve_warps(a), a.tab.npairs, a.tab.nnz, a.tab.ndr, sizeof(T), a.correct)
        .total;
}

template <typename T, int N> static cudaError_t launch_solve_n(const SolveArgs<T>& a, cudaStream_t st) {
    static bool attr_done = false;
    if (!attr_done) {
        cudaFuncSetAttribute(zfft_solve<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        attr_done = true;
    }
    const int nw = solve_warps<T>(a);
    const size_t bytes = solve_smem_bytes<T>(a);
    zfft_solve<T, N><<<a.nkx * N, nw * 32, bytes, st>>>(a);
    return cudaGetLastError();
}

template <typename T> cudaError_t launch_solve(int N, const SolveArgs<T>& a, cudaStream_t st) {
    switch (N) {
#define WLC_CASE(n) \
    case n:         \
        return launch_solve_n<T, n>(a, st);
        WLC_FOR_EACH_N(WLC_CASE)
#undef WLC_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

template <typename T>
cudaError_t launch_pivot_table(T* out, int nkeys, int L, double c0, double dcoef, double ds, double kf, const T* zoff,
                               cudaStream_t st) {
    pivot_table<T><<<(nkeys + 127) / 128, 128, 0, st>>>(out, nkeys, L, c0, dcoef, ds, kf, zoff);
    return cudaGetLastError();
}

template cudaError_t launch_solve<double>(int, const SolveArgs<double>&, cudaStream_t);
template cudaError_t launch_solve<float>(int, const SolveArgs<float>&, cudaStream_t);
template size_t solve_smem_bytes<double>(const SolveArgs<double>&);
template size_t solve_smem_bytes<float>(const SolveArgs<float>&);
template cudaError_t launch_pivot_table<double>(double*, int, int, double, double, double, double, const double*,
                                                cudaStream_t);
template cudaError_t launch_pivot_table<float>(float*, int, int, double, double, double, double, const float*,
                                               cudaStream_t);

}  // namespace wlc
