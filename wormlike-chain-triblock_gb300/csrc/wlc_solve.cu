// wlc_solve.cu -- pass B of a contour step: for one (kx, ky) column, the
// z-FFT of every harmonic coefficient, the per-wavevector solve of G(k)
// (replacing the stored dense G^-1 of Gmatrix_2dcomp_mod.f90:384-600 and
// its apply, wormlike_MDE_2dcomp_mod.f90:395-409) and the inverse z-FFT.
//
// Factorised solve (see wlc_host.cpp): G^-1 = D T^-1 D^T with
// D = Dz(alpha) Xm Dz(beta) Xp and T = A + i sigma ds |k| Rz, one
// tridiagonal system per m.  One thread owns one kz and runs the whole
// solve: the rotations block by block in registers with the generated
// constant codelets (wlc_rot_gen.cuh), the tridiagonal sweeps through its
// slot of the shared column (line stride N+1, conflict free).  Tridiagonal
// pivots come from a per-(order, block) table keyed by ix^2+iy^2+iz^2 when
// the grid spacing is isotropic.
#include <cstdio>

#include "wlc_attr.h"
#include "wlc_kernels.cuh"
#include "wlc_rot_gen.cuh"
#include "wlc_step.h"

namespace wlc {

__device__ __forceinline__ int fold_n(int i, int n) { return i <= n / 2 ? i : i - n; }

// ---------------------------------------------------------------------
// Per-wavevector solve, one thread per kz.  The thread's coefficient
// vector is column p of the shared column buffer (element i at v[i*vs]);
// lanes of a warp own consecutive p, so every access is bank-conflict free.
// Rotations work block by block (degree l) in registers with the
// generated constant codelets; the tridiagonal sweeps run through the
// shared column.

// Dz(sgn * gamma) on the (m, -m) pairs of register block a (index m+l)
template <int l, typename T, typename C>
__device__ __forceinline__ void dz_block(C* a, const T* cs, int sgn) {
#pragma unroll
    for (int m = 1; m <= l; ++m) {
        const T cm = cs[2 * m], sm = sgn > 0 ? cs[2 * m + 1] : -cs[2 * m + 1];
        const C x = a[l + m], y = a[l - m];
        a[l + m] = cmk<C>(cm * x.x - sm * y.x, cm * x.y - sm * y.y);
        a[l - m] = cmk<C>(sm * x.x + cm * y.x, sm * x.y + cm * y.y);
    }
}

// Dz(sgn * beta) on block a, with cos/sin(m beta) generated by the
// recurrence from (cb, sb) = (cos beta, sin beta) as the block goes (no
// table held in registers across blocks)
template <int l, typename T, typename C>
__device__ __forceinline__ void dz_block_rec(C* a, T cb, T sb, int sgn) {
    T cm = cb, sm = sb;
#pragma unroll
    for (int m = 1; m <= l; ++m) {
        const T s = sgn > 0 ? sm : -sm;
        const C x = a[l + m], y = a[l - m];
        a[l + m] = cmk<C>(cm * x.x - s * y.x, cm * x.y - s * y.y);
        a[l - m] = cmk<C>(s * x.x + cm * y.x, s * x.y + cm * y.y);
        const T cn = cm * cb - sm * sb, sn = sm * cb + cm * sb;
        cm = cn;
        sm = sn;
    }
}

// Block l of D^T (in = 1: Xm Dz(-beta) Xp Dz(-alpha)) or of D (in = 0:
// Dz(alpha) Xm Dz(beta) Xp).  Both directions share one copy of the Xp and
// Xm codelets (half the code of separate forward / backward bodies, which
// keeps the instruction working set of the solve small).
template <int l, typename T, typename C>
__device__ __forceinline__ void rot_block(C* v, int vs, const T* csa, T cb, T sb, int in) {
    constexpr int n = 2 * l + 1;
    C a[n], b[n];
#pragma unroll
    for (int j = 0; j < n; ++j) a[j] = v[(l * l + j) * vs];
    if (in) dz_block<l, T, C>(a, csa, -1);
    XRot<l>::template p<T, C>(a, b);
    dz_block_rec<l, T, C>(b, cb, sb, in ? -1 : +1);
    XRot<l>::template m<T, C>(b, a);
    if (!in) dz_block<l, T, C>(a, csa, +1);
#pragma unroll
    for (int j = 0; j < n; ++j) v[(l * l + j) * vs] = a[j];
}

// D^T (in = 1) or D (in = 0) on the degree blocks l set in lmask;
// cos/sin(m beta) by recurrence from (cb, sb).  Compiled once per precision.
template <typename T>
__device__ __noinline__ void rot_all(typename cvec<T>::t* __restrict__ v, int vs, int L, const T* __restrict__ csa, T cb,
                                     T sb, int in, unsigned lmask) {
    using C = typename cvec<T>::t;
#pragma unroll 1
    for (int l = 0; l <= L; ++l) {
        if (!((lmask >> l) & 1u)) continue;
        switch (l) {
#define WLC_ROT(q)                                      \
    case q:                                             \
        rot_block<q, T, C>(v, vs, csa, cb, sb, in);     \
        break;
            WLC_ROT(0) WLC_ROT(1) WLC_ROT(2) WLC_ROT(3) WLC_ROT(4) WLC_ROT(5) WLC_ROT(6)
            WLC_ROT(7) WLC_ROT(8) WLC_ROT(9) WLC_ROT(10) WLC_ROT(11) WLC_ROT(12)
#undef WLC_ROT
            default:
                break;
        }
    }
}

// Tridiagonal systems of one m (both +m and -m share the real pivots):
// d_0 = A_m, d_j = A_l + e^2/d_{j-1}, e = t z_{l-1}; forward
// y_l = b_l - i (e/d_{j-1}) y_{l-1}; back x_l = (y_l - i t z_l x_{l+1})/d_l.
template <typename T>
__device__ __noinline__ void tridiag_all(typename cvec<T>::t* __restrict__ v, int vs, int L, T t, T c0, T dcoef,
                                         const T* __restrict__ zoff, const T* __restrict__ pivrow, unsigned mmask) {
    using C = typename cvec<T>::t;
#pragma unroll 1
    for (int m = 0; m <= L; ++m) {
        if (!((mmask >> m) & 1u)) continue;
        const int n = L - m + 1;
        T dinv[16];
        // with a pivot table the inverse pivots are read from its row (L1-resident)
        // rather than copied into a runtime-indexed local array
        const T* pr = pivrow ? pivrow + m * (L + 1) - (m * (m - 1)) / 2 : dinv;
        if (!pivrow) {
            T d = c0 + dcoef * (T)(m * (m + 1));
            dinv[0] = (T)1 / d;
            for (int j = 1; j < n; ++j) {
                const int l = m + j;
                const T e = t * zoff[(l - 1) * (l - 1) + (l - 1) + m];
                d = (c0 + dcoef * (T)(l * (l + 1))) + e * (e * dinv[j - 1]);
                dinv[j] = (T)1 / d;
            }
        }
        if (m == 0) {
            int idx = 0;
            C yp = v[0];
            for (int j = 1; j < n; ++j) {
                const int prev = idx;
                idx = j * j + j;
                const T g = t * zoff[prev] * pr[j - 1];
                C y = v[idx * vs];
                y = cmk<C>(fma(g, yp.y, y.x), fma(-g, yp.x, y.y));
                v[idx * vs] = y;
                yp = y;
            }
            C xn = cmk<C>(yp.x * pr[n - 1], yp.y * pr[n - 1]);
            v[idx * vs] = xn;
            for (int j = n - 2; j >= 0; --j) {
                idx = j * j + j;
                const T e = t * zoff[idx];
                const C y = v[idx * vs];
                xn = cmk<C>(fma(e, xn.y, y.x) * pr[j], fma(-e, xn.x, y.y) * pr[j]);
                v[idx * vs] = xn;
            }
            continue;
        }
        // the +m and -m systems share the pivots: both chains advance in
        // lockstep (two independent dependency chains per step)
        int ip = m * m + 2 * m, im = m * m;
        C yp = v[ip * vs], ym = v[im * vs];
        for (int j = 1; j < n; ++j) {
            const int l = m + j;
            const int pp = ip, pm = im;
            ip = l * l + l + m;
            im = l * l + l - m;
            const T gp = t * zoff[pp] * pr[j - 1], gm = t * zoff[pm] * pr[j - 1];
            C y1 = v[ip * vs], y2 = v[im * vs];
            y1 = cmk<C>(fma(gp, yp.y, y1.x), fma(-gp, yp.x, y1.y));
            y2 = cmk<C>(fma(gm, ym.y, y2.x), fma(-gm, ym.x, y2.y));
            v[ip * vs] = y1;
            v[im * vs] = y2;
            yp = y1;
            ym = y2;
        }
        C xp = cmk<C>(yp.x * pr[n - 1], yp.y * pr[n - 1]);
        C xm = cmk<C>(ym.x * pr[n - 1], ym.y * pr[n - 1]);
        v[ip * vs] = xp;
        v[im * vs] = xm;
        for (int j = n - 2; j >= 0; --j) {
            const int l = m + j;
            ip = l * l + l + m;
            im = l * l + l - m;
            const T ep = t * zoff[ip], em = t * zoff[im];
            const C y1 = v[ip * vs], y2 = v[im * vs];
            xp = cmk<C>(fma(ep, xp.y, y1.x) * pr[j], fma(-ep, xp.x, y1.y) * pr[j]);
            xm = cmk<C>(fma(em, xm.y, y2.x) * pr[j], fma(-em, xm.x, y2.y) * pr[j]);
            v[ip * vs] = xp;
            v[im * vs] = xm;
        }
    }
}

// asynchronous global -> shared copy of one complex element (cp.async:
// the column loads are all in flight before the tables are staged)
template <typename C> __device__ __forceinline__ void cp_async_elem(C* sdst, const C* gsrc) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
    if constexpr (sizeof(C) == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gsrc) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(gsrc) : "memory");
}

template <typename X> __device__ __forceinline__ void stage(X* dst, const X* src, int n) {
    for (int e = threadIdx.x; e < n; e += blockDim.x) dst[e] = src[e];
}

template <typename T, int N, bool B = false>
__global__ void __launch_bounds__(kSolveThreads, (sizeof(T) == 4) ? 2 : 1)
    zfft_solve(SolveArgs<T> a0, const SolveArgs<T>* __restrict__ batch) {
    const SolveArgs<T> a = pick_args<B>(a0, batch);
    using C = typename cvec<T>::t;
    constexpr int NP = N + 1;
    const SolveTablesT<T>& g = a.tab;
    const int M = g.M, L = g.L;
    // the FP32 first-order correction exists in the FP64 path only
    const int correct = sizeof(T) == 8 ? a.correct : 0;
    const SolveSmem sm = solve_smem(N, M, L, g.ndr, sizeof(T), correct);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* col = reinterpret_cast<C*>(smem_raw + sm.col);
    C* tw = reinterpret_cast<C*>(smem_raw + sm.tw);
    T* csa = reinterpret_cast<T*>(smem_raw + sm.csa);
    float* csaf = reinterpret_cast<float*>(smem_raw + sm.csaf);
    T* s_zoff = reinterpret_cast<T*>(smem_raw + sm.zoff);
    float* s_zofff = reinterpret_cast<float*>(smem_raw + sm.zofff);
    int* s_drp = reinterpret_cast<int*>(smem_raw + sm.dr_ptr);
    int16_t* s_drc = reinterpret_cast<int16_t*>(smem_raw + sm.dr_col);
    int8_t* s_dra = reinterpret_cast<int8_t*>(smem_raw + sm.dr_axis);
    float* s_drv = reinterpret_cast<float*>(smem_raw + sm.dr_valf);
    float2* corr = reinterpret_cast<float2*>(smem_raw + sm.corr);
    const int colid = blockIdx.x;
    C* gcol = a.phat + (size_t)colid * M * N;
    for (int e = threadIdx.x; e < M * N; e += blockDim.x) cp_async_elem(col + (e / N) * NP + (e % N), gcol + e);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    stage(s_zoff, g.zoff, M);
    if (correct) {
        stage(s_zofff, g.zofff, M);
        stage(s_drp, g.dr_ptr, M + 1);
        stage(s_drc, g.dr_col, g.ndr);
        stage(s_dra, g.dr_axis, g.ndr);
        stage(s_drv, g.dr_valf, g.ndr);
    }
    const int kyi = colid / a.nkx, kxi = colid % a.nkx;
    const int ix = fold_n(kxi, N), iy = fold_n(kyi, N);
    const double kx = ix * a.kf[0], ky = iy * a.kf[1];
    for (int e = threadIdx.x; e < N; e += blockDim.x) tw[e] = a.twg[e];
    if (threadIdx.x == 0) {
        const double rho = sqrt(kx * kx + ky * ky);
        const double ca = rho > 0 ? kx / rho : 1.0, sa = rho > 0 ? ky / rho : 0.0;
        double cm = 1.0, sm2 = 0.0;
        for (int m = 0; m <= L; ++m) {
            csa[2 * m] = (T)cm;
            csa[2 * m + 1] = (T)sm2;
            csaf[2 * m] = (float)cm;
            csaf[2 * m + 1] = (float)sm2;
            const double cn = cm * ca - sm2 * sa, sn = sm2 * ca + cm * sa;
            cm = cn;
            sm2 = sn;
        }
    }
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    __syncthreads();
    fft_nat2perm<N, -1>(col, M, 1, NP, tw);

    // Work split: thread t owns kz position p = t % N and part t / N of its
    // solve (a greedy balance of the degree blocks and of the m systems
    // over S = blockDim / N parts); the parts meet at CTA barriers.
    const int S = max(1, (int)blockDim.x / N);
    unsigned* masks = reinterpret_cast<unsigned*>(smem_raw + sm.masks);  // [2][S]: l blocks, m systems
    if (threadIdx.x == 0) {
        float load[32];
        for (int q = 0; q < S; ++q) {
            masks[q] = 0u;
            masks[S + q] = 0u;
            load[q] = 0.f;
        }
        for (int l = L; l >= 0; --l) {  // costliest first
            int best = 0;
            for (int q = 1; q < S; ++q)
                if (load[q] < load[best]) best = q;
            masks[best] |= 1u << l;
            load[best] += (float)(l * l + 3 * l + 1);
        }
        for (int q = 0; q < S; ++q) load[q] = 0.f;
        for (int m = 0; m <= L; ++m) {
            int best = 0;
            for (int q = 1; q < S; ++q)
                if (load[q] < load[best]) best = q;
            masks[S + best] |= 1u << m;
            load[best] += (float)((L - m + 1) * (m > 0 ? 2 : 1));
        }
    }
    __syncthreads();
    const int p = threadIdx.x % N, part = threadIdx.x / N;
    const bool active = part < S && (int)threadIdx.x < N * S;
    const unsigned lmask = active ? masks[part] : 0u, mmask = active ? masks[S + part] : 0u;
    const T c0 = (T)a.c0, dcoef = (T)a.dcoef;
    const int iz = fold_n(perm_index<N>(p), N);
    const double kz = iz * a.kf[2];
    // angle of k to z and sigma ds |k|: in FP64 for FP64 propagators, in FP32
    // for FP32 ones (every thread runs this, and the FP64 pipe is a small
    // fraction of the FP32 pipe)
    const int key = ix * ix + iy * iy + iz * iz;
    const T* pivrow = a.pivtab ? a.pivtab + (size_t)key * a.npiv : nullptr;
    T cb, sb, t;
    if constexpr (sizeof(T) == 8) {
        const double rho = sqrt(kx * kx + ky * ky);
        const double kn = sqrt(rho * rho + kz * kz);
        cb = kn > 0 ? kz / kn : 1.0;
        sb = kn > 0 ? rho / kn : 0.0;
        t = a.sigma * a.ds * kn;
    } else {
        // every operation rounded explicitly (no contraction choices, so all
        // instantiations agree bit for bit); with a pivot table ds |k| is
        // formed from the key exactly as the table forms it
        const float kxf = __fmul_rn((float)ix, (float)a.kf[0]), kyf = __fmul_rn((float)iy, (float)a.kf[1]);
        const float kzf = __fmul_rn((float)iz, (float)a.kf[2]);
        const float rho = __fsqrt_rn(__fadd_rn(__fmul_rn(kxf, kxf), __fmul_rn(kyf, kyf)));
        const float kn = __fsqrt_rn(__fadd_rn(__fmul_rn(rho, rho), __fmul_rn(kzf, kzf)));
        cb = kn > 0.f ? __fdiv_rn(kzf, kn) : 1.f;
        sb = kn > 0.f ? __fdiv_rn(rho, kn) : 0.f;
        const float tk = pivrow ? __fmul_rn((float)(a.ds * a.kf[0]), __fsqrt_rn((float)key)) : __fmul_rn((float)a.ds, kn);
        t = a.sigma > 0 ? tk : -tk;
    }
    C* v = col + p;
    rot_all<T>(v, NP, L, csa, cb, sb, 1, lmask);
    __syncthreads();
    tridiag_all<T>(v, NP, L, t, c0, dcoef, s_zoff, pivrow, mmask);
    __syncthreads();
    rot_all<T>(v, NP, L, csa, cb, sb, 0, lmask);
    __syncthreads();
    if (correct) {
        // x -= G_cov^-1 (i sigma ds (k . dR) x), in FP32
        const float sds = (float)(a.sigma * a.ds);
        const float kk[3] = {(float)kx, (float)ky, (float)kz};
        float2* r = corr + p;
        for (int l = 0; l <= L; ++l) {
            if (!((lmask >> l) & 1u)) continue;
            for (int i = l * l; i < (l + 1) * (l + 1); ++i) {
                float ax = 0.f, ay = 0.f;
                for (int e = s_drp[i]; e < s_drp[i + 1]; ++e) {
                    const float gv = kk[s_dra[e]] * s_drv[e];
                    const C x = v[s_drc[e] * NP];
                    ax = fmaf(gv, (float)x.x, ax);
                    ay = fmaf(gv, (float)x.y, ay);
                }
                r[i * N] = make_float2(-sds * ay, sds * ax);
            }
        }
        __syncthreads();
        rot_all<float>(r, N, L, csaf, (float)cb, (float)sb, 1, lmask);
        __syncthreads();
        tridiag_all<float>(r, N, L, (float)t, (float)a.c0, (float)a.dcoef, s_zofff, nullptr, mmask);
        __syncthreads();
        rot_all<float>(r, N, L, csaf, (float)cb, (float)sb, 0, lmask);
        __syncthreads();
        for (int l = 0; l <= L; ++l) {
            if (!((lmask >> l) & 1u)) continue;
            for (int i = l * l; i < (l + 1) * (l + 1); ++i) {
                const float2 q = r[i * N];
                C x = v[i * NP];
                x.x -= (T)q.x;
                x.y -= (T)q.y;
                v[i * NP] = x;
            }
        }
    }
    __syncthreads();
    fft_perm2nat<N, +1>(col, M, 1, NP, tw);
    if (a.split) {
        // Crank-Nicolson operator (I + ds/2 A)^-1 (I - ds/2 A) = 2 (I + ds/2 A)^-1 - I
        // applied through the z transforms: IFFT_z(2x - b) = 2 IFFT_z(x) - N b,
        // with b the column as pass A wrote it (still in phat)
        for (int e = threadIdx.x; e < M * N; e += blockDim.x) {
            const C x = col[(e / N) * NP + (e % N)], b = gcol[e];
            gcol[e] = cmk<C>(fma((T)2, x.x, -(T)N * b.x), fma((T)2, x.y, -(T)N * b.y));
        }
    } else {
        for (int e = threadIdx.x; e < M * N; e += blockDim.x) gcol[e] = col[(e / N) * NP + (e % N)];
    }
}

// inverse pivots 1/d_j of the tridiagonal systems for every key
// ix^2+iy^2+iz^2 <= nkeys-1 (isotropic spacing), one (order, block)
template <typename T>
__global__ void pivot_table(T* out, int nkeys, int L, double c0, double dcoef, double ds, double kf,
                            const T* __restrict__ zoff) {
    const int npiv = (L + 1) * (L + 2) / 2;
    for (int key = blockIdx.x * blockDim.x + threadIdx.x; key < nkeys; key += gridDim.x * blockDim.x) {
        // ds |k| as the solve kernel forms it for this precision
        T t;
        if constexpr (sizeof(T) == 8)
            t = ds * kf * sqrt((double)key);
        else
            t = __fmul_rn((float)(ds * kf), __fsqrt_rn((float)key));
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

template <typename T> size_t solve_smem_bytes(const SolveArgs<T>& a) {
    const int N = 2 * (a.nkx - 1);
    return solve_smem(N, a.tab.M, a.tab.L, a.tab.ndr, sizeof(T), a.correct).total;
}

// threads per solve CTA: N x S with S parts per kz position (the solve
// splits each kz system over S threads); 0 = the default kSolveThreads
template <int N> static int solve_block(int threads) {
    if (threads <= 0) return kSolveThreads;
    const int S = threads / N < 1 ? 1 : threads / N;
    const int b = N * S;
    return b > kSolveThreads ? (kSolveThreads / N) * N : b;
}

template <typename T, int N> static cudaError_t launch_solve_n(const SolveArgs<T>& a, cudaStream_t st, int threads) {
    if (const cudaError_t e = smem_attr_once((const void*)zfft_solve<T, N>, 227 * 1024); e != cudaSuccess) return e;
    zfft_solve<T, N><<<a.nkx * N, solve_block<N>(threads), solve_smem_bytes<T>(a), st>>>(a, nullptr);
    return cudaGetLastError();
}

template <typename T> cudaError_t launch_solve(int N, const SolveArgs<T>& a, cudaStream_t st, int threads) {
    switch (N) {
#define WLC_CASE(n) \
    case n:         \
        return launch_solve_n<T, n>(a, st, threads);
        WLC_FOR_EACH_N(WLC_CASE)
#undef WLC_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

template <int N> static cudaError_t set_solve_batched_attr() {
    return smem_attr_once((const void*)zfft_solve<float, N, true>, 227 * 1024);
}

template <int N> static cudaError_t launch_solve_batched_n(const BatchLaunch<float>& b, cudaStream_t st) {
    if (const cudaError_t e = set_solve_batched_attr<N>(); e != cudaSuccess) return e;
    zfft_solve<float, N, true><<<dim3(b.nkx * N, 1, b.count), solve_block<N>(b.solve_threads), b.solve_smem, st>>>(
        SolveArgs<float>{}, b.dsolve);
    return cudaGetLastError();
}

cudaError_t launch_solve_batched(int N, const BatchLaunch<float>& b, cudaStream_t st) {
    switch (N) {
#define WLC_CASE(n) \
    case n:         \
        return launch_solve_batched_n<n>(b, st);
        WLC_FOR_EACH_BATCH_N(WLC_CASE)
#undef WLC_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

cudaError_t prepare_solve_batched(int N) {
    switch (N) {
#define WLC_CASE(n) \
    case n:         \
        return set_solve_batched_attr<n>();
        WLC_FOR_EACH_BATCH_N(WLC_CASE)
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

template cudaError_t launch_solve<double>(int, const SolveArgs<double>&, cudaStream_t, int);
template cudaError_t launch_solve<float>(int, const SolveArgs<float>&, cudaStream_t, int);
template size_t solve_smem_bytes<double>(const SolveArgs<double>&);
template size_t solve_smem_bytes<float>(const SolveArgs<float>&);
template cudaError_t launch_pivot_table<double>(double*, int, int, double, double, double, double, const double*,
                                                cudaStream_t);
template cudaError_t launch_pivot_table<float>(float*, int, int, double, double, double, double, const float*,
                                               cudaStream_t);

}  // namespace wlc
