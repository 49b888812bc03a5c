// wlc_step.cu -- kernels of one contour step (passes A, B, C; see
// wlc_kernels.cuh) and their host launchers, instantiated for every
// supported grid edge N and for FP64 / FP32.
#include <cstdio>

#include "wlc_kernels.cuh"
#include "wlc_step.h"

namespace wlc {

__device__ __forceinline__ int fold_idx(int i, int n) { return i <= n / 2 ? i : i - n; }

// BDF right-hand side at grid point r of coefficient i (init_pr,
// MDE_ABC.f90:245-375): order 1 (1 - ds w) q1; order 2
// 2 q1 - q2/2 - ds w (2 q1 - q2); order 3 sum_j c_j(r) q_j with
// c = (3 - 3 ds w, -3/2 + 3 ds w, 1/3 - ds w) precomputed per block.
template <typename T, int NR>
__device__ __forceinline__ T rhs_value(const StepArgs<T>& a, size_t off, size_t r) {
    T v;
    if (a.order == 0) {
        v = a.h1[off];
    } else if (a.order == 1) {
        const T W = (T)a.wb[r];
        v = ((T)1 - a.ds * W) * a.h1[off];
    } else if (a.order == 2) {
        const T W = (T)a.wb[r];
        const T q1 = a.h1[off], q2 = a.h2[off];
        v = (T)2 * q1 - (T)0.5 * q2 - a.ds * W * ((T)2 * q1 - q2);
    } else {
        v = a.cf[r] * a.h1[off];
        v = fma(a.cf[NR + r], a.h2[off], v);
        v = fma(a.cf[2 * (size_t)NR + r], a.h3[off], v);
    }
    if (a.msterm) v += a.msterm[off];
    return v;
}

// ---------------------------------------------------------------- pass A
template <typename T, int N>
__global__ void __launch_bounds__(256) rhs_fft_xy(StepArgs<T> a) {
    using C = typename cvec<T>::t;
    constexpr int Z = zg_planes(N, sizeof(T));
    constexpr int NKX = N / 2 + 1;
    constexpr int NR = N * N * N;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* zb = tw + N;              // (N/2) x N packed row pairs
    C* out = zb + (N / 2) * N;   // Z x N x NKX half spectra
    const int i = blockIdx.y;
    const int z0 = blockIdx.x * Z;
    for (int e = threadIdx.x; e < N; e += blockDim.x) tw[e] = a.twg[e];
    for (int zz = 0; zz < Z; ++zz) {
        const int z = z0 + zz;
        for (int e = threadIdx.x; e < (N / 2) * N; e += blockDim.x) {
            const int p = e / N, x = e % N;
            const size_t ra = ((size_t)z * N + 2 * p) * N + x, rb = ra + N;
            const T va = rhs_value<T, NR>(a, (size_t)i * NR + ra, ra);
            const T vb = rhs_value<T, NR>(a, (size_t)i * NR + rb, rb);
            zb[e] = cmk<C>(va, vb);
        }
        __syncthreads();
        fft_nat2perm<N, -1>(zb, N / 2, 1, N, tw);
        C* o = out + (size_t)zz * N * NKX;
        // split the transform of (row 2p) + i (row 2p+1) into two half spectra
        for (int e = threadIdx.x; e < (N / 2) * NKX; e += blockDim.x) {
            const int p = e / NKX, k = e % NKX;
            const C zk = zb[p * N + perm_pos<N>(k)];
            const C zm = zb[p * N + perm_pos<N>((N - k) % N)];
            o[(2 * p) * NKX + k] = cmk<C>((T)0.5 * (zk.x + zm.x), (T)0.5 * (zk.y - zm.y));
            o[(2 * p + 1) * NKX + k] = cmk<C>((T)0.5 * (zk.y + zm.y), (T)0.5 * (zm.x - zk.x));
        }
        __syncthreads();
        fft_nat2perm<N, -1>(o, NKX, NKX, 1, tw);
    }
    for (int e = threadIdx.x; e < N * NKX; e += blockDim.x) {
        const int ky = e / NKX, kx = e % NKX;
        const size_t colid = (size_t)ky * NKX + kx;
        C* dst = a.phat + (colid * a.M + i) * N + z0;
        const int pos = perm_pos<N>(ky) * NKX + kx;
#pragma unroll
        for (int zz = 0; zz < Z; ++zz) dst[zz] = out[(size_t)zz * N * NKX + pos];
    }
}

// ---------------------------------------------------------------- pass C
template <typename T, int N>
__global__ void __launch_bounds__(256) ifft_xy(StepArgs<T> a) {
    using C = typename cvec<T>::t;
    constexpr int Z = zg_planes(N, sizeof(T));
    constexpr int NKX = N / 2 + 1;
    constexpr int NR = N * N * N;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* zb = tw + N;
    C* out = zb + (N / 2) * N;
    const int i = blockIdx.y;
    const int z0 = blockIdx.x * Z;
    for (int e = threadIdx.x; e < N; e += blockDim.x) tw[e] = a.twg[e];
    for (int e = threadIdx.x; e < N * NKX; e += blockDim.x) {
        const C* src = a.phat + ((size_t)e * a.M + i) * N + z0;
#pragma unroll
        for (int zz = 0; zz < Z; ++zz) out[(size_t)zz * N * NKX + e] = src[zz];
    }
    __syncthreads();
    for (int zz = 0; zz < Z; ++zz) {
        C* o = out + (size_t)zz * N * NKX;
        fft_nat2perm<N, +1>(o, NKX, NKX, 1, tw);  // along y; row y now at perm_pos(y)
        // Hermitian extension of rows (2p, 2p+1) packed as one complex row;
        // the imaginary parts at kx = 0 and N/2 are discarded (c2r)
        for (int e = threadIdx.x; e < (N / 2) * N; e += blockDim.x) {
            const int p = e / N, k = e % N;
            const C* ra = o + perm_pos<N>(2 * p) * NKX;
            const C* rb = o + perm_pos<N>(2 * p + 1) * NKX;
            C xa, xb;
            if (k <= N / 2) {
                xa = ra[k];
                xb = rb[k];
                if (k == 0 || k == N / 2) {
                    xa.y = (T)0;
                    xb.y = (T)0;
                }
            } else {
                xa = ra[N - k];
                xb = rb[N - k];
                xa.y = -xa.y;
                xb.y = -xb.y;
            }
            zb[e] = cmk<C>(xa.x - xb.y, xa.y + xb.x);
        }
        __syncthreads();
        fft_nat2perm<N, +1>(zb, N / 2, 1, N, tw);  // along x; x at perm_pos(x)
        T* dst = a.qout + (size_t)i * NR + (size_t)(z0 + zz) * N * N;
        for (int e = threadIdx.x; e < N * N; e += blockDim.x) {
            const int y = e / N, x = e % N;
            const C v = zb[(y >> 1) * N + perm_pos<N>(x)];
            dst[e] = ((y & 1) ? v.y : v.x) * a.minv;
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- pass B
// Real-harmonic z rotation on the (m, -m) pairs of `v` (element (i, c) at
// v[i*vs + c]); cs holds cos/sin(m*gamma) for m = 0..L, per column c when
// percol (stride 2(L+1)).  sgn = -1 applies Dz(-gamma).
template <typename T, typename C>
__device__ __forceinline__ void dz_rotate(C* v, int vs, int nc, const T* cs, bool percol, int sgn,
                                          const SolveTablesT<T>& tb) {
    const int L = tb.L;
    for (int w = threadIdx.x; w < tb.npairs * nc; w += blockDim.x) {
        const int q = w / nc, c = w % nc;
        const int ic = tb.pairs[3 * q], is = tb.pairs[3 * q + 1], m = tb.pairs[3 * q + 2];
        const T* cc = percol ? cs + (size_t)c * 2 * (L + 1) : cs;
        const T cm = cc[2 * m], sm = sgn * cc[2 * m + 1];
        const C x = v[ic * vs + c], y = v[is * vs + c];
        v[ic * vs + c] = cmk<C>(cm * x.x - sm * y.x, cm * x.y - sm * y.y);
        v[is * vs + c] = cmk<C>(sm * x.x + cm * y.x, sm * x.y + cm * y.y);
    }
}

template <typename T, typename C>
__device__ __forceinline__ void csr_apply(const int* ptr, const int16_t* col, const T* val, const C* in, int is,
                                          C* out, int os, int M, int nc) {
    for (int w = threadIdx.x; w < M * nc; w += blockDim.x) {
        const int i = w / nc, c = w % nc;
        T ax = 0, ay = 0;
        for (int e = ptr[i]; e < ptr[i + 1]; ++e) {
            const T g = val[e];
            const C x = in[col[e] * is + c];
            ax = fma(g, x.x, ax);
            ay = fma(g, x.y, ay);
        }
        out[i * os + c] = cmk<C>(ax, ay);
    }
}

// One tridiagonal complex-symmetric system per m (real pivots):
// (A_l) x_l + i t (z_{l-1} x_{l-1} + z_l x_{l+1}) = b_l, l = |m|..L.
template <typename T, typename C>
__device__ __forceinline__ void tridiag(C* v, int vs, int nc, const T* tk, T c0, T dcoef, const SolveTablesT<T>& tb) {
    const int L = tb.L;
    for (int w = threadIdx.x; w < (2 * L + 1) * nc; w += blockDim.x) {
        const int m = w / nc - L, c = w % nc;
        const int am = m < 0 ? -m : m;
        const T t = tk[c];
        T dinv[16];
        int l = am;
        int idx = l * l + l + m;
        dinv[0] = (T)1 / (c0 + dcoef * (T)(l * (l + 1)));
        C yp = v[idx * vs + c];
        for (int j = 1; j <= L - am; ++j) {
            l = am + j;
            const int prev = idx;
            idx = l * l + l + m;
            const T e = t * tb.zoff[prev];
            const T g = e * dinv[j - 1];
            const T d = (c0 + dcoef * (T)(l * (l + 1))) + e * g;
            dinv[j] = (T)1 / d;
            C y = v[idx * vs + c];
            y = cmk<C>(fma(g, yp.y, y.x), fma(-g, yp.x, y.y));
            v[idx * vs + c] = y;
            yp = y;
        }
        C xn = cmk<C>(yp.x * dinv[L - am], yp.y * dinv[L - am]);
        v[idx * vs + c] = xn;
        for (int j = L - am - 1; j >= 0; --j) {
            l = am + j;
            idx = l * l + l + m;
            const T e = t * tb.zoff[idx];
            const C y = v[idx * vs + c];
            xn = cmk<C>(fma(e, xn.y, y.x) * dinv[j], fma(-e, xn.x, y.y) * dinv[j]);
            v[idx * vs + c] = xn;
        }
    }
}

// x <- D (A + i sigma ds |k| Rz)^-1 D^T x, D = Dz(alpha) Xm Dz(beta) Xp
template <typename T, typename C>
__device__ __forceinline__ void cov_solve(C* v, int vs, C* tmp, int ts, int nc, const T* csa, const T* csb,
                                          const T* tk, T c0, T dcoef, const SolveTablesT<T>& tb) {
    const int M = tb.M;
    dz_rotate<T, C>(v, vs, nc, csa, false, -1, tb);
    __syncthreads();
    csr_apply<T, C>(tb.xp_ptr, tb.xp_col, tb.xp_val, v, vs, tmp, ts, M, nc);
    __syncthreads();
    dz_rotate<T, C>(tmp, ts, nc, csb, true, -1, tb);
    __syncthreads();
    csr_apply<T, C>(tb.xm_ptr, tb.xm_col, tb.xm_val, tmp, ts, v, vs, M, nc);
    __syncthreads();
    tridiag<T, C>(v, vs, nc, tk, c0, dcoef, tb);
    __syncthreads();
    csr_apply<T, C>(tb.xp_ptr, tb.xp_col, tb.xp_val, v, vs, tmp, ts, M, nc);
    __syncthreads();
    dz_rotate<T, C>(tmp, ts, nc, csb, true, +1, tb);
    __syncthreads();
    csr_apply<T, C>(tb.xm_ptr, tb.xm_col, tb.xm_val, tmp, ts, v, vs, M, nc);
    __syncthreads();
    dz_rotate<T, C>(v, vs, nc, csa, false, +1, tb);
    __syncthreads();
}

template <typename T, int N>
__global__ void __launch_bounds__(256) zfft_solve(SolveArgs<T> a) {
    using C = typename cvec<T>::t;
    const SolveTablesT<T>& tb = a.tab;
    const int M = tb.M, L = tb.L, KC = a.kc;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* col = reinterpret_cast<C*>(smem_raw);
    C* tmp = col + (size_t)M * N;
    C* cor = tmp + (size_t)M * KC;
    C* tw = cor + (size_t)M * KC;
    T* csa = reinterpret_cast<T*>(tw + N);
    T* csb = csa + 2 * (L + 1);
    T* tk = csb + (size_t)KC * 2 * (L + 1);
    T* kz3 = tk + KC;

    const int colid = blockIdx.x;
    const int kyi = colid / a.nkx, kxi = colid % a.nkx;
    const double kx = fold_idx(kxi, N) * a.kf[0];
    const double ky = fold_idx(kyi, N) * a.kf[1];
    const double rho = sqrt(kx * kx + ky * ky);
    C* g = a.phat + (size_t)colid * M * N;
    for (int e = threadIdx.x; e < M * N; e += blockDim.x) col[e] = g[e];
    for (int e = threadIdx.x; e < N; e += blockDim.x) tw[e] = a.twg[e];
    if (threadIdx.x == 0) {
        const double ca = rho > 0 ? kx / rho : 1.0, sa = rho > 0 ? ky / rho : 0.0;
        double cm = 1.0, sm = 0.0;
        for (int m = 0; m <= L; ++m) {
            csa[2 * m] = (T)cm;
            csa[2 * m + 1] = (T)sm;
            const double cn = cm * ca - sm * sa, sn = sm * ca + cm * sa;
            cm = cn;
            sm = sn;
        }
    }
    __syncthreads();
    fft_nat2perm<N, -1>(col, M, 1, N, tw);
    const T c0 = (T)a.c0, dcoef = (T)a.dcoef;
    for (int p0 = 0; p0 < N; p0 += KC) {
        const int nc = min(KC, N - p0);
        for (int c = threadIdx.x; c < nc; c += blockDim.x) {
            const int kzi = perm_index<N>(p0 + c);
            const double kz = fold_idx(kzi, N) * a.kf[2];
            const double kn = sqrt(rho * rho + kz * kz);
            const double cb = kn > 0 ? kz / kn : 1.0, sb = kn > 0 ? rho / kn : 0.0;
            double cm = 1.0, sm = 0.0;
            T* cs = csb + (size_t)c * 2 * (L + 1);
            for (int m = 0; m <= L; ++m) {
                cs[2 * m] = (T)cm;
                cs[2 * m + 1] = (T)sm;
                const double cn = cm * cb - sm * sb, sn = sm * cb + cm * sb;
                cm = cn;
                sm = sn;
            }
            tk[c] = (T)(a.sigma * a.ds * kn);
            kz3[c] = (T)kz;
        }
        __syncthreads();
        C* v = col + p0;
        cov_solve<T, C>(v, N, tmp, KC, nc, csa, csb, tk, c0, dcoef, tb);
        if (tb.ndr > 0) {
            // first-order correction for the reference's non-covariant
            // rounding of Rx/Ry: x -= G_cov^-1 (i sigma ds dK x)
            const T sds = (T)(a.sigma * a.ds);
            for (int w = threadIdx.x; w < M * nc; w += blockDim.x) {
                const int i = w / nc, c = w % nc;
                const T kk[3] = {(T)kx, (T)ky, kz3[c]};
                T ax = 0, ay = 0;
                for (int e = tb.dr_ptr[i]; e < tb.dr_ptr[i + 1]; ++e) {
                    const T gv = kk[tb.dr_axis[e]] * tb.dr_val[e];
                    const C x = v[tb.dr_col[e] * N + c];
                    ax = fma(gv, x.x, ax);
                    ay = fma(gv, x.y, ay);
                }
                cor[i * KC + c] = cmk<C>(-sds * ay, sds * ax);
            }
            __syncthreads();
            cov_solve<T, C>(cor, KC, tmp, KC, nc, csa, csb, tk, c0, dcoef, tb);
            for (int w = threadIdx.x; w < M * nc; w += blockDim.x) {
                const int i = w / nc, c = w % nc;
                v[i * N + c] = csub(v[i * N + c], cor[i * KC + c]);
            }
            __syncthreads();
        }
    }
    fft_perm2nat<N, +1>(col, M, 1, N, tw);
    for (int e = threadIdx.x; e < M * N; e += blockDim.x) g[e] = col[e];
}

// right-hand side only (init_pr test hook), out[i][r]
template <typename T, int N>
__global__ void __launch_bounds__(256) rhs_only(StepArgs<T> a, T* out) {
    constexpr int NR = N * N * N;
    const int64_t n = (int64_t)a.M * NR;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        out[e] = rhs_value<T, NR>(a, (size_t)e, (size_t)(e % NR));
}

// ------------------------------------------------------------ launchers
template <typename T> size_t smem_xy(int N) {
    using C = typename cvec<T>::t;
    return sizeof(C) * ((size_t)N + (size_t)(N / 2) * N + (size_t)zg_planes(N, sizeof(T)) * N * (N / 2 + 1));
}

template <typename T> size_t smem_solve(int N, int M, int L, int kc) {
    using C = typename cvec<T>::t;
    return sizeof(C) * ((size_t)M * N + 2 * (size_t)M * kc + N) +
           sizeof(T) * (2 * (size_t)(L + 1) * (1 + kc) + 2 * (size_t)kc);
}

template <typename T, int N> static cudaError_t launch_n(const StepLaunch<T>& s, cudaStream_t st) {
    constexpr int Z = zg_planes(N, sizeof(T));
    const size_t sxy = smem_xy<T>(N);
    const size_t ssv = smem_solve<T>(N, s.solve.tab.M, s.solve.tab.L, s.solve.kc);
    static bool attr_done = false;
    if (!attr_done) {
        cudaFuncSetAttribute(rhs_fft_xy<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(ifft_xy<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        cudaFuncSetAttribute(zfft_solve<T, N>, cudaFuncAttributeMaxDynamicSharedMemorySize, 227 * 1024);
        attr_done = true;
    }
    const dim3 gxy(N / Z, s.step.M);
    if (s.events) cudaEventRecord(s.events[0], st);
    if (s.do_a) rhs_fft_xy<T, N><<<gxy, 256, sxy, st>>>(s.step);
    if (s.events) cudaEventRecord(s.events[1], st);
    if (s.do_b) zfft_solve<T, N><<<s.solve.nkx * N, 256, ssv, st>>>(s.solve);
    if (s.events) cudaEventRecord(s.events[2], st);
    if (s.do_c) ifft_xy<T, N><<<gxy, 256, sxy, st>>>(s.step);
    if (s.events) cudaEventRecord(s.events[3], st);
    return cudaGetLastError();
}

template <typename T> cudaError_t launch_step(int N, const StepLaunch<T>& s, cudaStream_t st) {
    switch (N) {
#define WLC_CASE(n) \
    case n:         \
        return launch_n<T, n>(s, st);
        WLC_FOR_EACH_N(WLC_CASE)
#undef WLC_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

template <typename T> cudaError_t launch_rhs_only(int N, const StepArgs<T>& a, T* out, cudaStream_t st) {
    switch (N) {
#define WLC_CASE(n)                                                                \
    case n: {                                                                      \
        const int64_t tot = (int64_t)a.M * n * n * n;                              \
        const int g = (int)((tot + 255) / 256 > 4096 ? 4096 : (tot + 255) / 256); \
        rhs_only<T, n><<<g, 256, 0, st>>>(a, out);                                 \
        return cudaGetLastError();                                                 \
    }
        WLC_FOR_EACH_N(WLC_CASE)
#undef WLC_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

template cudaError_t launch_rhs_only<double>(int, const StepArgs<double>&, double*, cudaStream_t);
template cudaError_t launch_rhs_only<float>(int, const StepArgs<float>&, float*, cudaStream_t);
template cudaError_t launch_step<double>(int, const StepLaunch<double>&, cudaStream_t);
template cudaError_t launch_step<float>(int, const StepLaunch<float>&, cudaStream_t);
template size_t smem_xy<double>(int);
template size_t smem_xy<float>(int);
template size_t smem_solve<double>(int, int, int, int);
template size_t smem_solve<float>(int, int, int, int);

}  // namespace wlc
