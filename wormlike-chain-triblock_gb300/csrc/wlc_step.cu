// wlc_step.cu -- kernels of one contour step (passes A, B, C; see
// wlc_kernels.cuh) and their host launchers, instantiated for every
// supported grid edge N and for FP64 / FP32.
#include <cstdio>

#include "wlc_attr.h"
#include "wlc_kernels.cuh"
#include "wlc_step.h"

namespace wlc {

__device__ __forceinline__ int fold_idx(int i, int n) { return i <= n / 2 ? i : i - n; }

// BDF right-hand side at grid point r of coefficient i (init_pr,
// MDE_ABC.f90:245-375): order 1 (1 - ds w) q1; order 2
// 2 q1 - q2/2 - ds w (2 q1 - q2); order 3 sum_j c_j(r) q_j with
// c = (3 - 3 ds w, -3/2 + 3 ds w, 1/3 - ds w) precomputed per block.
// FP32 form shared by both pass-A kernels (so that they give identical
// results): dw = ds w(r) rounded once, every operation rounded explicitly.
// Split-scheme steps (kSplitOrder) pass e^{-w ds/2} as dw: q1 e^{-w ds/2}.
__device__ __forceinline__ float rhs_f32(int order, float q1, float q2, float q3, float dw, float third) {
    if (order == 0) return q1;
    if (order == kSplitOrder) return __fmul_rn(dw, q1);
    if (order == 1) return __fmul_rn(__fsub_rn(1.0f, dw), q1);
    if (order == 2) {
        const float t = __fsub_rn(__fmul_rn(2.0f, q1), q2);
        return __fsub_rn(__fsub_rn(__fmul_rn(2.0f, q1), __fmul_rn(0.5f, q2)), __fmul_rn(dw, t));
    }
    const float dw3 = __fmul_rn(3.0f, dw);
    const float c1 = __fsub_rn(3.0f, dw3), c2 = __fadd_rn(-1.5f, dw3), c3 = __fsub_rn(third, dw);
    return __fmaf_rn(c3, q3, __fmaf_rn(c2, q2, __fmul_rn(c1, q1)));
}

template <typename T, int NR>
__device__ __forceinline__ T rhs_value(const StepArgs<T>& a, size_t off, size_t r) {
    if constexpr (sizeof(T) == 4) {
        const int o = a.order;
        const int nh = hist_slices(o);
        float v = rhs_f32(o, a.h1[off], nh >= 2 ? a.h2[off] : 0.0f, nh >= 3 ? a.h3[off] : 0.0f,
                          o >= 1 ? a.dsw[r] : 0.0f, a.third);
        if (a.msterm) v += a.msterm[off];
        return v;
    }
    T v;
    if (a.order == 0) {
        v = a.h1[off];
    } else if (a.order == kSplitOrder) {  // e^{-w ds/2} q(s-1)
        v = a.cf[r] * a.h1[off];
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

// rhs_value for four consecutive points (FP32; off and r multiples of 4)
__device__ __forceinline__ float4 ld4(const float* p) { return *reinterpret_cast<const float4*>(p); }
__device__ __forceinline__ float4 rhs_f32x4(const StepArgs<float>& a, size_t off, size_t r) {
    const int o = a.order;
    const int nh = hist_slices(o);
    const float4 z4 = make_float4(0.f, 0.f, 0.f, 0.f);
    const float4 q1 = ld4(a.h1 + off);
    const float4 q2 = nh >= 2 ? ld4(a.h2 + off) : z4;
    const float4 q3 = nh >= 3 ? ld4(a.h3 + off) : z4;
    const float4 dw = o >= 1 ? ld4(a.dsw + r) : z4;
    float4 v = make_float4(rhs_f32(o, q1.x, q2.x, q3.x, dw.x, a.third), rhs_f32(o, q1.y, q2.y, q3.y, dw.y, a.third),
                           rhs_f32(o, q1.z, q2.z, q3.z, dw.z, a.third), rhs_f32(o, q1.w, q2.w, q3.w, dw.w, a.third));
    if (a.msterm) {
        const float4 m = ld4(a.msterm + off);
        v.x += m.x;
        v.y += m.y;
        v.z += m.z;
        v.w += m.w;
    }
    return v;
}

// ------------------------------------------------------- async copies
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc) {
    const unsigned sa = (unsigned)__cvta_generic_to_shared(sdst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(sa), "l"(gsrc) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int n> __device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(n) : "memory");
}

// The half-spectrum planes of a CTA are kept z-fastest, out[(ky*NKX + kx)*Z + zz],
// so that the Z values of one (col, i) run in phat move as one 32-byte chunk.

// x-FFTs of ZB planes of packed row pairs (zb: ZB consecutive (N/2) x N
// blocks, row stride xrow(N)), split into two half spectra each: planes zz0 .. zz0+ZB-1 of out
// (the y-FFTs of all planes follow in one batched call, y_planes)
template <typename T, int N, int Z, int ZB>
__device__ __forceinline__ void fwd_x_planes(typename cvec<T>::t* zb, typename cvec<T>::t* out, int zz0,
                                             const typename cvec<T>::t* tw) {
    using C = typename cvec<T>::t;
    constexpr int NKX = N / 2 + 1;
    constexpr int XR = xrow(N);
    fft_nat2perm<N, -1>(zb, ZB * (N / 2), 1, XR, tw);
    for (int t = threadIdx.x; t < ZB * (N / 2) * NKX; t += blockDim.x) {
        const int q = t / ((N / 2) * NKX), e = t % ((N / 2) * NKX);
        const int p = e / NKX, k = e % NKX;
        const C* zq = zb + (size_t)q * xplane(N);
        const C zk = zq[p * XR + perm_pos<N>(k)];
        const C zm = zq[p * XR + perm_pos<N>((N - k) % N)];
        out[((2 * p) * NKX + k) * Z + zz0 + q] = cmk<C>((T)0.5 * (zk.x + zm.x), (T)0.5 * (zk.y - zm.y));
        out[((2 * p + 1) * NKX + k) * Z + zz0 + q] = cmk<C>((T)0.5 * (zk.y + zm.y), (T)0.5 * (zm.x - zk.x));
    }
    __syncthreads();
}

// y-FFTs of every (kx, plane) line of out: line kx*Z + zz starts at out + kx*Z + zz,
// element ky at stride NKX*Z
template <typename T, int N, int Z, int DIR>
__device__ __forceinline__ void y_planes(typename cvec<T>::t* out, const typename cvec<T>::t* tw) {
    constexpr int NKX = N / 2 + 1;
    fft_nat2perm<N, DIR>(out, NKX * Z, NKX * Z, 1, tw);
}

// one Z-run per (ky, kx) from the half spectra to phat, in 16-byte pieces
// when a run is a whole number of them (shared reads contiguous per lane)
template <typename T, int N, int Z>
__device__ __forceinline__ void store_phat(const StepArgs<T>& a, const typename cvec<T>::t* out, int i, int z0) {
    using C = typename cvec<T>::t;
    constexpr int NKX = N / 2 + 1;
    constexpr int CH = (Z * (int)sizeof(C)) % 16 == 0 ? (Z * (int)sizeof(C)) / 16 : 0;
    for (int e = threadIdx.x; e < N * NKX; e += blockDim.x) {
        const int ky = e / NKX, kx = e % NKX;
        const size_t colid = (size_t)ky * NKX + kx;
        C* dst = a.phat + (colid * a.M + i) * N + z0;
        const C* src = out + (size_t)(perm_pos<N>(ky) * NKX + kx) * Z;
        if constexpr (CH > 0) {
#pragma unroll
            for (int q = 0; q < CH; ++q) reinterpret_cast<uint4*>(dst)[q] = reinterpret_cast<const uint4*>(src)[q];
        } else {
#pragma unroll
            for (int zz = 0; zz < Z; ++zz) dst[zz] = src[zz];
        }
    }
}

// ---------------------------------------------------------------- pass A
// V: launch variant, bit 0 half the planes per CTA, bit 1 the x-FFTs of all
// planes in one batched call (one packed-row buffer per plane)
template <typename T, int N, int V> struct XyShape {
    static constexpr int Z = xy_planes(N, sizeof(T), V & 1);
    static constexpr int ZB = (V & 2) ? Z : 1;
};

template <typename T, int N, bool B = false, int V = 0>
__global__ void __launch_bounds__(512) rhs_fft_xy(StepArgs<T> a0, const StepArgs<T>* __restrict__ batch) {
    const StepArgs<T> a = pick_args<B>(a0, batch);
    using C = typename cvec<T>::t;
    constexpr int Z = XyShape<T, N, V>::Z, ZB = XyShape<T, N, V>::ZB;
    constexpr int NR = N * N * N;
    constexpr int PB = (N / 2) * N;  // packed row pairs per plane
    constexpr int XR = xrow(N), PBS = xplane(N);
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* zb = tw + N;                  // ZB x (N/2) x N packed row pairs (row stride XR)
    C* out = zb + (size_t)ZB * PBS;  // N x NKX x Z half spectra
    const int i = blockIdx.y;
    const int z0 = blockIdx.x * Z;
    for (int e = threadIdx.x; e < N; e += blockDim.x) tw[e] = a.twg[e];
    for (int zz0 = 0; zz0 < Z; zz0 += ZB) {
        if constexpr (sizeof(T) == 4) {
            // four consecutive x per thread: 16-byte loads of the history, ds*w
            // and Theta planes (N is a multiple of 4).  The four shared stores
            // go out in an order rotated by (t / 4) % 4, which spreads the
            // lanes of a warp over all bank pairs.
            for (int t = threadIdx.x; t < ZB * PB / 4; t += blockDim.x) {
                const int q = t / (PB / 4), e = 4 * (t % (PB / 4));
                const int p = e / N, x = e % N;
                const size_t ra = ((size_t)(z0 + zz0 + q) * N + 2 * p) * N + x, rb = ra + N;
                const float4 va = rhs_f32x4(a, (size_t)i * NR + ra, ra);
                const float4 vb = rhs_f32x4(a, (size_t)i * NR + rb, rb);
                C* zq = zb + (size_t)q * PBS + p * XR + x;
                const int rot = (t >> 2) & 3;
#pragma unroll
                for (int s = 0; s < 4; ++s) {
                    const int c = (s + rot) & 3;
                    const float xa = c == 0 ? va.x : c == 1 ? va.y : c == 2 ? va.z : va.w;
                    const float xb = c == 0 ? vb.x : c == 1 ? vb.y : c == 2 ? vb.z : vb.w;
                    zq[c] = cmk<C>(xa, xb);
                }
            }
        } else {
            for (int t = threadIdx.x; t < ZB * PB; t += blockDim.x) {
                const int q = t / PB, e = t % PB;
                const int p = e / N, x = e % N;
                const size_t ra = ((size_t)(z0 + zz0 + q) * N + 2 * p) * N + x, rb = ra + N;
                const T va = rhs_value<T, NR>(a, (size_t)i * NR + ra, ra);
                const T vb = rhs_value<T, NR>(a, (size_t)i * NR + rb, rb);
                zb[(size_t)q * PBS + p * XR + x] = cmk<C>(va, vb);
            }
        }
        __syncthreads();
        fwd_x_planes<T, N, Z, ZB>(zb, out, zz0, tw);
    }
    y_planes<T, N, Z, -1>(out, tw);
    store_phat<T, N, Z>(a, out, i, z0);
}

// FP32 pass A with the history planes staged by cp.async, double-buffered
// across the CTA's z planes (plane zz+1 in flight while zz is transformed).
template <int N> struct StagedA {
    static constexpr int Z = zg_planes(N, 4);
    static constexpr size_t P = (size_t)N * N;
    static constexpr size_t bytes = 8 * ((size_t)N + (size_t)xplane(N) + (size_t)Z * N * (N / 2 + 1)) + 2 * 4 * P * 4;
    static constexpr bool fits = bytes <= 220 * 1024;
};

__device__ __forceinline__ float rhs_staged(const float* st, int order, size_t P, size_t idx, float third) {
    const float q1 = st[idx];
    if (order == 0) return q1;
    if (order == 1 || order == kSplitOrder) return rhs_f32(order, q1, 0.0f, 0.0f, st[P + idx], third);
    if (order == 2) return rhs_f32(2, q1, st[P + idx], 0.0f, st[2 * P + idx], third);
    return rhs_f32(3, q1, st[P + idx], st[2 * P + idx], st[3 * P + idx], third);
}

template <int N, bool B = false>
__global__ void __launch_bounds__(512) rhs_fft_xy_staged(StepArgs<float> a0, const StepArgs<float>* __restrict__ batch) {
    const StepArgs<float> a = pick_args<B>(a0, batch);
    using C = float2;
    constexpr int Z = StagedA<N>::Z;
    constexpr int NKX = N / 2 + 1;
    constexpr int NR = N * N * N;
    constexpr size_t P = StagedA<N>::P;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* zb = tw + N;                   // packed row pairs, row stride xrow(N)
    C* out = zb + xplane(N);
    float* stage = reinterpret_cast<float*>(out + (size_t)Z * N * NKX);  // [2][4][P]
    const int i = blockIdx.y;
    const int z0 = blockIdx.x * Z;
    const int order = a.order;
    const float* src[4];
    int ns = 0;
    src[ns++] = a.h1 + (size_t)i * NR;
    if (hist_slices(order) >= 2) src[ns++] = a.h2 + (size_t)i * NR;
    if (hist_slices(order) >= 3) src[ns++] = a.h3 + (size_t)i * NR;
    if (order >= 1) src[ns++] = a.dsw;
    auto issue = [&](int zz, int buf) {
        const size_t zoff = (size_t)(z0 + zz) * P;
        for (int q = 0; q < ns; ++q) {
            const float* g = src[q] + zoff;
            float* d = stage + ((size_t)buf * 4 + q) * P;
            for (size_t e = (size_t)threadIdx.x * 4; e < P; e += (size_t)blockDim.x * 4) cp_async16(d + e, g + e);
        }
        cp_async_commit();
    };
    for (int e = threadIdx.x; e < N; e += blockDim.x) tw[e] = a.twg[e];
    issue(0, 0);
    for (int zz = 0; zz < Z; ++zz) {
        if (zz + 1 < Z) {
            issue(zz + 1, (zz + 1) & 1);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const float* st = stage + (size_t)(zz & 1) * 4 * P;
        const size_t zoff = (size_t)(z0 + zz) * P;
        for (int e = threadIdx.x; e < (N / 2) * N; e += blockDim.x) {
            const int p = e / N, x = e % N;
            const size_t ia = (size_t)(2 * p) * N + x, ib = ia + N;
            float va = rhs_staged(st, order, P, ia, a.third);
            float vb = rhs_staged(st, order, P, ib, a.third);
            if (a.msterm) {
                va += a.msterm[(size_t)i * NR + zoff + ia];
                vb += a.msterm[(size_t)i * NR + zoff + ib];
            }
            zb[p * xrow(N) + x] = make_float2(va, vb);
        }
        __syncthreads();
        fwd_x_planes<float, N, Z, 1>(zb, out, zz, tw);
    }
    y_planes<float, N, Z, -1>(out, tw);
    store_phat<float, N, Z>(a, out, i, z0);
}

// ---------------------------------------------------------------- pass C
template <typename T, int N, bool B = false, int V = 0>
__global__ void __launch_bounds__(512) ifft_xy(StepArgs<T> a0, const StepArgs<T>* __restrict__ batch) {
    const StepArgs<T> a = pick_args<B>(a0, batch);
    using C = typename cvec<T>::t;
    constexpr int Z = XyShape<T, N, V>::Z, ZB = XyShape<T, N, V>::ZB;
    constexpr int NKX = N / 2 + 1;
    constexpr int NR = N * N * N;
    constexpr int PB = (N / 2) * N;
    constexpr int XR = xrow(N), PBS = xplane(N);
    static_assert(PBS % 2 == 0, "the half-spectrum buffer must stay 16-byte aligned");
    extern __shared__ __align__(16) unsigned char smem_raw[];
    C* tw = reinterpret_cast<C*>(smem_raw);
    C* zb = tw + N;                   // packed row pairs, row stride XR
    C* out = zb + (size_t)ZB * PBS;
    const int i = blockIdx.y;
    const int z0 = blockIdx.x * Z;
    for (int e = threadIdx.x; e < N; e += blockDim.x) tw[e] = a.twg[e];
    // all loads issued up front: one Z-run (Z * sizeof(C) bytes) per (ky, kx)
    constexpr int CH = (Z * (int)sizeof(C)) / 16;  // 16-byte chunks per run
    static_assert((Z * sizeof(C)) % 16 == 0, "phat runs must be whole 16-byte chunks");
    for (int e = threadIdx.x; e < N * NKX * CH; e += blockDim.x) {
        const int col = e / CH, q = e % CH;
        const C* src = a.phat + ((size_t)col * a.M + i) * N + z0;
        cp_async16(reinterpret_cast<unsigned char*>(out + (size_t)col * Z) + 16 * q,
                   reinterpret_cast<const unsigned char*>(src) + 16 * q);
    }
    cp_async_commit();
    cp_async_wait<0>();
    __syncthreads();
    y_planes<T, N, Z, +1>(out, tw);  // along y for every plane; row y now at perm_pos(y)
    for (int zz0 = 0; zz0 < Z; zz0 += ZB) {
        // Hermitian extension of rows (2p, 2p+1) packed as one complex row;
        // the imaginary parts at kx = 0 and N/2 are discarded (c2r)
        // plane index fastest across the lanes: the ZB values read per
        // (row, k) are adjacent in out
        for (int t = threadIdx.x; t < ZB * PB; t += blockDim.x) {
            const int q = t % ZB, e = t / ZB;
            const int zz = zz0 + q;
            const int p = e / N, k = e % N;
            const C* ra = out + (size_t)perm_pos<N>(2 * p) * NKX * Z + zz;
            const C* rb = out + (size_t)perm_pos<N>(2 * p + 1) * NKX * Z + zz;
            C xa, xb;
            if (k <= N / 2) {
                xa = ra[k * Z];
                xb = rb[k * Z];
                if (k == 0 || k == N / 2) {
                    xa.y = (T)0;
                    xb.y = (T)0;
                }
            } else {
                xa = ra[(N - k) * Z];
                xb = rb[(N - k) * Z];
                xa.y = -xa.y;
                xb.y = -xb.y;
            }
            zb[(size_t)q * PBS + p * XR + k] = cmk<C>(xa.x - xb.y, xa.y + xb.x);
        }
        __syncthreads();
        fft_nat2perm<N, +1>(zb, ZB * (N / 2), 1, XR, tw);  // along x; x at perm_pos(x)
        // packed row pair p holds rows 2p (real part) and 2p+1 (imaginary part)
        for (int t = threadIdx.x; t < ZB * PB; t += blockDim.x) {
            const int q = t / PB, e = t % PB;
            const int p = e / N, x = e % N;
            const C v = zb[(size_t)q * PBS + p * XR + perm_pos<N>(x)];
            const size_t r = (size_t)(z0 + zz0 + q) * N * N + (size_t)(2 * p) * N + x;
            T* dst = a.qout + (size_t)i * NR + r;
            if (a.post) {  // split scheme: the second field half step
                dst[0] = (v.x * a.minv) * a.post[r];
                dst[N] = (v.y * a.minv) * a.post[r + N];
            } else {
                dst[0] = v.x * a.minv;
                dst[N] = v.y * a.minv;
            }
        }
        __syncthreads();
    }
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
template <typename T> size_t smem_xy(int N, int variant) {
    using C = typename cvec<T>::t;
    const int z = xy_planes(N, sizeof(T), variant & 1), zb = (variant & 2) ? z : 1;
    return sizeof(C) * ((size_t)N + (size_t)zb * xplane(N) + (size_t)z * N * (N / 2 + 1));
}

// shared-memory limits of the pass A / pass C kernels of (T, N, B), once per
// (kernel, device); returns the first error
template <typename T, int N, bool B> static cudaError_t set_xy_attrs() {
    constexpr int big = 200 * 1024;
    cudaError_t e = cudaSuccess;
    auto set = [&](const void* fn, int bytes) {
        const cudaError_t r = smem_attr_once(fn, bytes);
        if (e == cudaSuccess) e = r;
    };
    set((const void*)rhs_fft_xy<T, N, B, 0>, big);
    set((const void*)ifft_xy<T, N, B, 0>, big);
    set((const void*)rhs_fft_xy<T, N, B, 1>, big);
    set((const void*)ifft_xy<T, N, B, 1>, big);
    if (smem_xy<T>(N, 2) <= (size_t)big) {
        set((const void*)rhs_fft_xy<T, N, B, 2>, big);
        set((const void*)ifft_xy<T, N, B, 2>, big);
    }
    if (smem_xy<T>(N, 3) <= (size_t)big) {
        set((const void*)rhs_fft_xy<T, N, B, 3>, big);
        set((const void*)ifft_xy<T, N, B, 3>, big);
    }
    if constexpr (sizeof(T) == 4 && StagedA<N>::fits) set((const void*)rhs_fft_xy_staged<N, B>, (int)StagedA<N>::bytes);
    return e;
}

// threads per CTA of the generic pass A and of pass C: 256 (default) or 512
static inline int xy_block(int threads) { return threads == 512 ? 512 : 256; }

// pass A variant: 0 = default (staged where it fits), 1 = generic, 2 = staged
template <typename T, int N> static bool use_staged(int variant) {
    if constexpr (sizeof(T) == 4 && StagedA<N>::fits)
        return variant != 1;
    else
        return false;
}

// generic pass A / pass C launches in variant V (bit 0 half planes, bit 1
// batched x-FFTs)
template <typename T, int N, bool B, int V>
static void launch_xy(bool do_a, const StepArgs<T>& a, const StepArgs<T>* batch, int M, int count, int threads,
                      cudaStream_t st) {
    constexpr int Z = XyShape<T, N, V>::Z;
    const size_t sxy = smem_xy<T>(N, V);
    const dim3 g(N / Z, M, count);
    if (do_a)
        rhs_fft_xy<T, N, B, V><<<g, xy_block(threads), sxy, st>>>(a, batch);
    else
        ifft_xy<T, N, B, V><<<g, xy_block(threads), sxy, st>>>(a, batch);
}

template <typename T, int N, bool B>
static void launch_xy_any(int variant, bool do_a, const StepArgs<T>& a, const StepArgs<T>* batch, int M, int count,
                          int threads, cudaStream_t st) {
    if ((variant & 2) && smem_xy<T>(N, variant) > 200 * 1024) variant &= 1;  // batched x-FFTs do not fit
    switch (variant & 3) {
        case 1: launch_xy<T, N, B, 1>(do_a, a, batch, M, count, threads, st); break;
        case 2: launch_xy<T, N, B, 2>(do_a, a, batch, M, count, threads, st); break;
        case 3: launch_xy<T, N, B, 3>(do_a, a, batch, M, count, threads, st); break;
        default: launch_xy<T, N, B, 0>(do_a, a, batch, M, count, threads, st); break;
    }
}

template <typename T, int N> static cudaError_t launch_n(const StepLaunch<T>& s, cudaStream_t st) {
    constexpr int Z = zg_planes(N, sizeof(T));
    if (const cudaError_t ea = set_xy_attrs<T, N, false>(); ea != cudaSuccess) return ea;
    const dim3 gxy(N / Z, s.step.M);
    if (s.events) cudaEventRecord(s.events[0], st);
    if (s.do_a) {
        bool staged = false;
        if constexpr (sizeof(T) == 4 && StagedA<N>::fits) {
            staged = use_staged<T, N>(s.a_variant);
            if (staged) rhs_fft_xy_staged<N><<<gxy, 512, StagedA<N>::bytes, st>>>(s.step, nullptr);
        }
        if (!staged) launch_xy_any<T, N, false>(s.xy_z, true, s.step, nullptr, s.step.M, 1, s.xy_threads, st);
    }
    if (s.events) cudaEventRecord(s.events[1], st);
    if (s.do_b) launch_solve<T>(N, s.solve, st, s.solve_threads);
    if (s.events) cudaEventRecord(s.events[2], st);
    if (s.do_c) launch_xy_any<T, N, false>(s.xy_z, false, s.step, nullptr, s.step.M, 1, s.xy_threads, st);
    if (s.events) cudaEventRecord(s.events[3], st);
    return cudaGetLastError();
}

template <int N> static cudaError_t launch_batched_n(const BatchLaunch<float>& b, cudaStream_t st) {
    constexpr int Z = zg_planes(N, 4);
    if (const cudaError_t ea = set_xy_attrs<float, N, true>(); ea != cudaSuccess) return ea;
    const dim3 gxy(N / Z, b.M, b.count);
    bool staged = false;
    if constexpr (StagedA<N>::fits) {
        staged = use_staged<float, N>(b.a_variant);
        if (staged) rhs_fft_xy_staged<N, true><<<gxy, 512, StagedA<N>::bytes, st>>>(StepArgs<float>{}, b.dstep);
    }
    if (!staged) launch_xy_any<float, N, true>(b.xy_z, true, StepArgs<float>{}, b.dstep, b.M, b.count, b.xy_threads, st);
    cudaError_t e = launch_solve_batched(N, b, st);
    if (e != cudaSuccess) return e;
    launch_xy_any<float, N, true>(b.xy_z, false, StepArgs<float>{}, b.dstep, b.M, b.count, b.xy_threads, st);
    return cudaGetLastError();
}

cudaError_t launch_step_batched(int N, const BatchLaunch<float>& b, cudaStream_t st) {
    switch (N) {
#define WLC_CASE(n) \
    case n:         \
        return launch_batched_n<n>(b, st);
        WLC_FOR_EACH_BATCH_N(WLC_CASE)
#undef WLC_CASE
        default:
            return cudaErrorInvalidValue;
    }
}

// function attributes of the batched kernels, set outside any stream capture
cudaError_t prepare_step_batched(int N) {
    switch (N) {
#define WLC_CASE(n)                                                       \
    case n: {                                                             \
        const cudaError_t ea = set_xy_attrs<float, n, true>();            \
        return ea != cudaSuccess ? ea : prepare_solve_batched(n);         \
    }
        WLC_FOR_EACH_BATCH_N(WLC_CASE)
#undef WLC_CASE
        default:
            return cudaErrorInvalidValue;
    }
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
template size_t smem_xy<double>(int, int);
template size_t smem_xy<float>(int, int);

}  // namespace wlc
