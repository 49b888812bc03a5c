// wlc_reduce.cu -- layout conversion, field preprocessing, density / Q /
// orientation tensor / free energy kernels.
//
// Reference: density() SCFT_Density_FE_ABC.f90:3-271 (per-block
// restatement), SCFT_Density_FE.f90:48-220 (AB form), free_energy()
// SCFT_Density_FE.f90:273-342, integrators utility_mod.f90:195-374,
// Sum_sparse_2D utility_mod.f90:376-407.
//
// All reductions are deterministic: fixed partition per CTA, fixed-order
// tree in shared memory, one final CTA summing the partials in order.
#include <cstdint>

#include "wlc_attr.h"
#include "wlc_reduce.h"

namespace wlc {

// ------------------------------------------------------------ layouts
// reference layout [r][i] (coefficient fastest) <-> internal [i][r]
template <typename T>
__global__ void to_internal(const double* __restrict__ ref, T* __restrict__ out, int M, int64_t nr) {
    __shared__ double tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32;
    const int i0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t r = r0 + k;
        const int i = i0 + threadIdx.x;
        if (r < nr && i < M) tile[k][threadIdx.x] = ref[r * M + i];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int i = i0 + k;
        const int64_t r = r0 + threadIdx.x;
        if (r < nr && i < M) out[(int64_t)i * nr + r] = (T)tile[threadIdx.x][k];
    }
}

template <typename T>
__global__ void to_reference(const T* __restrict__ in, double* __restrict__ ref, int M, int64_t nr) {
    __shared__ double tile[32][33];
    const int64_t r0 = (int64_t)blockIdx.x * 32;
    const int i0 = blockIdx.y * 32;
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int i = i0 + k;
        const int64_t r = r0 + threadIdx.x;
        if (r < nr && i < M) tile[k][threadIdx.x] = (double)in[(int64_t)i * nr + r];
    }
    __syncthreads();
    for (int k = threadIdx.y; k < 32; k += blockDim.y) {
        const int64_t r = r0 + k;
        const int i = i0 + threadIdx.x;
        if (r < nr && i < M) ref[r * M + i] = tile[threadIdx.x][k];
    }
}

// q(0) = delta_{i0} (MDE_ABC.f90:40-45, :62-67)
template <typename T> __global__ void set_delta(T* q, int M, int64_t nr) {
    const int64_t n = (int64_t)M * nr;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        q[e] = e < nr ? (T)1 : (T)0;
}

// order-3 history coefficients per block: cf[blk][3][nr] =
// (3 - 3 ds w, -3/2 + 3 ds w, third - ds w); then dsw[blk][nr] = ds w at
// cf + 9 nr and the split scheme's field half-step factors e^{-w ds/2} at
// cf + 12 nr (split_operator_MDE_mod.f90:163-166)
template <typename T>
__global__ void make_cf(const double* __restrict__ w, T* __restrict__ cf, double ds, double third, int64_t nr) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x)
        for (int b = 0; b < 3; ++b) {
            const double W = w[b * nr + r];
            T* o = cf + (size_t)b * 3 * nr;
            o[r] = (T)(3.0 - 3.0 * ds * W);
            o[nr + r] = (T)(-1.5 + 3.0 * ds * W);
            o[2 * nr + r] = (T)(third - ds * W);
            cf[(size_t)(9 + b) * nr + r] = (T)(ds * W);
            cf[(size_t)(12 + b) * nr + r] = (T)exp(-0.5 * ds * W);
        }
}

// Maier-Saupe term ds * sum_j Theta_ij(r) h_j(r), h the BDF history
// combination of the given order (calc_THETAij and the Theta loop of
// init_pr, wormlike_MDE_2dcomp_mod.f90:5-110, MDE_ABC.f90:256-268).
// 16-byte vector access of 16/sizeof(T) consecutive values (16-byte aligned)
template <typename T> struct VecOf;
template <> struct VecOf<float> { using t = float4; };
template <> struct VecOf<double> { using t = double2; };
template <typename T> __device__ __forceinline__ void vload(const T* p, T* v) {
    const typename VecOf<T>::t x = *reinterpret_cast<const typename VecOf<T>::t*>(p);
    if constexpr (sizeof(T) == 4) {
        v[0] = x.x;
        v[1] = x.y;
        v[2] = x.z;
        v[3] = x.w;
    } else {
        v[0] = x.x;
        v[1] = x.y;
    }
}
template <typename T> __device__ __forceinline__ void vstore(T* p, const T* v) {
    typename VecOf<T>::t x;
    if constexpr (sizeof(T) == 4) {
        x.x = v[0];
        x.y = v[1];
        x.z = v[2];
        x.w = v[3];
    } else {
        x.x = v[0];
        x.y = v[1];
    }
    *reinterpret_cast<typename VecOf<T>::t*>(p) = x;
}

// shared-memory layout of ms_term: hc[M][TILE] (16-byte aligned rows) | val[5n] | rowptr[M+1] | col[n]
template <typename T> __host__ __device__ inline size_t ms_smem_bytes(int n, int M) {
    return sizeof(T) * ((size_t)5 * n + (size_t)M * PointTile<T>::value) + sizeof(int) * (size_t)(M + 1) +
           sizeof(int16_t) * (size_t)n;
}

// The Theta lists (values converted to the compute type) are staged once per
// CTA; the CTA then walks tiles of TILE points.  Thread (k, g) handles point
// k of the tile and rows i = g, g + kMsGroups, ... of its output.
template <typename T>
__global__ void __launch_bounds__(PointTile<T>::value * kMsGroups)
    ms_term(const T* __restrict__ h1, const T* __restrict__ h2, const T* __restrict__ h3, int order,
            const double* __restrict__ mop, ThetaLists tl, double ds, double thresh, int M, int64_t nr,
            T* __restrict__ out) {
    constexpr int TILE = PointTile<T>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    T* hc = reinterpret_cast<T*>(smem_raw);  // [M][TILE]: BDF history combination of the tile's points
    T* sval = hc + (size_t)M * TILE;
    int* srp = reinterpret_cast<int*>(sval + (size_t)5 * tl.n);
    int16_t* scol = reinterpret_cast<int16_t*>(srp + M + 1);
    for (int e = threadIdx.x; e < 5 * tl.n; e += blockDim.x) sval[e] = (T)tl.val[e];
    for (int e = threadIdx.x; e <= M; e += blockDim.x) srp[e] = tl.rowptr[e];
    for (int e = threadIdx.x; e < tl.n; e += blockDim.x) scol[e] = tl.col[e];
    const int k = threadIdx.x % TILE, g = threadIdx.x / TILE;
    const T th_min = (T)thresh;
    for (int64_t r0 = (int64_t)blockIdx.x * TILE; r0 < nr; r0 += (int64_t)gridDim.x * TILE) {
        __syncthreads();  // tables staged / previous tile consumed
        // 16-byte vectors of V consecutive points (nr and r0 are multiples of V)
        constexpr int V = 16 / sizeof(T);
        using VT = typename VecOf<T>::t;
        for (int idx = threadIdx.x; idx < M * (TILE / V); idx += blockDim.x) {
            const int j = idx / (TILE / V), kk = (idx % (TILE / V)) * V;
            const int64_t r = r0 + kk;
            T v[V] = {};
            if (r < nr) {
                const int64_t o = (int64_t)j * nr + r;
                T q1[V], q2[V], q3[V];
                vload<T>(h1 + o, q1);
                if (order >= 2) vload<T>(h2 + o, q2);
                if (order >= 3) vload<T>(h3 + o, q3);
#pragma unroll
                for (int u = 0; u < V; ++u) {
                    if (order == 1)
                        v[u] = q1[u];
                    else if (order == 2)
                        v[u] = (T)2 * q1[u] - q2[u];
                    else
                        v[u] = (T)3 * q1[u] - (T)3 * q2[u] + q3[u];
                }
            }
            vstore<T>(hc + j * TILE + kk, v);
        }
        (void)sizeof(VT);
        __syncthreads();
        const int64_t r = r0 + k;
        if (r >= nr) continue;
        // Theta_ij(r) = sum_c coef_c T_c(i,j), entries below the threshold dropped
        // (M01 = mop[0 + 3*1] = M_OP(k,0,1) in Fortran order; the tensor is symmetric)
        const T coef[5] = {(T)(mop[0 * nr + r] - mop[4 * nr + r]), (T)mop[8 * nr + r], (T)mop[3 * nr + r],
                           (T)mop[6 * nr + r], (T)mop[7 * nr + r]};
        const T* hv = hc + k;
        // entries in groups of four with independent partial sums (the list
        // loads and the coefficient gathers of four entries overlap)
        auto term = [&](int e) -> T {
            const T* v5 = sval + 5 * e;
            const T th = coef[0] * v5[0] + coef[1] * v5[1] + coef[2] * v5[2] + coef[3] * v5[3] + coef[4] * v5[4];
            return fabs(th) < th_min ? (T)0 : th * hv[scol[e] * TILE];
        };
        for (int i = g; i < M; i += kMsGroups) {
            T a0 = (T)0, a1 = (T)0, a2 = (T)0, a3 = (T)0;
            const int e1 = srp[i + 1];
            int e = srp[i];
            for (; e + 4 <= e1; e += 4) {
                a0 += term(e);
                a1 += term(e + 1);
                a2 += term(e + 2);
                a3 += term(e + 3);
            }
            for (; e < e1; ++e) a0 += term(e);
            out[(int64_t)i * nr + r] = (T)ds * ((a0 + a1) + (a2 + a3));
        }
    }
}

// ------------------------------------------------------------ densities
// raw[b][r] = sum_i S1_{s in block b}(q_i q*_i); junc[j][r] = sum_i q_i q*_i at
// s = NA, NA+NB, Nmax; qend[r] = q_0(r, Nmax).
// sum_i a[i*stride] c[i*stride] in FP64 with four independent partial sums
// (more loads in flight per thread; fixed order, so deterministic)
template <typename T>
__device__ __forceinline__ double dot_coeffs(const T* __restrict__ a, const T* __restrict__ c, int M, int64_t stride) {
    double s0 = 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
    int i = 0;
    for (; i + 4 <= M; i += 4) {
        s0 += (double)a[i * stride] * (double)c[i * stride];
        s1 += (double)a[(i + 1) * stride] * (double)c[(i + 1) * stride];
        s2 += (double)a[(i + 2) * stride] * (double)c[(i + 2) * stride];
        s3 += (double)a[(i + 3) * stride] * (double)c[(i + 3) * stride];
    }
    for (; i < M; ++i) s0 += (double)a[i * stride] * (double)c[i * stride];
    return (s0 + s1) + (s2 + s3);
}

template <typename T>
__global__ void density_accum(const T* __restrict__ qf, const T* __restrict__ qb, DensityArgs d,
                              double* __restrict__ raw, double* __restrict__ junc, double* __restrict__ qend) {
    const int64_t nr = d.nr;
    const int64_t sl = (int64_t)d.M * nr;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        for (int b = 0; b < 3; ++b) {
            double acc = 0.0;
            const int s0 = d.nstart[b], n = d.ns[b];
            if (n > 0) {
                for (int s = s0; s <= s0 + n; ++s) {
                    const int j = s - s0;
                    const double wgt = (j == 0 || j == n) ? 1.0 : ((j & 1) ? 4.0 : 2.0);
                    const double sum = dot_coeffs(qf + s * sl + r, qb + s * sl + r, d.M, nr);
                    acc += wgt * sum;
                }
                acc *= d.ds / 3.0;
            }
            raw[b * nr + r] = acc;
        }
        const int sj[3] = {d.nstart[1], d.nstart[2], d.nmax};
        for (int j = 0; j < 3; ++j) {
            junc[j * nr + r] = dot_coeffs(qf + sj[j] * sl + r, qb + sj[j] * sl + r, d.M, nr);
        }
        qend[r] = (double)qf[(int64_t)d.nmax * sl + r];
    }
}

// one J-list entry packed for a single broadcast load per entry (8 bytes
// in FP32, 16 in FP64) instead of three loads from separate arrays
template <typename T> struct alignas(sizeof(T) == 8 ? 16 : 8) JEnt {
    T val;
    int16_t row, col;
};

// shared-memory layout of the tiled density / tensor kernels:
// sa[M][TILE] | sc[M][TILE] | jent[nj] | jptr[6]
template <typename T> __host__ __device__ inline size_t slice_smem_bytes(int M, int nj, bool want_s) {
    size_t b = 2 * sizeof(T) * (size_t)M * PointTile<T>::value;
    if (want_s) b += sizeof(JEnt<T>) * (size_t)nj + sizeof(int) * 6;
    return b;
}

template <typename T> struct SliceSmem {
    T* sa;
    T* sc;
    JEnt<T>* jent;
    int* jptr;
};

template <typename T> __device__ __forceinline__ SliceSmem<T> slice_smem(unsigned char* raw, int M, int nj) {
    constexpr int TILE = PointTile<T>::value;
    SliceSmem<T> m;
    m.sa = reinterpret_cast<T*>(raw);
    m.sc = m.sa + (size_t)M * TILE;
    m.jent = reinterpret_cast<JEnt<T>*>(m.sc + (size_t)M * TILE);  // 2 M TILE sizeof(T) bytes in: 16-aligned
    m.jptr = reinterpret_cast<int*>(m.jent + nj);
    return m;
}

template <typename T> __device__ __forceinline__ void stage_jlists(const JLists& jl, const SliceSmem<T>& m) {
    for (int e = threadIdx.x; e < jl.n; e += blockDim.x) {
        JEnt<T> x;
        x.val = (T)jl.val[e];
        x.row = jl.row[e];
        x.col = jl.col[e];
        m.jent[e] = x;
    }
    for (int e = threadIdx.x; e < 6; e += blockDim.x) m.jptr[e] = jl.ptr[e];
}

// stage the coefficient vectors of one slice for the tile's points (zeros
// past the end of the grid), 16-byte vectors of consecutive points
template <typename T>
__device__ __forceinline__ void stage_tile(const T* __restrict__ a, const T* __restrict__ c, int M, int64_t nr,
                                           int64_t r0, T* sa, T* sc) {
    constexpr int TILE = PointTile<T>::value;
    constexpr int V = 16 / sizeof(T);
    for (int idx = threadIdx.x; idx < M * (TILE / V); idx += blockDim.x) {
        const int i = idx / (TILE / V), k = (idx % (TILE / V)) * V;
        const int64_t r = r0 + k;
        T va[V] = {}, vc[V] = {};
        if (r < nr) {
            vload<T>(a + (int64_t)i * nr + r, va);
            vload<T>(c + (int64_t)i * nr + r, vc);
        }
        vstore<T>(sa + i * TILE + k, va);
        vstore<T>(sc + i * TILE + k, vc);
    }
}

// q^T J_t q* at one point from staged vectors (stride TILE) and staged lists
template <typename T> __device__ __forceinline__ double jt_form(const SliceSmem<T>& m, int t, int k) {
    constexpr int TILE = PointTile<T>::value;
    T v = (T)0;
    for (int e = m.jptr[t]; e < m.jptr[t + 1]; ++e) {
        const JEnt<T> x = m.jent[e];
        v += x.val * m.sa[x.row * TILE + k] * m.sc[x.col * TILE + k];
    }
    return (double)v;
}

// orientation tensor per block (SCFT_Density_FE.f90:161-220):
// sraw[b][t][r] = S1_s( q^T J_t q* ), t = 11, 22, 12, 13, 23; thread (k, t)
template <typename T>
__global__ void __launch_bounds__(PointTile<T>::value * kSGroups)
    stensor_accum(const T* __restrict__ qf, const T* __restrict__ qb, DensityArgs d, JLists jl,
                  double* __restrict__ sraw) {
    constexpr int TILE = PointTile<T>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const SliceSmem<T> m = slice_smem<T>(smem_raw, d.M, jl.n);
    stage_jlists(jl, m);
    const int64_t nr = d.nr;
    const int64_t sl = (int64_t)d.M * nr;
    const int k = threadIdx.x % TILE, t = threadIdx.x / TILE;
    const int64_t r0 = (int64_t)blockIdx.x * TILE, r = r0 + k;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int b = 0; b < 3; ++b) {
        const int s0 = d.nstart[b], n = d.ns[b];
        if (n <= 0) continue;
        for (int s = s0; s <= s0 + n; ++s) {
            const int j = s - s0;
            const double wgt = (j == 0 || j == n) ? 1.0 : ((j & 1) ? 4.0 : 2.0);
            __syncthreads();
            stage_tile(qf + s * sl, qb + s * sl, d.M, nr, r0, m.sa, m.sc);
            __syncthreads();
            acc[b] += wgt * jt_form(m, t, k);
        }
    }
    if (r < nr)
        for (int b = 0; b < 3; ++b) sraw[((int64_t)b * 5 + t) * nr + r] = acc[b] * d.ds / 3.0;
}

// Streamed form of density_accum / stensor_accum: one slice s per launch,
// issued by the backward sweep right after q*(s) is computed (descending s),
// so the q* slices need not be stored.  Same Simpson weights per block.  One
// CTA per tile of points; the tile's coefficient vectors of q(s) and q*(s)
// are staged in shared memory once.
// One CTA walks tiles of TILE points of one instance; thread (k, g): point k,
// group g (g = 0 the densities, g = t the tensor component t when want_s;
// blockDim = TILE * kSGroups when any instance of the launch wants S).
template <typename T>
__device__ __forceinline__ void density_slice_tiles(const T* __restrict__ a, const T* __restrict__ c,
                                                    const DensityArgs& d, int s, int want_s, const JLists& jl,
                                                    double* __restrict__ raw, double* __restrict__ junc,
                                                    double* __restrict__ qend, double* __restrict__ sraw) {
    constexpr int TILE = PointTile<T>::value;
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const SliceSmem<T> m = slice_smem<T>(smem_raw, d.M, want_s ? jl.n : 0);
    if (want_s) stage_jlists(jl, m);
    const int64_t nr = d.nr;
    double wgt[3];
    bool any = false;
    for (int b = 0; b < 3; ++b) {
        const int j = s - d.nstart[b], n = d.ns[b];
        wgt[b] = 0.0;
        if (n > 0 && j >= 0 && j <= n) {
            wgt[b] = (j == 0 || j == n) ? 1.0 : ((j & 1) ? 4.0 : 2.0);
            any = true;
        }
    }
    const int sj[3] = {d.nstart[1], d.nstart[2], d.nmax};
    const double scl = d.ds / 3.0;
    const int k = threadIdx.x % TILE, g = threadIdx.x / TILE;
    for (int64_t r0 = (int64_t)blockIdx.x * TILE; r0 < nr; r0 += (int64_t)gridDim.x * TILE) {
        __syncthreads();  // lists staged / previous tile consumed
        stage_tile(a, c, d.M, nr, r0, m.sa, m.sc);
        __syncthreads();
        const int64_t r = r0 + k;
        if (r >= nr) continue;
        if (g == 0) {
            const double sum = dot_coeffs(m.sa + k, m.sc + k, d.M, (int64_t)TILE);
            if (any)
                for (int b = 0; b < 3; ++b)
                    if (wgt[b] != 0.0) raw[b * nr + r] += wgt[b] * sum;
            for (int j = 0; j < 3; ++j)
                if (s == sj[j]) junc[j * nr + r] = sum;
            if (s == d.nmax) qend[r] = (double)a[r];
            if (s == 0)  // last slice of the backward sweep
                for (int b = 0; b < 3; ++b) raw[b * nr + r] *= scl;
        }
        if (want_s && g < 5) {
            if (any) {
                const double st = jt_form(m, g, k);
                for (int b = 0; b < 3; ++b)
                    if (wgt[b] != 0.0) sraw[((int64_t)b * 5 + g) * nr + r] += wgt[b] * st;
            }
            if (s == 0)
                for (int b = 0; b < 3; ++b) sraw[((int64_t)b * 5 + g) * nr + r] *= scl;
        }
    }
}

template <typename T>
__global__ void __launch_bounds__(PointTile<T>::value * kSGroups)
    density_slice(const T* __restrict__ a, const T* __restrict__ c, DensityArgs d, int s, int want_s, JLists jl,
                  double* __restrict__ raw, double* __restrict__ junc, double* __restrict__ qend,
                  double* __restrict__ sraw) {
    density_slice_tiles<T>(a, c, d, s, want_s, jl, raw, junc, qend, sraw);
}

template <typename T>
__global__ void __launch_bounds__(PointTile<T>::value * kSGroups)
    density_slice_batched(const SliceBatchArgs<T>* __restrict__ args, int s) {
    const SliceBatchArgs<T> g = args[blockIdx.y];
    density_slice_tiles<T>(g.qf + (int64_t)s * g.sl, g.qb + (int64_t)(s & 3) * g.sl, g.d, s, g.want_s, g.jl, g.raw,
                           g.junc, g.qend, g.sraw);
}

// periodic Simpson weight product (utility_mod.f90:236-298): (h/3)*(2|4)
__device__ __forceinline__ double simpson_w(int64_t r, const S3Args& s) {
    const int x = (int)(r % s.n[0]);
    const int y = (int)((r / s.n[0]) % s.n[1]);
    const int z = (int)(r / ((int64_t)s.n[0] * s.n[1]));
    const double wx = (x & 1) ? 4.0 : 2.0, wy = (y & 1) ? 4.0 : 2.0, wz = (z & 1) ? 4.0 : 2.0;
    return (s.d[0] / 3.0 * wx) * (s.d[1] / 3.0 * wy) * (s.d[2] / 3.0 * wz);
}

// partial Simpson sums of sum_k a[k*stride + r] for k < nsum
__global__ void s3_partial(const double* __restrict__ a, int nsum, int64_t stride, S3Args s, double* __restrict__ part) {
    __shared__ double sh[256];
    const int64_t nr = (int64_t)s.n[0] * s.n[1] * s.n[2];
    const int64_t chunk = (nr + gridDim.x - 1) / gridDim.x;
    const int64_t beg = blockIdx.x * chunk, end = min(nr, beg + chunk);
    double acc = 0.0;
    for (int64_t r = beg + threadIdx.x; r < end; r += blockDim.x) {
        double v = 0.0;
        for (int k = 0; k < nsum; ++k) v += a[k * stride + r];
        acc += simpson_w(r, s) * v;
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void sum_partials(const double* __restrict__ part, int n, double* __restrict__ out) {
    __shared__ double sh[256];
    double acc = 0.0;
    for (int k = threadIdx.x; k < n; k += blockDim.x) acc += part[k];
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sh[0];
}

__global__ void scale_by(double* __restrict__ a, int64_t n, const double* __restrict__ denom, double vol) {
    const double f = vol / *denom;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        a[e] = a[e] * f;
}

// free-energy integrand, three-block form of SCFT_Density_FE.f90:296-320
__global__ void fe_integrand(const double* __restrict__ phi, const double* __restrict__ w,
                             const double* __restrict__ mop, FeArgs f, double* __restrict__ ar) {
    const int64_t nr = f.nr;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        const double pa = phi[r], pb = phi[nr + r], pc = phi[2 * nr + r];
        const double wa = w[r], wb = w[nr + r], wc = w[2 * nr + r];
        double v = f.chi[0] * pa * pb + f.chi[1] * pa * pc + f.chi[2] * pb * pc - wa * pa - wb * pb - wc * pc +
                   (wa + wb + wc) / 3.0 * (pa + pb + pc - 1.0);
        if (f.ms) {
            double dd = 0.0;
            for (int p = 0; p < 3; ++p)
                for (int q = 0; q < 3; ++q) dd += mop[(p * 3 + q) * nr + r] * mop[(q * 3 + p) * nr + r];
            v += 0.5 * (dd / f.nmu);
        }
        ar[r] = v;
    }
}

__global__ void count_nonfinite(const double* __restrict__ a, int64_t n, int* __restrict__ flag) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        if (!isfinite(a[e])) atomicOr(flag, 1);
}

// ------------------------------------------------------------ launchers
static int grid_for(int64_t n) {
    int64_t g = (n + 255) / 256;
    return (int)(g > 4096 ? 4096 : (g < 1 ? 1 : g));
}

template <typename T> void launch_to_internal(const double* ref, T* out, int M, int64_t nr, cudaStream_t st) {
    dim3 g((unsigned)((nr + 31) / 32), (unsigned)((M + 31) / 32));
    to_internal<T><<<g, dim3(32, 8), 0, st>>>(ref, out, M, nr);
}
template <typename T> void launch_to_reference(const T* in, double* ref, int M, int64_t nr, cudaStream_t st) {
    dim3 g((unsigned)((nr + 31) / 32), (unsigned)((M + 31) / 32));
    to_reference<T><<<g, dim3(32, 8), 0, st>>>(in, ref, M, nr);
}
template <typename T> void launch_set_delta(T* q, int M, int64_t nr, cudaStream_t st) {
    set_delta<T><<<grid_for((int64_t)M * nr), 256, 0, st>>>(q, M, nr);
}
template <typename T> void launch_make_cf(const double* w, T* cf, double ds, double third, int64_t nr, cudaStream_t st) {
    make_cf<T><<<grid_for(nr), 256, 0, st>>>(w, cf, ds, third, nr);
}
// CTAs of the tiled kernels: enough to fill the GPU, each walking several
// tiles so that the staged lists are reused
static unsigned tile_grid(int64_t nr, int tile) {
    const int64_t tiles = (nr + tile - 1) / tile;
    return (unsigned)(tiles < 1216 ? (tiles < 1 ? 1 : tiles) : 1216);
}

template <typename T>
void launch_ms_term(const T* h1, const T* h2, const T* h3, int order, const double* mop, const ThetaLists& tl,
                    double ds, double thresh, int M, int64_t nr, T* out, cudaStream_t st) {
    constexpr int TILE = PointTile<T>::value;
    ms_term<T><<<tile_grid(nr, TILE), TILE * kMsGroups, ms_smem_bytes<T>(tl.n, M), st>>>(h1, h2, h3, order, mop, tl,
                                                                                      ds, thresh, M, nr, out);
}
template <typename T>
void launch_density(const T* qf, const T* qb, const DensityArgs& d, double* raw, double* junc, double* qend,
                    cudaStream_t st) {
    density_accum<T><<<grid_for(d.nr), 256, 0, st>>>(qf, qb, d, raw, junc, qend);
}
template <typename T>
void launch_stensor(const T* qf, const T* qb, const DensityArgs& d, const JLists& jl, double* sraw, cudaStream_t st) {
    constexpr int TILE = PointTile<T>::value;
    stensor_accum<T><<<(unsigned)((d.nr + TILE - 1) / TILE), TILE * kSGroups, slice_smem_bytes<T>(d.M, jl.n, true),
                       st>>>(qf, qb, d, jl, sraw);
}

template <typename T>
void launch_density_slice(const T* qf_s, const T* qb_s, const DensityArgs& d, int s, int want_s, const JLists& jl,
                          double* raw, double* junc, double* qend, double* sraw, cudaStream_t st) {
    constexpr int TILE = PointTile<T>::value;
    density_slice<T><<<tile_grid(d.nr, TILE), TILE * (want_s ? kSGroups : 1),
                       slice_smem_bytes<T>(d.M, jl.n, want_s != 0), st>>>(qf_s, qb_s, d, s, want_s, jl, raw, junc,
                                                                          qend, sraw);
}

template <typename T>
void launch_density_slice_batched(const SliceBatchArgs<T>* args, int count, int64_t max_nr, int s, int M, int nj,
                                  int any_s, cudaStream_t st) {
    constexpr int TILE = PointTile<T>::value;
    density_slice_batched<T><<<dim3(tile_grid(max_nr, TILE), count), TILE * (any_s ? kSGroups : 1),
                               slice_smem_bytes<T>(M, nj, any_s != 0), st>>>(args, s);
}

void launch_s3(const double* a, int nsum, int64_t stride, const S3Args& s, double* part, double* out,
               cudaStream_t st) {
    s3_partial<<<kS3Blocks, 256, 0, st>>>(a, nsum, stride, s, part);
    sum_partials<<<1, 256, 0, st>>>(part, kS3Blocks, out);
}

void launch_scale(double* a, int64_t n, const double* denom, double vol, cudaStream_t st) {
    scale_by<<<grid_for(n), 256, 0, st>>>(a, n, denom, vol);
}

void launch_fe(const double* phi, const double* w, const double* mop, const FeArgs& f, double* ar, cudaStream_t st) {
    fe_integrand<<<grid_for(f.nr), 256, 0, st>>>(phi, w, mop, f, ar);
}

void launch_nonfinite(const double* a, int64_t n, int* flag, cudaStream_t st) {
    count_nonfinite<<<grid_for(n), 256, 0, st>>>(a, n, flag);
}

#define WLC_INST(T)                                                                                              \
    template void launch_to_internal<T>(const double*, T*, int, int64_t, cudaStream_t);                           \
    template void launch_to_reference<T>(const T*, double*, int, int64_t, cudaStream_t);                          \
    template void launch_set_delta<T>(T*, int, int64_t, cudaStream_t);                                           \
    template void launch_make_cf<T>(const double*, T*, double, double, int64_t, cudaStream_t);                    \
    template void launch_ms_term<T>(const T*, const T*, const T*, int, const double*, const ThetaLists&, double,  \
                                    double, int, int64_t, T*, cudaStream_t);                                     \
    template void launch_density<T>(const T*, const T*, const DensityArgs&, double*, double*, double*,           \
                                    cudaStream_t);                                                               \
    template void launch_stensor<T>(const T*, const T*, const DensityArgs&, const JLists&, double*, cudaStream_t); \
    template void launch_density_slice<T>(const T*, const T*, const DensityArgs&, int, int, const JLists&, double*, \
                                          double*, double*, double*, cudaStream_t);                              \
    template void launch_density_slice_batched<T>(const SliceBatchArgs<T>*, int, int64_t, int, int, int, int,        \
                                                  cudaStream_t);
WLC_INST(double)
WLC_INST(float)
#undef WLC_INST

cudaError_t prepare_reduce_kernels() {
    // per (kernel, device): a context may be created on any device
    const int big = 200 * 1024;
    const void* fns[] = {(const void*)stensor_accum<double>, (const void*)stensor_accum<float>,
                         (const void*)density_slice<double>, (const void*)density_slice<float>,
                         (const void*)density_slice_batched<double>, (const void*)density_slice_batched<float>,
                         (const void*)ms_term<double>, (const void*)ms_term<float>};
    for (const void* fn : fns)
        if (const cudaError_t e = smem_attr_once(fn, big); e != cudaSuccess) return e;
    return cudaSuccess;
}

}  // namespace wlc
