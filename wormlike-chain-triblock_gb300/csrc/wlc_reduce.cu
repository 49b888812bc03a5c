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
// (3 - 3 ds w, -3/2 + 3 ds w, third - ds w); then dsw[blk][nr] = ds w at cf + 9 nr
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
        }
}

// Maier-Saupe term ds * sum_j Theta_ij(r) h_j(r), h the BDF history
// combination of the given order (calc_THETAij and the Theta loop of
// init_pr, wormlike_MDE_2dcomp_mod.f90:5-110, MDE_ABC.f90:256-268).
template <typename T>
__global__ void ms_term(const T* __restrict__ h1, const T* __restrict__ h2, const T* __restrict__ h3, int order,
                        const double* __restrict__ mop, ThetaLists tl, double ds, double thresh, int M, int64_t nr,
                        T* __restrict__ out) {
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        const double a0 = mop[0 * nr + r] - mop[4 * nr + r];  // M00 - M11
        const double coef[5] = {a0, mop[8 * nr + r], mop[3 * nr + r], mop[6 * nr + r], mop[7 * nr + r]};
        // note M01 = mop[(0 + 3*1)] = M_OP(k,0,1) in Fortran order; the tensor is symmetric
        for (int i = 0; i < M; ++i) out[(int64_t)i * nr + r] = (T)0;
        // Theta_ij(r) = sum_c coef_c T_c(i,j), thresholded per entry
        for (int e = 0; e < tl.n; ++e) {
            const int i = tl.row[e], j = tl.col[e];
            double th = 0.0;
            for (int c = 0; c < 5; ++c) th += coef[c] * tl.val[5 * e + c];
            if (fabs(th) < thresh) continue;
            double hj;
            const int64_t o = (int64_t)j * nr + r;
            if (order == 1)
                hj = (double)h1[o];
            else if (order == 2)
                hj = 2.0 * (double)h1[o] - (double)h2[o];
            else
                hj = 3.0 * (double)h1[o] - 3.0 * (double)h2[o] + (double)h3[o];
            const int64_t oi = (int64_t)i * nr + r;
            out[oi] = (T)((double)out[oi] + ds * th * hj);
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

// orientation tensor per block (SCFT_Density_FE.f90:161-220):
// sraw[b][t][r] = S1_s( q^T J_t q* ), t = 11, 22, 12, 13, 23
template <typename T>
__global__ void stensor_accum(const T* __restrict__ qf, const T* __restrict__ qb, DensityArgs d, JLists jl,
                              double* __restrict__ sraw) {
    const int64_t nr = d.nr;
    const int64_t sl = (int64_t)d.M * nr;
    for (int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; r < nr; r += (int64_t)gridDim.x * blockDim.x) {
        for (int b = 0; b < 3; ++b) {
            double acc[5] = {0, 0, 0, 0, 0};
            const int s0 = d.nstart[b], n = d.ns[b];
            if (n > 0) {
                for (int s = s0; s <= s0 + n; ++s) {
                    const int j = s - s0;
                    const double wgt = (j == 0 || j == n) ? 1.0 : ((j & 1) ? 4.0 : 2.0);
                    const T* a = qf + s * sl + r;
                    const T* c = qb + s * sl + r;
                    for (int t = 0; t < 5; ++t) {
                        double sum = 0.0;
                        for (int e = jl.ptr[t]; e < jl.ptr[t + 1]; ++e)
                            sum += jl.val[e] * (double)a[(int64_t)jl.row[e] * nr] * (double)c[(int64_t)jl.col[e] * nr];
                        acc[t] += wgt * sum;
                    }
                }
            }
            for (int t = 0; t < 5; ++t) sraw[((int64_t)b * 5 + t) * nr + r] = acc[t] * d.ds / 3.0;
        }
    }
}

template <typename T>
__device__ __forceinline__ void density_slice_body(const T* __restrict__ a, const T* __restrict__ c,
                                                   const DensityArgs& d, int s, int want_s, const JLists& jl,
                                                   double* __restrict__ raw, double* __restrict__ junc,
                                                   double* __restrict__ qend, double* __restrict__ sraw,
                                                   int64_t r0, int64_t rstep) {
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
    const bool last = s == 0;
    const double sc = d.ds / 3.0;
    for (int64_t r = r0; r < nr; r += rstep) {
        const double sum = dot_coeffs(a + r, c + r, d.M, nr);
        if (any)
            for (int b = 0; b < 3; ++b)
                if (wgt[b] != 0.0) raw[b * nr + r] += wgt[b] * sum;
        for (int j = 0; j < 3; ++j)
            if (s == sj[j]) junc[j * nr + r] = sum;
        if (s == d.nmax) qend[r] = (double)a[r];
        if (want_s && any) {
            for (int t = 0; t < 5; ++t) {
                double st = 0.0;
                for (int e = jl.ptr[t]; e < jl.ptr[t + 1]; ++e)
                    st += jl.val[e] * (double)a[(int64_t)jl.row[e] * nr + r] * (double)c[(int64_t)jl.col[e] * nr + r];
                for (int b = 0; b < 3; ++b)
                    if (wgt[b] != 0.0) sraw[((int64_t)b * 5 + t) * nr + r] += wgt[b] * st;
            }
        }
        if (last) {
            for (int b = 0; b < 3; ++b) raw[b * nr + r] *= sc;
            if (want_s)
                for (int q = 0; q < 15; ++q) sraw[(int64_t)q * nr + r] *= sc;
        }
    }
}

// Streamed form of density_accum / stensor_accum: one slice s per launch,
// issued by the backward sweep right after q*(s) is computed (descending s),
// so the q* slices need not be stored.  Same Simpson weights per block.
template <typename T>
__global__ void density_slice(const T* __restrict__ a, const T* __restrict__ c, DensityArgs d, int s, int want_s,
                              JLists jl, double* __restrict__ raw, double* __restrict__ junc,
                              double* __restrict__ qend, double* __restrict__ sraw) {
    density_slice_body<T>(a, c, d, s, want_s, jl, raw, junc, qend, sraw,
                          blockIdx.x * (int64_t)blockDim.x + threadIdx.x, (int64_t)gridDim.x * blockDim.x);
}

template <typename T>
__global__ void density_slice_batched(const SliceBatchArgs<T>* __restrict__ args, int s) {
    const SliceBatchArgs<T> g = args[blockIdx.y];
    density_slice_body<T>(g.qf + (int64_t)s * g.sl, g.qb + (int64_t)(s & 3) * g.sl, g.d, s, g.want_s, g.jl, g.raw,
                          g.junc, g.qend, g.sraw, blockIdx.x * (int64_t)blockDim.x + threadIdx.x,
                          (int64_t)gridDim.x * blockDim.x);
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
template <typename T>
void launch_ms_term(const T* h1, const T* h2, const T* h3, int order, const double* mop, const ThetaLists& tl,
                    double ds, double thresh, int M, int64_t nr, T* out, cudaStream_t st) {
    ms_term<T><<<grid_for(nr), 128, 0, st>>>(h1, h2, h3, order, mop, tl, ds, thresh, M, nr, out);
}
template <typename T>
void launch_density(const T* qf, const T* qb, const DensityArgs& d, double* raw, double* junc, double* qend,
                    cudaStream_t st) {
    density_accum<T><<<grid_for(d.nr), 256, 0, st>>>(qf, qb, d, raw, junc, qend);
}
template <typename T>
void launch_stensor(const T* qf, const T* qb, const DensityArgs& d, const JLists& jl, double* sraw, cudaStream_t st) {
    stensor_accum<T><<<grid_for(d.nr), 128, 0, st>>>(qf, qb, d, jl, sraw);
}

template <typename T>
void launch_density_slice(const T* qf_s, const T* qb_s, const DensityArgs& d, int s, int want_s, const JLists& jl,
                          double* raw, double* junc, double* qend, double* sraw, cudaStream_t st) {
    density_slice<T><<<grid_for(d.nr), 256, 0, st>>>(qf_s, qb_s, d, s, want_s, jl, raw, junc, qend, sraw);
}

template <typename T>
void launch_density_slice_batched(const SliceBatchArgs<T>* args, int count, int64_t max_nr, int s, cudaStream_t st) {
    density_slice_batched<T><<<dim3(grid_for(max_nr), count), 256, 0, st>>>(args, s);
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
    template void launch_density_slice_batched<T>(const SliceBatchArgs<T>*, int, int64_t, int, cudaStream_t);
WLC_INST(double)
WLC_INST(float)
#undef WLC_INST

}  // namespace wlc
