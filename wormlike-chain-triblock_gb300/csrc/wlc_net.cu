// wlc_net.cu -- learned warm start for the SCFT field iteration: a small 3D
// convolutional encoder-decoder (periodic padding, 4 grid levels) that maps
// (a coarse noise field, the instance parameters) to the three block fields.
// It has no counterpart in the reference.
//
// Everything runs on the device with kernels written here: BF16 weights and
// activations, FP32 accumulation on the tensor cores (mma.sync m16n8k16 --
// the network costs seconds next to the solver, so the simple warp-level
// tensor instruction is used rather than tcgen05), FP32 activation gradients
// and FP32 Adam state / master weights.  The convolutions are implicit GEMMs
// with the neighbour gather done in the operand loads:
//   forward    out[p][co]  = sum_kk sum_ci  x[nb(p,kk)][ci] W[kk][ci][co]
//   data grad  dx[p][ci]  += sum_kk sum_co dz[nb^-1(p,kk)][co] W[kk][ci][co]
//   weight grad dW[kk][ci][co] = sum_q x[nb(q,kk)][ci] dz[q][co]
// Activations are channel-last [point][channel], point = x + g (y + g z).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "wlc.h"

namespace wlcnet {

using bf16 = __nv_bfloat16;

// ------------------------------------------------------------ device helpers
__device__ __forceinline__ int wrapi(int v, int g) {
    v %= g;
    return v < 0 ? v + g : v;
}

// input point of output point m (grid go) for neighbour kk at the given stride
// (input grid gi = go * stride), periodic
__device__ __forceinline__ int nb_fwd(int m, int kk, int gi, int go, int stride) {
    const int x = m % go, y = (m / go) % go, z = m / (go * go);
    const int dx = kk % 3 - 1, dy = (kk / 3) % 3 - 1, dz = kk / 9 - 1;
    return wrapi(stride * x + dx, gi) + gi * (wrapi(stride * y + dy, gi) + gi * wrapi(stride * z + dz, gi));
}

// output point whose neighbour kk is input point p, or -1 (stride 2: only
// points of matching parity)
__device__ __forceinline__ int nb_bwd(int p, int kk, int gi, int go, int stride) {
    const int x = p % gi, y = (p / gi) % gi, z = p / (gi * gi);
    const int dx = kk % 3 - 1, dy = (kk / 3) % 3 - 1, dz = kk / 9 - 1;
    int tx = wrapi(x - dx, gi), ty = wrapi(y - dy, gi), tz = wrapi(z - dz, gi);
    if (stride == 2) {
        if ((tx | ty | tz) & 1) return -1;
        tx >>= 1;
        ty >>= 1;
        tz >>= 1;
    }
    return tx + go * (ty + go * tz);
}

__device__ __forceinline__ uint32_t ld_pair(const bf16* p) { return *reinterpret_cast<const uint32_t*>(p); }

__device__ __forceinline__ uint32_t pack2(bf16 lo, bf16 hi) {
    return (uint32_t)__bfloat16_as_ushort(lo) | ((uint32_t)__bfloat16_as_ushort(hi) << 16);
}

__device__ __forceinline__ void mma_bf16(float c[4], uint32_t a0, uint32_t a1, uint32_t a2, uint32_t a3, uint32_t b0,
                                         uint32_t b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// ------------------------------------------------------------ kernels
// Gather GEMM for the forward pass (MODE 0) and the data gradient (MODE 1).
// out[m][n] = sum_kk sum_k A[row(m,kk)][k] * B[kk][n][k]; A rows of K BF16,
// B [27][N][K] BF16.  MODE 0: rows = nb_fwd, output BF16 with bias and
// optional ReLU (or FP32 when outf is given).  MODE 1: rows = nb_bwd, FP32
// accumulated into outf.  A warp computes 16 rows x 16 columns; a CTA four
// warps (64 rows).  K and N are multiples of 16.
template <int MODE>
__global__ void __launch_bounds__(128) gather_gemm(const bf16* __restrict__ A, int K, const bf16* __restrict__ B, int N,
                                                   int M, int gi, int go, int stride, const float* __restrict__ bias,
                                                   int relu, bf16* __restrict__ outb, float* __restrict__ outf) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int gid = lane >> 2, tig = lane & 3;
    const int r0 = blockIdx.x * 64 + warp * 16;
    const int n0 = blockIdx.y * 16;
    const int m0 = r0 + gid, m1 = r0 + gid + 8;
    float c[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    for (int kk = 0; kk < 27; ++kk) {
        int p0 = -1, p1 = -1;
        if (MODE == 0) {
            if (m0 < M) p0 = nb_fwd(m0, kk, gi, go, stride);
            if (m1 < M) p1 = nb_fwd(m1, kk, gi, go, stride);
        } else {
            if (m0 < M) p0 = nb_bwd(m0, kk, gi, go, stride);
            if (m1 < M) p1 = nb_bwd(m1, kk, gi, go, stride);
        }
        const bf16* a0p = A + (size_t)(p0 < 0 ? 0 : p0) * K;
        const bf16* a1p = A + (size_t)(p1 < 0 ? 0 : p1) * K;
        const bf16* bp = B + (size_t)kk * N * K;
        for (int k0 = 0; k0 < K; k0 += 16) {
            const uint32_t a0 = p0 >= 0 ? ld_pair(a0p + k0 + tig * 2) : 0u;
            const uint32_t a1 = p1 >= 0 ? ld_pair(a1p + k0 + tig * 2) : 0u;
            const uint32_t a2 = p0 >= 0 ? ld_pair(a0p + k0 + 8 + tig * 2) : 0u;
            const uint32_t a3 = p1 >= 0 ? ld_pair(a1p + k0 + 8 + tig * 2) : 0u;
#pragma unroll
            for (int j = 0; j < 2; ++j) {
                const bf16* b = bp + (size_t)(n0 + j * 8 + gid) * K + k0 + tig * 2;
                mma_bf16(c[j], a0, a1, a2, a3, ld_pair(b), ld_pair(b + 8));
            }
        }
    }
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int col = n0 + j * 8 + tig * 2;
#pragma unroll
        for (int h = 0; h < 2; ++h) {
            const int m = h == 0 ? m0 : m1;
            if (m >= M) continue;
            for (int e = 0; e < 2; ++e) {
                float v = c[j][2 * h + e];
                const size_t o = (size_t)m * N + col + e;
                if (MODE == 1) {
                    outf[o] += v;
                } else {
                    v += bias[col + e];
                    if (outf) {
                        outf[o] = v;
                    } else {
                        if (relu) v = fmaxf(v, 0.0f);
                        outb[o] = __float2bfloat16(v);
                    }
                }
            }
        }
    }
}

// Weight gradient, one kk per CTA column (blockIdx.z = kk * splits + split):
// part[split][kk][ci][co] = sum over q in the split's range of
// x[nb_fwd(q,kk)][ci] dz[q][co].  A warp computes 16 ci x 16 co.
__global__ void __launch_bounds__(32) wgrad(const bf16* __restrict__ X, int Ci, const bf16* __restrict__ dZ, int Co,
                                            int Mq, int gi, int go, int stride, int splits,
                                            float* __restrict__ part) {
    const int lane = threadIdx.x & 31, gid = lane >> 2, tig = lane & 3;
    const int ci0 = blockIdx.x * 16, co0 = blockIdx.y * 16;
    const int kk = blockIdx.z / splits, sp = blockIdx.z % splits;
    const int per = ((Mq + splits - 1) / splits + 15) / 16 * 16;
    const int qb = sp * per, qe = min(Mq, qb + per);
    float c[2][4] = {{0, 0, 0, 0}, {0, 0, 0, 0}};
    auto xval = [&](int q, int ci) -> bf16 {
        return q < qe ? X[(size_t)nb_fwd(q, kk, gi, go, stride) * Ci + ci] : __float2bfloat16(0.0f);
    };
    auto zval = [&](int q, int co) -> bf16 { return q < qe ? dZ[(size_t)q * Co + co] : __float2bfloat16(0.0f); };
    for (int q0 = qb; q0 < qe; q0 += 16) {
        const int qa = q0 + tig * 2;
        const uint32_t a0 = pack2(xval(qa, ci0 + gid), xval(qa + 1, ci0 + gid));
        const uint32_t a1 = pack2(xval(qa, ci0 + gid + 8), xval(qa + 1, ci0 + gid + 8));
        const uint32_t a2 = pack2(xval(qa + 8, ci0 + gid), xval(qa + 9, ci0 + gid));
        const uint32_t a3 = pack2(xval(qa + 8, ci0 + gid + 8), xval(qa + 9, ci0 + gid + 8));
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const int co = co0 + j * 8 + gid;
            mma_bf16(c[j], a0, a1, a2, a3, pack2(zval(qa, co), zval(qa + 1, co)),
                     pack2(zval(qa + 8, co), zval(qa + 9, co)));
        }
    }
    float* out = part + ((size_t)sp * 27 + kk) * Ci * Co;
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const int col = co0 + j * 8 + tig * 2;
        out[(size_t)(ci0 + gid) * Co + col] = c[j][0];
        out[(size_t)(ci0 + gid) * Co + col + 1] = c[j][1];
        out[(size_t)(ci0 + gid + 8) * Co + col] = c[j][2];
        out[(size_t)(ci0 + gid + 8) * Co + col + 1] = c[j][3];
    }
}

// grad[e] += sum over splits of part[split][e] (fixed order)
__global__ void sum_splits(const float* __restrict__ part, int splits, int64_t n, float* __restrict__ grad) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        float s = 0.0f;
        for (int k = 0; k < splits; ++k) s += part[(size_t)k * n + e];
        grad[e] += s;
    }
}

// db[co] += sum_q dz[q][co]
__global__ void bias_grad(const bf16* __restrict__ dZ, int Co, int Mq, float* __restrict__ db) {
    const int co = blockIdx.x * blockDim.x + threadIdx.x;
    if (co >= Co) return;
    float s = 0.0f;
    for (int q = 0; q < Mq; ++q) s += __bfloat162float(dZ[(size_t)q * Co + co]);
    db[co] += s;
}

// dz = bf16(dy * relu'(y)) (relu = 0: no mask)
__global__ void relu_back(const float* __restrict__ dy, const bf16* __restrict__ y, int relu, int64_t n,
                          bf16* __restrict__ dz) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float g = (relu && !(__bfloat162float(y[e]) > 0.0f)) ? 0.0f : dy[e];
        dz[e] = __float2bfloat16(g);
    }
}

// nearest x2 upsampling of src [gc^3][C] into channels [off, off+C) of dst
// [(2gc)^3][Ct]; and copy of src [g^3][C] into channels [off, off+C)
__global__ void up_into(const bf16* __restrict__ src, int gc, int C, bf16* __restrict__ dst, int Ct, int off) {
    const int gf = 2 * gc;
    const int64_t n = (int64_t)gf * gf * gf * C;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const int p = (int)(e / C);
        const int x = p % gf, y = (p / gf) % gf, z = p / (gf * gf);
        const int pc = (x >> 1) + gc * ((y >> 1) + gc * (z >> 1));
        dst[(size_t)p * Ct + off + c] = src[(size_t)pc * C + c];
    }
}
__global__ void copy_into(const bf16* __restrict__ src, int64_t npts, int C, bf16* __restrict__ dst, int Ct, int off) {
    const int64_t n = npts * C;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        dst[(size_t)(e / C) * Ct + off + e % C] = src[e];
}
// gradient of up_into: dsrc[pc][c] += sum of the 8 children; of copy_into: dsrc += slice
__global__ void up_back(const float* __restrict__ dcat, int gc, int C, int Ct, int off, float* __restrict__ dsrc) {
    const int gf = 2 * gc;
    const int64_t n = (int64_t)gc * gc * gc * C;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int c = (int)(e % C);
        const int pc = (int)(e / C);
        const int x = pc % gc, y = (pc / gc) % gc, z = pc / (gc * gc);
        float s = 0.0f;
        for (int k = 0; k < 8; ++k) {
            const int p = (2 * x + (k & 1)) + gf * ((2 * y + ((k >> 1) & 1)) + gf * (2 * z + (k >> 2)));
            s += dcat[(size_t)p * Ct + off + c];
        }
        dsrc[e] += s;
    }
}
__global__ void copy_back(const float* __restrict__ dcat, int64_t npts, int C, int Ct, int off, float* __restrict__ dsrc) {
    const int64_t n = npts * C;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x)
        dsrc[e] += dcat[(size_t)(e / C) * Ct + off + e % C];
}

// loss = sum_{p, c<3} (out - t)^2 / (3 npts); dout = d loss / d out
// (partials per CTA, fixed-order final sum)
__global__ void mse_loss(const float* __restrict__ out, int Co, const float* __restrict__ tgt, int npts,
                         float* __restrict__ dout, double* __restrict__ part) {
    __shared__ double sm[256];
    double acc = 0.0;
    const float scale = 2.0f / (3.0f * (float)npts);
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < npts * Co; e += gridDim.x * blockDim.x) {
        const int p = e / Co, c = e % Co;
        float g = 0.0f;
        if (c < 3) {
            const float d = out[e] - tgt[(size_t)c * npts + p];
            acc += (double)d * d;
            g = scale * d;
        }
        dout[e] = g;
    }
    sm[threadIdx.x] = acc;
    __syncthreads();
    for (int s = 128; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) part[blockIdx.x] = sm[0];
}

// Adam on the FP32 master weights, then the BF16 copies W[kk][ci][co] and
// WT[kk][co][ci] of a layer's weights
__global__ void adam(float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                     int64_t n, float lr, float b1, float b2, float eps, float c1, float c2, float gscale) {
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const float gr = g[e] * gscale;
        const float mm = b1 * m[e] + (1.0f - b1) * gr;
        const float vv = b2 * v[e] + (1.0f - b2) * gr * gr;
        m[e] = mm;
        v[e] = vv;
        w[e] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
    }
}
__global__ void to_bf16_pair(const float* __restrict__ w, int Ci, int Co, bf16* __restrict__ wb, bf16* __restrict__ wt) {
    const int64_t n = (int64_t)27 * Ci * Co;
    for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < n; e += (int64_t)gridDim.x * blockDim.x) {
        const int co = (int)(e % Co), ci = (int)((e / Co) % Ci), kk = (int)(e / ((int64_t)Ci * Co));
        const bf16 b = __float2bfloat16(w[e]);
        wb[e] = b;
        wt[((size_t)kk * Co + co) * Ci + ci] = b;
    }
}
__global__ void input_pack(const float* __restrict__ in, int nch, int npts, bf16* __restrict__ x, int Cpad) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < npts * Cpad; e += gridDim.x * blockDim.x) {
        const int p = e / Cpad, c = e % Cpad;
        x[e] = __float2bfloat16(c < nch ? in[(size_t)c * npts + p] : 0.0f);
    }
}
__global__ void output_unpack(const float* __restrict__ out, int Co, int npts, float* __restrict__ o3) {
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < npts * 3; e += gridDim.x * blockDim.x) {
        const int c = e / npts, p = e % npts;
        o3[e] = out[(size_t)p * Co + c];
    }
}

static int gridn(int64_t n) { return (int)std::min<int64_t>(4096, std::max<int64_t>(1, (n + 255) / 256)); }

// ------------------------------------------------------------ the network
struct Layer {
    int ci, co, stride, gin, gout, relu;
    int64_t woff, boff;  // offsets in the flat parameter vector
    bf16 *wb = nullptr, *wt = nullptr;
};

}  // namespace wlcnet

using namespace wlcnet;

struct wlc_net {
    int G = 0, C = 0;
    std::string err;
    std::vector<Layer> L;  // e1..e6, d1..d3, out
    int64_t np = 0;
    float *w = nullptr, *g = nullptr, *m = nullptr, *v = nullptr;  // params, grads, Adam moments
    int64_t step = 0;
    std::vector<void*> allocs;
    // activations (BF16) and their gradients (FP32)
    bf16 *x0 = nullptr, *e[7] = {}, *d[4] = {}, *cat[4] = {};
    float* outf = nullptr;
    float *ge[7] = {}, *gd[4] = {}, *gcat[4] = {}, *gout = nullptr;
    bf16* dz = nullptr;   // BF16 copy of the current layer's output gradient
    float* part = nullptr;  // weight-gradient partials
    int splits = 1;
    double* lpart = nullptr;
    float* tgt = nullptr;
    float* inbuf = nullptr;
    cudaStream_t st = nullptr;
};

static int nerr(wlc_net* n, int code, const std::string& m) {
    if (n) n->err = m;
    return code;
}

#define NCK(call)                                                                                           \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess) return nerr(n, WLC_E_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

template <typename X> static int nalloc(wlc_net* n, X** p, size_t count) {
    void* q = nullptr;
    if (cudaMalloc(&q, sizeof(X) * std::max<size_t>(count, 1)) != cudaSuccess) {
        cudaGetLastError();
        return nerr(n, WLC_E_ALLOC, "cudaMalloc failed");
    }
    n->allocs.push_back(q);
    *p = (X*)q;
    return WLC_OK;
}

static int64_t pts(int g) { return (int64_t)g * g * g; }

extern "C" int wlc_net_create(int32_t grid, int32_t width, uint64_t seed, wlc_net** out) {
    if (!out) return WLC_E_PARAM;
    wlc_net* n = new wlc_net();
    *out = n;
    if (grid < 8 || grid > 64 || (grid & 7) || width < 16 || width > 64 || (width & 15))
        return nerr(n, WLC_E_PARAM, "grid must be a multiple of 8 in [8, 64], width a multiple of 16 in [16, 64]");
    n->G = grid;
    n->C = width;
    const int G = grid, C = width;
    // (ci, co, stride, gin, relu): encoder e1..e6, decoder d1..d3, output
    const int spec[10][5] = {{16, C, 1, G, 1},          {C, 2 * C, 2, G, 1},         {2 * C, 2 * C, 1, G / 2, 1},
                             {2 * C, 4 * C, 2, G / 2, 1}, {4 * C, 4 * C, 1, G / 4, 1}, {4 * C, 4 * C, 2, G / 4, 1},
                             {8 * C, 4 * C, 1, G / 4, 1}, {6 * C, 2 * C, 1, G / 2, 1}, {3 * C, C, 1, G, 1},
                             {C, 16, 1, G, 0}};
    int64_t off = 0;
    for (auto& s : spec) {
        Layer l;
        l.ci = s[0];
        l.co = s[1];
        l.stride = s[2];
        l.gin = s[3];
        l.gout = s[3] / s[2];
        l.relu = s[4];
        l.woff = off;
        off += (int64_t)27 * l.ci * l.co;
        l.boff = off;
        off += l.co;
        n->L.push_back(l);
    }
    n->np = off;
    int rc;
    if ((rc = nalloc(n, &n->w, off)) || (rc = nalloc(n, &n->g, off)) || (rc = nalloc(n, &n->m, off)) ||
        (rc = nalloc(n, &n->v, off)))
        return rc;
    for (auto& l : n->L) {
        if ((rc = nalloc(n, &l.wb, (size_t)27 * l.ci * l.co)) || (rc = nalloc(n, &l.wt, (size_t)27 * l.ci * l.co)))
            return rc;
    }
    // activations: e1 G C, e2 G/2 2C, e3 G/2 2C, e4 G/4 4C, e5 G/4 4C, e6 G/8 4C;
    // cat1 G/4 8C -> d1 G/4 4C; cat2 G/2 6C -> d2 G/2 2C; cat3 G 3C -> d3 G C; out G 16
    const int eg[7] = {0, G, G / 2, G / 2, G / 4, G / 4, G / 8}, ec[7] = {0, C, 2 * C, 2 * C, 4 * C, 4 * C, 4 * C};
    const int dg[4] = {0, G / 4, G / 2, G}, dc[4] = {0, 4 * C, 2 * C, C}, cc[4] = {0, 8 * C, 6 * C, 3 * C};
    if ((rc = nalloc(n, &n->x0, pts(G) * 16))) return rc;
    for (int k = 1; k <= 6; ++k)
        if ((rc = nalloc(n, &n->e[k], pts(eg[k]) * ec[k])) || (rc = nalloc(n, &n->ge[k], pts(eg[k]) * ec[k])))
            return rc;
    for (int k = 1; k <= 3; ++k)
        if ((rc = nalloc(n, &n->d[k], pts(dg[k]) * dc[k])) || (rc = nalloc(n, &n->gd[k], pts(dg[k]) * dc[k])) ||
            (rc = nalloc(n, &n->cat[k], pts(dg[k]) * cc[k])) || (rc = nalloc(n, &n->gcat[k], pts(dg[k]) * cc[k])))
            return rc;
    if ((rc = nalloc(n, &n->outf, pts(G) * 16)) || (rc = nalloc(n, &n->gout, pts(G) * 16))) return rc;
    if ((rc = nalloc(n, &n->dz, pts(G) * 8 * C))) return rc;
    n->splits = (int)std::max<int64_t>(1, std::min<int64_t>(64, pts(G) / 512));
    int64_t maxw = 0;
    for (auto& l : n->L) maxw = std::max<int64_t>(maxw, (int64_t)27 * l.ci * l.co);
    if ((rc = nalloc(n, &n->part, (size_t)n->splits * maxw))) return rc;
    if ((rc = nalloc(n, &n->lpart, 256)) || (rc = nalloc(n, &n->tgt, pts(G) * 3)) ||
        (rc = nalloc(n, &n->inbuf, pts(G) * 6)))
        return rc;
    NCK(cudaStreamCreateWithFlags(&n->st, cudaStreamNonBlocking));
    // He-uniform initialisation from a seeded SplitMix64 stream; biases 0
    std::vector<float> h(off, 0.0f);
    uint64_t s = seed ? seed : 0x9E3779B97F4A7C15ull;
    auto next = [&]() {
        s += 0x9E3779B97F4A7C15ull;
        uint64_t z = s;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    for (size_t li = 0; li < n->L.size(); ++li) {
        const Layer& l = n->L[li];
        const double a = (li + 1 == n->L.size() ? 0.1 : 1.0) * std::sqrt(6.0 / (27.0 * l.ci));
        for (int64_t e = 0; e < (int64_t)27 * l.ci * l.co; ++e) h[l.woff + e] = (float)((2.0 * next() - 1.0) * a);
    }
    NCK(cudaMemcpy(n->w, h.data(), sizeof(float) * off, cudaMemcpyHostToDevice));
    NCK(cudaMemset(n->m, 0, sizeof(float) * off));
    NCK(cudaMemset(n->v, 0, sizeof(float) * off));
    for (auto& l : n->L) to_bf16_pair<<<gridn((int64_t)27 * l.ci * l.co), 256, 0, n->st>>>(n->w + l.woff, l.ci, l.co, l.wb, l.wt);
    NCK(cudaStreamSynchronize(n->st));
    n->err.clear();
    return WLC_OK;
}

extern "C" int wlc_net_destroy(wlc_net* n) {
    if (!n) return WLC_OK;
    if (n->st) cudaStreamSynchronize(n->st);
    for (void* p : n->allocs) cudaFree(p);
    if (n->st) cudaStreamDestroy(n->st);
    delete n;
    return WLC_OK;
}

extern "C" const char* wlc_net_last_error(const wlc_net* n) { return n ? n->err.c_str() : "null network"; }
extern "C" int64_t wlc_net_param_count(const wlc_net* n) { return n ? n->np : 0; }

static void conv_fwd(wlc_net* n, const Layer& l, const bf16* x, bf16* y, float* yf) {
    const int M = (int)pts(l.gout);
    const dim3 grid((M + 63) / 64, l.co / 16);
    gather_gemm<0><<<grid, 128, 0, n->st>>>(x, l.ci, l.wt, l.co, M, l.gin, l.gout, l.stride, n->w + l.boff, l.relu, y,
                                            yf);
}

// from dy (FP32, layer output gradient) and the layer output y: weight and
// bias gradients, and (dx != null) dx += data gradient
static void conv_bwd(wlc_net* n, const Layer& l, const bf16* x, const bf16* y, const float* dy, float* dx) {
    const int64_t Mq = pts(l.gout), Mp = pts(l.gin);
    relu_back<<<gridn(Mq * l.co), 256, 0, n->st>>>(dy, y, l.relu, Mq * l.co, n->dz);
    const int splits = (int)std::max<int64_t>(1, std::min<int64_t>(n->splits, Mq / 16));
    wgrad<<<dim3(l.ci / 16, l.co / 16, 27 * splits), 32, 0, n->st>>>(x, l.ci, n->dz, l.co, (int)Mq, l.gin, l.gout,
                                                                     l.stride, splits, n->part);
    const int64_t nw = (int64_t)27 * l.ci * l.co;
    sum_splits<<<gridn(nw), 256, 0, n->st>>>(n->part, splits, nw, n->g + l.woff);
    bias_grad<<<(l.co + 63) / 64, 64, 0, n->st>>>(n->dz, l.co, (int)Mq, n->g + l.boff);
    if (dx) {
        const dim3 grid((unsigned)((Mp + 63) / 64), l.ci / 16);
        gather_gemm<1><<<grid, 128, 0, n->st>>>(n->dz, l.co, l.wb, l.ci, (int)Mp, l.gin, l.gout, l.stride, nullptr, 0,
                                                nullptr, dx);
    }
}

static void forward(wlc_net* n) {
    const int G = n->G, C = n->C;
    const auto& L = n->L;
    conv_fwd(n, L[0], n->x0, n->e[1], nullptr);
    for (int k = 2; k <= 6; ++k) conv_fwd(n, L[k - 1], n->e[k - 1], n->e[k], nullptr);
    // d1: cat(up(e6), e5) at G/4
    up_into<<<gridn(pts(G / 4) * 4 * C), 256, 0, n->st>>>(n->e[6], G / 8, 4 * C, n->cat[1], 8 * C, 0);
    copy_into<<<gridn(pts(G / 4) * 4 * C), 256, 0, n->st>>>(n->e[5], pts(G / 4), 4 * C, n->cat[1], 8 * C, 4 * C);
    conv_fwd(n, L[6], n->cat[1], n->d[1], nullptr);
    up_into<<<gridn(pts(G / 2) * 4 * C), 256, 0, n->st>>>(n->d[1], G / 4, 4 * C, n->cat[2], 6 * C, 0);
    copy_into<<<gridn(pts(G / 2) * 2 * C), 256, 0, n->st>>>(n->e[3], pts(G / 2), 2 * C, n->cat[2], 6 * C, 4 * C);
    conv_fwd(n, L[7], n->cat[2], n->d[2], nullptr);
    up_into<<<gridn(pts(G) * 2 * C), 256, 0, n->st>>>(n->d[2], G / 2, 2 * C, n->cat[3], 3 * C, 0);
    copy_into<<<gridn(pts(G) * C), 256, 0, n->st>>>(n->e[1], pts(G), C, n->cat[3], 3 * C, 2 * C);
    conv_fwd(n, L[8], n->cat[3], n->d[3], nullptr);
    conv_fwd(n, L[9], n->d[3], nullptr, n->outf);
}

// gradients of the loss w.r.t. all parameters, accumulated into n->g
static int backward(wlc_net* n) {
    const int G = n->G, C = n->C;
    const auto& L = n->L;
    for (int k = 1; k <= 6; ++k) NCK(cudaMemsetAsync(n->ge[k], 0, sizeof(float) * pts(L[k - 1].gout) * L[k - 1].co, n->st));
    const int dg[4] = {0, G / 4, G / 2, G}, dc[4] = {0, 4 * C, 2 * C, C}, cc[4] = {0, 8 * C, 6 * C, 3 * C};
    for (int k = 1; k <= 3; ++k) {
        NCK(cudaMemsetAsync(n->gd[k], 0, sizeof(float) * pts(dg[k]) * dc[k], n->st));
        NCK(cudaMemsetAsync(n->gcat[k], 0, sizeof(float) * pts(dg[k]) * cc[k], n->st));
    }
    conv_bwd(n, L[9], n->d[3], nullptr, n->gout, n->gd[3]);  // linear output layer (relu = 0: y unused)
    conv_bwd(n, L[8], n->cat[3], n->d[3], n->gd[3], n->gcat[3]);
    up_back<<<gridn(pts(G / 2) * 2 * C), 256, 0, n->st>>>(n->gcat[3], G / 2, 2 * C, 3 * C, 0, n->gd[2]);
    copy_back<<<gridn(pts(G) * C), 256, 0, n->st>>>(n->gcat[3], pts(G), C, 3 * C, 2 * C, n->ge[1]);
    conv_bwd(n, L[7], n->cat[2], n->d[2], n->gd[2], n->gcat[2]);
    up_back<<<gridn(pts(G / 4) * 4 * C), 256, 0, n->st>>>(n->gcat[2], G / 4, 4 * C, 6 * C, 0, n->gd[1]);
    copy_back<<<gridn(pts(G / 2) * 2 * C), 256, 0, n->st>>>(n->gcat[2], pts(G / 2), 2 * C, 6 * C, 4 * C, n->ge[3]);
    conv_bwd(n, L[6], n->cat[1], n->d[1], n->gd[1], n->gcat[1]);
    up_back<<<gridn(pts(G / 8) * 4 * C), 256, 0, n->st>>>(n->gcat[1], G / 8, 4 * C, 8 * C, 0, n->ge[6]);
    copy_back<<<gridn(pts(G / 4) * 4 * C), 256, 0, n->st>>>(n->gcat[1], pts(G / 4), 4 * C, 8 * C, 4 * C, n->ge[5]);
    for (int k = 6; k >= 2; --k) conv_bwd(n, L[k - 1], n->e[k - 1], n->e[k], n->ge[k], n->ge[k - 1]);
    conv_bwd(n, L[0], n->x0, n->e[1], n->ge[1], nullptr);
    NCK(cudaGetLastError());
    return WLC_OK;
}

static int upload_input(wlc_net* n, const float* in) {
    const int64_t P = pts(n->G);
    NCK(cudaMemcpyAsync(n->inbuf, in, sizeof(float) * 6 * P, cudaMemcpyHostToDevice, n->st));
    input_pack<<<gridn(P * 16), 256, 0, n->st>>>(n->inbuf, 6, (int)P, n->x0, 16);
    return WLC_OK;
}

// loss of the current output against tgt (device), with gout filled
static int loss_of(wlc_net* n, double* loss) {
    const int P = (int)pts(n->G);
    mse_loss<<<64, 256, 0, n->st>>>(n->outf, 16, n->tgt, P, n->gout, n->lpart);
    double h[64];
    NCK(cudaMemcpyAsync(h, n->lpart, sizeof(double) * 64, cudaMemcpyDeviceToHost, n->st));
    NCK(cudaStreamSynchronize(n->st));
    double s = 0.0;
    for (int k = 0; k < 64; ++k) s += h[k];
    *loss = s / (3.0 * P);
    return WLC_OK;
}

extern "C" int wlc_net_forward(wlc_net* n, const float* input, float* output) {
    if (!n || !n->st || !input || !output) return WLC_E_PARAM;
    int rc;
    if ((rc = upload_input(n, input))) return rc;
    forward(n);
    const int64_t P = pts(n->G);
    output_unpack<<<gridn(P * 3), 256, 0, n->st>>>(n->outf, 16, (int)P, n->inbuf);
    NCK(cudaMemcpyAsync(output, n->inbuf, sizeof(float) * 3 * P, cudaMemcpyDeviceToHost, n->st));
    NCK(cudaStreamSynchronize(n->st));
    return WLC_OK;
}

extern "C" int wlc_net_loss_grad(wlc_net* n, const float* input, const float* target, double* loss, float* grad) {
    if (!n || !n->st || !input || !target || !loss) return WLC_E_PARAM;
    const int64_t P = pts(n->G);
    int rc;
    if ((rc = upload_input(n, input))) return rc;
    NCK(cudaMemcpyAsync(n->tgt, target, sizeof(float) * 3 * P, cudaMemcpyHostToDevice, n->st));
    forward(n);
    if ((rc = loss_of(n, loss))) return rc;
    NCK(cudaMemsetAsync(n->g, 0, sizeof(float) * n->np, n->st));
    if ((rc = backward(n))) return rc;
    if (grad) NCK(cudaMemcpyAsync(grad, n->g, sizeof(float) * n->np, cudaMemcpyDeviceToHost, n->st));
    NCK(cudaStreamSynchronize(n->st));
    return WLC_OK;
}

extern "C" int wlc_net_get_params(const wlc_net* nc, float* out) {
    wlc_net* n = const_cast<wlc_net*>(nc);
    if (!n || !out) return WLC_E_PARAM;
    NCK(cudaMemcpy(out, n->w, sizeof(float) * n->np, cudaMemcpyDeviceToHost));
    return WLC_OK;
}

extern "C" int wlc_net_set_params(wlc_net* n, const float* in) {
    if (!n || !in) return WLC_E_PARAM;
    NCK(cudaMemcpy(n->w, in, sizeof(float) * n->np, cudaMemcpyHostToDevice));
    for (auto& l : n->L)
        to_bf16_pair<<<gridn((int64_t)27 * l.ci * l.co), 256, 0, n->st>>>(n->w + l.woff, l.ci, l.co, l.wb, l.wt);
    NCK(cudaStreamSynchronize(n->st));
    n->step = 0;
    NCK(cudaMemset(n->m, 0, sizeof(float) * n->np));
    NCK(cudaMemset(n->v, 0, sizeof(float) * n->np));
    return WLC_OK;
}

// Adam training on nsamples (inputs [s][6][G^3], targets [s][3][G^3], host):
// minibatches of `batch` samples in a seeded shuffled order for `epochs`
// epochs; loss_hist[epoch] = mean training loss of the epoch.
extern "C" int wlc_net_train(wlc_net* n, const float* inputs, const float* targets, int32_t nsamples, int32_t batch,
                             int32_t epochs, float lr, uint64_t seed, double* loss_hist) {
    if (!n || !n->st || !inputs || !targets || nsamples < 1 || batch < 1 || epochs < 1) return WLC_E_PARAM;
    const int64_t P = pts(n->G);
    float *din = nullptr, *dt = nullptr;
    int rc;
    if ((rc = nalloc(n, &din, (size_t)nsamples * 6 * P)) || (rc = nalloc(n, &dt, (size_t)nsamples * 3 * P))) return rc;
    NCK(cudaMemcpyAsync(din, inputs, sizeof(float) * nsamples * 6 * P, cudaMemcpyHostToDevice, n->st));
    NCK(cudaMemcpyAsync(dt, targets, sizeof(float) * nsamples * 3 * P, cudaMemcpyHostToDevice, n->st));
    std::vector<int> order(nsamples);
    for (int i = 0; i < nsamples; ++i) order[i] = i;
    uint64_t s = seed ? seed : 1;
    auto rnd = [&]() {
        s ^= s << 13;
        s ^= s >> 7;
        s ^= s << 17;
        return s;
    };
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int i = nsamples - 1; i > 0; --i) std::swap(order[i], order[rnd() % (uint64_t)(i + 1)]);
        double tot = 0.0;
        for (int b0 = 0; b0 < nsamples; b0 += batch) {
            const int nb = std::min(batch, nsamples - b0);
            NCK(cudaMemsetAsync(n->g, 0, sizeof(float) * n->np, n->st));
            for (int k = 0; k < nb; ++k) {
                const int i = order[b0 + k];
                input_pack<<<gridn(P * 16), 256, 0, n->st>>>(din + (size_t)i * 6 * P, 6, (int)P, n->x0, 16);
                NCK(cudaMemcpyAsync(n->tgt, dt + (size_t)i * 3 * P, sizeof(float) * 3 * P, cudaMemcpyDeviceToDevice,
                                    n->st));
                forward(n);
                double l;
                if ((rc = loss_of(n, &l))) return rc;
                tot += l;
                if ((rc = backward(n))) return rc;
            }
            ++n->step;
            const float c1 = 1.0f - std::pow(b1, (float)n->step), c2 = 1.0f - std::pow(b2, (float)n->step);
            adam<<<gridn(n->np), 256, 0, n->st>>>(n->w, n->g, n->m, n->v, n->np, lr, b1, b2, eps, c1, c2, 1.0f / nb);
            for (auto& l : n->L)
                to_bf16_pair<<<gridn((int64_t)27 * l.ci * l.co), 256, 0, n->st>>>(n->w + l.woff, l.ci, l.co, l.wb,
                                                                                  l.wt);
        }
        if (loss_hist) loss_hist[ep] = tot / nsamples;
    }
    NCK(cudaStreamSynchronize(n->st));
    // the staging buffers are released with the network; free them now
    for (void* p : {(void*)din, (void*)dt}) {
        n->allocs.erase(std::find(n->allocs.begin(), n->allocs.end(), p));
        cudaFree(p);
    }
    return WLC_OK;
}
