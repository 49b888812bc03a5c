// wlc_kernels.cuh -- the three kernels of one contour step and their
// arguments.  One BDF step of the reference (init_pr + mde_one_step,
// MDE_ABC.f90:90-383; wormlike_MDE_2dcomp_mod.f90:323-455) runs as
//   pass A  rhs_fft_xy : BDF right-hand side of one coefficient plane group,
//                        R2C along x, C2C along y        -> phat[col][i][z]
//   pass B  zfft_solve : per (kx, ky) column: C2C along z for every
//                        coefficient, the per-k solve of G(k), inverse z
//   pass C  ifft_xy    : inverse y, C2R along x, 1/N^3 -> q_s[i][r]
// phat (the k-space intermediate) is laid out [col = ky*nkx + kx][i][z] so
// that pass B reads one column as a single contiguous run.
#pragma once
#include <cstdint>

#include "wlc_fft.cuh"

namespace wlc {

// Element stride of one packed x row in the shared buffers of passes A and
// C: N + 1 (odd), so that the line-fastest x-FFT work split puts the lanes
// of a warp on distinct banks.  (N/2) rows of a plane then take
// (N/2)(N+1) elements, an even count for the supported N (multiples of 4),
// which keeps the buffers after them 16-byte aligned.
__host__ __device__ constexpr int xrow(int N) { return N + 1; }
__host__ __device__ constexpr int xplane(int N) { return (N / 2) * xrow(N); }

// z planes per CTA of passes A and C: 32-byte runs per (col, i) in phat,
// fewer when the half-spectrum planes would not fit in shared memory
__host__ __device__ constexpr int zg_planes(int N, int tsize) {
    int z = 32 / (2 * tsize);
    while (z > 1 && (size_t)(N + xplane(N) + z * N * (N / 2 + 1)) * 2 * tsize > 200 * 1024) z /= 2;
    return z;
}

// planes per CTA of the generic pass A and pass C in launch variant zd
// (0: zg_planes; 1: half of it while a plane run stays a whole 16-byte chunk)
__host__ __device__ constexpr int xy_planes(int N, int tsize, int zd) {
    const int z = zg_planes(N, tsize);
    return (zd == 1 && z / 2 >= 1 && ((z / 2) * 2 * tsize) % 16 == 0) ? z / 2 : z;
}

// StepArgs::order of a step of the operator-split scheme (WLC_SCHEME_SPLIT):
// pass A multiplies q(s-1) by e^{-w ds/2} (cf / dsw hold that factor),
// pass B applies the Crank-Nicolson operator, pass C multiplies by
// e^{-w ds/2} again (post)
constexpr int kSplitOrder = 4;
// history slices read by a step of the given order (0: the given RHS)
__host__ __device__ constexpr int hist_slices(int order) { return order == 2 ? 2 : order == 3 ? 3 : 1; }

template <typename T> struct StepArgs {
    using C = typename cvec<T>::t;
    // pass A
    const T* h1;        // history slices [M][nr] (q(s-1) / q*(s+1) ...), or Pr
    const T* h2;
    const T* h3;
    const double* wb;   // block field [nr] (orders 1, 2)
    const T* cf;        // order-3 coefficient planes [3][nr]; split: e^{-w ds/2} [nr]
    const T* dsw;       // ds * w of the block [nr] (FP32 path); split: e^{-w ds/2} [nr]
    T third;            // 1/3 of the BDF3 history (literal semantics)
    const T* msterm;    // optional ds*Theta*h term [M][nr] (Maier-Saupe) or null
    int order;          // 0: h1 is the right-hand side itself; 1..3 BDF order; kSplitOrder
    T ds;
    C* phat;            // [nkx*N][M][N]
    const C* twg;       // twiddle table exp(-2 pi i j/N), j < N
    int M;
    // pass C
    T* qout;            // [M][nr]
    T minv;             // 1/N^3
    const T* post = nullptr;  // split scheme: e^{-w ds/2} [nr] applied after 1/N^3; null: none
};

// Per-context constant data of the factorised solve (device pointers).
// Values are in the compute type T; the *f copies in FP32 serve the
// first-order correction, which runs in FP32 inside the FP64 path.
template <typename T> struct SolveTablesT {
    int L, M;
    int npairs;              // (l, m>0) pairs
    const int16_t* pairs;    // [npairs][3]: index of (l, m), index of (l, -m), m
    int nnz;                 // entries of Xp (= entries of Xm)
    const int* xp_ptr;       // CSR of Xp over output rows
    const int16_t* xp_col;
    const T* xp_val;
    const float* xp_valf;
    const int* xm_ptr;       // CSR of Xm = Xp^T
    const int16_t* xm_col;
    const T* xm_val;
    const float* xm_valf;
    const T* zoff;           // [M] Rz coupling (l, m) -> (l+1, m)
    const float* zofff;
    int ndr;                 // correction entries (0: none)
    const int* dr_ptr;       // CSR over rows
    const int16_t* dr_col;
    const int8_t* dr_axis;   // 0 x, 1 y, 2 z
    const float* dr_valf;
};

template <typename T> struct SolveArgs {
    using C = typename cvec<T>::t;
    C* phat;
    const C* twg;
    SolveTablesT<T> tab;
    double kf[3];       // 2 pi / (SIDE * d) per axis
    double ds;
    double c0;          // BDF diagonal
    double dcoef;       // ds * Loa / (2 kappa)
    int sigma;          // +1 forward, -1 backward
    int nkx;
    int correct;        // apply the FP32 first-order correction (tab.ndr > 0)
    const T* pivtab;    // [key][npiv] inverse tridiagonal pivots of this
                        // (order, block), key = ix^2+iy^2+iz^2; null: on the fly
    int npiv;           // (L+1)(L+2)/2
    int split = 0;      // 1: Crank-Nicolson output 2 G^-1 b - b (G = I + ds/2 A, ds here = half step)
};

// Shared-memory carve-up of the solve kernel (bytes, 16-aligned), shared by
// the host launcher and the kernel.
struct SolveSmem {
    size_t col, tw, csa, csaf, zoff, zofff, dr_ptr, dr_col, dr_axis, dr_valf, corr, masks;
    size_t total;
};

__host__ __device__ inline size_t al16(size_t v) { return (v + 15) & ~(size_t)15; }

__host__ __device__ inline SolveSmem solve_smem(int N, int M, int L, int ndr, int tsize, int correct) {
    SolveSmem s;
    size_t o = 0;
    const size_t cs = 2 * (size_t)tsize;
    auto take = [&](size_t bytes) {
        const size_t at = o;
        o = al16(o + bytes);
        return at;
    };
    s.col = take(cs * (size_t)M * (N + 1));
    s.tw = take(cs * N);
    s.csa = take((size_t)tsize * 2 * (L + 1));
    s.csaf = take(4 * 2 * (size_t)(L + 1));
    s.zoff = take((size_t)tsize * M);
    s.zofff = take(correct ? 4 * (size_t)M : 0);
    s.dr_ptr = take(correct ? 4 * (size_t)(M + 1) : 0);
    s.dr_col = take(correct ? 2 * (size_t)ndr : 0);
    s.dr_axis = take(correct ? (size_t)ndr : 0);
    s.dr_valf = take(correct ? 4 * (size_t)ndr : 0);
    s.corr = take(correct ? 8 * (size_t)M * N : 0);  // FP32 correction vectors [i][kz]
    s.masks = take(4 * 2 * 32);                      // work split of the solve phase
    s.total = o;
    return s;
}

constexpr int kSolveThreads = 256;  // threads per CTA of the solve kernel (kz x parts in the solve phase)

// Kernel arguments of one launch: the by-value parameter, or (batched
// launches over several instances) entry blockIdx.z of a device array.
template <bool B, typename A> __device__ __forceinline__ A pick_args(const A& a0, const A* batch) {
    if constexpr (B)
        return batch[blockIdx.z];
    else
        return a0;
}

}  // namespace wlc
