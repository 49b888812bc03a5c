// wlc_mix.h -- launch interface of the SCFT field-update kernels.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace wlc {

constexpr int kMixBlocks = 256;   // CTAs of the deterministic reductions
constexpr int kMaxAnderson = 10;  // Anderson history depth limit
// accumulators of one Anderson reduction: U (upper triangle), V, 3 x (|dW_K|^2, |w_out_K|^2)
constexpr int kMaxMixAcc = kMaxAnderson * (kMaxAnderson + 1) / 2 + kMaxAnderson + 6;

struct MixGrid {
    int n[3];
    double d[3];
};

// chi_KJ N (symmetric, zero diagonal) and the mean-composition terms
struct MixChi {
    double c[3][3];
    double cf[3];  // sum_J chi_KJ f_J, f_J = N_J / N
    double f[3];   // f_J
    double fsum;   // sum_K cf[K]
};

// mode of launch_mix_out
enum MixMode { kMixSimple = 0, kMixSimpleStore = 1, kMixStore = 2 };

// history slots of one Anderson step: k (current) and km[m] = k - m - 1 (mod depth + 1)
struct AndersonSlots {
    const double* dwk;
    const double* woutk;
    const double* dwm[kMaxAnderson];
};

void launch_mix_out(const double* phi, double* w, const MixChi& chi, int64_t nr, int mode, double lambda, double* wout,
                    double* dw, double* maxpart, double* maxout, cudaStream_t st);
// Maier-Saupe tensor update by simple mixing (SCFT_iterate.f90:351-372):
// M_ab += lambda (NMu S_ab - M_ab) for the 9 components, S the orientation
// tensor summed over the blocks (srs[blk][t][r], t = xx, yy, xy, xz, yz;
// S_zz = -S_xx - S_yy); max |NMu S - M| into *maxout
void launch_mix_m(double* mop, const double* srs, double nmu, double lambda, int64_t nr, double* maxpart,
                  double* maxout, cudaStream_t st);
// U_mn = <dW_k - dW_km, dW_k - dW_kn>, V_m = <dW_k - dW_km, dW_k> (summed over the
// blocks), then <dW_k,K, dW_k,K> and <w_out_k,K, w_out_k,K> per block K: out[0 .. nacc)
int anderson_acc_count(int nrt);
void launch_anderson_dots(const AndersonSlots& s, int nrt, const MixGrid& g, int64_t nr, double vol, double* part,
                          double* out, cudaStream_t st);
// solve U c = V (from launch_anderson_dots' out) and form the new fields
void launch_anderson(const double* acc, int nrt, double* coef, double* w, const double* wout_hist,
                     const double* dw_hist, int64_t slot_stride, int k, const int* km, double lambda, int64_t n,
                     cudaStream_t st);

}  // namespace wlc
