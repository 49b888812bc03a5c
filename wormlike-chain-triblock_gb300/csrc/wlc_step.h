// wlc_step.h -- host-side launch interface of the contour-step kernels.
#pragma once
#include <cuda_runtime.h>

#include "wlc_kernels.cuh"

// Grid edges with compiled kernels (cubic grids).
#define WLC_FOR_EACH_N(X) X(8) X(12) X(16) X(24) X(32) X(40) X(48) X(64) X(96) X(128)
// Grid edges with batched (several instances per launch) FP32 kernels.
#define WLC_FOR_EACH_BATCH_N(X) X(16) X(24) X(32) X(40) X(48) X(64)

namespace wlc {

template <typename T> struct StepLaunch {
    StepArgs<T> step;
    SolveArgs<T> solve;
    bool do_a = true, do_b = true, do_c = true;
    int a_variant = 0;      // pass A: 0 default, 1 generic, 2 staged (FP32, where it fits)
    int solve_threads = 0;  // pass B threads per CTA (0: default)
    int xy_threads = 0;     // generic pass A and pass C threads per CTA (256 or 512; 0: 256)
    int xy_z = 0;           // generic pass A and pass C planes per CTA: 0 default, 1 half
    cudaEvent_t* events = nullptr;  // 4 events around the three passes, or null
};

// One batched contour step: instance j of the launch takes dstep[j] /
// dsolve[j] (device arrays); all instances share N, M and the solve layout.
template <typename T> struct BatchLaunch {
    const StepArgs<T>* dstep = nullptr;
    const SolveArgs<T>* dsolve = nullptr;
    int count = 0, M = 0, nkx = 0;
    size_t solve_smem = 0;
    int a_variant = 0, solve_threads = 0, xy_threads = 0, xy_z = 0;
};

template <typename T> cudaError_t launch_step(int N, const StepLaunch<T>& s, cudaStream_t st);
template <typename T> cudaError_t launch_rhs_only(int N, const StepArgs<T>& a, T* out, cudaStream_t st);
template <typename T> size_t smem_xy(int N, int zd = 0);
template <typename T> cudaError_t launch_solve(int N, const SolveArgs<T>& a, cudaStream_t st, int threads = 0);
cudaError_t launch_step_batched(int N, const BatchLaunch<float>& b, cudaStream_t st);
cudaError_t launch_solve_batched(int N, const BatchLaunch<float>& b, cudaStream_t st);
cudaError_t prepare_step_batched(int N);
cudaError_t prepare_solve_batched(int N);
template <typename T> size_t solve_smem_bytes(const SolveArgs<T>& a);
template <typename T>
cudaError_t launch_pivot_table(T* out, int nkeys, int L, double c0, double dcoef, double ds, double kf, const T* zoff,
                               cudaStream_t st);

inline bool supported_n(int n) {
    switch (n) {
#define WLC_CASE(v) case v:
        WLC_FOR_EACH_N(WLC_CASE)
#undef WLC_CASE
        return true;
        default:
            return false;
    }
}

inline bool supported_batch_n(int n) {
    switch (n) {
#define WLC_CASE(v) case v:
        WLC_FOR_EACH_BATCH_N(WLC_CASE)
#undef WLC_CASE
        return true;
        default:
            return false;
    }
}

}  // namespace wlc
