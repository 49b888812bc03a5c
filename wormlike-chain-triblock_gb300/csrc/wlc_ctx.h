// wlc_ctx.h -- internal: the context structure behind the C ABI and the
// helpers shared by the single-instance API (wlc_api.cu) and the batch
// engine (wlc_batch.cu).  Not installed; not part of the ABI.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "wlc.h"
#include "wlc_internal.h"
#include "wlc_mix.h"
#include "wlc_reduce.h"
#include "wlc_step.h"

using namespace wlc;

struct wlc_ctx {
    wlc_params p{};
    int N = 0, L = 0, M = 0, nkx = 0;
    int64_t nr = 0, nk = 0;
    bool fp32 = false;
    int real4 = 1;
    double ds = 0, vol = 0, kf[3] = {0, 0, 0};
    int nstart[3] = {0, 0, 0};
    void* pivtab = nullptr;  // [order 1..3][blk][key][npiv] compute type, isotropic spacing only
    int nkeys = 0, npiv = 0;
    bool have_piv = false;
    cudaStream_t st = nullptr;
    // overlapped sweeps (stored mode, own stream): the backward sweep runs on
    // st2 with its own k-space buffer phat2, after ev_inputs (recorded on st
    // by every call that changes what the sweep reads) and before ev_join
    // (which st waits on), so it overlaps the forward sweep on st
    cudaStream_t st2 = nullptr;
    cudaEvent_t ev_inputs = nullptr, ev_join = nullptr;
    void* phat2 = nullptr;
    std::string err;
    BasisTables tab;
    std::vector<void*> allocs;
    SolveTablesT<double> sd{};
    SolveTablesT<float> sf{};
    ThetaLists thl{};
    JLists jl{};
    void* twg = nullptr;
    // per-precision operator data ([0] FP64, [1] FP32); twg / pivtab /
    // have_piv above alias the active one
    struct PrecState {
        bool built = false;
        void* twg = nullptr;
        void* pivtab = nullptr;
        bool have_piv = false;
        int piv_gen = -1;
    } prec[2];
    int box_gen = 0;   // incremented by every wlc_set_box
    size_t elem = 0;   // bytes per real of the propagator buffers as allocated
    // propagator storage: qf holds all Nmax+1 slices of q, or (q_checkpoint K
    // > 0) a 4-slice ring, the BDF3 history triple at every K-th slice and a
    // (K+2)-slice segment buffer; qb holds all slices of q* or (streamed
    // densities) a 4-slice ring
    void* qf = nullptr;
    void* qb = nullptr;
    int K = 0, nck = 0;
    bool stream = false;
    bool own_stream = true;   // false: the stream belongs to a batch
    bool batch_owned = false;
    int a_variant = 0, solve_threads = 0, xy_threads = 0, xy_z = 0;  // launch configuration (autotuned or default)
    void* phat = nullptr;
    void* cf = nullptr;
    void* work = nullptr;    // [M][nr] compute type: RHS / one-step scratch
    void* msterm = nullptr;  // [M][nr] compute type: Maier-Saupe term
    double* w = nullptr;
    double* mop = nullptr;
    double* raw = nullptr;   // [3][nr]
    double* junc = nullptr;  // [3][nr] (unscaled)
    double* juncs = nullptr; // [3][nr] scaled copy
    double* qend = nullptr;  // [nr]
    double* phi = nullptr;   // [3][nr]
    double* part = nullptr;  // [kS3Blocks]
    double* scal = nullptr;  // [8]
    double* sraw = nullptr;  // [3][5][nr] (unscaled)
    double* srs = nullptr;   // [3][5][nr] scaled copy
    double* ar = nullptr;    // [nr]
    double* stage = nullptr; // [M*nr] double, host transfer staging
    int* flag = nullptr;
    bool have_fields = false, have_mop = false, have_fwd = false, have_bwd = false, have_density = false;
    double lnq = 0.0, totden = 0.0;
    int64_t launches = 0;
    bool timing = false;
    std::vector<cudaEvent_t> ev;
    double tms[4] = {0, 0, 0, 0};
    // field update (wlc_iterate)
    int mix_iter = 0, mix_depth = -1;
    double* wout_hist = nullptr;  // [depth+1][3][nr]
    double* dw_hist = nullptr;    // [depth+1][3][nr]
    double* mixbuf = nullptr;     // partials / results / coefficients
};

inline int set_err(wlc_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}

#define CK(call)                                                                                          \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess)                                                                            \
            return set_err(c, WLC_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));            \
    } while (0)

template <typename X> inline int dalloc(wlc_ctx* c, X** ptr, size_t bytes) {
    void* p = nullptr;
    cudaError_t e = cudaMalloc(&p, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        char buf[200];
        std::snprintf(buf, sizeof buf, "cudaMalloc(%zu bytes) failed: %s", bytes, cudaGetErrorString(e));
        return set_err(c, WLC_E_ALLOC, buf);
    }
    c->allocs.push_back(p);
    *ptr = reinterpret_cast<X*>(p);
    return WLC_OK;
}

template <typename X> inline int upload(wlc_ctx* c, X** dst, const std::vector<X>& v) {
    int rc = dalloc(c, dst, sizeof(X) * v.size());
    if (rc) return rc;
    if (!v.empty()) CK(cudaMemcpy((void*)*dst, v.data(), sizeof(X) * v.size(), cudaMemcpyHostToDevice));
    return WLC_OK;
}

inline bool ready(const wlc_ctx* c) { return c && c->st; }

// (order, sigma, block) of one contour step
struct StepKind {
    int order, sigma, blk;
};

// Maier-Saupe coupling switched on (|NMu| >= 1e-5, as the reference tests it)
inline bool ms_on(const wlc_ctx* c) { return std::fabs(c->p.nmu) >= 1.0e-5; }
// orientation tensor accumulated by a streamed backward sweep
inline bool stream_s(const wlc_ctx* c) { return c->p.store_qstar == 2 || ms_on(c); }

inline int blk_fwd(const wlc_ctx* c, int s) {  // MDE_ABC.f90:44-57
    if (s <= c->nstart[1]) return 0;
    if (s <= c->nstart[2]) return 1;
    return 2;
}
inline int blk_bwd(const wlc_ctx* c, int s) {  // MDE_ABC.f90:69-83
    if (s >= c->nstart[2]) return 2;
    if (s >= c->nstart[1]) return 1;
    return 0;
}

inline bool split_scheme(const wlc_ctx* c) { return c->p.scheme == WLC_SCHEME_SPLIT; }
// the step to slice s of the forward sweep / of the backward sweep: BDF order
// ramp 1, 2, 3 at the chain ends (MDE_ABC.f90:50-56,70-82), or the split step
inline StepKind fwd_kind(const wlc_ctx* c, int s) {
    return StepKind{split_scheme(c) ? kSplitOrder : (s < 3 ? s : 3), 1, blk_fwd(c, s)};
}
inline StepKind bwd_kind(const wlc_ctx* c, int s) {
    const int n = c->p.nmax - s;
    return StepKind{split_scheme(c) ? kSplitOrder : (n < 3 ? n : 3), -1, blk_bwd(c, s)};
}
// diagonal constant of the solved operator: BDF c0, or 1 for I + ds/2 A
inline double step_c0(const wlc_ctx* c, int order) {
    return order == kSplitOrder ? 1.0 : lit_c0(order, c->real4);
}
// pivot tables per precision: (BDF order 1..3) x block, plus the split operator per block
inline int pivot_tables(const wlc_ctx* c) { return split_scheme(c) ? 12 : 9; }
// e^{-w_blk ds/2} plane of block blk in the coefficient array cf
// ([blk][3][nr] BDF3 coefficients, [blk][nr] ds*w, [blk][nr] half-step factors)
template <typename T> inline const T* ehalf_plane(const wlc_ctx* c, int blk) {
    return (const T*)c->cf + (size_t)(12 + blk) * (size_t)c->nr;
}

// Fill the launch description of one step.  h1..h3: history (or the RHS
// for order 0), qout: destination slice.
template <typename T>
inline StepLaunch<T> make_launch(wlc_ctx* c, StepKind k, const T* h1, const T* h2, const T* h3, T* qout) {
    using C = typename cvec<T>::t;
    StepLaunch<T> L;
    L.a_variant = c->a_variant;
    L.solve_threads = c->solve_threads;
    L.xy_threads = c->xy_threads;
    L.xy_z = c->xy_z;
    const size_t nr = (size_t)c->nr;
    StepArgs<T>& a = L.step;
    a.h1 = h1;
    a.h2 = h2;
    a.h3 = h3;
    a.wb = c->w + (size_t)k.blk * nr;
    a.cf = (const T*)c->cf + (size_t)k.blk * 3 * nr;
    a.dsw = (const T*)c->cf + (size_t)(9 + k.blk) * nr;
    a.third = (T)lit_third(c->real4);
    a.msterm = nullptr;
    a.order = k.order;
    a.ds = (T)c->ds;
    a.phat = (C*)c->phat;
    a.twg = (const C*)c->twg;
    a.M = c->M;
    a.qout = qout;
    a.minv = (T)(1.0 / (double)c->nr);  // M_grid_inv, wormlike_MDE_2dcomp_mod.f90:307
    SolveArgs<T>& s = L.solve;
    s.phat = (C*)c->phat;
    s.twg = (const C*)c->twg;
    if constexpr (sizeof(T) == 8)
        s.tab = c->sd;
    else
        s.tab = c->sf;
    for (int q = 0; q < 3; ++q) s.kf[q] = c->kf[q];
    s.ds = c->ds;
    s.sigma = k.sigma;
    s.nkx = c->nkx;
    s.correct = (!c->fp32 && s.tab.ndr > 0) ? 1 : 0;
    s.npiv = c->npiv;
    s.pivtab = nullptr;
    if (c->have_piv && k.order >= 1 && k.order <= 3)
        s.pivtab = (const T*)c->pivtab + ((size_t)((k.order - 1) * 3 + k.blk) * c->nkeys) * c->npiv;
    // diagonal of G (Gmatrix_2dcomp_mod.f90:394): c0 + ds*Loa*l(l+1)/(2 kappa)
    s.dcoef = c->ds * c->p.loa / (2.0 * c->p.kappa[k.blk]);
    if (k.order == kSplitOrder) {
        // e^{-w ds/2} before and after; pass B solves I + ds/2 A (the G of
        // c0 = 1 at half the step) and forms the Crank-Nicolson output
        const T* eh = ehalf_plane<T>(c, k.blk);
        a.cf = eh;
        a.dsw = eh;
        a.post = eh;
        s.ds = 0.5 * c->ds;
        s.dcoef = 0.5 * c->ds * c->p.loa / (2.0 * c->p.kappa[k.blk]);
        s.split = 1;
        if (c->have_piv)
            s.pivtab = (const T*)c->pivtab + ((size_t)(9 + k.blk) * c->nkeys) * c->npiv;
    }
    return L;
}

// the backward sweep may run on its own stream, overlapping the forward
// sweep: q* does not depend on q when every slice is stored (the densities
// come after both sweeps); not with streamed densities, the Maier-Saupe term
// (one Theta buffer), timing (per-pass events) or a stream shared with a batch
inline bool overlap_sweeps(const wlc_ctx* c) {
    return c->st2 && c->phat2 && c->p.store_qstar == 1 && !ms_on(c) && !c->timing && !c->batch_owned;
}
// the inputs of a backward sweep (fields, coefficient planes, tables, box,
// stored slices) are final up to here on the context stream
inline cudaError_t mark_inputs(wlc_ctx* c) { return c->ev_inputs ? cudaEventRecord(c->ev_inputs, c->st) : cudaSuccess; }

// slice addressing of the storage modes
template <typename T> inline T* qf_ring(wlc_ctx* c, int s) {
    return (T*)c->qf + (size_t)(s & 3) * (size_t)c->M * c->nr;
}
template <typename T> inline T* qf_ckpt(wlc_ctx* c, int m, int j) {  // q(mK - 2 + j), m >= 1
    return (T*)c->qf + (size_t)(4 + 3 * (m - 1) + j) * (size_t)c->M * c->nr;
}
template <typename T> inline T* qf_seg(wlc_ctx* c, int idx) {  // segment slot idx = s - mK + 2
    return (T*)c->qf + (size_t)(4 + 3 * c->nck + idx) * (size_t)c->M * c->nr;
}
// q(s) as the backward sweep sees it
template <typename T> inline T* qf_at(wlc_ctx* c, int s) {
    if (c->K == 0) return (T*)c->qf + (size_t)s * (size_t)c->M * c->nr;
    return qf_seg<T>(c, s - (s / c->K) * c->K + 2);
}
template <typename T> inline T* qb_at(wlc_ctx* c, int s) {
    return (T*)c->qb + (size_t)(c->stream ? (s & 3) : s) * (size_t)c->M * c->nr;
}

inline DensityArgs density_args(const wlc_ctx* c) {
    DensityArgs d;
    d.nr = c->nr;
    d.M = c->M;
    d.nmax = c->p.nmax;
    for (int b = 0; b < 3; ++b) {
        d.nstart[b] = c->nstart[b];
        d.ns[b] = c->p.ns[b];
    }
    d.ds = c->ds;
    return d;
}

// ------------------------------------------------------------ launch autotuning helpers
inline std::vector<int> solve_thread_candidates(int N) {
    std::vector<int> out;
    const int smax = std::max(1, kSolveThreads / N);
    for (int S : {1, 2, 3, 4, 6, 8, 12, 16})
        if (S <= smax) out.push_back(N * S);
    if (out.empty() || out.back() != N * smax) out.push_back(N * smax);
    return out;
}

template <typename F> inline float time_ms(cudaStream_t st, F&& body, int reps) {
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    body();  // warm-up
    cudaEventRecord(e0, st);
    for (int r = 0; r < reps; ++r) body();
    cudaEventRecord(e1, st);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    return ms / (float)reps;
}


// context creation on a given stream (null: its own) and destruction
int create_impl(const wlc_params* p, cudaStream_t ext, wlc_ctx** out);
int destroy_impl(wlc_ctx* c);
