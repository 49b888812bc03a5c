/*
 * wlc.h -- C ABI of the GB300 (sm_103a) wormlike-chain MDE hot path.
 *
 * Drop-in boundary for the propagator / density entry points of
 * tjz2026/wormlike-chain-triblock.  The reference keeps all state in Fortran
 * module globals (global_parameters.f90:17-376) and has no bind(C) interface;
 * each entry point below replaces one reference routine (file:line cited) and
 * keeps that routine's meaning.  A Fortran host binds these through
 * ISO_C_BINDING.
 *
 * Conventions
 *  - Every function returns 0 on success or a negative WLC_E_* code;
 *    wlc_last_error() gives a message.  No call aborts the process and no
 *    call falls back to a CPU path.
 *  - Host arrays are plain pointers with the reference's Fortran
 *    (column-major) layouts, written here as C index expressions.  Grid
 *    point r = x + nx*(y + ny*z) (the reference's x-pencil index on one
 *    rank, grid_mod.f90:356-379).  The library copies in and out; it never
 *    keeps a host pointer.
 *  - A context owns one CUDA stream and all device memory of one SCFT
 *    instance; it is not thread-safe.  One context per host thread.
 */
#ifndef WLC_H
#define WLC_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define WLC_ABI_VERSION 1

enum {
    WLC_OK = 0,
    WLC_E_PARAM = -1,     /* invalid parameter (odd block length, bad size ...) */
    WLC_E_ALLOC = -2,     /* device or host allocation failed                   */
    WLC_E_CUDA = -3,      /* CUDA runtime error                                 */
    WLC_E_STATE = -4,     /* call order violated (e.g. density before sweeps)   */
    WLC_E_NONFINITE = -5, /* NaN/Inf detected in a result                       */
    WLC_E_UNSUPPORTED = -6, /* size/option combination not built                */
    WLC_E_SELFTEST = -7,  /* host-side consistency check of the G(k) factorisation failed */
    WLC_E_IO = -8         /* a file could not be opened, written or parsed          */
};

enum { WLC_FP64 = 0, WLC_FP32 = 1 };

/* Fortran literal semantics of the reference's default-kind constants
 * (11.0/6.0, 1.0/3.0, 1.0/sqrt(3.0), sqrt(1.0*...) in triple_product, PI of
 * kind SP): WLC_LIT_REAL4 = standard build (single precision),
 * WLC_LIT_REAL8 = build with a default-real-8 promotion flag. */
enum { WLC_LIT_REAL4 = 0, WLC_LIT_REAL8 = 1 };

/* Contour-step scheme.
 * WLC_SCHEME_BDF: the reference's semi-implicit BDF1/2/3 step with the
 *   per-k solve of G(k) (mde_one_step / init_pr, MDE_ABC.f90:90-383) -- the
 *   drop-in.
 * WLC_SCHEME_SPLIT: no counterpart in the reference's harmonic-basis
 *   solver.  Operator split of each step,
 *     q(s) = e^{-w ds/2} C2R[ G_CN(k) R2C[ e^{-w ds/2} q(s-1) ] ] / N^3,
 *     G_CN = (I + ds/2 A)^-1 (I - ds/2 A), A = Loa l(l+1)/(2 kappa) + i sigma k.R
 *   (Strang splitting of the field term around a Crank-Nicolson step;
 *   second order in ds, one history slice per step).  The field half steps
 *   follow the reference's angular-grid split-operator solver
 *   (split_operator_MDE_mod.f90:163-166,290-420).  Needs nmu = 0; not in
 *   batches; wlc_init_pr and wlc_mde_one_step keep the BDF meaning. */
enum { WLC_SCHEME_BDF = 0, WLC_SCHEME_SPLIT = 1 };

/* Parameters of one ABC triblock instance: the union of input.txt
 * (initialize_mod.f90:59-84) and the reference's compile-time constants
 * (global_parameters.f90:32,52-60), with one L for all blocks. */
typedef struct wlc_params {
    int32_t n[3];       /* SIDEx, SIDEy, SIDEz (even)                              */
    int32_t lmax;       /* L <= 12: harmonics l = 0..L, M = (L+1)^2 coefficients    */
    int32_t nmax;       /* Nmax contour steps, ds = 1/Nmax                          */
    int32_t ns[3];      /* NA, NB, NC (even, NA+NB+NC = Nmax, initialize_mod.f90:190) */
    double dx[3];       /* grid spacing dx, dy, dz (box edge / SIDE)                */
    double loa;         /* Loa (L over a)                                           */
    double kappa[3];    /* kapa_A (0.5 in the reference), kapa_B, kapa_C            */
    double chi[3];      /* NxAB, NxAC, NxBC                                         */
    double nmu;         /* Maier-Saupe NMu (0 disables the Theta term)              */
    int32_t precision;  /* WLC_FP64 (drop-in) or WLC_FP32 propagators               */
    int32_t literals;   /* WLC_LIT_REAL4 or WLC_LIT_REAL8                            */
    int32_t store_qstar;/* 1: keep every q* slice (wlc_get_q / wlc_init_pr on dir -1);
                           0: keep a 4-slice ring of q* and accumulate the densities
                              during the backward sweep (half the memory);
                           2: as 0, also accumulating the orientation tensor      */
    int32_t q_checkpoint;/* 0: keep every q slice; K >= 3: keep the BDF3 history at
                           every K-th slice and recompute each segment of q during
                           the backward sweep (needs store_qstar 0 or 2; K ~ sqrt(3 Nmax)
                           minimises memory, at one extra forward sweep)           */
    int32_t scheme;     /* WLC_SCHEME_BDF (drop-in) or WLC_SCHEME_SPLIT                 */
    int32_t reserved[3];
} wlc_params;

typedef struct wlc_ctx wlc_ctx;

/* ABI version of the loaded library (WLC_ABI_VERSION). */
int wlc_abi_version(void);

/* Allocate an instance on the current CUDA device, build the harmonic
 * algebra (init_arrays_2decomp, init_array_2dcomp_mod.f90:7-375) and the
 * k-space operator data (init_inverse_sparse_GAB,
 * Gmatrix_2dcomp_mod.f90:222-652). */
int wlc_create(const wlc_params* p, wlc_ctx** out);
int wlc_destroy(wlc_ctx* ctx);
const char* wlc_last_error(const wlc_ctx* ctx);

/* Change the grid spacing and rebuild the k-space data; the reference calls
 * init_inverse_sparse_GAB every time the box changes
 * (Gmatrix_2dcomp_mod.f90:222-224, SCFT_control.f90:166-183). */
int wlc_set_box(wlc_ctx* ctx, double dx, double dy, double dz);

/* Upload the block fields W_blk(0:LS,1:3) (w[blk*nr + r]) and, when
 * nmu != 0, M_OP(0:LS,0:2,0:2) (m_op[r + nr*(a + 3*b)]; may be NULL).
 * Replaces the module-global assignment the Fortran host does before
 * calc_THETAij / MDE_q (SCFT_control.f90:237-243). */
int wlc_set_fields(wlc_ctx* ctx, const double* w, const double* m_op);

/* Forward (dir=+1, MDE_q, wormlike_MDE_2dcomp_mod.f90:231-959) or backward
 * (dir=-1, MDE_qstar, :961-1557) propagator sweep over the three blocks, as
 * ABC_melt_driver (MDE_ABC.f90:8-88) orders them. */
int wlc_propagate(wlc_ctx* ctx, int32_t dir);

/* density() (SCFT_Density_FE_ABC.f90:3-271, per-block restatement).
 * phi:  R_blk(0:LS,1:3)            -> phi[blk*nr + r]            (may be NULL)
 * junc: junction densities at s = NA, NA+NB, Nmax -> junc[j*nr + r] (may be NULL)
 * s_op: S_OP_blk(0:LS,0:2,0:2,1:3) -> s_op[r + nr*(a + 3*b + 9*blk)] (may be NULL;
 *       computing it costs ~ nnz(J)*Nmax*nr flops)
 * lnq:  pff_global = ln Q            (may be NULL) */
int wlc_density(wlc_ctx* ctx, double* phi, double* junc, double* s_op, double* lnq);

/* free_energy() (SCFT_Density_FE.f90:273-342, three-block form): uses the
 * last wlc_density result and the current fields. */
int wlc_free_energy(wlc_ctx* ctx, double* fe);

/* Field-update parameters (the reference's iteration constants,
 * global_parameters.f90:126-139, input.txt line 8, SCFT_main.f90:41). */
typedef struct wlc_mix_params {
    int32_t anderson_depth;   /* Anderson_nim_AB: history depth (1..10)                   */
    int32_t num_simple;       /* Num_simple_mixing_AB = 20: simple-mixing iterations      */
    double lambda_simple;     /* lanbtwA = lanbtwB = 0.1                                   */
    double lambda_anderson;   /* lambda_WAB_anderson = 0.1                                 */
    double tol;               /* CC = 1e-4: every block error below it means converged     */
    int32_t min_iter;         /* 20: converged stays 0 while n_iter < min_iter             */
    int32_t relax_iter;       /* 150: from this n_iter on (nmu == 0 only) ...              */
    double relax_tol;         /* ... 5e-4 is enough; relax_iter <= 0 disables it           */
    double lambda_m;          /* lanbtM = 0.08: Maier-Saupe tensor mixing (nmu != 0)       */
    int32_t reserved[2];
} wlc_mix_params;

/* iterate(converge) (AB_iterate, SCFT_iterate.f90:27-522, three-block
 * form): from the last wlc_density result, update the fields on the device
 * by simple mixing (n_iter <= num_simple) or Anderson mixing (least squares
 * in FP64 on the device).  With f_J = N_J/Nmax, the simple-mixing residual is
 * dW_K = sum_J chi_KJ (phi_J - f_J) + (1/3) sum_J w_J - w_K and the Anderson
 * output field w_K^out = sum_J chi_KJ phi_J + (1/3)(sum_J w_J - sum_KJ chi_KJ f_J)
 * (both reduce to the reference's two-block formulas).
 * err[0..2]: block errors (max |dW_K| while simple mixing,
 * sqrt(<dW_K,dW_K>/<w_K^out,w_K^out>) with Anderson; global, not a mean of
 * per-rank maxima); err[3]: incompressibility residual max |sum_K phi_K - 1|;
 * err[4]: with nmu != 0, tm_diff = max |NMu S - M| before the Maier-Saupe
 * update M += lambda_m (NMu S - M) (S summed over the blocks; 0 otherwise),
 * and convergence also needs err[4] < 5 tol (SCFT_iterate.f90:1124-1139).
 * err has 5 entries.
 * n_iter counts the calls since creation, the last wlc_reset_mixing or a
 * change of anderson_depth.  The fields of the next wlc_propagate are the
 * updated ones; wlc_get_fields reads them. */
int wlc_iterate(wlc_ctx* ctx, const wlc_mix_params* mp, double* err, int32_t* converged);
int wlc_reset_mixing(wlc_ctx* ctx);

/* Copy the current fields W_blk(0:LS,1:3) to the host (w[blk*nr + r]). */
int wlc_get_fields(wlc_ctx* ctx, double* w);
/* Copy the current Maier-Saupe tensor M_OP(0:LS,0:2,0:2) to the host
 * (m_op[r + nr*(a + 3*b)], the layout of wlc_set_fields). */
int wlc_get_mop(wlc_ctx* ctx, double* m_op);

/* No counterpart in the reference (which is FP64 only).  Switch the
 * propagator precision of an existing context between WLC_FP64 and WLC_FP32
 * (precision schedules: FP32 sweeps far from convergence, FP64 to finish).
 * Fields, mixing history and box are kept; propagator slices and the last
 * density are invalidated.  The first switch to a precision builds its
 * operator tables; switching FP32 -> FP64 in a context created FP32
 * reallocates the propagator storage at twice the size. */
int wlc_set_precision(wlc_ctx* ctx, int32_t precision);

/* Copy one contour slice q_f(0:M-1,0:LS,s) (dir=+1) or q_star(...,s)
 * (dir=-1) to the host: out[r*M + i] (coefficient fastest, as the
 * reference's q_f(i,K,s)). */
int wlc_get_q(wlc_ctx* ctx, int32_t dir, int32_t s, double* out);

/* Overwrite one contour slice (test hook; same layout as wlc_get_q). */
int wlc_set_q(wlc_ctx* ctx, int32_t dir, int32_t s, const double* in);

/* init_pr(s, blk_indx, dir, M_Bar, Pr) (MDE_ABC.f90:223-383): BDF right-hand
 * side of contour index s from the stored slices; pr[r*M + i]. */
int wlc_init_pr(wlc_ctx* ctx, int32_t dir, int32_t s, double* pr);

/* mde_one_step(M_Bar, q_out, Pr, G_index, blk_indx, dir) (MDE_ABC.f90:90-221):
 * q_out = C2R(G^-1 . R2C(Pr))/N^3 for the ABC G_index table of
 * Gmatrix_mod-old.f90:446-518 (1 GA1, 2 GA2, 3 GA3, 4 GB3, 5 GC3, 6 GA3*,
 * 7 GB3*, 8 GC3*, 9 GC2*, 10 GC1*).  pr, q_out: [r*M + i] host arrays. */
int wlc_mde_one_step(wlc_ctx* ctx, int32_t g_index, const double* pr, double* q_out);

/* No counterpart in the reference.  wlc_mde_one_step for callers that
 * cannot allocate device memory (code handed only device pointers by its
 * framework, fixed memory pools, driver-level plugins): FP64 only, no
 * context, nothing allocated.  pr_dev / q_out_dev are DEVICE arrays in the
 * coefficient-major layout [i*nr + r] (may alias).  The k-space scratch and
 * operator tables live in one static 64 MiB device array per GPU, so sizes
 * needing more (M * (N/2+1) * N^2 * 16 bytes plus ~100 kB of tables) are
 * rejected with WLC_E_UNSUPPORTED.  The first call on a device looks up the
 * array's address and uploads the tables: make it before any stream
 * capture.  A call whose (N, L, literals) differs from the previous call's
 * on that device uploads its own tables over the old ones and waits for the
 * copy (WLC_E_STATE while its stream is being captured); work still queued
 * on other streams then reads the new tables.  All calls share the array;
 * calls that overlap on the GPU race.
 * stream: cudaStream_t or NULL; errbuf (may be NULL) receives a message. */
int wlc_mde_one_step_noalloc(const wlc_params* p, int32_t g_index, const double* pr_dev, double* q_out_dev,
                             void* stream, char* errbuf, int32_t errlen);

/* Number of the library's own kernel launches issued on the context's
 * stream since creation (instrumentation). */
int64_t wlc_launch_count(const wlc_ctx* ctx);

/* The CUDA stream the context launches on (cudaStream_t as void*), for
 * event timing by the caller. */
void* wlc_stream(const wlc_ctx* ctx);

/* Device time (ms, CUDA events on the context stream) of the last
 * wlc_propagate, split by kernel family: [0] rhs+xy-FFT, [1] z-FFT+G solve,
 * [2] inverse xy-FFT, [3] total.  Only filled when timing is enabled
 * (wlc_enable_timing). */
int wlc_enable_timing(wlc_ctx* ctx, int32_t on);
int wlc_last_timing(const wlc_ctx* ctx, double* ms4);

/* No counterpart in the reference.  Launch autotuning: time the candidate
 * launch configurations of one contour step on this context's own data
 * (pass A variant, threads per solve CTA; all give identical results) and
 * keep the fastest.  Runs a forward sweep first if none is current.
 * config (may be NULL) receives {a_variant, solve_threads, xy_threads,
 * xy_variant} (pass A variant 1 generic / 2 staged; threads per solve CTA;
 * threads per CTA of the generic pass A and pass C, 256 or 512; their
 * variant: bit 0 half the default number of z planes per CTA, bit 1 the
 * x-FFTs of all planes in one batched call).
 * wlc_set_launch_config sets them by hand (0, 0, 0, 0 = defaults). */
int wlc_autotune(wlc_ctx* ctx, int32_t* config);
int wlc_set_launch_config(wlc_ctx* ctx, int32_t a_variant, int32_t solve_threads, int32_t xy_threads,
                          int32_t xy_variant);

/* No counterpart in the reference (one instance per MPI job there).
 * Batches: independent FP32 instances (own grid, box, composition, chi,
 * kappa, Loa, fields; one nmax and lmax; grid edges 16, 24, 32, 40, 48, 64)
 * advanced together.  One kernel launch per pass per grid-size group per
 * contour step covers every instance of the group, the streamed density
 * slices of all instances share one launch per step, and the whole
 * forward + backward contour loop is captured once as a CUDA graph and
 * replayed by wlc_batch_propagate.  Each instance is an ordinary context
 * (wlc_batch_get) for wlc_set_fields, wlc_set_box, wlc_density,
 * wlc_free_energy, wlc_iterate ...; it shares the batch stream and is
 * destroyed with the batch only. */
typedef struct wlc_batch wlc_batch;
int wlc_batch_create(const wlc_params* p, int32_t count, wlc_batch** out);  /* p[count] */
int wlc_batch_destroy(wlc_batch* b);
const char* wlc_batch_last_error(const wlc_batch* b);
int32_t wlc_batch_size(const wlc_batch* b);
int32_t wlc_batch_groups(const wlc_batch* b);
int wlc_batch_get(wlc_batch* b, int32_t i, wlc_ctx** ctx);
/* MDE_q and MDE_qstar of every instance (wormlike_MDE_2dcomp_mod.f90:231-1557
 * per instance); the graph is re-captured after a box or Maier-Saupe change. */
int wlc_batch_propagate(wlc_batch* b);
/* per grid-size group: config[5g..5g+4] = {N, a_variant, solve_threads, xy_threads, xy_variant}
 * (may be NULL) */
int wlc_batch_autotune(wlc_batch* b, int32_t* config);
int wlc_batch_use_graph(wlc_batch* b, int32_t on);  /* 0: issue the launches directly */
void* wlc_batch_stream(const wlc_batch* b);
int64_t wlc_batch_launch_count(const wlc_batch* b);

/* The reference's files (host arrays only, no context needed), for
 * starting from the Fortran code's output and the other way round.
 *  W<rank>.dat: "K W_A W_B W_C" per grid point (W_dump, SCFT_dump.f90:296-300);
 *    wlc_io_read_w also takes the two-block "K W_A W_B" form (readW,
 *    init_array_2dcomp_mod.f90:1088-1093), with w_C = 0.  w[blk*nr + r].
 *  M_OP<rank>.dat: three lines "Lx Ly Lz M(a,0) M(a,1) M(a,2)" per point
 *    (SCFT_dump.f90:302-308); m_op[r + nr*(a + 3*b)], box = {Lx, Ly, Lz}.
 *  RHO_total.dat: '(3f10.6,3f12.8)' x y z phi_A phi_B phi_C, z outermost
 *    (SCFT_dump.f90:116-127); phi[blk*nr + r].
 *  FreeEG.dat: "n_iter F lnQ F+lnQ F-F_FH" and "n_iter box FE-FH F-F_FH"
 *    (SCFT_dump.f90:40-42), F_FH = sum_{K<J} chi_KJ f_K f_J; chi = (AB, AC, BC).
 *  error.dat: "n_iter err..." (SCFT_dump.f90:36-38).
 * Return WLC_E_IO when a file cannot be opened, written or parsed. */
int wlc_io_write_w(const char* path, const double* w, int64_t nr);
int wlc_io_read_w(const char* path, double* w, int64_t nr);
int wlc_io_write_mop(const char* path, const double* m_op, int64_t nr, const double* box);
int wlc_io_read_mop(const char* path, double* m_op, int64_t nr);
int wlc_io_write_rho(const char* path, const double* phi, const int32_t* n, const double* dx);
int wlc_io_append_free_energy(const char* path, int32_t n_iter, double fe, double lnq, double box,
                              const double* chi, const int32_t* ns, int32_t nmax);
int wlc_io_append_errors(const char* path, int32_t n_iter, const double* err, int32_t nerr);

/* No counterpart in the reference.  Learned warm start of the field
 * iteration: a 3D convolutional encoder-decoder (periodic padding; grid
 * levels G, G/2, G/4, G/8; widths C, 2C, 4C; skip connections) mapping six
 * input channels on a G^3 grid (a noise field and five instance parameters
 * as constant fields) to three output fields (the normalised block fields).
 * BF16 weights and activations, FP32 accumulation on the tensor cores, FP32
 * Adam; forward, backward and training all run on the device.
 * Layouts: input [6][G^3], output / target [3][G^3] (channel, then point
 * x + G(y + Gz)).  grid: multiple of 8 in [8, 64]; width: multiple of 16 in
 * [16, 64]; seed: weight initialisation. */
typedef struct wlc_net wlc_net;
int wlc_net_create(int32_t grid, int32_t width, uint64_t seed, wlc_net** out);
int wlc_net_destroy(wlc_net* net);
const char* wlc_net_last_error(const wlc_net* net);
int64_t wlc_net_param_count(const wlc_net* net);
/* FP32 master parameters: per layer (e1..e6, d1..d3, out) W[27][ci][co] then b[co] */
int wlc_net_get_params(const wlc_net* net, float* params);
int wlc_net_set_params(wlc_net* net, const float* params);
int wlc_net_forward(wlc_net* net, const float* input, float* output);
/* mean-squared-error loss of one sample and its gradient w.r.t. the parameters (grad may be NULL) */
int wlc_net_loss_grad(wlc_net* net, const float* input, const float* target, double* loss, float* grad);
/* Adam training: inputs [n][6][G^3], targets [n][3][G^3]; loss_hist[epochs] (may be NULL) */
int wlc_net_train(wlc_net* net, const float* inputs, const float* targets, int32_t nsamples, int32_t batch,
                  int32_t epochs, float lr, uint64_t seed, double* loss_hist);

#ifdef __cplusplus
}
#endif
#endif /* WLC_H */
