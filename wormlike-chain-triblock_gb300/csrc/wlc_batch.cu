// wlc_batch.cu -- the batch engine (wlc_batch_*): several independent FP32
// instances advanced together with batched launches and a captured
// contour loop.  No counterpart in the reference (one instance per MPI job
// there).
#include "wlc_ctx.h"

// ------------------------------------------------------------ batches
// Several independent FP32 instances advanced together: one launch per pass
// per grid-size group per contour step covers every instance of the group
// (arguments from device arrays, instance = blockIdx.z), the streamed
// density slices of all instances share one launch per step, and the whole
// forward + backward contour loop is captured once into a CUDA graph and
// replayed.
struct wlc_batch {
    std::vector<wlc_ctx*> inst;
    cudaStream_t st = nullptr;
    std::string err;
    int nmax = 0, M = 0;
    struct Group {
        int N = 0;
        std::vector<int> idx;
        StepArgs<float>* dstep = nullptr;  // [2 directions][nmax + 1][count]
        SolveArgs<float>* dsolve = nullptr;
        size_t smem = 0;
        int a_variant = 0, solve_threads = 0, xy_threads = 0, xy_z = 0;
        std::vector<int> streamed;              // members with streamed densities
        SliceBatchArgs<float>* dslice = nullptr;  // [streamed]
        bool any_s = false;
        cudaStream_t st = nullptr;  // the group's stream inside the captured contour loop
        cudaEvent_t done = nullptr;
    };
    cudaEvent_t fork = nullptr;
    std::vector<Group> groups;
    std::vector<int> streamed;  // instances with streamed densities
    std::vector<void*> allocs;
    std::vector<long> sig;  // per instance: box generation and Maier-Saupe state at the last build
    bool built = false;
    bool use_graph = true;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t gexec = nullptr;
    int64_t launches = 0;
    int64_t per_replay = 0;  // kernel launches in one replay of the graph
};

static int bset_err(wlc_batch* b, int code, const std::string& msg) {
    if (b) b->err = msg;
    return code;
}

#define BCK(call)                                                                                         \
    do {                                                                                                  \
        cudaError_t e_ = (call);                                                                          \
        if (e_ != cudaSuccess) return bset_err(b, WLC_E_CUDA, std::string(#call ": ") + cudaGetErrorString(e_)); \
    } while (0)

template <typename X> static int balloc(wlc_batch* b, X** p, size_t bytes) {
    void* q = nullptr;
    cudaError_t e = cudaMalloc(&q, bytes ? bytes : 16);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return bset_err(b, WLC_E_ALLOC, std::string("cudaMalloc: ") + cudaGetErrorString(e));
    }
    b->allocs.push_back(q);
    *p = (X*)q;
    return WLC_OK;
}

static void drop_graph(wlc_batch* b) {
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->graph) cudaGraphDestroy(b->graph);
    b->gexec = nullptr;
    b->graph = nullptr;
}

static bool ms_active(const wlc_ctx* c) { return std::fabs(c->p.nmu) >= 1.0e-5 && c->have_mop; }

static std::vector<long> batch_signature(const wlc_batch* b) {
    std::vector<long> v;
    for (auto* c : b->inst) v.push_back(2L * c->box_gen + (ms_active(c) ? 1 : 0));
    return v;
}

// history / output pointers of step n of direction dir for one instance
static void step_ptrs(wlc_ctx* c, int dir, int n, const float** h, float** out, StepKind* k) {
    const size_t sl = (size_t)c->M * c->nr;
    const int nmax = c->p.nmax;
    const int s = dir > 0 ? n : nmax - n;
    const int order = n < 3 ? n : 3;
    *k = StepKind{order, dir, dir > 0 ? blk_fwd(c, s) : blk_bwd(c, s)};
    for (int j = 1; j <= 3; ++j) {
        if (j > order) {
            h[j - 1] = nullptr;
            continue;
        }
        h[j - 1] = dir > 0 ? (const float*)c->qf + (size_t)(s - j) * sl : qb_at<float>(c, s + j);
    }
    *out = dir > 0 ? (float*)c->qf + (size_t)s * sl : qb_at<float>(c, s);
}

static int batch_build(wlc_batch* b) {
    const int nmax = b->nmax;
    for (auto& g : b->groups) {
        const int cnt = (int)g.idx.size();
        const size_t tot = (size_t)2 * (nmax + 1) * cnt;
        std::vector<StepArgs<float>> hs(tot);
        std::vector<SolveArgs<float>> hv(tot);
        for (int d = 0; d < 2; ++d)
            for (int n = 1; n <= nmax; ++n)
                for (int j = 0; j < cnt; ++j) {
                    wlc_ctx* c = b->inst[g.idx[j]];
                    const float* h[3];
                    float* out;
                    StepKind k;
                    step_ptrs(c, d == 0 ? 1 : -1, n, h, &out, &k);
                    StepLaunch<float> L = make_launch<float>(c, k, h[0], h[1], h[2], out);
                    L.solve.c0 = lit_c0(k.order, c->real4);
                    if (ms_active(c)) L.step.msterm = (const float*)c->msterm;
                    const size_t e = ((size_t)d * (nmax + 1) + n) * cnt + j;
                    hs[e] = L.step;
                    hv[e] = L.solve;
                    const size_t sm = solve_smem_bytes<float>(L.solve);
                    if (j == 0 && d == 0 && n == 1)
                        g.smem = sm;
                    else if (sm != g.smem)
                        return bset_err(b, WLC_E_UNSUPPORTED, "instances of one grid size need one solve layout");
                }
        int rc;
        if (!g.dstep) {
            if ((rc = balloc(b, &g.dstep, sizeof(StepArgs<float>) * tot))) return rc;
            if ((rc = balloc(b, &g.dsolve, sizeof(SolveArgs<float>) * tot))) return rc;
        }
        BCK(cudaMemcpy(g.dstep, hs.data(), sizeof(StepArgs<float>) * tot, cudaMemcpyHostToDevice));
        BCK(cudaMemcpy(g.dsolve, hv.data(), sizeof(SolveArgs<float>) * tot, cudaMemcpyHostToDevice));
    }
    for (auto& g : b->groups) {
        if (g.streamed.empty()) continue;
        std::vector<SliceBatchArgs<float>> ha;
        g.any_s = false;
        for (int i : g.streamed) {
            wlc_ctx* c = b->inst[i];
            SliceBatchArgs<float> a;
            a.qf = (const float*)c->qf;
            a.qb = (const float*)c->qb;
            a.sl = (int64_t)c->M * c->nr;
            a.d = density_args(c);
            a.want_s = stream_s(c) ? 1 : 0;
            a.jl = c->jl;
            a.raw = c->raw;
            a.junc = c->junc;
            a.qend = c->qend;
            a.sraw = c->sraw;
            g.any_s = g.any_s || a.want_s;
            ha.push_back(a);
        }
        int rc;
        if (!g.dslice && (rc = balloc(b, &g.dslice, sizeof(SliceBatchArgs<float>) * ha.size()))) return rc;
        BCK(cudaMemcpy(g.dslice, ha.data(), sizeof(SliceBatchArgs<float>) * ha.size(), cudaMemcpyHostToDevice));
    }
    b->sig = batch_signature(b);
    b->built = true;
    return WLC_OK;
}

// enqueue the forward and backward sweeps of one grid-size group on stream st
static int batch_issue_group(wlc_batch* b, wlc_batch::Group& g, cudaStream_t st) {
    const int nmax = b->nmax;
    const int cnt = (int)g.idx.size();
    auto step = [&](int d, int n) -> int {
        const int dir = d == 0 ? 1 : -1;
        for (int i : g.idx) {
            wlc_ctx* c = b->inst[i];
            if (!ms_active(c)) continue;
            const float* h[3];
            float* out;
            StepKind k;
            step_ptrs(c, dir, n, h, &out, &k);
            launch_ms_term<float>(h[0], h[1], h[2], k.order, c->mop, c->thl, c->ds, lit_thresh(c->real4), c->M,
                                  c->nr, (float*)c->msterm, st);
            b->launches++;
        }
        BatchLaunch<float> bl;
        const size_t e = ((size_t)d * (nmax + 1) + n) * cnt;
        bl.dstep = g.dstep + e;
        bl.dsolve = g.dsolve + e;
        bl.count = cnt;
        bl.M = b->M;
        bl.nkx = g.N / 2 + 1;
        bl.solve_smem = g.smem;
        bl.a_variant = g.a_variant;
        bl.solve_threads = g.solve_threads;
        bl.xy_threads = g.xy_threads;
        bl.xy_z = g.xy_z;
        cudaError_t err = launch_step_batched(g.N, bl, st);
        b->launches += 3;
        if (err != cudaSuccess) return bset_err(b, WLC_E_CUDA, std::string("batched step: ") + cudaGetErrorString(err));
        return WLC_OK;
    };
    auto slices = [&](int s) {
        if (g.streamed.empty()) return;
        const wlc_ctx* c0 = b->inst[g.streamed[0]];
        launch_density_slice_batched<float>(g.dslice, (int)g.streamed.size(), c0->nr, s, b->M, c0->jl.n,
                                            g.any_s ? 1 : 0, st);
        b->launches++;
    };
    int rc;
    for (int i : g.idx) {
        wlc_ctx* c = b->inst[i];
        launch_set_delta<float>((float*)c->qf, c->M, c->nr, st);
        b->launches++;
    }
    for (int n = 1; n <= nmax; ++n)
        if ((rc = step(0, n))) return rc;
    for (int i : g.streamed) {
        wlc_ctx* c = b->inst[i];
        BCK(cudaMemsetAsync(c->raw, 0, sizeof(double) * 3 * (size_t)c->nr, st));
        if (stream_s(c)) BCK(cudaMemsetAsync(c->sraw, 0, sizeof(double) * 15 * (size_t)c->nr, st));
    }
    for (int i : g.idx) {
        wlc_ctx* c = b->inst[i];
        launch_set_delta<float>(qb_at<float>(c, nmax), c->M, c->nr, st);
        b->launches++;
    }
    slices(nmax);
    for (int n = 1; n <= nmax; ++n) {
        if ((rc = step(1, n))) return rc;
        slices(nmax - n);
    }
    BCK(cudaGetLastError());
    return WLC_OK;
}

// enqueue the sweeps of every instance: the groups are independent, so each
// runs on its own stream (forked from and joined back into the batch
// stream; inside stream capture this becomes parallel branches of the graph)
static int batch_issue(wlc_batch* b) {
    if (b->groups.size() == 1) return batch_issue_group(b, b->groups[0], b->st);
    BCK(cudaEventRecord(b->fork, b->st));
    int rc = WLC_OK;
    for (auto& g : b->groups) {
        BCK(cudaStreamWaitEvent(g.st, b->fork, 0));
        if ((rc = batch_issue_group(b, g, g.st))) break;
        BCK(cudaEventRecord(g.done, g.st));
    }
    for (auto& g : b->groups) BCK(cudaStreamWaitEvent(b->st, g.done, 0));
    return rc;
}

extern "C" int wlc_batch_create(const wlc_params* p, int32_t count, wlc_batch** out) {
    if (!p || !out || count < 1) return WLC_E_PARAM;
    wlc_batch* b = new wlc_batch();
    *out = b;
    for (int i = 0; i < count; ++i) {
        const wlc_params& q = p[i];
        char buf[200];
        if (q.precision != WLC_FP32 || !supported_batch_n(q.n[0]) || q.q_checkpoint != 0 || q.nmax != p[0].nmax ||
            q.lmax != p[0].lmax || q.scheme != WLC_SCHEME_BDF) {
            std::snprintf(buf, sizeof buf,
                          "instance %d: batches take FP32 BDF-scheme instances with one nmax and lmax, no "
                          "q_checkpoint, and a grid edge in {16, 24, 32, 40, 48, 64}",
                          i);
            return bset_err(b, WLC_E_UNSUPPORTED, buf);
        }
    }
    b->nmax = p[0].nmax;
    b->M = (p[0].lmax + 1) * (p[0].lmax + 1);
    BCK(cudaStreamCreateWithFlags(&b->st, cudaStreamNonBlocking));
    for (int i = 0; i < count; ++i) {
        wlc_ctx* c = nullptr;
        int rc = create_impl(&p[i], b->st, &c);
        if (rc) {
            b->err = "instance " + std::to_string(i) + ": " + (c ? c->err : std::string("create failed"));
            if (c) destroy_impl(c);
            return rc;
        }
        c->batch_owned = true;
        b->inst.push_back(c);
        bool found = false;
        for (auto& g : b->groups)
            if (g.N == c->N) {
                g.idx.push_back(i);
                found = true;
            }
        if (!found) {
            wlc_batch::Group g;
            g.N = c->N;
            g.idx.push_back(i);
            b->groups.push_back(g);
        }
        if (c->stream) {
            b->streamed.push_back(i);
            for (auto& g : b->groups)
                if (g.N == c->N) g.streamed.push_back(i);
        }
    }
    for (auto& g : b->groups) {
        BCK(prepare_step_batched(g.N));
        BCK(cudaStreamCreateWithFlags(&g.st, cudaStreamNonBlocking));
        BCK(cudaEventCreateWithFlags(&g.done, cudaEventDisableTiming));
    }
    BCK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    return WLC_OK;
}

extern "C" int wlc_batch_destroy(wlc_batch* b) {
    if (!b) return WLC_OK;
    if (b->st) cudaStreamSynchronize(b->st);
    drop_graph(b);
    for (auto* c : b->inst) destroy_impl(c);
    for (void* q : b->allocs) cudaFree(q);
    for (auto& g : b->groups) {
        if (g.st) {
            cudaStreamSynchronize(g.st);
            cudaStreamDestroy(g.st);
        }
        if (g.done) cudaEventDestroy(g.done);
    }
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->st) cudaStreamDestroy(b->st);
    delete b;
    return WLC_OK;
}

extern "C" const char* wlc_batch_last_error(const wlc_batch* b) { return b ? b->err.c_str() : "null batch"; }

extern "C" int32_t wlc_batch_size(const wlc_batch* b) { return b ? (int32_t)b->inst.size() : 0; }

extern "C" int wlc_batch_get(wlc_batch* b, int32_t i, wlc_ctx** ctx) {
    if (!b || !ctx || i < 0 || i >= (int)b->inst.size()) return bset_err(b, WLC_E_PARAM, "bad instance index");
    *ctx = b->inst[i];
    return WLC_OK;
}

extern "C" void* wlc_batch_stream(const wlc_batch* b) { return b ? (void*)b->st : nullptr; }

extern "C" int64_t wlc_batch_launch_count(const wlc_batch* b) { return b ? b->launches : 0; }

extern "C" int wlc_batch_use_graph(wlc_batch* b, int32_t on) {
    if (!b) return WLC_E_PARAM;
    b->use_graph = on != 0;
    drop_graph(b);
    return WLC_OK;
}

extern "C" int wlc_batch_propagate(wlc_batch* b) {
    if (!b || !b->st) return WLC_E_STATE;
    for (auto* c : b->inst)
        if (!c->have_fields) return bset_err(b, WLC_E_STATE, "every instance needs wlc_set_fields first");
    for (auto* c : b->inst)
        if (c->fp32 == false) return bset_err(b, WLC_E_STATE, "batch instances must stay FP32");
    int rc;
    if (!b->built || b->sig != batch_signature(b)) {
        drop_graph(b);
        if ((rc = batch_build(b))) return rc;
    }
    if (b->use_graph) {
        if (!b->gexec) {
            BCK(cudaStreamSynchronize(b->st));
            BCK(cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
            const int64_t l0 = b->launches;
            rc = batch_issue(b);
            cudaGraph_t gr = nullptr;
            cudaError_t e = cudaStreamEndCapture(b->st, &gr);
            if (rc) {
                if (gr) cudaGraphDestroy(gr);
                return rc;
            }
            if (e != cudaSuccess) return bset_err(b, WLC_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
            b->graph = gr;
            BCK(cudaGraphInstantiate(&b->gexec, b->graph, 0));
            b->per_replay = b->launches - l0;
            b->launches = l0;  // counted per replay below
        }
        BCK(cudaGraphLaunch(b->gexec, b->st));
        b->launches += b->per_replay;
    } else {
        if ((rc = batch_issue(b))) return rc;
    }
    for (auto* c : b->inst) {
        c->have_fwd = c->have_bwd = true;
        c->have_density = false;
    }
    return WLC_OK;
}

// Time the batched step of each grid-size group under every candidate
// launch configuration (on the last forward step, which re-runs with the
// same inputs and output) and keep the fastest; the graph is re-captured.
extern "C" int wlc_batch_autotune(wlc_batch* b, int32_t* config) {
    if (!b || !b->st) return WLC_E_STATE;
    int rc;
    if ((rc = wlc_batch_propagate(b))) return rc;
    const int nmax = b->nmax;
    for (size_t gi = 0; gi < b->groups.size(); ++gi) {
        auto& g = b->groups[gi];
        const int cnt = (int)g.idx.size();
        float best = 1e30f;
        int best_a = g.a_variant, best_t = g.solve_threads, best_x = g.xy_threads, best_z = g.xy_z;
        for (int xz : {0, 1, 2, 3})
        for (int xt : {256, 512})
        for (int av : {1, 2})
            for (int th : solve_thread_candidates(g.N)) {
                BatchLaunch<float> bl;
                const size_t e = (size_t)nmax * cnt;  // direction 0, step nmax
                bl.dstep = g.dstep + e;
                bl.dsolve = g.dsolve + e;
                bl.count = cnt;
                bl.M = b->M;
                bl.nkx = g.N / 2 + 1;
                bl.solve_smem = g.smem;
                bl.a_variant = av;
                bl.solve_threads = th;
                bl.xy_threads = xt;
                bl.xy_z = xz;
                for (int i : g.idx) {  // Theta terms of that step
                    wlc_ctx* c = b->inst[i];
                    if (!ms_active(c)) continue;
                    const float* h[3];
                    float* out;
                    StepKind k;
                    step_ptrs(c, 1, nmax, h, &out, &k);
                    launch_ms_term<float>(h[0], h[1], h[2], k.order, c->mop, c->thl, c->ds, lit_thresh(c->real4),
                                          c->M, c->nr, (float*)c->msterm, b->st);
                }
                const float t = time_ms(b->st, [&] { launch_step_batched(g.N, bl, b->st); }, 3);
                BCK(cudaGetLastError());
                if (t < best) {
                    best = t;
                    best_a = av;
                    best_t = th;
                    best_x = xt;
                    best_z = xz;
                }
            }
        g.a_variant = best_a;
        g.solve_threads = best_t;
        g.xy_threads = best_x;
        g.xy_z = best_z;
        if (config) {
            config[5 * gi] = g.N;
            config[5 * gi + 1] = best_a;
            config[5 * gi + 2] = best_t;
            config[5 * gi + 3] = best_x;
            config[5 * gi + 4] = best_z;
        }
    }
    drop_graph(b);
    return WLC_OK;
}

extern "C" int32_t wlc_batch_groups(const wlc_batch* b) { return b ? (int32_t)b->groups.size() : 0; }
