// wlc_api.cu -- the C ABI (include/wlc.h): one context per SCFT instance,
// owning its CUDA stream and device memory.  Sweep drivers follow
// ABC_melt_driver (MDE_ABC.f90:8-88); density / free energy follow
// SCFT_Density_FE_ABC.f90:3-271 and SCFT_Density_FE.f90:273-342.
#include "wlc_ctx.h"
#include "wlc_rot_gen.cuh"

template <typename T> static int build_solve_tables(wlc_ctx* c, SolveTablesT<T>& s) {
    const BasisTables& t = c->tab;
    s.L = t.L;
    s.M = t.M;
    std::vector<int16_t> pairs;
    for (int l = 1; l <= t.L; ++l)
        for (int m = 1; m <= l; ++m) {
            pairs.push_back((int16_t)(l * l + l + m));
            pairs.push_back((int16_t)(l * l + l - m));
            pairs.push_back((int16_t)m);
        }
    s.npairs = (int)pairs.size() / 3;
    s.nnz = (int)t.xp_val.size();
    auto cvt = [](const std::vector<double>& v) { return std::vector<T>(v.begin(), v.end()); };
    auto cvf = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
    float* pf;
    auto i16 = [](const std::vector<int>& v) {
        std::vector<int16_t> o(v.size());
        for (size_t k = 0; k < v.size(); ++k) o[k] = (int16_t)v[k];
        return o;
    };
    int rc;
    int16_t* p16;
    int* pi;
    T* pv;
    if ((rc = upload(c, &p16, pairs))) return rc;
    s.pairs = p16;
    if ((rc = upload(c, &pi, t.xp_ptr))) return rc;
    s.xp_ptr = pi;
    if ((rc = upload(c, &p16, i16(t.xp_col)))) return rc;
    s.xp_col = p16;
    if ((rc = upload(c, &pv, cvt(t.xp_val)))) return rc;
    s.xp_val = pv;
    if ((rc = upload(c, &pf, cvf(t.xp_val)))) return rc;
    s.xp_valf = pf;
    if ((rc = upload(c, &pi, t.xm_ptr))) return rc;
    s.xm_ptr = pi;
    if ((rc = upload(c, &p16, i16(t.xm_col)))) return rc;
    s.xm_col = p16;
    if ((rc = upload(c, &pv, cvt(t.xm_val)))) return rc;
    s.xm_val = pv;
    if ((rc = upload(c, &pf, cvf(t.xm_val)))) return rc;
    s.xm_valf = pf;
    if ((rc = upload(c, &pv, cvt(t.zoff)))) return rc;
    s.zoff = pv;
    if ((rc = upload(c, &pf, cvf(t.zoff)))) return rc;
    s.zofff = pf;
    // correction entries, CSR over rows
    std::vector<std::vector<std::pair<int, std::pair<int, double>>>> rows(t.M);
    for (int a = 0; a < 3; ++a)
        for (size_t e = 0; e < t.dR[a].size(); ++e)
            rows[t.dR[a].row[e]].push_back({t.dR[a].col[e], {a, t.dR[a].val[e]}});
    std::vector<int> ptr(t.M + 1, 0);
    std::vector<int16_t> col;
    std::vector<int8_t> axis;
    std::vector<float> val;
    for (int i = 0; i < t.M; ++i) {
        for (auto& e : rows[i]) {
            col.push_back((int16_t)e.first);
            axis.push_back((int8_t)e.second.first);
            val.push_back((float)e.second.second);
        }
        ptr[i + 1] = (int)val.size();
    }
    s.ndr = (int)val.size();
    int8_t* p8;
    if ((rc = upload(c, &pi, ptr))) return rc;
    s.dr_ptr = pi;
    if ((rc = upload(c, &p16, col))) return rc;
    s.dr_col = p16;
    if ((rc = upload(c, &p8, axis))) return rc;
    s.dr_axis = p8;
    if ((rc = upload(c, &pf, val))) return rc;
    s.dr_valf = pf;
    return WLC_OK;
}

template <typename T> static int build_twiddles(wlc_ctx* c) {
    using C = typename cvec<T>::t;
    std::vector<C> tw(c->N);
    for (int j = 0; j < c->N; ++j) {
        const double a = 2.0 * M_PI * (double)j / (double)c->N;
        tw[j].x = (T)std::cos(a);
        tw[j].y = (T)(-std::sin(a));
    }
    C* d;
    int rc = upload(c, &d, tw);
    c->twg = d;
    return rc;
}

extern "C" int wlc_abi_version(void) { return WLC_ABI_VERSION; }

extern "C" const char* wlc_last_error(const wlc_ctx* c) { return c ? c->err.c_str() : "null context"; }

extern "C" int64_t wlc_launch_count(const wlc_ctx* c) { return c ? c->launches : 0; }

extern "C" void* wlc_stream(const wlc_ctx* c) { return c ? (void*)c->st : nullptr; }

static int validate(const wlc_params* p, std::string& why) {
    char buf[256];
    if (p->n[0] != p->n[1] || p->n[1] != p->n[2]) {
        why = "only cubic grids (SIDEx = SIDEy = SIDEz) are built";
        return WLC_E_UNSUPPORTED;
    }
    if (!supported_n(p->n[0])) {
        std::snprintf(buf, sizeof buf, "grid edge %d has no compiled kernels", p->n[0]);
        why = buf;
        return WLC_E_UNSUPPORTED;
    }
    if (p->lmax < 0 || p->lmax > kRotLmax) {
        why = "lmax must be in [0, 12] (the rotation codelets cover l <= 12)";
        return WLC_E_PARAM;
    }
    if (p->nmax < 3) {
        why = "nmax must be >= 3";
        return WLC_E_PARAM;
    }
    int sum = 0;
    for (int b = 0; b < 3; ++b) {
        if (p->ns[b] < 0 || (p->ns[b] % 2) != 0) {
            std::snprintf(buf, sizeof buf, "block lengths must be even and >= 0 (NA,NB,NC = %d,%d,%d)", p->ns[0],
                          p->ns[1], p->ns[2]);
            why = buf;
            return WLC_E_PARAM;
        }
        sum += p->ns[b];
        if (!(p->kappa[b] > 0)) {
            why = "kappa must be > 0";
            return WLC_E_PARAM;
        }
        if (!(p->dx[b] > 0)) {
            why = "grid spacing must be > 0";
            return WLC_E_PARAM;
        }
    }
    if (sum != p->nmax) {
        why = "NA + NB + NC must equal nmax";
        return WLC_E_PARAM;
    }
    if (p->precision != WLC_FP64 && p->precision != WLC_FP32) {
        why = "precision must be WLC_FP64 or WLC_FP32";
        return WLC_E_PARAM;
    }
    if (p->literals != WLC_LIT_REAL4 && p->literals != WLC_LIT_REAL8) {
        why = "literals must be WLC_LIT_REAL4 or WLC_LIT_REAL8";
        return WLC_E_PARAM;
    }
    if (p->store_qstar < 0 || p->store_qstar > 2) {
        why = "store_qstar must be 0, 1 or 2";
        return WLC_E_PARAM;
    }
    if (p->q_checkpoint != 0 && (p->q_checkpoint < 3 || p->q_checkpoint > p->nmax || p->store_qstar == 1)) {
        why = "q_checkpoint must be 0 or in [3, nmax], and needs store_qstar 0 or 2";
        return WLC_E_PARAM;
    }
    if (p->scheme != WLC_SCHEME_BDF && p->scheme != WLC_SCHEME_SPLIT) {
        why = "scheme must be WLC_SCHEME_BDF or WLC_SCHEME_SPLIT";
        return WLC_E_PARAM;
    }
    if (p->scheme == WLC_SCHEME_SPLIT && std::fabs(p->nmu) >= 1.0e-5) {
        why = "the split scheme has no Maier-Saupe term (nmu must be 0)";
        return WLC_E_UNSUPPORTED;
    }
    return WLC_OK;
}

static void apply_box(wlc_ctx* c) {
    for (int a = 0; a < 3; ++a) c->kf[a] = lit_kfactor(c->N, c->p.dx[a], c->real4);
    c->vol = c->p.dx[0] * c->p.dx[1] * c->p.dx[2] * (double)c->nr;  // SCFT_control.f90:180
}

// Inverse tridiagonal pivots for every (order, block) when the spacing is
// isotropic (|k|^2 then depends on ix^2+iy^2+iz^2 only).
template <typename T> static int build_pivots(wlc_ctx* c) {
    c->have_piv = false;
    if (!c->pivtab) return WLC_OK;
    if (!(c->kf[0] == c->kf[1] && c->kf[1] == c->kf[2])) return WLC_OK;
    const T* zoff = sizeof(T) == 8 ? (const T*)c->sd.zoff : (const T*)c->sf.zoff;
    for (int order = 1; order <= 3; ++order)
        for (int b = 0; b < 3; ++b) {
            T* out = (T*)c->pivtab + ((size_t)((order - 1) * 3 + b) * c->nkeys) * c->npiv;
            const double dcoef = c->ds * c->p.loa / (2.0 * c->p.kappa[b]);
            cudaError_t e = launch_pivot_table<T>(out, c->nkeys, c->L, lit_c0(order, c->real4), dcoef, c->ds, c->kf[0],
                                                  zoff, c->st);
            c->launches++;
            if (e != cudaSuccess) return set_err(c, WLC_E_CUDA, std::string("pivot table: ") + cudaGetErrorString(e));
        }
    if (split_scheme(c))  // I + ds/2 A per block: c0 = 1 at half the step
        for (int b = 0; b < 3; ++b) {
            T* out = (T*)c->pivtab + ((size_t)(9 + b) * c->nkeys) * c->npiv;
            const double dcoef = 0.5 * c->ds * c->p.loa / (2.0 * c->p.kappa[b]);
            cudaError_t e = launch_pivot_table<T>(out, c->nkeys, c->L, 1.0, dcoef, 0.5 * c->ds, c->kf[0], zoff, c->st);
            c->launches++;
            if (e != cudaSuccess) return set_err(c, WLC_E_CUDA, std::string("pivot table: ") + cudaGetErrorString(e));
        }
    c->have_piv = true;
    return WLC_OK;
}

template <typename T> static int alloc_fields(wlc_ctx* c) {
    using C = typename cvec<T>::t;
    const size_t sl = (size_t)c->M * c->nr;
    int rc;
    T* pt;
    C* pc;
    const size_t nqf = c->K > 0 ? (size_t)(4 + 3 * c->nck + c->K + 2) : (size_t)(c->p.nmax + 1);
    const size_t nqb = c->stream ? 4 : (size_t)(c->p.nmax + 1);
    if ((rc = dalloc(c, &pt, sizeof(T) * sl * nqf))) return rc;
    c->qf = pt;
    if ((rc = dalloc(c, &pt, sizeof(T) * sl * nqb))) return rc;
    c->qb = pt;
    if ((rc = dalloc(c, &pc, sizeof(C) * (size_t)c->nk * c->M))) return rc;
    c->phat = pc;
    if (c->st2) {  // k-space buffer of the overlapped backward sweep
        if ((rc = dalloc(c, &pc, sizeof(C) * (size_t)c->nk * c->M))) return rc;
        c->phat2 = pc;
    }
    if ((rc = dalloc(c, &pt, sizeof(T) * 15 * (size_t)c->nr))) return rc;  // cf[3][3][nr] + dsw[3][nr] + ehalf[3][nr]
    c->cf = pt;
    if ((rc = dalloc(c, &pt, sizeof(T) * sl))) return rc;
    c->work = pt;
    if (std::fabs(c->p.nmu) >= 1.0e-5) {
        if ((rc = dalloc(c, &pt, sizeof(T) * sl))) return rc;
        c->msterm = pt;
    }
    c->elem = sizeof(T);
    return WLC_OK;
}

static int check_smem(wlc_ctx* c, bool fp32) {
    const size_t sxy = fp32 ? smem_xy<float>(c->N) : smem_xy<double>(c->N);
    int ndr = 0;
    for (int a = 0; a < 3; ++a) ndr += (int)c->tab.dR[a].size();
    const bool corr = !fp32 && ndr > 0;
    const size_t ssv = solve_smem(c->N, c->M, c->L, ndr, fp32 ? 4 : 8, corr ? 1 : 0).total;
    if (ssv > 227 * 1024 || sxy > 227 * 1024)
        return set_err(c, WLC_E_UNSUPPORTED, "one coefficient column (M x N) does not fit in shared memory for "
                                             "this (N, L, precision)");
    return WLC_OK;
}

// Make precision T the active one: operator tables, twiddles and pivots of
// T (built once, pivots rebuilt after a box change), propagator buffers wide
// enough for T, coefficient planes refreshed from the fields.
template <typename T> static int use_precision(wlc_ctx* c) {
    constexpr int idx = sizeof(T) == 4 ? 1 : 0;
    int rc;
    if ((rc = check_smem(c, idx == 1))) return rc;
    auto& ps = c->prec[idx];
    if (!ps.built) {
        if constexpr (idx == 1) {
            if ((rc = build_solve_tables<float>(c, c->sf))) return rc;
        } else {
            if ((rc = build_solve_tables<double>(c, c->sd))) return rc;
        }
        if ((rc = build_twiddles<T>(c))) return rc;
        ps.twg = c->twg;
        void* pv = nullptr;
        if ((rc = dalloc(c, (unsigned char**)&pv, (size_t)pivot_tables(c) * c->nkeys * c->npiv * sizeof(T)))) return rc;
        ps.pivtab = pv;
        ps.built = true;
        ps.piv_gen = -1;
    }
    c->fp32 = idx == 1;
    c->p.precision = idx == 1 ? WLC_FP32 : WLC_FP64;
    c->twg = ps.twg;
    c->pivtab = ps.pivtab;
    if (ps.piv_gen != c->box_gen) {
        if ((rc = build_pivots<T>(c))) return rc;
        ps.have_piv = c->have_piv;
        ps.piv_gen = c->box_gen;
    } else {
        c->have_piv = ps.have_piv;
    }
    if (c->elem < sizeof(T)) {  // widen the propagator buffers
        for (void** b : {&c->qf, &c->qb, &c->phat, &c->phat2, &c->cf, &c->work, &c->msterm}) {
            if (*b) {
                for (size_t i = 0; i < c->allocs.size(); ++i)
                    if (c->allocs[i] == *b) {
                        c->allocs.erase(c->allocs.begin() + (long)i);
                        break;
                    }
                cudaFree(*b);
                *b = nullptr;
            }
        }
        if ((rc = alloc_fields<T>(c))) return rc;
    }
    if (c->have_fields) {
        launch_make_cf<T>(c->w, (T*)c->cf, c->ds, lit_third(c->real4), c->nr, c->st);
        c->launches++;
        CK(cudaGetLastError());
    }
    c->have_fwd = c->have_bwd = c->have_density = false;
    CK(mark_inputs(c));
    return WLC_OK;
}

int create_impl(const wlc_params* p, cudaStream_t ext, wlc_ctx** out) {
    if (!p || !out) return WLC_E_PARAM;
    *out = nullptr;
    wlc_ctx* c = new wlc_ctx();
    std::string why;
    int rc = validate(p, why);
    if (rc) {
        // the caller gets the code; keep the message reachable through a
        // context that only carries the error
        c->err = why;
        *out = c;
        return rc;
    }
    c->p = *p;
    c->N = p->n[0];
    c->L = p->lmax;
    c->M = (c->L + 1) * (c->L + 1);
    c->nkx = c->N / 2 + 1;
    c->nr = (int64_t)c->N * c->N * c->N;
    c->nk = (int64_t)c->nkx * c->N * c->N;
    c->fp32 = p->precision == WLC_FP32;
    c->real4 = p->literals == WLC_LIT_REAL4 ? 1 : 0;
    c->ds = 1.0 / (double)p->nmax;  // initialize_mod.f90:140
    c->nstart[0] = 0;
    c->nstart[1] = p->ns[0];
    c->nstart[2] = p->ns[0] + p->ns[1];
    c->stream = p->store_qstar != 1;
    c->K = p->q_checkpoint;
    c->nck = c->K > 0 ? p->nmax / c->K : 0;
    *out = c;
    if (!build_basis_tables(c->L, c->real4, c->tab, why)) return set_err(c, WLC_E_SELFTEST, why);
    if ((rc = check_smem(c, c->fp32))) return rc;
    CK(prepare_reduce_kernels());
    if (ext) {
        c->st = ext;
        c->own_stream = false;
    } else {
        CK(cudaStreamCreateWithFlags(&c->st, cudaStreamNonBlocking));
        if (p->store_qstar == 1 && std::fabs(p->nmu) < 1.0e-5) {  // overlapped sweeps (overlap_sweeps)
            CK(cudaStreamCreateWithFlags(&c->st2, cudaStreamNonBlocking));
            CK(cudaEventCreateWithFlags(&c->ev_inputs, cudaEventDisableTiming));
            CK(cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming));
        }
    }
    apply_box(c);
    // Theta and J lists
    {
        std::vector<int16_t> tr, tcol;
        std::vector<double> tv;
        const int M = c->M;
        for (int i = 0; i < M; ++i)
            for (int j = 0; j < M; ++j) {
                bool any = false;
                for (int a = 0; a < 5; ++a) any = any || c->tab.T[a][(size_t)i * M + j] != 0.0;
                if (!any) continue;
                tr.push_back((int16_t)i);
                tcol.push_back((int16_t)j);
                for (int a = 0; a < 5; ++a) tv.push_back(c->tab.T[a][(size_t)i * M + j]);
            }
        int16_t* p16;
        double* pd;
        if ((rc = upload(c, &p16, tr))) return rc;
        c->thl.row = p16;
        if ((rc = upload(c, &p16, tcol))) return rc;
        c->thl.col = p16;
        if ((rc = upload(c, &pd, tv))) return rc;
        c->thl.val = pd;
        c->thl.n = (int)tr.size();
        std::vector<int> rp(M + 1, 0);  // entries are emitted row by row
        for (int16_t i : tr) rp[i + 1]++;
        for (int i = 0; i < M; ++i) rp[i + 1] += rp[i];
        int* pr;
        if ((rc = upload(c, &pr, rp))) return rc;
        c->thl.rowptr = pr;
        std::vector<int> jp(6, 0);
        std::vector<int16_t> jr, jc;
        std::vector<double> jv;
        for (int a = 0; a < 5; ++a) {
            for (size_t e = 0; e < c->tab.Jsp[a].size(); ++e) {
                jr.push_back((int16_t)c->tab.Jsp[a].row[e]);
                jc.push_back((int16_t)c->tab.Jsp[a].col[e]);
                jv.push_back(c->tab.Jsp[a].val[e]);
            }
            jp[a + 1] = (int)jv.size();
        }
        int* pi;
        if ((rc = upload(c, &pi, jp))) return rc;
        c->jl.ptr = pi;
        if ((rc = upload(c, &p16, jr))) return rc;
        c->jl.row = p16;
        if ((rc = upload(c, &p16, jc))) return rc;
        c->jl.col = p16;
        if ((rc = upload(c, &pd, jv))) return rc;
        c->jl.val = pd;
        c->jl.n = (int)jv.size();
    }
    c->nkeys = 3 * (c->N / 2) * (c->N / 2) + 1;
    c->npiv = (c->L + 1) * (c->L + 2) / 2;
    if ((rc = c->fp32 ? alloc_fields<float>(c) : alloc_fields<double>(c))) return rc;
    if ((rc = c->fp32 ? use_precision<float>(c) : use_precision<double>(c))) return rc;
    const size_t nr = (size_t)c->nr;
    if ((rc = dalloc(c, &c->w, sizeof(double) * 3 * nr))) return rc;
    if ((rc = dalloc(c, &c->mop, sizeof(double) * 9 * nr))) return rc;
    if ((rc = dalloc(c, &c->raw, sizeof(double) * 3 * nr))) return rc;
    if ((rc = dalloc(c, &c->junc, sizeof(double) * 3 * nr))) return rc;
    if ((rc = dalloc(c, &c->qend, sizeof(double) * nr))) return rc;
    if ((rc = dalloc(c, &c->phi, sizeof(double) * 3 * nr))) return rc;
    if ((rc = dalloc(c, &c->part, sizeof(double) * kS3Blocks))) return rc;
    if ((rc = dalloc(c, &c->scal, sizeof(double) * 8))) return rc;
    if ((rc = dalloc(c, &c->sraw, sizeof(double) * 15 * nr))) return rc;
    if ((rc = dalloc(c, &c->srs, sizeof(double) * 15 * nr))) return rc;
    if ((rc = dalloc(c, &c->juncs, sizeof(double) * 3 * nr))) return rc;
    if ((rc = dalloc(c, &c->ar, sizeof(double) * nr))) return rc;
    if ((rc = dalloc(c, &c->stage, sizeof(double) * (size_t)c->M * nr))) return rc;
    if ((rc = dalloc(c, &c->flag, sizeof(int)))) return rc;
    CK(cudaMemsetAsync(c->mop, 0, sizeof(double) * 9 * nr, c->st));
    CK(mark_inputs(c));
    CK(cudaStreamSynchronize(c->st));
    c->err.clear();
    return WLC_OK;
}

extern "C" int wlc_create(const wlc_params* p, wlc_ctx** out) { return create_impl(p, nullptr, out); }

extern "C" int wlc_destroy(wlc_ctx* c) {
    if (!c) return WLC_OK;
    if (c->batch_owned) return set_err(c, WLC_E_STATE, "this context belongs to a batch (wlc_batch_destroy)");
    return destroy_impl(c);
}

int destroy_impl(wlc_ctx* c) {
    if (!c) return WLC_OK;
    if (c->st) cudaStreamSynchronize(c->st);
    if (c->st2) cudaStreamSynchronize(c->st2);
    for (void* p : c->allocs) cudaFree(p);
    for (auto e : c->ev) cudaEventDestroy(e);
    if (c->ev_inputs) cudaEventDestroy(c->ev_inputs);
    if (c->ev_join) cudaEventDestroy(c->ev_join);
    if (c->st2) cudaStreamDestroy(c->st2);
    if (c->st && c->own_stream) cudaStreamDestroy(c->st);
    delete c;
    return WLC_OK;
}

extern "C" int wlc_set_box(wlc_ctx* c, double dx, double dy, double dz) {
    if (!ready(c)) return WLC_E_STATE;
    if (!(dx > 0 && dy > 0 && dz > 0)) return set_err(c, WLC_E_PARAM, "grid spacing must be > 0");
    c->p.dx[0] = dx;
    c->p.dx[1] = dy;
    c->p.dx[2] = dz;
    apply_box(c);
    c->box_gen++;
    int rc = c->fp32 ? build_pivots<float>(c) : build_pivots<double>(c);
    if (rc) return rc;
    auto& ps = c->prec[c->fp32 ? 1 : 0];
    ps.have_piv = c->have_piv;
    ps.piv_gen = c->box_gen;
    c->have_fwd = c->have_bwd = c->have_density = false;
    CK(mark_inputs(c));
    return WLC_OK;
}

extern "C" int wlc_set_precision(wlc_ctx* c, int32_t precision) {
    if (!ready(c)) return WLC_E_STATE;
    if (c->batch_owned) return set_err(c, WLC_E_STATE, "batch instances stay FP32");
    if (precision != WLC_FP64 && precision != WLC_FP32)
        return set_err(c, WLC_E_PARAM, "precision must be WLC_FP64 or WLC_FP32");
    if ((precision == WLC_FP32) == c->fp32) return WLC_OK;
    return precision == WLC_FP32 ? use_precision<float>(c) : use_precision<double>(c);
}

extern "C" int wlc_set_fields(wlc_ctx* c, const double* w, const double* m_op) {
    if (!ready(c)) return WLC_E_STATE;
    if (!w) return set_err(c, WLC_E_PARAM, "w is null");
    const size_t nr = (size_t)c->nr;
    CK(cudaMemcpyAsync(c->w, w, sizeof(double) * 3 * nr, cudaMemcpyHostToDevice, c->st));
    if (m_op) {
        CK(cudaMemcpyAsync(c->mop, m_op, sizeof(double) * 9 * nr, cudaMemcpyHostToDevice, c->st));
        c->have_mop = true;
    } else {
        CK(cudaMemsetAsync(c->mop, 0, sizeof(double) * 9 * nr, c->st));
        c->have_mop = false;
    }
    // one launch covers the three blocks: cf[blk][3][nr] from w[blk][nr]
    const double third = lit_third(c->real4);
    if (c->fp32)
        launch_make_cf<float>(c->w, (float*)c->cf, c->ds, third, c->nr, c->st);
    else
        launch_make_cf<double>(c->w, (double*)c->cf, c->ds, third, c->nr, c->st);
    c->launches++;
    CK(cudaGetLastError());
    c->have_fields = true;
    c->have_fwd = c->have_bwd = c->have_density = false;
    CK(mark_inputs(c));
    return WLC_OK;
}

template <typename T> static int run_step(wlc_ctx* c, StepLaunch<T>& L, double c0, int slot) {
    L.solve.c0 = c0;
    L.events = (c->timing && slot >= 0) ? &c->ev[4 * (size_t)slot] : nullptr;
    cudaError_t e = launch_step<T>(c->N, L, c->st);
    c->launches += 3;
    if (e != cudaSuccess) return set_err(c, WLC_E_CUDA, std::string("step launch: ") + cudaGetErrorString(e));
    return WLC_OK;
}

// one contour step of either sweep: out = G^-1 . RHS(h1, h2, h3)
template <typename T>
static int contour_step(wlc_ctx* c, StepKind k, const T* h1, const T* h2, const T* h3, T* out, int slot) {
    StepLaunch<T> L = make_launch<T>(c, k, h1, h2, h3, out);
    if (std::fabs(c->p.nmu) >= 1.0e-5 && c->have_mop) {
        launch_ms_term<T>(h1, h2, h3, k.order, c->mop, c->thl, c->ds, lit_thresh(c->real4), c->M, c->nr,
                          (T*)c->msterm, c->st);
        c->launches++;
        L.step.msterm = (const T*)c->msterm;
    }
    return run_step<T>(c, L, step_c0(c, k.order), slot);
}

// recompute q over segment m (slices mK+1 .. min(mK+K-1, Nmax)) into the
// segment buffer from the stored BDF3 history at mK (bit-identical to the
// forward sweep: same kernels, same inputs)
template <typename T> static int recompute_segment(wlc_ctx* c, int m) {
    const size_t sl = (size_t)c->M * c->nr;
    const int base = m * c->K, top = std::min(base + c->K - 1, c->p.nmax);
    if (m == 0) {
        launch_set_delta<T>(qf_seg<T>(c, 2), c->M, c->nr, c->st);
        c->launches++;
    } else {
        CK(cudaMemcpyAsync(qf_seg<T>(c, 0), qf_ckpt<T>(c, m, 0), sizeof(T) * sl * 3, cudaMemcpyDeviceToDevice,
                           c->st));
    }
    for (int s = base + 1; s <= top; ++s) {
        const StepKind k = fwd_kind(c, s);
        const int nh = hist_slices(k.order);
        const int i = s - base + 2;
        int rc = contour_step<T>(c, k, qf_seg<T>(c, i - 1), nh >= 2 ? qf_seg<T>(c, i - 2) : nullptr,
                                 nh >= 3 ? qf_seg<T>(c, i - 3) : nullptr, qf_seg<T>(c, i), -1);
        if (rc) return rc;
    }
    return WLC_OK;
}

template <typename T> static int sweep(wlc_ctx* c, int dir) {
    const size_t sl = (size_t)c->M * c->nr;
    const int nmax = c->p.nmax;
    if (c->timing && c->ev.size() < 4 * (size_t)(nmax + 1)) {
        for (auto e : c->ev) cudaEventDestroy(e);
        c->ev.assign(4 * (size_t)(nmax + 1), nullptr);
        for (auto& e : c->ev) CK(cudaEventCreate(&e));
    }
    int rc;
    if (dir > 0) {
        // forward: all slices, or a ring with the BDF3 history copied out at
        // every K-th slice
        auto at = [&](int s) -> T* { return c->K ? qf_ring<T>(c, s) : (T*)c->qf + (size_t)s * sl; };
        launch_set_delta<T>(at(0), c->M, c->nr, c->st);  // q(0) = delta_i0
        c->launches++;
        for (int s = 1; s <= nmax; ++s) {
            const StepKind k = fwd_kind(c, s);
            const int nh = hist_slices(k.order);
            if ((rc = contour_step<T>(c, k, at(s - 1), nh >= 2 ? at(s - 2) : nullptr, nh >= 3 ? at(s - 3) : nullptr,
                                      at(s), s)))
                return rc;
            if (c->K) {
                const int m = (s + 2) / c->K, j = s + 2 - m * c->K;
                if (m >= 1 && j <= 2 && m * c->K <= nmax)
                    CK(cudaMemcpyAsync(qf_ckpt<T>(c, m, j), at(s), sizeof(T) * sl, cudaMemcpyDeviceToDevice, c->st));
            }
        }
    } else {
        const DensityArgs d = density_args(c);
        const int want_s = stream_s(c) ? 1 : 0;
        if (c->stream) {
            CK(cudaMemsetAsync(c->raw, 0, sizeof(double) * 3 * (size_t)c->nr, c->st));
            if (want_s) CK(cudaMemsetAsync(c->sraw, 0, sizeof(double) * 15 * (size_t)c->nr, c->st));
            if (c->K && (rc = recompute_segment<T>(c, nmax / c->K))) return rc;
        }
        auto slice = [&](int s) -> int {  // streamed density contribution of slice s
            if (!c->stream) return WLC_OK;
            launch_density_slice<T>(qf_at<T>(c, s), qb_at<T>(c, s), d, s, want_s, c->jl, c->raw, c->junc, c->qend,
                                    c->sraw, c->st);
            c->launches++;
            return WLC_OK;
        };
        launch_set_delta<T>(qb_at<T>(c, nmax), c->M, c->nr, c->st);  // q*(Nmax) = delta_i0
        c->launches++;
        slice(nmax);
        for (int n = 1; n <= nmax; ++n) {
            const int s = nmax - n;
            const StepKind k = bwd_kind(c, s);
            const int nh = hist_slices(k.order);
            if ((rc = contour_step<T>(c, k, qb_at<T>(c, s + 1), nh >= 2 ? qb_at<T>(c, s + 2) : nullptr,
                                      nh >= 3 ? qb_at<T>(c, s + 3) : nullptr, qb_at<T>(c, s), n)))
                return rc;
            if (c->K && (s + 1) % c->K == 0 && (rc = recompute_segment<T>(c, s / c->K))) return rc;
            slice(s);
        }
    }
    CK(cudaGetLastError());
    if (c->timing) {
        CK(cudaStreamSynchronize(c->st));
        for (int q2 = 0; q2 < 4; ++q2) c->tms[q2] = 0.0;
        for (int n = 1; n <= nmax; ++n) {
            float t;
            for (int q2 = 0; q2 < 3; ++q2) {
                CK(cudaEventElapsedTime(&t, c->ev[4 * n + q2], c->ev[4 * n + q2 + 1]));
                c->tms[q2] += t;
            }
            CK(cudaEventElapsedTime(&t, c->ev[4 * n], c->ev[4 * n + 3]));
            c->tms[3] += t;
        }
    }
    return WLC_OK;
}

extern "C" int wlc_propagate(wlc_ctx* c, int32_t dir) {
    if (!ready(c)) return WLC_E_STATE;
    if (dir != 1 && dir != -1) return set_err(c, WLC_E_PARAM, "dir must be +1 or -1");
    if (!c->have_fields) return set_err(c, WLC_E_STATE, "wlc_set_fields must be called before wlc_propagate");
    if (dir < 0 && c->stream && !c->have_fwd)
        return set_err(c, WLC_E_STATE, "with streamed densities (store_qstar 0/2) the forward sweep must come first");
    int rc;
    if (dir < 0 && overlap_sweeps(c)) {
        // q* does not read q: run the backward sweep on the second stream
        // with its own k-space buffer, after the inputs and overlapping the
        // forward sweep; the context stream waits for it before anything else
        CK(cudaStreamWaitEvent(c->st2, c->ev_inputs, 0));
        std::swap(c->st, c->st2);
        std::swap(c->phat, c->phat2);
        rc = c->fp32 ? sweep<float>(c, dir) : sweep<double>(c, dir);
        std::swap(c->st, c->st2);
        std::swap(c->phat, c->phat2);
        if (rc) return rc;
        CK(cudaEventRecord(c->ev_join, c->st2));
        CK(cudaStreamWaitEvent(c->st, c->ev_join, 0));
    } else {
        rc = c->fp32 ? sweep<float>(c, dir) : sweep<double>(c, dir);
        if (rc) return rc;
    }
    if (dir > 0)
        c->have_fwd = true;
    else
        c->have_bwd = true;
    c->have_density = false;
    return WLC_OK;
}

extern "C" int wlc_enable_timing(wlc_ctx* c, int32_t on) {
    if (!ready(c)) return WLC_E_STATE;
    c->timing = on != 0;
    return WLC_OK;
}

extern "C" int wlc_last_timing(const wlc_ctx* c, double* ms4) {
    if (!c || !ms4) return WLC_E_PARAM;
    for (int q = 0; q < 4; ++q) ms4[q] = c->tms[q];
    return WLC_OK;
}

template <typename T> static void density_launch(wlc_ctx* c, const DensityArgs& d) {
    launch_density<T>((const T*)c->qf, (const T*)c->qb, d, c->raw, c->junc, c->qend, c->st);
}
template <typename T> static void stensor_launch(wlc_ctx* c, const DensityArgs& d) {
    launch_stensor<T>((const T*)c->qf, (const T*)c->qb, d, c->jl, c->sraw, c->st);
}

extern "C" int wlc_density(wlc_ctx* c, double* phi, double* junc, double* s_op, double* lnq) {
    if (!ready(c)) return WLC_E_STATE;
    if (!c->have_fwd || !c->have_bwd)
        return set_err(c, WLC_E_STATE, "both sweeps (wlc_propagate +1 and -1) must precede wlc_density");
    const size_t nr = (size_t)c->nr;
    if (s_op && c->stream && !stream_s(c))
        return set_err(c, WLC_E_STATE, "the orientation tensor is not accumulated with store_qstar = 0 (use 2)");
    const DensityArgs d = density_args(c);
    S3Args s3;
    for (int a = 0; a < 3; ++a) {
        s3.n[a] = c->N;
        s3.d[a] = c->p.dx[a];
    }
    if (!c->stream) {  // streamed densities were accumulated by the backward sweep
        if (c->fp32)
            density_launch<float>(c, d);
        else
            density_launch<double>(c, d);
    }
    launch_s3(c->qend, 1, 0, s3, c->part, c->scal + 0, c->st);          // S3(q_0(Nmax))
    launch_s3(c->raw, 3, (int64_t)nr, s3, c->part, c->scal + 1, c->st);  // totden
    CK(cudaMemcpyAsync(c->phi, c->raw, sizeof(double) * 3 * nr, cudaMemcpyDeviceToDevice, c->st));
    launch_scale(c->phi, 3 * (int64_t)nr, c->scal + 1, c->vol, c->st);
    CK(cudaMemcpyAsync(c->juncs, c->junc, sizeof(double) * 3 * nr, cudaMemcpyDeviceToDevice, c->st));
    launch_scale(c->juncs, 3 * (int64_t)nr, c->scal + 1, c->vol, c->st);
    c->launches += 7;
    double hs[2];
    CK(cudaMemcpyAsync(hs, c->scal, sizeof(double) * 2, cudaMemcpyDeviceToHost, c->st));
    CK(cudaMemsetAsync(c->flag, 0, sizeof(int), c->st));
    launch_nonfinite(c->phi, 3 * (int64_t)nr, c->flag, c->st);
    c->launches++;
    int hflag = 0;
    CK(cudaMemcpyAsync(&hflag, c->flag, sizeof(int), cudaMemcpyDeviceToHost, c->st));
    if (phi) CK(cudaMemcpyAsync(phi, c->phi, sizeof(double) * 3 * nr, cudaMemcpyDeviceToHost, c->st));
    if (junc) CK(cudaMemcpyAsync(junc, c->juncs, sizeof(double) * 3 * nr, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    c->totden = hs[1];
    c->lnq = std::log(hs[0] / c->vol);  // pff_global = ln[(1/V) S3(q_0)], SCFT_Density_FE_ABC.f90:82-92
    if (lnq) *lnq = c->lnq;
    if (hflag || !std::isfinite(c->lnq) || !std::isfinite(c->totden))
        return set_err(c, WLC_E_NONFINITE, "non-finite density or partition function");
    if (s_op || ms_on(c)) {  // the Maier-Saupe update needs S on the device
        if (!c->stream) {
            if (c->fp32)
                stensor_launch<float>(c, d);
            else
                stensor_launch<double>(c, d);
            c->launches++;
        }
        CK(cudaMemcpyAsync(c->srs, c->sraw, sizeof(double) * 15 * nr, cudaMemcpyDeviceToDevice, c->st));
        launch_scale(c->srs, 15 * (int64_t)nr, c->scal + 1, c->vol, c->st);
        c->launches++;
    }
    if (s_op) {
        std::vector<double> h(15 * nr);
        CK(cudaMemcpyAsync(h.data(), c->srs, sizeof(double) * 15 * nr, cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        // S_OP_blk(r, a, b, blk) at s_op[r + nr*(a + 3b + 9 blk)]; S_zz = -S_xx - S_yy
        for (int b = 0; b < 3; ++b)
            for (size_t r = 0; r < nr; ++r) {
                const double* t = h.data() + (size_t)b * 5 * nr + r;
                const double sxx = t[0], syy = t[nr], sxy = t[2 * nr], sxz = t[3 * nr], syz = t[4 * nr];
                const double S[9] = {sxx, sxy, sxz, sxy, syy, syz, sxz, syz, -(sxx + syy)};
                for (int q = 0; q < 9; ++q) s_op[r + nr * (q + 9 * (size_t)b)] = S[q];
            }
    }
    c->have_density = true;
    return WLC_OK;
}

extern "C" int wlc_free_energy(wlc_ctx* c, double* fe) {
    if (!ready(c)) return WLC_E_STATE;
    if (!fe) return set_err(c, WLC_E_PARAM, "fe is null");
    if (!c->have_density) return set_err(c, WLC_E_STATE, "wlc_density must precede wlc_free_energy");
    FeArgs f;
    f.nr = c->nr;
    for (int a = 0; a < 3; ++a) f.chi[a] = c->p.chi[a];
    f.nmu = c->p.nmu;
    f.ms = (std::fabs(c->p.nmu) >= 1.0e-5 && c->have_mop) ? 1 : 0;
    S3Args s3;
    for (int a = 0; a < 3; ++a) {
        s3.n[a] = c->N;
        s3.d[a] = c->p.dx[a];
    }
    launch_fe(c->phi, c->w, c->mop, f, c->ar, c->st);
    launch_s3(c->ar, 1, 0, s3, c->part, c->scal + 2, c->st);
    c->launches += 3;
    double h = 0;
    CK(cudaMemcpyAsync(&h, c->scal + 2, sizeof(double), cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    *fe = -c->lnq + h / c->vol;  // FE_global = -pff_global + tempEE_global
    if (!std::isfinite(*fe)) return set_err(c, WLC_E_NONFINITE, "non-finite free energy");
    return WLC_OK;
}

template <typename T> static int get_q(wlc_ctx* c, int dir, int s, double* out) {
    const size_t sl = (size_t)c->M * c->nr;
    const T* q = (const T*)(dir > 0 ? c->qf : c->qb) + (size_t)s * sl;
    launch_to_reference<T>(q, c->stage, c->M, c->nr, c->st);
    c->launches++;
    CK(cudaMemcpyAsync(out, c->stage, sizeof(double) * sl, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return WLC_OK;
}

template <typename T> static int set_q(wlc_ctx* c, int dir, int s, const double* in) {
    const size_t sl = (size_t)c->M * c->nr;
    T* q = (T*)(dir > 0 ? c->qf : c->qb) + (size_t)s * sl;
    CK(cudaMemcpyAsync(c->stage, in, sizeof(double) * sl, cudaMemcpyHostToDevice, c->st));
    launch_to_internal<T>(c->stage, q, c->M, c->nr, c->st);
    c->launches++;
    CK(cudaStreamSynchronize(c->st));
    return WLC_OK;
}

extern "C" int wlc_get_q(wlc_ctx* c, int32_t dir, int32_t s, double* out) {
    if (!ready(c)) return WLC_E_STATE;
    if ((dir != 1 && dir != -1) || s < 0 || s > c->p.nmax || !out)
        return set_err(c, WLC_E_PARAM, "wlc_get_q: bad dir / s / out");
    if ((dir > 0 && c->K) || (dir < 0 && c->stream))
        return set_err(c, WLC_E_STATE, "that propagator is not stored (store_qstar / q_checkpoint)");
    return c->fp32 ? get_q<float>(c, dir, s, out) : get_q<double>(c, dir, s, out);
}

extern "C" int wlc_set_q(wlc_ctx* c, int32_t dir, int32_t s, const double* in) {
    if (!ready(c)) return WLC_E_STATE;
    if ((dir != 1 && dir != -1) || s < 0 || s > c->p.nmax || !in)
        return set_err(c, WLC_E_PARAM, "wlc_set_q: bad dir / s / in");
    if ((dir > 0 && c->K) || (dir < 0 && c->stream))
        return set_err(c, WLC_E_STATE, "that propagator is not stored (store_qstar / q_checkpoint)");
    const int rc = c->fp32 ? set_q<float>(c, dir, s, in) : set_q<double>(c, dir, s, in);
    if (rc) return rc;
    CK(mark_inputs(c));
    return WLC_OK;
}

template <typename T> static int init_pr_impl(wlc_ctx* c, int dir, int s, double* pr) {
    const size_t sl = (size_t)c->M * c->nr;
    T* q = (T*)(dir > 0 ? c->qf : c->qb);
    const int n = dir > 0 ? s : c->p.nmax - s;
    const int order = n < 3 ? n : 3;
    StepKind k{order, dir, dir > 0 ? blk_fwd(c, s) : blk_bwd(c, s)};
    const T* h1 = q + (size_t)(s - dir) * sl;
    const T* h2 = order >= 2 ? q + (size_t)(s - 2 * dir) * sl : nullptr;
    const T* h3 = order >= 3 ? q + (size_t)(s - 3 * dir) * sl : nullptr;
    StepLaunch<T> L = make_launch<T>(c, k, h1, h2, h3, (T*)c->work);
    if (std::fabs(c->p.nmu) >= 1.0e-5 && c->have_mop) {
        launch_ms_term<T>(h1, h2, h3, order, c->mop, c->thl, c->ds, lit_thresh(c->real4), c->M, c->nr, (T*)c->msterm,
                          c->st);
        c->launches++;
        L.step.msterm = (const T*)c->msterm;
    }
    cudaError_t e = launch_rhs_only<T>(c->N, L.step, (T*)c->work, c->st);
    c->launches++;
    if (e != cudaSuccess) return set_err(c, WLC_E_CUDA, cudaGetErrorString(e));
    launch_to_reference<T>((const T*)c->work, c->stage, c->M, c->nr, c->st);
    c->launches++;
    CK(cudaMemcpyAsync(pr, c->stage, sizeof(double) * sl, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return WLC_OK;
}

extern "C" int wlc_init_pr(wlc_ctx* c, int32_t dir, int32_t s, double* pr) {
    if (!ready(c)) return WLC_E_STATE;
    if (!pr || (dir != 1 && dir != -1)) return set_err(c, WLC_E_PARAM, "wlc_init_pr: bad dir / pr");
    if ((dir > 0 && (s < 1 || s > c->p.nmax)) || (dir < 0 && (s < 0 || s > c->p.nmax - 1)))
        return set_err(c, WLC_E_PARAM, "wlc_init_pr: s out of range");
    if (!c->have_fields) return set_err(c, WLC_E_STATE, "wlc_set_fields must precede wlc_init_pr");
    if ((dir > 0 && c->K) || (dir < 0 && c->stream))
        return set_err(c, WLC_E_STATE, "that propagator is not stored (store_qstar / q_checkpoint)");
    if (split_scheme(c))
        return set_err(c, WLC_E_UNSUPPORTED, "wlc_init_pr is the BDF right-hand side; this context runs the split scheme");
    return c->fp32 ? init_pr_impl<float>(c, dir, s, pr) : init_pr_impl<double>(c, dir, s, pr);
}

// ABC G_index table, Gmatrix_mod-old.f90:446-518
static bool g_index_kind(int g, StepKind& k) {
    static const StepKind tab[10] = {{1, 1, 0}, {2, 1, 0}, {3, 1, 0}, {3, 1, 1}, {3, 1, 2},
                                     {3, -1, 0}, {3, -1, 1}, {3, -1, 2}, {2, -1, 2}, {1, -1, 2}};
    if (g < 1 || g > 10) return false;
    k = tab[g - 1];
    return true;
}

template <typename T> static int one_step_impl(wlc_ctx* c, StepKind k, const double* pr, double* qout) {
    const size_t sl = (size_t)c->M * c->nr;
    CK(cudaMemcpyAsync(c->stage, pr, sizeof(double) * sl, cudaMemcpyHostToDevice, c->st));
    launch_to_internal<T>(c->stage, (T*)c->work, c->M, c->nr, c->st);
    c->launches++;
    // the solve uses the BDF order of G_index; the right-hand side is given
    StepLaunch<T> L = make_launch<T>(c, k, (const T*)c->work, nullptr, nullptr, (T*)c->work);
    L.step.order = 0;
    int rc = run_step<T>(c, L, lit_c0(k.order, c->real4), 0);
    if (rc) return rc;
    launch_to_reference<T>((const T*)c->work, c->stage, c->M, c->nr, c->st);
    c->launches++;
    CK(cudaMemcpyAsync(qout, c->stage, sizeof(double) * sl, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return WLC_OK;
}

extern "C" int wlc_mde_one_step(wlc_ctx* c, int32_t g_index, const double* pr, double* q_out) {
    if (!ready(c)) return WLC_E_STATE;
    StepKind k;
    if (!g_index_kind(g_index, k)) return set_err(c, WLC_E_PARAM, "G_index must be in 1..10");
    if (!pr || !q_out) return set_err(c, WLC_E_PARAM, "null pr / q_out");
    if (c->timing && c->ev.size() < 4) {
        c->ev.assign(4, nullptr);
        for (auto& e : c->ev) CK(cudaEventCreate(&e));
    }
    return c->fp32 ? one_step_impl<float>(c, k, pr, q_out) : one_step_impl<double>(c, k, pr, q_out);
}

// ------------------------------------------------------------ field update
static int anderson_index(int i, int nr) {  // Anderson_index, SCFT_iterate.f90:1-25
    int a = i % (nr + 1);
    if (i < 0) {
        a = nr + 1 + a;
        if (a == nr + 1) a = 0;
    }
    return a;
}

static void dfree(wlc_ctx* c, void* p) {
    if (!p) return;
    for (size_t i = 0; i < c->allocs.size(); ++i)
        if (c->allocs[i] == p) {
            c->allocs.erase(c->allocs.begin() + (long)i);
            break;
        }
    cudaFree(p);
}

extern "C" int wlc_reset_mixing(wlc_ctx* c) {
    if (!ready(c)) return WLC_E_STATE;
    c->mix_iter = 0;
    return WLC_OK;
}

extern "C" int wlc_get_fields(wlc_ctx* c, double* w) {
    if (!ready(c)) return WLC_E_STATE;
    if (!w) return set_err(c, WLC_E_PARAM, "w is null");
    if (!c->have_fields) return set_err(c, WLC_E_STATE, "wlc_set_fields must come first");
    CK(cudaMemcpyAsync(w, c->w, sizeof(double) * 3 * (size_t)c->nr, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return WLC_OK;
}

extern "C" int wlc_get_mop(wlc_ctx* c, double* m_op) {
    if (!ready(c)) return WLC_E_STATE;
    if (!m_op) return set_err(c, WLC_E_PARAM, "m_op is null");
    CK(cudaMemcpyAsync(m_op, c->mop, sizeof(double) * 9 * (size_t)c->nr, cudaMemcpyDeviceToHost, c->st));
    CK(cudaStreamSynchronize(c->st));
    return WLC_OK;
}

extern "C" int wlc_iterate(wlc_ctx* c, const wlc_mix_params* mp, double* err, int32_t* converged) {
    if (!ready(c)) return WLC_E_STATE;
    if (!mp || !err || !converged) return set_err(c, WLC_E_PARAM, "null argument");
    if (!c->have_density) return set_err(c, WLC_E_STATE, "wlc_density must precede wlc_iterate");
    const int depth = mp->anderson_depth;
    if (depth < 1 || depth > kMaxAnderson) return set_err(c, WLC_E_PARAM, "anderson_depth must be in 1..10");
    if (mp->num_simple < 1) return set_err(c, WLC_E_PARAM, "num_simple must be >= 1");
    if (ms_on(c) && !(mp->lambda_m > 0.0)) return set_err(c, WLC_E_PARAM, "lambda_m must be > 0 when nmu != 0");
    const int64_t nr = c->nr;
    const size_t slot = 3 * (size_t)nr;
    int rc;
    if (c->mix_depth != depth) {  // (re)allocate the history; a depth change restarts the mixing
        dfree(c, c->wout_hist);
        dfree(c, c->dw_hist);
        c->wout_hist = c->dw_hist = nullptr;
        c->mix_depth = -1;
        double* p;
        if ((rc = dalloc(c, &p, sizeof(double) * slot * (depth + 1)))) return rc;
        c->wout_hist = p;
        if ((rc = dalloc(c, &p, sizeof(double) * slot * (depth + 1)))) return rc;
        c->dw_hist = p;
        if (!c->mixbuf) {
            if ((rc = dalloc(c, &p, sizeof(double) * ((4 + kMaxMixAcc) * kMixBlocks + 256)))) return rc;
            c->mixbuf = p;
        }
        c->mix_depth = depth;
        c->mix_iter = 0;
    }
    double* maxpart = c->mixbuf;                    // [4][kMixBlocks]
    double* dotpart = c->mixbuf + 4 * kMixBlocks;   // [kMaxMixAcc][kMixBlocks]
    double* res = dotpart + kMaxMixAcc * kMixBlocks;  // 0..3 maxima, 8.. Anderson sums, 160.. coefficients
    const int n = ++c->mix_iter;
    const int ns = mp->num_simple;
    const int k = n <= ns ? 0 : (n - ns) % (depth + 1);
    double* wout = c->wout_hist + (size_t)k * slot;
    double* dw = c->dw_hist + (size_t)k * slot;
    MixChi chi;
    chi.c[0][0] = chi.c[1][1] = chi.c[2][2] = 0.0;
    chi.c[0][1] = chi.c[1][0] = c->p.chi[0];  // AB
    chi.c[0][2] = chi.c[2][0] = c->p.chi[1];  // AC
    chi.c[1][2] = chi.c[2][1] = c->p.chi[2];  // BC
    for (int J = 0; J < 3; ++J) chi.f[J] = (double)c->p.ns[J] / (double)c->p.nmax;
    chi.fsum = 0.0;
    for (int K = 0; K < 3; ++K) {
        chi.cf[K] = chi.c[K][0] * chi.f[0] + chi.c[K][1] * chi.f[1] + chi.c[K][2] * chi.f[2];
        chi.fsum += chi.cf[K];
    }
    double h[96];
    if (n <= ns) {  // simple mixing; the last one also fills history slot 0 (SCFT_iterate.f90:167-197)
        launch_mix_out(c->phi, c->w, chi, nr, n == ns ? kMixSimpleStore : kMixSimple, mp->lambda_simple, wout, dw,
                       maxpart, res, c->st);
        c->launches += 2;
        CK(cudaMemcpyAsync(h, res, sizeof(double) * 4, cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        for (int q = 0; q < 4; ++q) err[q] = h[q];
    } else {  // Anderson mixing (SCFT_iterate.f90:200-331)
        launch_mix_out(c->phi, c->w, chi, nr, kMixStore, 0.0, wout, dw, maxpart, res, c->st);
        const int nrt = std::min(n - ns, depth);
        int km[kMaxAnderson];
        AndersonSlots sl;
        sl.dwk = dw;
        sl.woutk = wout;
        for (int m = 1; m <= nrt; ++m) {
            km[m - 1] = anderson_index(k - m, depth);
            sl.dwm[m - 1] = c->dw_hist + (size_t)km[m - 1] * slot;
        }
        for (int m = nrt; m < kMaxAnderson; ++m) sl.dwm[m] = dw;
        MixGrid g;
        for (int a = 0; a < 3; ++a) {
            g.n[a] = c->N;
            g.d[a] = c->p.dx[a];
        }
        const int nacc = anderson_acc_count(nrt);
        launch_anderson_dots(sl, nrt, g, nr, c->vol, dotpart, res + 8, c->st);
        launch_anderson(res + 8, nrt, res + 160, c->w, c->wout_hist, c->dw_hist, (int64_t)slot, k, km,
                        mp->lambda_anderson, (int64_t)slot, c->st);
        c->launches += 6;
        CK(cudaMemcpyAsync(h, res, sizeof(double) * (8 + nacc), cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        const double* nrm = h + 8 + (nacc - 6);
        for (int K = 0; K < 3; ++K) err[K] = nrm[2 * K + 1] != 0.0 ? std::sqrt(std::fabs(nrm[2 * K] / nrm[2 * K + 1])) : 0.0;
        err[3] = h[3];
    }
    // Maier-Saupe tensor: simple mixing towards NMu S (SCFT_iterate.f90:351-372;
    // the reference's Anderson branch for M starts after Num_simple_mixing_M
    // = 5000 iterations, beyond MAXITS, and never runs)
    err[4] = 0.0;
    if (ms_on(c)) {
        launch_mix_m(c->mop, c->srs, c->p.nmu, mp->lambda_m, nr, maxpart, res + 4, c->st);
        c->launches += 2;
        CK(cudaMemcpyAsync(&err[4], res + 4, sizeof(double), cudaMemcpyDeviceToHost, c->st));
        CK(cudaStreamSynchronize(c->st));
        c->have_mop = true;
    }
    // the fields changed: refresh the BDF3 coefficient planes
    const double third = lit_third(c->real4);
    if (c->fp32)
        launch_make_cf<float>(c->w, (float*)c->cf, c->ds, third, c->nr, c->st);
    else
        launch_make_cf<double>(c->w, (double*)c->cf, c->ds, third, c->nr, c->st);
    c->launches++;
    CK(cudaGetLastError());
    CK(mark_inputs(c));
    // convergence test (SCFT_iterate.f90:1124-1160) and the minimum iteration
    // count of the driver loop (SCFT_control.f90:270-272)
    const bool strict = err[0] < mp->tol && err[1] < mp->tol && err[2] < mp->tol &&
                        (!ms_on(c) || err[4] < 5.0 * mp->tol);
    const bool relaxed = c->p.nmu == 0.0 && mp->relax_iter > 0 && n >= mp->relax_iter && err[0] < mp->relax_tol &&
                         err[1] < mp->relax_tol && err[2] < mp->relax_tol;
    *converged = ((strict || relaxed) && n >= mp->min_iter) ? 1 : 0;
    c->have_fwd = c->have_bwd = c->have_density = false;
    return WLC_OK;
}

// ------------------------------------------------------------ launch autotuning
// Candidate launch configurations give bit-identical results (the solve
// split only changes which thread owns which degree block / m system, and
// both pass-A variants compute the same sums), so the tuner times them on
// the instance's own data and keeps the fastest.
template <typename T> static int autotune_impl(wlc_ctx* c) {
    int rc;
    if (!c->have_fwd && (rc = sweep<T>(c, 1))) return rc;
    c->have_fwd = true;
    // re-run the last forward step (same inputs, same output) per candidate
    const size_t sl = (size_t)c->M * c->nr;
    const int s = c->p.nmax;
    auto at = [&](int q) -> T* { return c->K ? qf_ring<T>(c, q) : (T*)c->qf + (size_t)q * sl; };
    const StepKind k = fwd_kind(c, s);
    float best = 1e30f;
    int best_a = c->a_variant, best_t = c->solve_threads, best_x = c->xy_threads, best_z = c->xy_z;
    const bool ms = std::fabs(c->p.nmu) >= 1.0e-5 && c->have_mop;
    for (int xz : {0, 1, 2, 3})
    for (int xt : {256, 512})
    for (int av : {1, 2}) {
        if (av == 2 && sizeof(T) != 4) continue;
        for (int th : solve_thread_candidates(c->N)) {
            c->a_variant = av;
            c->solve_threads = th;
            c->xy_threads = xt;
            c->xy_z = xz;
            StepLaunch<T> L = make_launch<T>(c, k, at(s - 1), at(s - 2), at(s - 3), at(s));
            if (ms) {  // the Theta term of this step (the buffer holds the last step of the last sweep)
                launch_ms_term<T>(at(s - 1), at(s - 2), at(s - 3), 3, c->mop, c->thl, c->ds, lit_thresh(c->real4),
                                  c->M, c->nr, (T*)c->msterm, c->st);
                L.step.msterm = (const T*)c->msterm;
            }
            L.solve.c0 = step_c0(c, k.order);
            const float ms_t = time_ms(c->st, [&] { launch_step<T>(c->N, L, c->st); }, 3);
            CK(cudaGetLastError());
            if (ms_t < best) {
                best = ms_t;
                best_a = av;
                best_t = th;
                best_x = xt;
                best_z = xz;
            }
        }
    }
    c->a_variant = best_a;
    c->solve_threads = best_t;
    c->xy_threads = best_x;
    c->xy_z = best_z;
    return WLC_OK;
}

extern "C" int wlc_autotune(wlc_ctx* c, int32_t* config) {
    if (!ready(c)) return WLC_E_STATE;
    if (!c->have_fields) return set_err(c, WLC_E_STATE, "wlc_set_fields must precede wlc_autotune");
    int rc = c->fp32 ? autotune_impl<float>(c) : autotune_impl<double>(c);
    if (rc) return rc;
    if (config) {
        config[0] = c->a_variant;
        config[1] = c->solve_threads;
        config[2] = c->xy_threads;
        config[3] = c->xy_z;
    }
    return WLC_OK;
}

extern "C" int wlc_set_launch_config(wlc_ctx* c, int32_t a_variant, int32_t solve_threads, int32_t xy_threads,
                                     int32_t xy_variant) {
    if (!ready(c)) return WLC_E_STATE;
    if (a_variant < 0 || a_variant > 2 || solve_threads < 0 || solve_threads > kSolveThreads ||
        (xy_threads != 0 && xy_threads != 256 && xy_threads != 512) || xy_variant < 0 || xy_variant > 3)
        return set_err(c, WLC_E_PARAM,
                       "a_variant must be 0..2, solve_threads 0..256, xy_threads 0, 256 or 512, xy_variant 0..3");
    c->xy_z = xy_variant;
    c->a_variant = a_variant;
    c->solve_threads = solve_threads;
    c->xy_threads = xy_threads;
    return WLC_OK;
}
