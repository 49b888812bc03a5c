// wlc_noalloc.cu -- one FP64 contour step (the work of wlc_mde_one_step)
// for callers that cannot allocate device memory.
//
// Who needs it: code that runs where cudaMalloc is unavailable or
// forbidden -- inside a host callback or a driver-level plugin that only
// receives device pointers from its framework, under a memory pool that
// must not grow, or in a process that has handed all memory to another
// allocator.  Those callers own their input and output buffers but cannot
// ask for the k-space scratch or the operator tables that wlc_create
// allocates.
//
// How: the scratch lives in one file-scope __device__ array of a fixed
// size (kScratchBytes).  Every GPU that loads libwlc holds this array
// until the process exits.  Host code cannot use the array's name as a
// device address (on the host it names a shadow symbol), so the first
// call on each device, with that device current, looks up the real
// address with cudaGetSymbolAddress and keeps it.  That first call also
// copies the operator tables for (N, L, literal semantics) into the array;
// make it before any stream capture.  A later call with a different
// (N, L, literals) copies that configuration's tables over them and waits
// for the copy on its stream; while its stream is being captured such a
// call is refused with WLC_E_STATE.  Work queued earlier on other streams
// that still reads the array sees the new tables.  Nothing here calls
// cudaMalloc, cudaFree or an allocating library routine.
//
// All calls share the one array: calls that overlap on the GPU (on
// different streams, or from different host threads) race and corrupt
// each other's results.  The array keeps the last call's contents; no
// part of it has to start at zero (every byte a call reads was written
// earlier in the same call or by the table upload).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "wlc.h"
#include "wlc_rot_gen.cuh"
#include "wlc_internal.h"
#include "wlc_step.h"

namespace {

constexpr size_t kScratchBytes = 64ull << 20;  // 64 MiB per device
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_scratch[kScratchBytes];

struct DevState {
    bool ready = false;
    unsigned char* base = nullptr;  // device address of g_scratch
    int L = -1, real4 = -1, N = -1;  // configuration whose tables the array holds
    wlc::SolveTablesT<double> tab{};
    double2* twg = nullptr;
    double2* phat = nullptr;
};

// host-side tables of one (L, literal semantics) and the size of their
// device image (which does not depend on the base address)
struct HostTables {
    wlc::BasisTables t;
    size_t image_bytes = 0;
};

std::mutex g_mu;
DevState g_dev[kMaxDevices];
std::map<std::pair<int, int>, HostTables> g_tables;

int fail(char* errbuf, int errlen, int code, const std::string& msg) {
    if (errbuf && errlen > 0) {
        std::strncpy(errbuf, msg.c_str(), (size_t)errlen - 1);
        errbuf[errlen - 1] = '\0';
    }
    return code;
}

size_t align256(size_t v) { return (v + 255) & ~(size_t)255; }

// Byte image of the solve tables, each array 256-byte aligned, with the
// device pointers patched in for the given base address.
struct TableImage {
    std::vector<unsigned char> bytes;
    wlc::SolveTablesT<double> tab{};
};

template <typename X> size_t put(std::vector<unsigned char>& img, const std::vector<X>& v) {
    const size_t off = align256(img.size());
    img.resize(off + sizeof(X) * v.size());
    if (!v.empty()) std::memcpy(img.data() + off, v.data(), sizeof(X) * v.size());
    return off;
}

TableImage make_image(const wlc::BasisTables& t, unsigned char* base) {
    TableImage im;
    std::vector<int16_t> pairs;
    for (int l = 1; l <= t.L; ++l)
        for (int m = 1; m <= l; ++m) {
            pairs.push_back((int16_t)(l * l + l + m));
            pairs.push_back((int16_t)(l * l + l - m));
            pairs.push_back((int16_t)m);
        }
    auto i16 = [](const std::vector<int>& v) {
        std::vector<int16_t> o(v.size());
        for (size_t k = 0; k < v.size(); ++k) o[k] = (int16_t)v[k];
        return o;
    };
    std::vector<std::vector<std::pair<int, std::pair<int, double>>>> rows(t.M);
    for (int a = 0; a < 3; ++a)
        for (size_t e = 0; e < t.dR[a].size(); ++e)
            rows[t.dR[a].row[e]].push_back({t.dR[a].col[e], {a, t.dR[a].val[e]}});
    std::vector<int> dptr(t.M + 1, 0);
    std::vector<int16_t> dcol;
    std::vector<int8_t> dax;
    std::vector<double> dval;
    for (int i = 0; i < t.M; ++i) {
        for (auto& e : rows[i]) {
            dcol.push_back((int16_t)e.first);
            dax.push_back((int8_t)e.second.first);
            dval.push_back(e.second.second);
        }
        dptr[i + 1] = (int)dval.size();
    }
    auto& img = im.bytes;
    wlc::SolveTablesT<double>& s = im.tab;
    auto f32 = [](const std::vector<double>& v) { return std::vector<float>(v.begin(), v.end()); };
    s.L = t.L;
    s.M = t.M;
    s.npairs = (int)pairs.size() / 3;
    s.nnz = (int)t.xp_val.size();
    s.pairs = reinterpret_cast<const int16_t*>(base + put(img, pairs));
    s.xp_ptr = reinterpret_cast<const int*>(base + put(img, t.xp_ptr));
    s.xp_col = reinterpret_cast<const int16_t*>(base + put(img, i16(t.xp_col)));
    s.xp_val = reinterpret_cast<const double*>(base + put(img, t.xp_val));
    s.xp_valf = reinterpret_cast<const float*>(base + put(img, f32(t.xp_val)));
    s.xm_ptr = reinterpret_cast<const int*>(base + put(img, t.xm_ptr));
    s.xm_col = reinterpret_cast<const int16_t*>(base + put(img, i16(t.xm_col)));
    s.xm_val = reinterpret_cast<const double*>(base + put(img, t.xm_val));
    s.xm_valf = reinterpret_cast<const float*>(base + put(img, f32(t.xm_val)));
    s.zoff = reinterpret_cast<const double*>(base + put(img, t.zoff));
    s.zofff = reinterpret_cast<const float*>(base + put(img, f32(t.zoff)));
    s.ndr = (int)dval.size();
    s.dr_ptr = reinterpret_cast<const int*>(base + put(img, dptr));
    s.dr_col = reinterpret_cast<const int16_t*>(base + put(img, dcol));
    s.dr_axis = reinterpret_cast<const int8_t*>(base + put(img, dax));
    s.dr_valf = reinterpret_cast<const float*>(base + put(img, f32(dval)));
    img.resize(align256(img.size()));
    return im;
}

}  // namespace

extern "C" int wlc_mde_one_step_noalloc(const wlc_params* p, int32_t g_index, const double* pr_dev,
                                        double* q_out_dev, void* stream, char* errbuf, int32_t errlen) {
    using namespace wlc;
    if (!p || !pr_dev || !q_out_dev) return fail(errbuf, errlen, WLC_E_PARAM, "null params / pr_dev / q_out_dev");
    if (p->precision != WLC_FP64) return fail(errbuf, errlen, WLC_E_UNSUPPORTED, "only WLC_FP64 is built here");
    if (p->n[0] != p->n[1] || p->n[1] != p->n[2] || !supported_n(p->n[0]))
        return fail(errbuf, errlen, WLC_E_UNSUPPORTED, "grid must be cubic with a compiled edge length");
    if (p->lmax < 0 || p->lmax > kRotLmax || p->nmax < 1)
        return fail(errbuf, errlen, WLC_E_PARAM, "lmax must be in [0, 12] and nmax >= 1");
    if (p->literals != WLC_LIT_REAL4 && p->literals != WLC_LIT_REAL8)
        return fail(errbuf, errlen, WLC_E_PARAM, "literals must be WLC_LIT_REAL4 or WLC_LIT_REAL8");
    for (int a = 0; a < 3; ++a)
        if (!(p->dx[a] > 0) || !(p->kappa[a] > 0))
            return fail(errbuf, errlen, WLC_E_PARAM, "grid spacing and kappa must be > 0");
    // ABC G_index table, Gmatrix_mod-old.f90:446-518
    static const int kind[10][3] = {{1, 1, 0}, {2, 1, 0}, {3, 1, 0}, {3, 1, 1}, {3, 1, 2},
                                    {3, -1, 0}, {3, -1, 1}, {3, -1, 2}, {2, -1, 2}, {1, -1, 2}};
    if (g_index < 1 || g_index > 10) return fail(errbuf, errlen, WLC_E_PARAM, "G_index must be in 1..10");
    const int order = kind[g_index - 1][0], sigma = kind[g_index - 1][1], blk = kind[g_index - 1][2];
    const int N = p->n[0], L = p->lmax, M = (L + 1) * (L + 1);
    const int real4 = p->literals == WLC_LIT_REAL4 ? 1 : 0;
    const size_t nk = (size_t)(N / 2 + 1) * N * N;
    const size_t phat_bytes = sizeof(double2) * nk * (size_t)M;

    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices)
        return fail(errbuf, errlen, WLC_E_CUDA, "no current CUDA device");
    cudaStream_t st = reinterpret_cast<cudaStream_t>(stream);

    std::lock_guard<std::mutex> lock(g_mu);
    DevState& ds = g_dev[dev];
    if (!ds.ready) {
        void* addr = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&addr, g_scratch);
        if (e != cudaSuccess)
            return fail(errbuf, errlen, WLC_E_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
        ds.base = reinterpret_cast<unsigned char*>(addr);
        ds.ready = true;
    }
    const auto key = std::make_pair(L, real4);
    auto it = g_tables.find(key);
    if (it == g_tables.end()) {
        HostTables h;
        std::string why;
        if (!build_basis_tables(L, real4, h.t, why)) return fail(errbuf, errlen, WLC_E_SELFTEST, why);
        h.image_bytes = make_image(h.t, ds.base).bytes.size();
        it = g_tables.emplace(key, std::move(h)).first;
    }
    const size_t tw_off = it->second.image_bytes;
    const size_t phat_off = align256(tw_off + sizeof(double2) * (size_t)N);
    const size_t need = phat_off + phat_bytes;
    if (need > kScratchBytes) {
        char buf[256];
        std::snprintf(buf, sizeof buf,
                      "scratch for N=%d, L=%d needs %zu bytes, above the %zu-byte static limit of "
                      "wlc_mde_one_step_noalloc; use wlc_create / wlc_mde_one_step",
                      N, L, need, kScratchBytes);
        return fail(errbuf, errlen, WLC_E_UNSUPPORTED, buf);
    }
    {
        const BasisTables& t = it->second.t;
        const int ndr = (int)(t.dR[0].size() + t.dR[1].size() + t.dR[2].size());
        const size_t ssv =
            solve_smem(N, M, L, ndr, 8, ndr > 0 ? 1 : 0).total;
        if (ssv > 227 * 1024 || smem_xy<double>(N) > 227 * 1024)
            return fail(errbuf, errlen, WLC_E_UNSUPPORTED, "one coefficient column does not fit in shared memory");
    }
    if (ds.L != L || ds.real4 != real4 || ds.N != N) {
        // (N, L, literals) changed since the last call on this device: the
        // tables are re-uploaded, which blocks on the stream -- refused
        // while the stream is being captured
        cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
        if (cudaStreamIsCapturing(st, &cap) != cudaSuccess || cap != cudaStreamCaptureStatusNone) {
            cudaGetLastError();
            return fail(errbuf, errlen, WLC_E_STATE,
                        "the operator tables of these (N, L, literals) must be uploaded outside stream capture: "
                        "make one call with them before capturing");
        }
        const TableImage im = make_image(it->second.t, ds.base);
        std::vector<double2> tw(N);
        for (int j = 0; j < N; ++j) {
            const double a = 2.0 * M_PI * (double)j / (double)N;
            tw[j].x = std::cos(a);
            tw[j].y = -std::sin(a);
        }
        cudaError_t e = cudaMemcpyAsync(ds.base, im.bytes.data(), im.bytes.size(), cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess)
            e = cudaMemcpyAsync(ds.base + tw_off, tw.data(), sizeof(double2) * N, cudaMemcpyHostToDevice, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess)
            return fail(errbuf, errlen, WLC_E_CUDA, std::string("table upload: ") + cudaGetErrorString(e));
        ds.L = L;
        ds.real4 = real4;
        ds.N = N;
        ds.tab = im.tab;
    }
    ds.twg = reinterpret_cast<double2*>(ds.base + tw_off);
    ds.phat = reinterpret_cast<double2*>(ds.base + phat_off);

    StepLaunch<double> Lh;
    StepArgs<double>& a = Lh.step;
    a.h1 = pr_dev;
    a.h2 = nullptr;
    a.h3 = nullptr;
    a.wb = nullptr;
    a.cf = nullptr;
    a.dsw = nullptr;
    a.third = lit_third(real4);
    a.msterm = nullptr;
    a.order = 0;  // the right-hand side is given
    a.ds = 1.0 / (double)p->nmax;
    a.phat = ds.phat;
    a.twg = ds.twg;
    a.M = M;
    a.qout = q_out_dev;
    a.minv = 1.0 / ((double)N * N * N);
    SolveArgs<double>& s = Lh.solve;
    s.phat = ds.phat;
    s.twg = ds.twg;
    s.tab = ds.tab;
    for (int q = 0; q < 3; ++q) s.kf[q] = lit_kfactor(N, p->dx[q], real4);
    s.ds = 1.0 / (double)p->nmax;
    s.c0 = lit_c0(order, real4);
    s.dcoef = s.ds * p->loa / (2.0 * p->kappa[blk]);
    s.sigma = sigma;
    s.nkx = N / 2 + 1;
    s.correct = ds.tab.ndr > 0 ? 1 : 0;
    s.pivtab = nullptr;  // pivots computed in the kernel: no table to hold
    s.npiv = (L + 1) * (L + 2) / 2;
    cudaError_t e = launch_step<double>(N, Lh, st);
    if (e != cudaSuccess) return fail(errbuf, errlen, WLC_E_CUDA, std::string("launch: ") + cudaGetErrorString(e));
    return WLC_OK;
}
