// wlc_reduce.h -- launch interface of the layout, density and reduction
// kernels (wlc_reduce.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace wlc {

constexpr int kS3Blocks = 512;  // CTAs of the deterministic Simpson reduction

struct DensityArgs {
    int64_t nr;
    int M;
    int nmax;
    int nstart[3], ns[3];
    double ds;
};

struct S3Args {
    int n[3];
    double d[3];
};

struct FeArgs {
    int64_t nr;
    double chi[3];  // AB, AC, BC
    double nmu;
    int ms;
};

// union of the five Theta basis tensors: entry e couples (row, col) with
// values val[5e + c], c = T1122, T33, T12, T13, T23
struct ThetaLists {
    int n;
    const int* rowptr;  // [M+1]: entries of row i at [rowptr[i], rowptr[i+1]) (entries are sorted by row)
    const int16_t* row;
    const int16_t* col;
    const double* val;
};

// five J lists (J11, J22, J12, J13, J23) concatenated; ptr[6]
struct JLists {
    int n;  // total entries (ptr[5])
    const int* ptr;
    const int16_t* row;
    const int16_t* col;
    const double* val;
};

// points per CTA of the tiled per-point coefficient kernels (ms_term,
// density slices, orientation tensor): the coefficient vectors of the tile
// are staged in shared memory once
template <typename T> struct PointTile {
    static constexpr int value = sizeof(T) == 8 ? 32 : 64;
};
// function attributes of the tiled kernels (large shared memory) on the
// current device; call on each device before any stream capture (repeat
// calls on a device return at once)
cudaError_t prepare_reduce_kernels();
constexpr int kMsGroups = 4;  // ms_term: row groups per point (threads per point)
constexpr int kSGroups = 5;   // orientation tensor: one thread per component per point

template <typename T> void launch_to_internal(const double* ref, T* out, int M, int64_t nr, cudaStream_t st);
template <typename T> void launch_to_reference(const T* in, double* ref, int M, int64_t nr, cudaStream_t st);
template <typename T> void launch_set_delta(T* q, int M, int64_t nr, cudaStream_t st);
template <typename T>
void launch_make_cf(const double* w, T* cf, double ds, double third, int64_t nr, cudaStream_t st);
template <typename T>
void launch_ms_term(const T* h1, const T* h2, const T* h3, int order, const double* mop, const ThetaLists& tl,
                    double ds, double thresh, int M, int64_t nr, T* out, cudaStream_t st);
template <typename T>
void launch_density(const T* qf, const T* qb, const DensityArgs& d, double* raw, double* junc, double* qend,
                    cudaStream_t st);
template <typename T>
void launch_stensor(const T* qf, const T* qb, const DensityArgs& d, const JLists& jl, double* sraw, cudaStream_t st);
// one contour slice s of the streamed density integrals (q(s), q*(s) given):
// raw/sraw += Simpson weight x q.q* for the blocks containing s, junction
// and Q(end) slices copied; at the last slice (s = 0) scaled by ds/3
// per-instance arguments of a batched density_slice launch (instance j =
// blockIdx.y): q(s) = qf + s*sl, q*(s) = qb + (s & 3)*sl (streamed ring)
template <typename T> struct SliceBatchArgs {
    const T* qf;
    const T* qb;
    int64_t sl;
    DensityArgs d;
    int want_s;
    JLists jl;
    double* raw;
    double* junc;
    double* qend;
    double* sraw;
};
template <typename T>
void launch_density_slice_batched(const SliceBatchArgs<T>* args, int count, int64_t max_nr, int s, int M, int nj,
                                  int any_s, cudaStream_t st);

template <typename T>
void launch_density_slice(const T* qf_s, const T* qb_s, const DensityArgs& d, int s, int want_s, const JLists& jl,
                          double* raw, double* junc, double* qend, double* sraw, cudaStream_t st);
void launch_s3(const double* a, int nsum, int64_t stride, const S3Args& s, double* part, double* out,
               cudaStream_t st);
void launch_scale(double* a, int64_t n, const double* denom, double vol, cudaStream_t st);
void launch_fe(const double* phi, const double* w, const double* mop, const FeArgs& f, double* ar, cudaStream_t st);
void launch_nonfinite(const double* a, int64_t n, int* flag, cudaStream_t st);

}  // namespace wlc
