// wlc_fft.cuh -- shared-memory batched FFTs for the 3D R2C/C2R transforms
// of the harmonic coefficients (replacing decomp_2d_fft_3d,
// 2dcomp_fft_mod.f90:18-236, called from wormlike_MDE_2dcomp_mod.f90:357-455).
//
// Sign convention is FFTW's: DIR = -1 forward (e^{-i}), DIR = +1 backward,
// both unnormalised.  A length-N line is split N = N1*N2 (N1 the first
// radix).  fft_nat2perm takes natural-order input and leaves X[k1 + N1*k2]
// at position k1*N2 + k2 ("permuted"); fft_perm2nat is its transpose and
// takes permuted input to natural-order output.  Every small DFT runs in
// registers of one thread; the CTA cooperates over (line, sub-transform)
// work items with one __syncthreads between the two passes.
#pragma once
#include <cuda_runtime.h>

namespace wlc {

template <typename T> struct cvec;
template <> struct cvec<double> { using t = double2; };
template <> struct cvec<float> { using t = float2; };

template <typename C> __device__ __forceinline__ C cmk(decltype(C::x) a, decltype(C::x) b) {
    C r;
    r.x = a;
    r.y = b;
    return r;
}
template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return cmk<C>(a.x + b.x, a.y + b.y); }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return cmk<C>(a.x - b.x, a.y - b.y); }
template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return cmk<C>(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
template <typename C, typename R> __device__ __forceinline__ C cscale(C a, R s) { return cmk<C>(a.x * s, a.y * s); }
// multiply by DIR*i
template <int DIR, typename C> __device__ __forceinline__ C cmuli(C a) {
    return DIR > 0 ? cmk<C>(-a.y, a.x) : cmk<C>(a.y, -a.x);
}

// ------------------------------------------------------------ small DFTs
template <int R> struct Dft;

template <> struct Dft<1> {
    template <int DIR, typename C> __device__ __forceinline__ static void run(C*) {}
};

template <> struct Dft<2> {
    template <int DIR, typename C> __device__ __forceinline__ static void run(C* v) {
        C a = v[0], b = v[1];
        v[0] = cadd(a, b);
        v[1] = csub(a, b);
    }
};

template <> struct Dft<3> {
    template <int DIR, typename C> __device__ __forceinline__ static void run(C* v) {
        using T = decltype(C::x);
        const T s = (T)0.86602540378443864676;
        C t1 = cadd(v[1], v[2]);
        C t2 = csub(v[0], cscale(t1, (T)0.5));
        C t3 = cmuli<DIR>(cscale(csub(v[1], v[2]), s));
        v[0] = cadd(v[0], t1);
        v[1] = cadd(t2, t3);
        v[2] = csub(t2, t3);
    }
};

template <> struct Dft<4> {
    template <int DIR, typename C> __device__ __forceinline__ static void run(C* v) {
        C a = cadd(v[0], v[2]), b = csub(v[0], v[2]);
        C c = cadd(v[1], v[3]), d = cmuli<DIR>(csub(v[1], v[3]));
        v[0] = cadd(a, c);
        v[2] = csub(a, c);
        v[1] = cadd(b, d);
        v[3] = csub(b, d);
    }
};

template <> struct Dft<5> {
    template <int DIR, typename C> __device__ __forceinline__ static void run(C* v) {
        using T = decltype(C::x);
        const T c1 = (T)0.30901699437494742410, c2 = (T)-0.80901699437494742410;
        const T s1 = (T)0.95105651629515357212, s2 = (T)0.58778525229247312917;
        C t1 = cadd(v[1], v[4]), t2 = cadd(v[2], v[3]);
        C t3 = csub(v[1], v[4]), t4 = csub(v[2], v[3]);
        C a1 = cadd(v[0], cadd(cscale(t1, c1), cscale(t2, c2)));
        C a2 = cadd(v[0], cadd(cscale(t1, c2), cscale(t2, c1)));
        C b1 = cmuli<DIR>(cadd(cscale(t3, s1), cscale(t4, s2)));
        C b2 = cmuli<DIR>(csub(cscale(t3, s2), cscale(t4, s1)));
        v[0] = cadd(v[0], cadd(t1, t2));
        v[1] = cadd(a1, b1);
        v[4] = csub(a1, b1);
        v[2] = cadd(a2, b2);
        v[3] = csub(a2, b2);
    }
};

template <> struct Dft<8> {
    template <int DIR, typename C> __device__ __forceinline__ static void run(C* v) {
        using T = decltype(C::x);
        const T h = (T)0.70710678118654752440;
        C e[4] = {v[0], v[2], v[4], v[6]};
        C o[4] = {v[1], v[3], v[5], v[7]};
        Dft<4>::run<DIR>(e);
        Dft<4>::run<DIR>(o);
        // o[k] *= w8^k, w8 = h*(1 + DIR i)
        C o1 = cmk<C>(h * (o[1].x - DIR * o[1].y), h * (o[1].y + DIR * o[1].x));
        C o2 = cmuli<DIR>(o[2]);
        C o3 = cmk<C>(h * (-o[3].x - DIR * o[3].y), h * (-o[3].y + DIR * o[3].x));
        v[0] = cadd(e[0], o[0]);
        v[4] = csub(e[0], o[0]);
        v[1] = cadd(e[1], o1);
        v[5] = csub(e[1], o1);
        v[2] = cadd(e[2], o2);
        v[6] = csub(e[2], o2);
        v[3] = cadd(e[3], o3);
        v[7] = csub(e[3], o3);
    }
};

// cos/sin(2 pi e / R) for the composite radices (R divides 16 or 6)
template <int R> __device__ __forceinline__ double root_cos(int e) {
    if (R == 6 || R == 3) {
        const int f = e * (6 / R) % 6;
        return f == 0 ? 1.0 : (f == 1 || f == 5) ? 0.5 : (f == 3) ? -1.0 : -0.5;
    }
    const int f = e * (16 / R) % 16;
    const double c[5] = {1.0, 0.92387953251128675613, 0.70710678118654752440, 0.38268343236508977173, 0.0};
    if (f <= 4) return c[f];
    if (f <= 8) return -c[8 - f];
    if (f <= 12) return -c[f - 8];
    return c[16 - f];
}
template <int R> __device__ __forceinline__ double root_sin(int e) {
    if (R == 6 || R == 3) {
        const int f = e * (6 / R) % 6;
        const double s = 0.86602540378443864676;
        return (f == 0 || f == 3) ? 0.0 : (f < 3) ? s : -s;
    }
    const int f = e * (16 / R) % 16;
    return root_cos<16>((f + 12) % 16);  // sin(x) = cos(x - pi/2)
}

// composite R = A*B in registers (compile-time twiddles)
template <int A, int B> struct DftCT {
    template <int DIR, typename C> __device__ __forceinline__ static void run(C* v) {
        using T = decltype(C::x);
        constexpr int R = A * B;
        C tmp[R];
#pragma unroll
        for (int n2 = 0; n2 < B; ++n2) {
            C u[A];
#pragma unroll
            for (int n1 = 0; n1 < A; ++n1) u[n1] = v[B * n1 + n2];
            Dft<A>::template run<DIR>(u);
#pragma unroll
            for (int k1 = 0; k1 < A; ++k1) {
                const int e = (n2 * k1) % R;
                C w = u[k1];
                if (e != 0) w = cmul(u[k1], cmk<C>((T)root_cos<R>(e), (T)(DIR * root_sin<R>(e))));
                tmp[k1 * B + n2] = w;
            }
        }
#pragma unroll
        for (int k1 = 0; k1 < A; ++k1) {
            C u[B];
#pragma unroll
            for (int n2 = 0; n2 < B; ++n2) u[n2] = tmp[k1 * B + n2];
            Dft<B>::template run<DIR>(u);
#pragma unroll
            for (int k2 = 0; k2 < B; ++k2) v[k1 + A * k2] = u[k2];
        }
    }
};
template <> struct Dft<6> : DftCT<2, 3> {};
template <> struct Dft<16> : DftCT<4, 4> {};

// ------------------------------------------------------------ line plans
template <int N> struct Plan;
template <> struct Plan<4> { static constexpr int N1 = 4, N2 = 1; };
template <> struct Plan<6> { static constexpr int N1 = 6, N2 = 1; };
template <> struct Plan<8> { static constexpr int N1 = 8, N2 = 1; };
template <> struct Plan<12> { static constexpr int N1 = 4, N2 = 3; };
template <> struct Plan<16> { static constexpr int N1 = 16, N2 = 1; };
template <> struct Plan<24> { static constexpr int N1 = 8, N2 = 3; };
template <> struct Plan<32> { static constexpr int N1 = 8, N2 = 4; };
template <> struct Plan<40> { static constexpr int N1 = 8, N2 = 5; };
template <> struct Plan<48> { static constexpr int N1 = 8, N2 = 6; };
template <> struct Plan<64> { static constexpr int N1 = 8, N2 = 8; };
template <> struct Plan<96> { static constexpr int N1 = 16, N2 = 6; };
template <> struct Plan<128> { static constexpr int N1 = 16, N2 = 8; };

// position of frequency (or output) index k after fft_nat2perm
template <int N> __device__ __forceinline__ int perm_pos(int k) {
    constexpr int N1 = Plan<N>::N1, N2 = Plan<N>::N2;
    return (k % N1) * N2 + k / N1;
}
// index held at position p after fft_nat2perm
template <int N> __device__ __forceinline__ int perm_index(int p) {
    constexpr int N1 = Plan<N>::N1, N2 = Plan<N>::N2;
    return (p / N2) + N1 * (p % N2);
}

// tw[j] = exp(-2 pi i j / N) (forward); the backward twiddle is its conjugate
template <int DIR, typename C> __device__ __forceinline__ C twid(const C* tw, int e) {
    C w = tw[e];
    if (DIR > 0) w.y = -w.y;
    return w;
}

// Work items (line b, sub-transform j) of one sub-pass are dealt to the
// threads line-fastest, j = w / nlines, b = w % nlines, stepped without a
// division.  Lanes of a warp then touch different lines at the same element
// offset: consecutive words for interleaved lines (lstride 1), and distinct
// banks for contiguous lines when lstride is odd.
struct LineWalk {
    int b, j, sb, sj, nl;
    __device__ __forceinline__ explicit LineWalk(int nlines)
        : b((int)threadIdx.x % nlines), j((int)threadIdx.x / nlines), sb((int)blockDim.x % nlines),
          sj((int)blockDim.x / nlines), nl(nlines) {}
    __device__ __forceinline__ void next() {
        b += sb;
        j += sj;
        if (b >= nl) {
            b -= nl;
            ++j;
        }
    }
};

// Batched in-place line FFTs: line b, element e at data[b*lstride + e*estride].
template <int N, int DIR, typename C>
__device__ __forceinline__ void fft_nat2perm(C* data, int nlines, int estride, int lstride, const C* tw) {
    constexpr int N1 = Plan<N>::N1, N2 = Plan<N>::N2;
    if constexpr (N2 == 1) {
        for (int w = threadIdx.x; w < nlines; w += blockDim.x) {
            C* ln = data + (size_t)w * lstride;
            C v[N1];
#pragma unroll
            for (int n = 0; n < N1; ++n) v[n] = ln[n * estride];
            Dft<N1>::template run<DIR>(v);
#pragma unroll
            for (int n = 0; n < N1; ++n) ln[n * estride] = v[n];
        }
        __syncthreads();
    } else {
    for (LineWalk it(nlines); it.j < N2; it.next()) {
        const int j2 = it.j;
        C* ln = data + (size_t)it.b * lstride;
        C v[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) v[n1] = ln[(n1 * N2 + j2) * estride];
        Dft<N1>::template run<DIR>(v);
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) {
            C x = v[k1];
            if (k1 != 0 && j2 != 0) x = cmul(x, twid<DIR>(tw, (j2 * k1) % N));
            ln[(k1 * N2 + j2) * estride] = x;
        }
    }
    __syncthreads();
    for (LineWalk it(nlines); it.j < N1; it.next()) {
        const int k1 = it.j;
        C* ln = data + (size_t)it.b * lstride;
        C v[N2];
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) v[n2] = ln[(k1 * N2 + n2) * estride];
        Dft<N2>::template run<DIR>(v);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) ln[(k1 * N2 + k2) * estride] = v[k2];
    }
    __syncthreads();
    }
}

template <int N, int DIR, typename C>
__device__ __forceinline__ void fft_perm2nat(C* data, int nlines, int estride, int lstride, const C* tw) {
    constexpr int N1 = Plan<N>::N1, N2 = Plan<N>::N2;
    if constexpr (N2 == 1) {
        fft_nat2perm<N, DIR>(data, nlines, estride, lstride, tw);
    } else {
    for (LineWalk it(nlines); it.j < N1; it.next()) {
        const int k1 = it.j;
        C* ln = data + (size_t)it.b * lstride;
        C v[N2];
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) v[k2] = ln[(k1 * N2 + k2) * estride];
        Dft<N2>::template run<DIR>(v);
#pragma unroll
        for (int n2 = 0; n2 < N2; ++n2) {
            C x = v[n2];
            if (k1 != 0 && n2 != 0) x = cmul(x, twid<DIR>(tw, (n2 * k1) % N));
            ln[(k1 * N2 + n2) * estride] = x;
        }
    }
    __syncthreads();
    for (LineWalk it(nlines); it.j < N2; it.next()) {
        const int n2 = it.j;
        C* ln = data + (size_t)it.b * lstride;
        C v[N1];
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v[k1] = ln[(k1 * N2 + n2) * estride];
        Dft<N1>::template run<DIR>(v);
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) ln[(n1 * N2 + n2) * estride] = v[n1];
    }
    __syncthreads();
    }
}

}  // namespace wlc
