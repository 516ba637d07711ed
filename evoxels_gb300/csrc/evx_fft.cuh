// In-register FFT building blocks shared by the spectral passes (evx_fftx.cu:
// x-pass; evx_fftyz.cu: fused (y, z) transforms).
//
// Four-step FFT of length N = N1*N2 over a "column" held by N2 threads
// (n = N2*n1 + n2; thread n2 holds n1 = 0..N1-1 in registers), k = k1 + N1*k2:
//   forward  A[k1][n2]     = W_N^{n2 k1} * DFT_N1(x[N2 n1 + n2])[k1]     thread n2, registers
//            X[k1 + N1 k2] = DFT_N2(A[k1][.])[k2]                      after a shared exchange
//   inverse  B[k1][n2]     = W_N^{-n2 k1} * IDFT_N2(X[k1 + N1 .])[n2]   the thread holding X
//            y[N2 n1 + n2] = IDFT_N1(B[.][n2])[n1]                     after a shared exchange
// Between the exchanges thread n2 holds the Q = N1/N2 values k1 = n2*Q + q.
// The exchange slot of (k1, j) is xs[(k1*N2 + j)*stride + p]: a [N][stride]
// array of which the column uses entry p of each row, so it may alias the
// [n][p] array the column was read from (the same addresses, k1 <-> n1).
//
// The in-register DFTs use twiddles fixed at compile time (cos/sin of
// 2*pi*j/L evaluated by Taylor series in double, so multiplications by 1, -1
// and +-i vanish); the inter-stage twiddles W_N^{n2 k1} depend on the thread
// and come from a per-translation-unit table of W_512^j computed on the host
// in double precision (upload_w512 once per device).  Everything here has
// internal linkage: each including unit owns its table and its uploader.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <type_traits>

namespace evx {
namespace fft {
namespace {

__constant__ float2 c_w512[512];   // (cos, -sin)(2*pi*j/512): forward roots of unity

// Host: fill this translation unit's twiddle table on the current device.
inline cudaError_t upload_w512() {
    float2 h[512];
    for (int j = 0; j < 512; ++j) {
        const double a = 2.0 * M_PI * (double)j / 512.0;
        h[j] = make_float2((float)std::cos(a), (float)-std::sin(a));
    }
    return cudaMemcpyToSymbol(c_w512, h, sizeof(h));
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
// Complex sums and differences as one two-lane instruction each (sm_100 FADD2 / FFMA2): each lane
// rounds as the scalar operation (b*(-1) is exact), so results are those of the scalar forms.
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return __ffma2_rn(b, make_float2(-1.f, -1.f), a); }
__device__ __forceinline__ float2 conjf2(float2 a) { return make_float2(a.x, -a.y); }

// W_512^j of the forward (INV = false) or inverse (conjugate) transform
template <bool INV>
__device__ __forceinline__ float2 w512(int j) {
    const float2 w = c_w512[j & 511];
    return INV ? make_float2(w.x, -w.y) : w;
}

// ---- compile-time twiddles ----------------------------------------------------
constexpr double kPi = 3.141592653589793238462643383279502884;
// Taylor series on [-pi, pi]; 16 terms leave an error below 1e-18
__host__ __device__ constexpr double cx_sin(double x) {
    double t = x, s = x;
    for (int k = 1; k < 16; ++k) {
        t *= -x * x / ((2.0 * k) * (2.0 * k + 1.0));
        s += t;
    }
    return s;
}
__host__ __device__ constexpr double cx_cos(double x) {
    double t = 1.0, s = 1.0;
    for (int k = 1; k < 16; ++k) {
        t *= -x * x / ((2.0 * k - 1.0) * (2.0 * k));
        s += t;
    }
    return s;
}
// 2*pi*j/L reduced to [-pi, pi]
__host__ __device__ constexpr double cx_angle(int j, int L) {
    j %= L;
    if (2 * j > L) j -= L;
    return 2.0 * kPi * (double)j / (double)L;
}

// a * W_L^J (forward, W = exp(-2*pi*i/L)) or a * conj(W_L^J) (inverse)
template <int J, int L, bool INV>
__device__ __forceinline__ float2 twiddle(float2 a) {
    constexpr int j = J % L;
    if constexpr (j == 0) {
        return a;
    } else if constexpr (2 * j == L) {
        return make_float2(-a.x, -a.y);
    } else if constexpr (4 * j == L) {        // forward -i, inverse +i
        return INV ? make_float2(-a.y, a.x) : make_float2(a.y, -a.x);
    } else if constexpr (4 * j == 3 * L) {    // forward +i, inverse -i
        return INV ? make_float2(a.y, -a.x) : make_float2(-a.y, a.x);
    } else {
        constexpr float c = (float)cx_cos(cx_angle(j, L));
        constexpr float s = (float)(INV ? cx_sin(cx_angle(j, L)) : -cx_sin(cx_angle(j, L)));
        return make_float2(a.x * c - a.y * s, a.x * s + a.y * c);
    }
}

template <int B, int E, int S = 1, class F>
__device__ __forceinline__ void static_for(F&& f) {
    if constexpr (B < E) {
        f(std::integral_constant<int, B>{});
        static_for<B + S, E, S>(f);
    }
}

template <int L>
__host__ __device__ constexpr int bitrev(int i) {
    int r = 0;
    for (int b = 1; b < L; b <<= 1) {
        r = (r << 1) | (i & 1);
        i >>= 1;
    }
    return r;
}

// In-register DFT of length L (power of two <= 64), natural order in and out:
// radix-2 decimation in time on the bit-reversed input (the permutation is a
// compile-time register renaming).
template <int L, bool INV>
__device__ __forceinline__ void dft(float2 (&v)[L]) {
#pragma unroll
    for (int i = 0; i < L; ++i) {
        const int j = bitrev<L>(i);
        if (j > i) {
            const float2 t = v[i];
            v[i] = v[j];
            v[j] = t;
        }
    }
    static_for<1, 7>([&](auto S) {
        constexpr int len = 1 << decltype(S)::value;
        if constexpr (len <= L) {
            static_for<0, L, len>([&](auto I) {
                static_for<0, len / 2>([&](auto K) {
                    constexpr int i = decltype(I)::value, k = decltype(K)::value;
                    const float2 a = v[i + k], b = twiddle<k, len, INV>(v[i + k + len / 2]);
                    v[i + k] = cadd(a, b);
                    v[i + k + len / 2] = csub(a, b);
                });
            });
        }
    });
}

// Barrier of the exchange: the block, or the warp when all threads of a
// column sit in one warp (WARP = true).
template <bool WARP>
__device__ __forceinline__ void exchange_sync() {
    if constexpr (WARP) __syncwarp();
    else __syncthreads();
}

// Per-thread context of one column: entry p of each row of a [N][stride] array.
// (The stage functions take any type with n2 and xi(k1, j).)
template <int N1, int N2>
struct Col {
    static constexpr int N = N1 * N2, Q = N1 / N2;
    static_assert(N1 >= N2 && N1 % N2 == 0 && N <= 512, "unsupported split");
    int p, n2, stride;
    __device__ __forceinline__ int xi(int k1, int j) const { return (k1 * N2 + j) * stride + p; }
};

// Forward stage 1 on the thread's column v (x = N2*n1 + n2): DFT over n1,
// twiddle, exchange; afterwards v[q*N2 + j] = A[n2*Q + q][j].  The gathered
// rows are rewritten only by their gathering thread, so no barrier follows.
template <int N1, int N2, bool WARP = false, class C>
__device__ __forceinline__ void fwd_stage1(float2 (&v)[N1], float2* xs, const C& c) {
    constexpr int N = N1 * N2, Q = N1 / N2;
    dft<N1, false>(v);
    if constexpr (N2 > 1) {
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) xs[c.xi(k1, c.n2)] = cmul(v[k1], w512<false>((c.n2 * k1) * (512 / N)));
        exchange_sync<WARP>();
#pragma unroll
        for (int q = 0; q < Q; ++q)
#pragma unroll
            for (int j = 0; j < N2; ++j) v[q * N2 + j] = xs[c.xi(c.n2 * Q + q, j)];
    }
}

// Forward stage 2 (no multiplier): v[q*N2 + k2] = X[k1 + N1*k2], k1 = n2*Q + q
// (N2 == 1: v[q] = X[q]).
template <int N1, int N2>
__device__ __forceinline__ void fwd_stage2(float2 (&v)[N1]) {
    constexpr int Q = N1 / N2;
    if constexpr (N2 > 1) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            float2 a[N2];
#pragma unroll
            for (int j = 0; j < N2; ++j) a[j] = v[q * N2 + j];
            dft<N2, false>(a);
#pragma unroll
            for (int j = 0; j < N2; ++j) v[q * N2 + j] = a[j];
        }
    }
}

// Inverse stage 2: from v[q*N2 + k2] = X[k1 + N1*k2] (k1 = n2*Q + q), IDFT over
// k2, conjugate twiddle, into xs[k1][j] (N2 > 1; N2 == 1 leaves v as is).
template <int N1, int N2, class C>
__device__ __forceinline__ void inv_stage2(float2 (&v)[N1], float2* xs, const C& c) {
    constexpr int N = N1 * N2, Q = N1 / N2;
    if constexpr (N2 > 1) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int k1 = c.n2 * Q + q;
            float2 a[N2];
#pragma unroll
            for (int j = 0; j < N2; ++j) a[j] = v[q * N2 + j];
            dft<N2, true>(a);
#pragma unroll
            for (int j = 0; j < N2; ++j) xs[c.xi(k1, j)] = cmul(a[j], w512<true>((j * k1) * (512 / N)));
        }
    }
}

// Inverse stage 1: gather B[.][n2] (after a barrier), IDFT over k1; v then
// holds the output column x = N2*n1 + n2 (same addresses as the gather).
template <int N1, int N2, bool WARP = false, class C>
__device__ __forceinline__ void inv_stage1(float2 (&v)[N1], const float2* xs, const C& c) {
    if constexpr (N2 > 1) {
        exchange_sync<WARP>();
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) v[k1] = xs[c.xi(k1, c.n2)];
    }
    dft<N1, true>(v);
}

// Variants with the inter-stage twiddles in registers, for columns whose
// threads in a warp hold different n2 (one table load per thread instead of
// divergent reads of the constant table in every stage).
// tw[k1] = W_N^{n2*k1} (forward stage 1)
template <int N1, int N2>
__device__ __forceinline__ void fwd_twiddles(float2 (&tw)[N1], int n2) {
    constexpr int N = N1 * N2;
#pragma unroll
    for (int k1 = 0; k1 < N1; ++k1) tw[k1] = w512<false>((n2 * k1) * (512 / N));
}
// tw[q*N2 + j] = conj W_N^{j*k1}, k1 = n2*Q + q (inverse stage 2)
template <int N1, int N2>
__device__ __forceinline__ void inv_twiddles(float2 (&tw)[N1], int n2) {
    constexpr int N = N1 * N2, Q = N1 / N2;
#pragma unroll
    for (int q = 0; q < Q; ++q)
#pragma unroll
        for (int j = 0; j < N2; ++j) tw[q * N2 + j] = w512<true>((j * (n2 * Q + q)) * (512 / N));
}

template <int N1, int N2, bool WARP = false, class C>
__device__ __forceinline__ void fwd_stage1_tw(float2 (&v)[N1], float2* xs, const C& c, const float2 (&tw)[N1]) {
    constexpr int Q = N1 / N2;
    dft<N1, false>(v);
    if constexpr (N2 > 1) {
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) xs[c.xi(k1, c.n2)] = cmul(v[k1], tw[k1]);
        exchange_sync<WARP>();
#pragma unroll
        for (int q = 0; q < Q; ++q)
#pragma unroll
            for (int j = 0; j < N2; ++j) v[q * N2 + j] = xs[c.xi(c.n2 * Q + q, j)];
    }
}

// Split twiddles for N1 = N2 = 16 columns (thread n2 = t): W^{t*k} for k = 4i + j
// as W^{t*j} * W^{t*4i}, six registers instead of fifteen (one more rounding on
// the nine k with i, j both nonzero).  INV: the conjugate roots.
template <bool INV>
struct Tw16 {
    float2 a[4], b[4];   // a[j] = W^{t*j}, b[i] = W^{t*4i}
    __device__ __forceinline__ void init(int t) {
#pragma unroll
        for (int j = 0; j < 4; ++j) a[j] = w512<INV>((t * j) * 2);
#pragma unroll
        for (int i = 0; i < 4; ++i) b[i] = w512<INV>((t * 4 * i) * 2);
    }
    __device__ __forceinline__ float2 at(int k) const {   // k a compile-time constant after unrolling
        const int j = k & 3, i = k >> 2;
        if (i == 0) return a[j];
        if (j == 0) return b[i];
        return cmul(a[j], b[i]);
    }
};

template <bool WARP = false, class C>
__device__ __forceinline__ void fwd_stage1_tw16(float2 (&v)[16], float2* xs, const C& c, const Tw16<false>& tw) {
    dft<16, false>(v);
#pragma unroll
    for (int k1 = 0; k1 < 16; ++k1) xs[c.xi(k1, c.n2)] = k1 ? cmul(v[k1], tw.at(k1)) : v[k1];
    exchange_sync<WARP>();
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = xs[c.xi(c.n2, j)];
}

template <int N1, int N2, class C>
__device__ __forceinline__ void inv_stage2_tw(float2 (&v)[N1], float2* xs, const C& c, const float2 (&tw)[N1]) {
    constexpr int Q = N1 / N2;
    if constexpr (N2 > 1) {
#pragma unroll
        for (int q = 0; q < Q; ++q) {
            const int k1 = c.n2 * Q + q;
            float2 a[N2];
#pragma unroll
            for (int j = 0; j < N2; ++j) a[j] = v[q * N2 + j];
            dft<N2, true>(a);
#pragma unroll
            for (int j = 0; j < N2; ++j) xs[c.xi(k1, j)] = cmul(a[j], tw[q * N2 + j]);
        }
    }
}

}  // namespace
}  // namespace fft
}  // namespace evx
