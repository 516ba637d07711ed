// Spectral x-pass: for every (ky, kz) pencil of a half spectrum that has been
// transformed over (y, z) only, FFT along x, multiply by the IMEX prefactor,
// inverse FFT along x - one read and one write of the spectrum instead of two
// cuFFT passes plus a separate k-space pass.
//
// Layout: spec[x][ky][kz] complex (cuFFT's 2-D R2C over (y, z), batched over
// x), so pencil m = ky*nzh + kz is contiguous across m at fixed x and element
// x sits at spec[x*M + m] (M = ny*nzh).  A block of 256 threads owns P = 256/N2
// consecutive pencils; pencil p is handled by N2 threads (N = N1*N2 along x).
//
// Four-step FFT with N = N1*N2, n = N2*n1 + n2, k = k1 + N1*k2:
//   forward  A[k1][n2]     = W_N^{n2 k1} * DFT_N1(x[N2 n1 + n2])[k1]     thread n2, registers
//            X[k1 + N1 k2] = DFT_N2(A[k1][.])[k2]                      after a shared exchange
//   inverse  B[k1][n2]     = W_N^{-n2 k1} * IDFT_N2(X[k1 + N1 .])[n2]   the thread holding X
//            y[N2 n1 + n2] = IDFT_N1(B[.][n2])[n1]                     after a shared exchange
// The frequency data never needs natural order, so there is no bit-reversal
// pass, and every thread writes back exactly the elements it loaded.  Roots
// of unity come from a table of W_512^j computed on the host in double
// precision.  The transforms are compiled with FMA contraction (no bitwise
// requirement; cuFFT rounds differently anyway); the forward multiplier uses
// explicit round-to-nearest operations as the k-space kernels do.
// Multipliers (same float32 expressions as the k-space kernels):
//   forward  X * prefac(k) * invN                    (evoxels/timesteppers.py:77,87)
//   adjoint  X * (prefac*invN), and X * (prefac*invN*k^4) into a second spectrum
#include <cmath>
#include <mutex>

#include "evx_ch_plan.cuh"

namespace evx {
namespace {

__constant__ float2 c_w512[512];   // (cos, -sin)(2*pi*j/512): forward roots of unity

std::once_flag g_tw_once;
int g_tw_rc = EVX_OK;

__device__ __forceinline__ float2 cmul(float2 a, float2 b) {
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// W_512^j of the forward (INV = false) or inverse (conjugate) transform
template <bool INV>
__device__ __forceinline__ float2 w512(int j) {
    const float2 w = c_w512[j & 511];
    return INV ? make_float2(w.x, -w.y) : w;
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

// In-register DFT of length L (power of two <= 32), natural order in and out:
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
#pragma unroll
    for (int len = 2; len <= L; len <<= 1) {
#pragma unroll
        for (int i = 0; i < L; i += len) {
#pragma unroll
            for (int k = 0; k < len / 2; ++k) {
                const float2 w = w512<INV>(k * (512 / len));
                const float2 a = v[i + k], b = cmul(v[i + k + len / 2], w);
                v[i + k] = cadd(a, b);
                v[i + k + len / 2] = csub(a, b);
            }
        }
    }
}

#ifndef EVX_XPASS_MIN_BLOCKS
#define EVX_XPASS_MIN_BLOCKS 2   // resident blocks per SM the register budget is sized for
#endif

template <int N1, int N2, int MODE>   // MODE 0 forward, 1 adjoint (g), 2 adjoint (g and h)
__global__ void __launch_bounds__(256, MODE == 2 ? 2 : EVX_XPASS_MIN_BLOCKS)
xpass_kernel(float2* __restrict__ spec, float2* __restrict__ spec_h, int M, int nzh,
             const float* __restrict__ kx2, const float* __restrict__ ky2, const float* __restrict__ kz2,
             float sym_coef, float dt, float invN) {
    constexpr int N = N1 * N2;
    constexpr int P = 256 / N2;          // pencils per block
    constexpr int Q = N1 / N2;           // k1 values per thread between the exchanges
    static_assert(N1 >= N2 && N1 % N2 == 0 && 256 % N2 == 0, "unsupported split");
    extern __shared__ float2 xs[];       // [N1][N2][P], pencil index fastest (conflict-free)
    const int tid = threadIdx.x;
    const int p = tid % P, n2 = tid / P;
    const int m = blockIdx.x * P + p;
    const bool live = m < M;
    const int mc = live ? m : 0;
    const int ky = mc / nzh, kz = mc - ky * nzh;
    const float ky2v = __ldg(ky2 + ky), kz2v = __ldg(kz2 + kz);
    auto at = [&](int k1, int j) -> float2& { return xs[(k1 * N2 + j) * P + p]; };

    // ---- forward stage 1: load the thread's column, DFT over n1, twiddle
    float2 v[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1)
        v[n1] = live ? spec[(size_t)(N2 * n1 + n2) * M + m] : make_float2(0.f, 0.f);
    dft<N1, false>(v);
    if (N2 > 1) {
#pragma unroll
        for (int k1 = 0; k1 < N1; ++k1) at(k1, n2) = cmul(v[k1], w512<false>((n2 * k1) * (512 / N)));
        __syncthreads();
#pragma unroll
        for (int q = 0; q < Q; ++q)
#pragma unroll
            for (int j = 0; j < N2; ++j) v[q * N2 + j] = at(n2 * Q + q, j);   // A[k1][.] for the thread's k1
        __syncthreads();
    }
    // ---- forward stage 2, multiply, inverse stage 2 (registers); stash B[k1][.]
    float2 hv[MODE == 2 ? N1 : 1];
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int k1 = N2 > 1 ? n2 * Q + q : q;
        float2 a[N2], b[N2];
#pragma unroll
        for (int j = 0; j < N2; ++j) a[j] = v[N2 > 1 ? q * N2 + j : q];
        if (N2 > 1) dft<N2, false>(a);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) {
            const int kx = k1 + N1 * k2;
            const float k2s = __fadd_rn(__fadd_rn(__ldg(kx2 + kx), ky2v), kz2v);
            if (MODE == 0) {
                const float pre = imex_prefac(k2s, sym_coef, dt);
                a[k2] = make_float2(__fmul_rn(__fmul_rn(a[k2].x, pre), invN), __fmul_rn(__fmul_rn(a[k2].y, pre), invN));
            } else {
                const float k4 = k2s * k2s;
                const float sg = (dt / (1.f - dt * (sym_coef * k4))) * invN;
                if (MODE == 2) b[k2] = make_float2(a[k2].x * (sg * k4), a[k2].y * (sg * k4));
                a[k2] = make_float2(a[k2].x * sg, a[k2].y * sg);
            }
        }
        if (N2 > 1) {
            dft<N2, true>(a);
            if (MODE == 2) dft<N2, true>(b);
#pragma unroll
            for (int j = 0; j < N2; ++j) {
                at(k1, j) = cmul(a[j], w512<true>((j * k1) * (512 / N)));
                if (MODE == 2) hv[q * N2 + j] = cmul(b[j], w512<true>((j * k1) * (512 / N)));
            }
        } else {
            v[q] = a[0];
            if (MODE == 2) hv[q] = b[0];
        }
    }
    // ---- inverse stage 1: gather B[.][n2], IDFT over k1, store
    auto finish = [&](float2* dst) {
        if (N2 > 1) {
            __syncthreads();
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) v[k1] = at(k1, n2);
        }
        dft<N1, true>(v);
        if (live) {
#pragma unroll
            for (int n1 = 0; n1 < N1; ++n1) dst[(size_t)(N2 * n1 + n2) * M + m] = v[n1];
        }
    };
    finish(spec);
    if (MODE == 2) {
        if (N2 > 1) {
            __syncthreads();   // everyone has gathered the g data
#pragma unroll
            for (int q = 0; q < Q; ++q)
#pragma unroll
                for (int j = 0; j < N2; ++j) at(n2 * Q + q, j) = hv[q * N2 + j];
        } else {
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) v[k1] = hv[k1];
        }
        finish(spec_h);
    }
}

template <int N1, int N2>
int xpass_launch_t(int mode, float2* spec, float2* spec_h, int M, int nzh, const float* kx2, const float* ky2,
                   const float* kz2, float sym, float dt, float invN, cudaStream_t st) {
    constexpr int P = 256 / N2;
    const size_t smem = (size_t)N1 * N2 * P * sizeof(float2);
    static bool attr[3] = {false, false, false};
    const dim3 grid((M + P - 1) / P);
    if (mode == 0) {
        if (!attr[0]) { cudaFuncSetAttribute(xpass_kernel<N1, N2, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); attr[0] = true; }
        EVX_TIMED("ch_xpass_fwd", st, xpass_kernel<N1, N2, 0><<<grid, 256, smem, st>>>(spec, nullptr, M, nzh, kx2, ky2, kz2, sym, dt, invN));
    } else if (mode == 1) {
        if (!attr[1]) { cudaFuncSetAttribute(xpass_kernel<N1, N2, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); attr[1] = true; }
        EVX_TIMED("ch_xpass_adj", st, xpass_kernel<N1, N2, 1><<<grid, 256, smem, st>>>(spec, nullptr, M, nzh, kx2, ky2, kz2, sym, dt, invN));
    } else {
        if (!attr[2]) { cudaFuncSetAttribute(xpass_kernel<N1, N2, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem); attr[2] = true; }
        EVX_TIMED("ch_xpass_adj", st, xpass_kernel<N1, N2, 2><<<grid, 256, smem, st>>>(spec, spec_h, M, nzh, kx2, ky2, kz2, sym, dt, invN));
    }
    count_launch();
    return check_launch("xpass_kernel");
}

}  // namespace

bool xpass_supported(int nx) {
    return nx >= 8 && nx <= 512 && (nx & (nx - 1)) == 0;
}

int xpass_init() {
    std::call_once(g_tw_once, [] {
        float2 h[512];
        for (int j = 0; j < 512; ++j) {
            const double a = 2.0 * M_PI * (double)j / 512.0;
            h[j] = make_float2((float)std::cos(a), (float)-std::sin(a));
        }
        g_tw_rc = check_cuda(cudaMemcpyToSymbol(c_w512, h, sizeof(h)), "twiddle table upload");
    });
    return g_tw_rc;
}

// mode 0: forward multiply; 1: adjoint g; 2: adjoint g and h (spec_h)
int xpass_launch(int mode, int nx, float2* spec, float2* spec_h, int M, int nzh, const float* kx2, const float* ky2,
                 const float* kz2, float sym, float dt, float invN, cudaStream_t st) {
    int rc = xpass_init();
    if (rc) return rc;
    switch (nx) {
        case 8: return xpass_launch_t<8, 1>(mode, spec, spec_h, M, nzh, kx2, ky2, kz2, sym, dt, invN, st);
        case 16: return xpass_launch_t<16, 1>(mode, spec, spec_h, M, nzh, kx2, ky2, kz2, sym, dt, invN, st);
        case 32: return xpass_launch_t<16, 2>(mode, spec, spec_h, M, nzh, kx2, ky2, kz2, sym, dt, invN, st);
        case 64: return xpass_launch_t<16, 4>(mode, spec, spec_h, M, nzh, kx2, ky2, kz2, sym, dt, invN, st);
        case 128: return xpass_launch_t<16, 8>(mode, spec, spec_h, M, nzh, kx2, ky2, kz2, sym, dt, invN, st);
        case 256: return xpass_launch_t<16, 16>(mode, spec, spec_h, M, nzh, kx2, ky2, kz2, sym, dt, invN, st);
        case 512: return xpass_launch_t<32, 16>(mode, spec, spec_h, M, nzh, kx2, ky2, kz2, sym, dt, invN, st);
        default: return fail(EVX_ERR_UNSUPPORTED, "x-pass needs a power-of-two nx in [8, 512]");
    }
}

}  // namespace evx
