// Spectral x-pass: for every (ky, kz) pencil of a half spectrum that has been
// transformed over (y, z) only, FFT along x, multiply by the IMEX prefactor,
// inverse FFT along x - one read and one write of the spectrum instead of two
// cuFFT passes plus a separate k-space pass.
//
// Layout: spec[x][ky][kz] complex (cuFFT's 2-D R2C over (y, z), batched over
// x), so pencil m = ky*nzh + kz is contiguous across m at fixed x and element
// x sits at spec[x*M + m] (M = ny*nzh).  A tile of P = 256/N2 consecutive
// pencils x all nx rows is owned by one block of 256 threads; pencil p is
// handled by N2 threads (N = N1*N2 along x).
//
// The transform along x is the four-step FFT of evx_fft.cuh (N = N1*N2,
// compile-time twiddles in the register DFTs); the frequency data never needs
// natural order, so there is no bit-reversal pass, and every thread writes
// back exactly the elements it loaded.  Compiled with FMA contraction (no
// bitwise requirement; cuFFT rounds differently anyway); the forward
// multiplier uses explicit round-to-nearest operations as the k-space kernels
// do.
// Multipliers (same float32 expressions as the k-space kernels):
//   forward  X * prefac(k) * invN                    (evoxels/timesteppers.py:77,87)
//   adjoint  X * (prefac*invN), and X * (prefac*invN*k^4) into a second spectrum
//
// Stored increment spectra.  The forward pass can also write the multiplied
// spectrum dU(k) = prefac*invN*R(k) (whose inverse transform is u_{s+1} - u_s)
// in the kernel's own register order, [tile][element][thread], so that the
// adjoint pass of the same step reads it back coalesced at the same positions.
// With it the adjoint forms the two mobility sums by Parseval over the half
// spectrum (weight 1 on the kz = 0 and kz = nz/2 planes, 2 elsewhere):
//   <lam', u_{s+1} - u_s>   = sum_k wz Re(L(k) conj dU(k))
//   <K lam', u_{s+1} - u_s> = sum_k wz prefac k^4 Re(L(k) conj dU(k))
// with L = R2C(lam') unnormalised; per-block partial sums go out in double.
//
// Two kernels share this math.  The pipelined one (even M >= 256, modes 0, 1
// and 3) is persistent: a 3-slot ring of tiles in shared memory is filled by
// TMA tensor loads (cp.async.bulk.tensor, one thread, mbarrier completion)
// one tile ahead of the compute, and results leave by TMA tensor stores from
// the same slot, so the load of tile i+1 and the store of tile i-1 overlap the
// transforms of tile i.  The per-tile kernel (any M, all modes) loads and
// stores with plain coalesced accesses.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <mutex>
#include <type_traits>

#include "evx_ch_plan.cuh"
#include "evx_fft.cuh"

namespace evx {
namespace {

using namespace fft;

__device__ int g_dev_status;       // bit 0: an x-pass barrier wait gave up
constexpr int WAIT_POLLS = 1 << 22;
__device__ int g_wait_polls = WAIT_POLLS;   // poll limit of the x-pass's tile-load waits

#ifndef EVX_XPASS_MIN_BLOCKS
#define EVX_XPASS_MIN_BLOCKS 2   // resident blocks per SM the register budget is sized for
#endif

// Multiplier stage: forward DFT over k2, multiply, inverse DFT, conjugate
// twiddle into xs[k1][j] (N2 > 1) or back into v (N2 == 1).  MODE 0 forward
// (optional store of the product to dsp), 1 adjoint g, 2 adjoint g and h (into
// hv), 3 adjoint g with the Parseval sums against dsp, 4 multiplier table
// (mult[kx*M + m] in the spectrum's own pencil order, mrow = mult + m: a warp's
// reads are consecutive whichever of y or z is contiguous).  dsp points at the tile's stored
// spectrum ([element][thread], thread offset included).
// PRE (mode 3): the stored spectrum values come preloaded in dpre[q*N2 + k2].
// KX: where kx^2 comes from - 0 the global table kx2, 1 the thread's values preloaded in
// kxr[q*N2 + k2] (they depend on the thread only), 2 a copy of the table in shared memory (kx2).
// TW (N1 = N2 = 16 only): the inverse inter-stage twiddles are the conjugates of the thread's split
// forward twiddles tw (W^{n2*j} = tw->at(j)) instead of reads of the constant table.
template <int N1, int N2, int MODE, bool PRE = false, int KX = 0, bool TW = false>
__device__ __forceinline__ void mid_stage(float2 (&v)[N1], float2 (&hv)[MODE == 2 ? N1 : 1], float2* xs,
                                          const Col<N1, N2>& c, float ky2v, float kz2v, float wz,
                                          const float* __restrict__ kx2, float sym_coef, float dt, float invN,
                                          float2* __restrict__ dsp, float& t1, float& t2,
                                          const float* __restrict__ mrow = nullptr, int M = 0,
                                          const float2 (*dpre)[PRE ? N1 : 1] = nullptr,
                                          const float (*kxr)[KX == 1 ? N1 : 1] = nullptr,
                                          const Tw16<false>* tw = nullptr) {
    constexpr int N = N1 * N2, Q = N1 / N2;
#pragma unroll
    for (int q = 0; q < Q; ++q) {
        const int k1 = N2 > 1 ? c.n2 * Q + q : q;
        float2 a[N2], b[N2];
#pragma unroll
        for (int j = 0; j < N2; ++j) a[j] = v[N2 > 1 ? q * N2 + j : q];
        if constexpr (N2 > 1) dft<N2, false>(a);
#pragma unroll
        for (int k2 = 0; k2 < N2; ++k2) {
            const int kx = k1 + N1 * k2;
            float kx2v;
            if constexpr (KX == 1) kx2v = (*kxr)[q * N2 + k2];
            else if constexpr (KX == 2) kx2v = kx2[kx];
            else kx2v = __ldg(kx2 + kx);
            const float k2s = __fadd_rn(__fadd_rn(kx2v, ky2v), kz2v);
            if constexpr (MODE == 4) {
                const float mv = __ldg(mrow + (size_t)kx * M);
                a[k2] = make_float2(__fmul_rn(__fmul_rn(a[k2].x, mv), invN), __fmul_rn(__fmul_rn(a[k2].y, mv), invN));
            } else if constexpr (MODE == 0) {
                const float pre = imex_prefac(k2s, sym_coef, dt);
                a[k2] = make_float2(__fmul_rn(__fmul_rn(a[k2].x, pre), invN), __fmul_rn(__fmul_rn(a[k2].y, pre), invN));
                if (dsp) dsp[(q * N2 + k2) * 256] = a[k2];
            } else {
                const float k4 = k2s * k2s;
                const float pre = dt / (1.f - dt * (sym_coef * k4));
                const float sg = pre * invN;
                if constexpr (MODE == 2) b[k2] = make_float2(a[k2].x * (sg * k4), a[k2].y * (sg * k4));
                if constexpr (MODE == 3) {
                    float2 d;
                    if constexpr (PRE) d = (*dpre)[q * N2 + k2];
                    else d = dsp[(q * N2 + k2) * 256];
                    const float re = wz * (a[k2].x * d.x + a[k2].y * d.y);
                    t1 += re;
                    t2 += re * (pre * k4);
                }
                a[k2] = make_float2(a[k2].x * sg, a[k2].y * sg);
            }
        }
        if constexpr (N2 > 1) {
            dft<N2, true>(a);
            if constexpr (MODE == 2) dft<N2, true>(b);
#pragma unroll
            for (int j = 0; j < N2; ++j) {
                if constexpr (TW) {
                    static_assert(N1 == 16 && N2 == 16 && MODE != 2, "split twiddles: 16 x 16 columns");
                    xs[c.xi(k1, j)] = j ? cmul(a[j], conjf2(tw->at(j))) : a[j];
                } else {
                    xs[c.xi(k1, j)] = cmul(a[j], w512<true>((j * k1) * (512 / N)));
                    if constexpr (MODE == 2) hv[q * N2 + j] = cmul(b[j], w512<true>((j * k1) * (512 / N)));
                }
            }
        } else {
            v[q] = a[0];
            if constexpr (MODE == 2) hv[q] = b[0];
        }
    }
}

__device__ __forceinline__ float kz_weight(int kz, int nz) { return (kz == 0 || 2 * kz == nz) ? 1.f : 2.f; }

// Block sums of (t1, t2) in double, fixed order, into out[0..1].
__device__ __forceinline__ void block_sum2(float t1, float t2, double* out) {
    __shared__ double red[2][8];
    const int tid = threadIdx.x;
    double d1 = t1, d2 = t2;
    for (int o = 16; o > 0; o >>= 1) {
        d1 += __shfl_down_sync(0xffffffffu, d1, o);
        d2 += __shfl_down_sync(0xffffffffu, d2, o);
    }
    if ((tid & 31) == 0) {
        red[0][tid >> 5] = d1;
        red[1][tid >> 5] = d2;
    }
    __syncthreads();
    if (tid < 2) {
        double x = 0.0;
        for (int w = 0; w < 8; ++w) x += red[tid][w];
        out[tid] = x;
    }
}

// ---- per-tile kernel (plain loads and stores) -------------------------------------
// MODE 0 forward (dspec: optional store of the increment spectrum), 1 adjoint (g),
// 2 adjoint (g and h into spec_h), 3 adjoint (g and the two Parseval sums
// against dspec into xpart[2*block .. 2*block+1]).  EXT 1 / 2: the spectrum
// holds N/2 x rows and the transformed sequence is its even / odd mirror
// extension, x' = N-1-x for x >= N/2 (the mirrored-x step of a Neumann /
// Dirichlet x axis); only the first N/2 rows are written back.  xb (batched
// path): instance blockIdx.y of a shape group, its spectrum offset and IMEX
// constants taken from xb.
template <int N1, int N2, int MODE, int EXT = 0>
__global__ void __launch_bounds__(256, MODE == 2 ? 2 : EVX_XPASS_MIN_BLOCKS)
xpass_kernel(float2* __restrict__ spec, float2* __restrict__ spec_h, float2* __restrict__ dspec,
             double* __restrict__ xpart, int M, int nzh, int nz,
             const float* __restrict__ kx2, const float* __restrict__ ky2, const float* __restrict__ kz2,
             float sym_coef, float dt, float invN, const XBatchInst* __restrict__ xb,
             const float* __restrict__ mult = nullptr, int nyk = 0) {
    if (xb) {
        const XBatchInst X = xb[blockIdx.y];
        spec += X.soff;
        if (spec_h) spec_h += X.soff;
        if (dspec) dspec += X.doff;
        if (xpart) xpart += (size_t)X.xoff * 2;
        sym_coef = X.sym;
        dt = X.dt;
        invN = X.invN;
    }
    using C = Col<N1, N2>;
    constexpr int P = 256 / N2, Q = C::Q;
    extern __shared__ float2 xs[];       // [N1][N2][P], pencil index fastest (conflict-free)
    const int tid = threadIdx.x;
    const C c{tid % P, tid / P, P};
    const int m = blockIdx.x * P + c.p;
    const bool live = m < M;
    const int mc = live ? m : 0;
    // pencil m = ky*nzh + kz, or kz*ny + ky for the y-contiguous spectrum (nyk = ny)
    const int ky = nyk ? mc % nyk : mc / nzh, kz = nyk ? mc / nyk : mc % nzh;
    const float ky2v = __ldg(ky2 + ky), kz2v = __ldg(kz2 + kz);
    float2* dsp = dspec ? dspec + (size_t)blockIdx.x * N1 * 256 + tid : nullptr;
    float t1 = 0.f, t2 = 0.f;
    // mode 3: the tile's stored spectrum into registers first, in flight with the tile's own loads
    // (nx <= 128: at 256 the registers would spill)
    constexpr bool PRE = MODE == 3 && N1 <= 16 && N1 * N2 <= 128;
    float2 dpre[PRE ? N1 : 1];
    if constexpr (PRE) {
#pragma unroll
        for (int e = 0; e < N1; ++e) dpre[e] = __ldcs(dsp + e * 256);
    }

    // kx^2 of the thread's frequencies (modes 0, 1 and 4 up to nx = 128: in registers, loaded with the
    // tile) or the whole table in shared memory (where the registers are taken)
    constexpr int KX = (MODE == 0 || MODE == 1 || MODE == 4) && N1 * N2 <= 128 ? 1 : 2;
    float kxr[KX == 1 ? N1 : 1];
    __shared__ float s_kx2[KX == 2 ? N1 * N2 : 1];
    if constexpr (KX == 1) {
#pragma unroll
        for (int q = 0; q < Q; ++q)
#pragma unroll
            for (int k2 = 0; k2 < N2; ++k2) kxr[q * N2 + k2] = __ldg(kx2 + (N2 > 1 ? c.n2 * Q + q : q) + N1 * k2);
    } else {
        for (int i = tid; i < N1 * N2; i += 256) s_kx2[i] = __ldg(kx2 + i);
        __syncthreads();
    }

    constexpr int NH = (N1 * N2) / 2;   // physical rows with EXT
    float2 v[N1];
#pragma unroll
    for (int n1 = 0; n1 < N1; ++n1) {
        const int x = N2 * n1 + c.n2;
        if (EXT && x >= NH) {
            const float2 w = live ? spec[(size_t)(2 * NH - 1 - x) * M + m] : make_float2(0.f, 0.f);
            v[n1] = EXT == 2 ? make_float2(-w.x, -w.y) : w;
        } else {
            v[n1] = live ? spec[(size_t)x * M + m] : make_float2(0.f, 0.f);
        }
    }
    fwd_stage1<N1, N2>(v, xs, c);
    float2 hv[MODE == 2 ? N1 : 1];
    mid_stage<N1, N2, MODE, PRE, KX>(v, hv, xs, c, ky2v, kz2v, kz_weight(kz, nz), KX == 2 ? s_kx2 : kx2, sym_coef, dt,
                                     invN, dsp, t1, t2, mult + mc, M, &dpre, &kxr);
    auto store = [&](float2* dst) {
        if (live) {
#pragma unroll
            for (int n1 = 0; n1 < N1; ++n1) {
                const int x = N2 * n1 + c.n2;
                if (!EXT || x < NH) dst[(size_t)x * M + m] = v[n1];
            }
        }
    };
    inv_stage1<N1, N2>(v, xs, c);
    store(spec);
    if constexpr (MODE == 2) {
        if constexpr (N2 > 1) {
            __syncthreads();   // everyone has gathered the g data
#pragma unroll
            for (int q = 0; q < Q; ++q)
#pragma unroll
                for (int j = 0; j < N2; ++j) xs[c.xi(c.n2 * Q + q, j)] = hv[q * N2 + j];
        } else {
#pragma unroll
            for (int k1 = 0; k1 < N1; ++k1) v[k1] = hv[k1];
        }
        inv_stage1<N1, N2>(v, xs, c);
        store(spec_h);
    }
    if constexpr (MODE == 3) block_sum2(t1, t2, xpart + (size_t)blockIdx.x * 2);
}

// ---- pipelined persistent kernel (TMA) ----------------------------------------
constexpr int XSTAGES = 3;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
// Bounded wait on a phase; false if it did not complete within `polls` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int polls) {
    const uint32_t a = smem_u32(bar);
    for (int i = 0; i < polls; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
    }
    return false;
}
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* tm, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
        ::"r"(smem_u32(dst)), "l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* tm, int x, int y, const void* src) {
    asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];"
                 ::"l"(reinterpret_cast<uint64_t>(tm)), "r"(x), "r"(y), "r"(smem_u32(src))
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read %0;" ::"n"(N) : "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void prefetch_l2(const void* p, uint32_t bytes) {
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(p), "r"(bytes) : "memory");
}

// Tile t = pencils [t*P, t*P + P) x all N rows, moved as ROWS-row boxes
// (ROWS <= 256); the tensor map describes spec as N rows of M complex values.
template <int N1, int N2, int MODE>
__global__ void __launch_bounds__(256, N1 >= 32 ? 1 : 2)
xpass_tma_kernel(const __grid_constant__ CUtensorMap tm, float2* __restrict__ dspec, double* __restrict__ xpart,
                 int M, int nzh, int nz, int ntiles, const float* __restrict__ kx2, const float* __restrict__ ky2,
                 const float* __restrict__ kz2, float sym_coef, float dt, float invN,
                 const float* __restrict__ mult, int nyk) {
    using C = Col<N1, N2>;
    constexpr int P = 256 / N2, N = C::N;
    constexpr int TILE = N * P;                       // complex values per tile
    constexpr int BOXES = (N + 255) / 256, ROWS = N / BOXES;
    constexpr uint32_t TILE_BYTES = TILE * sizeof(float2);
    extern __shared__ __align__(128) float2 ring[];   // [XSTAGES][TILE], each [x][p]
    __shared__ __align__(8) uint64_t bar[XSTAGES];
    // the thread's kx^2 values are the same for every tile: in registers where there are registers to
    // spare (modes 0, 1 and 4), else read from a copy of the table in shared memory
    constexpr int KX = (MODE == 0 || MODE == 1 || MODE == 4) ? 1 : 2;
    __shared__ float s_kx2[KX == 2 ? N : 1];
    const int tid = threadIdx.x;
    const C c{tid % P, tid / P, P};
    if constexpr (KX == 2)
        for (int i = tid; i < N; i += 256) s_kx2[i] = __ldg(kx2 + i);   // published by the barrier below

    auto issue_load = [&](int slot, int tile) {
        mbar_expect_tx(&bar[slot], TILE_BYTES);
#pragma unroll
        for (int b = 0; b < BOXES; ++b)
            tma_load_2d(ring + (size_t)slot * TILE + b * ROWS * P, &tm, tile * P, b * ROWS, &bar[slot]);
    };
    if (tid == 0) {
        for (int s = 0; s < XSTAGES; ++s) mbar_init(&bar[s], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        if ((int)blockIdx.x < ntiles) issue_load(0, blockIdx.x);
    }
    __syncthreads();
    const int polls = g_wait_polls;
    float t1 = 0.f, t2 = 0.f;
    int it = 0;
    // mode 3: a tile's stored spectrum goes into registers as soon as the previous tile's multiplier
    // stage has consumed its own, so the loads are in flight through that tile's inverse stage, its
    // store and this tile's first stage (N1 = 32: one block per SM, 236 registers)
    constexpr bool PRE = MODE == 3;
    float2 dpre[PRE ? N1 : 1];
    auto load_pre = [&](int t) {
        const float2* dp = dspec + (size_t)t * N1 * 256 + tid;
#pragma unroll
        for (int e = 0; e < N1; ++e) dpre[e] = __ldcs(dp + e * 256);
    };
    if constexpr (PRE) {
        if ((int)blockIdx.x < ntiles) load_pre(blockIdx.x);
    }
    // 16 x 16 columns: the thread's inter-stage twiddles in registers (split form)
    constexpr bool TW = (MODE == 0 || MODE == 1 || MODE == 3) && N1 == 16 && N2 == 16;
    Tw16<false> tw;
    if constexpr (TW) tw.init(c.n2);
    float kxr[KX == 1 ? N1 : 1];
    if constexpr (KX == 1) {
        constexpr int Q = N1 / N2;
#pragma unroll
        for (int q = 0; q < Q; ++q)
#pragma unroll
            for (int k2 = 0; k2 < N2; ++k2) kxr[q * N2 + k2] = __ldg(kx2 + (N2 > 1 ? c.n2 * Q + q : q) + N1 * k2);
    }
    for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++it) {
        const int slot = it % XSTAGES;
        const int next = tile + gridDim.x;
        if (tid == 0 && next < ntiles) {
            // the next slot last held tile it-2, whose store is the older of the
            // (at most two) bulk groups that may still be reading shared memory
            bulk_wait_read<1>();
            issue_load((it + 1) % XSTAGES, next);
            if (MODE == 3) prefetch_l2(dspec + (size_t)next * N1 * 256, N1 * 256 * sizeof(float2));
        }
        const bool landed = mbar_wait(&bar[slot], (uint32_t)(it / XSTAGES) & 1u, polls);
        float2* xs = ring + (size_t)slot * TILE;
        const int m = tile * P + c.p;
        const int mc = m < M ? m : 0;
        const int ky = nyk ? mc % nyk : mc / nzh, kz = nyk ? mc / nyk : mc % nzh;
        const float ky2v = __ldg(ky2 + ky), kz2v = __ldg(kz2 + kz);
        float2* dsp = dspec ? dspec + (size_t)tile * N1 * 256 + tid : nullptr;

        float2 v[N1];
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) v[n1] = xs[(N2 * n1 + c.n2) * P + c.p];
        if constexpr (TW) fwd_stage1_tw16(v, xs, c, tw);
        else fwd_stage1<N1, N2>(v, xs, c);
        float2 hv[1];
        mid_stage<N1, N2, MODE, PRE, KX, TW>(v, hv, xs, c, ky2v, kz2v, kz_weight(kz, nz), KX == 2 ? s_kx2 : kx2,
                                             sym_coef, dt, invN, dsp, t1, t2, mult + mc, M, &dpre, &kxr, &tw);
        if constexpr (PRE) {
            if (next < ntiles) load_pre(next);
        }
        inv_stage1<N1, N2>(v, xs, c);
#pragma unroll
        for (int n1 = 0; n1 < N1; ++n1) xs[(N2 * n1 + c.n2) * P + c.p] = v[n1];
        fence_async_smem();
        if (__syncthreads_or(!landed)) {
            // a wait gave up: flag it, store nothing more, and leave once this tile's and the
            // next tile's loads (the only ones in flight) have landed - again a bounded wait
            if (tid == 0) {
                atomicOr(&g_dev_status, 1);
                mbar_wait(&bar[slot], (uint32_t)(it / XSTAGES) & 1u, WAIT_POLLS);
                if (next < ntiles)
                    mbar_wait(&bar[(it + 1) % XSTAGES], (uint32_t)((it + 1) / XSTAGES) & 1u, WAIT_POLLS);
            }
            break;
        }
        if (tid == 0) {
#pragma unroll
            for (int b = 0; b < BOXES; ++b) tma_store_2d(&tm, tile * P, b * ROWS, xs + b * ROWS * P);
            bulk_commit();
        }
    }
    if (MODE == 3) block_sum2(t1, t2, xpart + (size_t)blockIdx.x * 2);
    if (tid == 0) bulk_wait_read<0>();   // shared memory must outlive the stores' reads
}

// ---- host side -------------------------------------------------------------------
constexpr int MAX_DEVICES = 64;
int g_tw_rc[MAX_DEVICES];
std::once_flag g_tw_once[MAX_DEVICES];
bool g_tma_off = false;   // EVX_XPASS_TMA=0 selects the per-tile kernel everywhere

int xpass_split_n2(int nx) {
    switch (nx) {
        case 8: case 16: return 1;
        case 32: return 2;
        case 64: return 4;
        case 128: return 8;
        case 256: case 512: return 16;
        default: return 0;
    }
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) !=
                cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    return fn;
}

template <int N1, int N2, int MODE, int EXT = 0>
int xpass_launch_tile(const XpassArgs& A, cudaStream_t st, const char* slot) {
    constexpr int P = 256 / N2;
    const size_t smem = (size_t)N1 * N2 * P * sizeof(float2);
    // the attribute belongs to the current device's context: set it for every launch (cheap)
    const int rc = check_cuda(cudaFuncSetAttribute(xpass_kernel<N1, N2, MODE, EXT>,
                                                   cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                              "x-pass shared memory attribute");
    if (rc) return rc;
    const int blocks = (A.M + P - 1) / P;
    if (A.n_xpart_out) *A.n_xpart_out = blocks;
    EVX_TIMED(slot, st,
              (xpass_kernel<N1, N2, MODE, EXT><<<blocks, 256, smem, st>>>(A.spec, A.spec_h, A.dspec, A.xpart, A.M,
                                                                        A.nzh, A.nz, A.kx2, A.ky2, A.kz2, A.sym,
                                                                        A.dt, A.invN, nullptr, A.mult, A.nyk)));
    count_launch();
    return check_launch("xpass_kernel");
}

template <int N1, int N2, int MODE>
int xpass_launch_tma(const XpassArgs& A, cudaStream_t st, const char* slot) {
    constexpr int P = 256 / N2, N = N1 * N2;
    constexpr int BOXES = (N + 255) / 256, ROWS = N / BOXES;
    const size_t smem = (size_t)XSTAGES * N * P * sizeof(float2);
    // attribute and residency belong to the current device: queried for every launch (cheap)
    int rc = check_cuda(cudaFuncSetAttribute(xpass_tma_kernel<N1, N2, MODE>,
                                             cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "x-pass shared memory attribute");
    if (rc) return rc;
    int dev = 0, sms = 0, per = 0;
    if ((rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice"))) return rc;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, xpass_tma_kernel<N1, N2, MODE>, 256, smem),
                    "x-pass occupancy");
    if (rc) return rc;
    const int grid_cap = std::max(1, sms) * (per > 0 ? per : 1);
    CUtensorMap tm;
    const cuuint64_t dims[2] = {(cuuint64_t)A.M, (cuuint64_t)N};
    const cuuint64_t strides[1] = {(cuuint64_t)A.M * sizeof(float2)};
    const cuuint32_t box[2] = {(cuuint32_t)P, (cuuint32_t)ROWS};
    const cuuint32_t estr[2] = {1, 1};
    const CUresult r = encode_fn()(&tm, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 2, A.spec, dims, strides, box, estr,
                                   CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                                   CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) return fail(EVX_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)r);
    const int ntiles = (A.M + P - 1) / P;
    const int blocks = ntiles < grid_cap ? ntiles : grid_cap;
    if (A.n_xpart_out) *A.n_xpart_out = blocks;
    EVX_TIMED(slot, st,
              xpass_tma_kernel<N1, N2, MODE><<<blocks, 256, smem, st>>>(tm, A.dspec, A.xpart, A.M, A.nzh, A.nz, ntiles,
                                                                      A.kx2, A.ky2, A.kz2, A.sym, A.dt, A.invN,
                                                                      A.mult, A.nyk));
    count_launch();
    return check_launch("xpass_tma_kernel");
}

template <int N1, int N2, int MODE>
int xpass_launch_m(const XpassArgs& A, cudaStream_t st) {
    const char* slot = MODE == 0 ? (A.dspec ? "ch_xpass_fwd_store" : "ch_xpass_fwd")
                                 : (MODE == 3 ? "ch_xpass_adj_spec" : (MODE == 4 ? "xpass_mult" : "ch_xpass_adj"));
    if constexpr (MODE != 2) {
        // TMA needs 16-byte row strides (even M) and a 16-byte aligned base; small M keeps the per-tile kernel
        const bool tma = !g_tma_off && (A.M % 2) == 0 && A.M >= 256 &&
                         (reinterpret_cast<uintptr_t>(A.spec) & 15) == 0 && encode_fn() != nullptr;
        if (tma) return xpass_launch_tma<N1, N2, MODE>(A, st, slot);
    }
    return xpass_launch_tile<N1, N2, MODE>(A, st, slot);
}

template <int N1, int N2>
int xpass_launch_t(const XpassArgs& A, cudaStream_t st) {
    if (A.ext) {   // mirrored-x step: per-tile kernel (odd or even extension)
        if ((A.mode != 0 && A.mode != 2 && A.mode != 4) || A.dspec)
            return fail(EVX_ERR_UNSUPPORTED, "mirrored-x x-pass: modes 0, 2 and 4 without stored spectra");
        if (A.mode == 2)   // adjoint g and h (parameter gradients of the mirrored step)
            return A.ext == 2 ? xpass_launch_tile<N1, N2, 2, 2>(A, st, "ch_xpass_adj_mirror")
                              : xpass_launch_tile<N1, N2, 2, 1>(A, st, "ch_xpass_adj_mirror");
        if (A.mode == 4)
            return A.ext == 2 ? xpass_launch_tile<N1, N2, 4, 2>(A, st, "xpass_mult_mirror")
                              : xpass_launch_tile<N1, N2, 4, 1>(A, st, "xpass_mult_mirror");
        return A.ext == 2 ? xpass_launch_tile<N1, N2, 0, 2>(A, st, "ch_xpass_fwd_mirror")
                          : xpass_launch_tile<N1, N2, 0, 1>(A, st, "ch_xpass_fwd_mirror");
    }
    switch (A.mode) {
        case 0: return xpass_launch_m<N1, N2, 0>(A, st);
        case 1: return xpass_launch_m<N1, N2, 1>(A, st);
        case 2: return xpass_launch_m<N1, N2, 2>(A, st);
        case 3: return xpass_launch_m<N1, N2, 3>(A, st);
        default: return xpass_launch_m<N1, N2, 4>(A, st);
    }
}

}  // namespace

bool xpass_supported(int nx) {
    return nx >= 8 && nx <= 512 && (nx & (nx - 1)) == 0;
}

int xpass_init() {
    int dev = 0;
    int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= MAX_DEVICES) return fail(EVX_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::call_once(g_tw_once[dev], [dev] {
        g_tw_rc[dev] = check_cuda(upload_w512(), "twiddle table upload");
        const char* e = std::getenv("EVX_XPASS_TMA");
        if (e && e[0] == '0') g_tma_off = true;
    });
    return g_tw_rc[dev];
}

size_t xpass_blocks(int nx, int M) {
    const int n2 = xpass_split_n2(nx);
    if (!n2) return 0;
    const int P = 256 / n2;
    return (size_t)((M + P - 1) / P);
}

size_t xpass_spectrum_floats(int nx, int M) {
    // [tile][element < N1][thread < 256] complex values; N1 = nx / N2
    const int n2 = xpass_split_n2(nx);
    return n2 ? xpass_blocks(nx, M) * (size_t)(nx / n2) * 256 * 2 : 0;
}

template <int N1, int N2>
int xpass_batch_t(int mode, float2* spec, float2* spec_h, const XBatchInst* xb, int count, int M, int nzh, int nz,
                  const float* kx2, const float* ky2, const float* kz2, cudaStream_t st, int nyk, float2* dspec,
                  double* xpart) {
    constexpr int P = 256 / N2;
    const size_t smem = (size_t)N1 * N2 * P * sizeof(float2);
    const dim3 grid((M + P - 1) / P, count);
    auto go = [&](auto kern, const char* slot) {
        const int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                                  "x-pass shared memory attribute");
        if (rc) return rc;
        EVX_TIMED(slot, st, (kern<<<grid, 256, smem, st>>>(spec, spec_h, dspec, xpart, M, nzh, nz, kx2, ky2, kz2,
                                                           0.f, 0.f, 0.f, xb, nullptr, nyk)));
        count_launch();
        return check_launch("xpass_kernel (batched)");
    };
    switch (mode) {
        case 0: return go(xpass_kernel<N1, N2, 0>, dspec ? "batch_xpass_fwd_store" : "batch_xpass_fwd");
        case 1: return go(xpass_kernel<N1, N2, 1>, "batch_xpass_adj");
        case 2: return go(xpass_kernel<N1, N2, 2>, "batch_xpass_adj");
        default: return go(xpass_kernel<N1, N2, 3>, "batch_xpass_adj_spec");
    }
}

int xpass_batch_launch(int mode, int nx, float2* spec, float2* spec_h, const XBatchInst* xb, int count, int M,
                       int nzh, int nz, const float* kx2, const float* ky2, const float* kz2, cudaStream_t st,
                       int nyk, float2* dspec, double* xpart) {
    int rc = xpass_init();
    if (rc) return rc;
    if (count < 1 || count > 65535) return fail(EVX_ERR_BAD_ARG, "batched x-pass: %d instances", count);
    if (mode < 0 || mode > 3) return fail(EVX_ERR_BAD_ARG, "batched x-pass mode %d", mode);
    if ((mode == 2 && !spec_h) || (mode == 3 && (!dspec || !xpart)))
        return fail(EVX_ERR_BAD_ARG, "x-pass mode %d is missing a buffer", mode);
    if (mode != 0 && mode != 3) dspec = nullptr;
    if (mode != 3) xpart = nullptr;
    switch (nx) {
        case 8: return xpass_batch_t<8, 1>(mode, spec, spec_h, xb, count, M, nzh, nz, kx2, ky2, kz2, st, nyk, dspec, xpart);
        case 16: return xpass_batch_t<16, 1>(mode, spec, spec_h, xb, count, M, nzh, nz, kx2, ky2, kz2, st, nyk, dspec, xpart);
        case 32: return xpass_batch_t<16, 2>(mode, spec, spec_h, xb, count, M, nzh, nz, kx2, ky2, kz2, st, nyk, dspec, xpart);
        case 64: return xpass_batch_t<16, 4>(mode, spec, spec_h, xb, count, M, nzh, nz, kx2, ky2, kz2, st, nyk, dspec, xpart);
        case 128: return xpass_batch_t<16, 8>(mode, spec, spec_h, xb, count, M, nzh, nz, kx2, ky2, kz2, st, nyk, dspec, xpart);
        case 256: return xpass_batch_t<16, 16>(mode, spec, spec_h, xb, count, M, nzh, nz, kx2, ky2, kz2, st, nyk, dspec, xpart);
        case 512: return xpass_batch_t<32, 16>(mode, spec, spec_h, xb, count, M, nzh, nz, kx2, ky2, kz2, st, nyk, dspec, xpart);
        default: return fail(EVX_ERR_UNSUPPORTED, "x-pass needs a power-of-two nx in [8, 512]");
    }
}

int xpass_launch(const XpassArgs& A, cudaStream_t st) {
    int rc = xpass_init();
    if (rc) return rc;
    if ((A.mode == 3 && (!A.dspec || !A.xpart)) || (A.mode == 2 && !A.spec_h) || (A.mode == 4 && !A.mult))
        return fail(EVX_ERR_BAD_ARG, "x-pass mode %d is missing a buffer", A.mode);
    if (A.mode < 0 || A.mode > 4) return fail(EVX_ERR_BAD_ARG, "x-pass mode %d", A.mode);
    switch (A.nx) {
        case 8: return xpass_launch_t<8, 1>(A, st);
        case 16: return xpass_launch_t<16, 1>(A, st);
        case 32: return xpass_launch_t<16, 2>(A, st);
        case 64: return xpass_launch_t<16, 4>(A, st);
        case 128: return xpass_launch_t<16, 8>(A, st);
        case 256: return xpass_launch_t<16, 16>(A, st);
        case 512: return xpass_launch_t<32, 16>(A, st);
        default: return fail(EVX_ERR_UNSUPPORTED, "x-pass needs a power-of-two nx in [8, 512]");
    }
}

}  // namespace evx

extern "C" int evx_device_status_async(int* dst, void* stream) {
    if (!dst) return evx::fail(EVX_ERR_BAD_ARG, "evx_device_status_async: null destination");
    return evx::check_cuda(cudaMemcpyFromSymbolAsync(dst, evx::g_dev_status, sizeof(int), 0, cudaMemcpyDefault,
                                                     evx::as_stream(stream)),
                           "queue device status read");
}

extern "C" int evx_set_wait_polls(int polls) {
    const int v = polls < 0 ? evx::WAIT_POLLS : polls;
    return evx::check_cuda(cudaMemcpyToSymbol(evx::g_wait_polls, &v, sizeof(int)), "set wait poll limit");
}

extern "C" int evx_device_status(int reset) {
    int v = 0;
    if (evx::check_cuda(cudaMemcpyFromSymbol(&v, evx::g_dev_status, sizeof(int)), "read device status")) return -1;
    if (reset && v) {
        const int z = 0;
        if (evx::check_cuda(cudaMemcpyToSymbol(evx::g_dev_status, &z, sizeof(int)), "reset device status")) return -1;
    }
    return v;
}
