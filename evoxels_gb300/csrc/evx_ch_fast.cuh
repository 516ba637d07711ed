// Tile geometry and helpers shared by the periodic fast-path stencil kernels
// (Cahn-Hilliard rhs and its adjoint pullback), single-grid and batched.
//
// A block of 256 threads owns a TY x TZ (y, z) tile and streams along x.
// Every thread owns a 2 x 2 (y, z) patch of outputs, so faces inside a patch
// are evaluated once and the x face of a patch is carried in registers from
// one plane to the next.  Field planes are staged in shared memory with a halo
// of 2 rows in y and 4 columns in z (4 keeps every row float4-aligned for
// nz % 4 == 0); chemical-potential planes cover the tile grown by one cell.
// Wrap-around (periodic) offsets are computed once per tile, so the per-plane
// loads are plain float4 loads.  Two tile shapes are built: 16 x 64 (wide in
// z) and 32 x 32 (for grids whose nz is a multiple of 32 but not of 64).
#pragma once

#include <initializer_list>

#include "evx_ch_plan.cuh"

namespace evx {
namespace fast {

constexpr int THREADS = 256;

template <int TZ_, int TY_>
struct Tile {
    static constexpr int TZ = TZ_, TY = TY_;
    static constexpr int BX = TZ / 2, BY = TY / 2;  // thread grid over 2x2 patches
    static constexpr int W = TZ + 8;          // shared row width: z in [k0-4, k0+TZ+4)
    static constexpr int CR = TY + 4;         // field rows: y in [j0-2, j0+TY+2)
    static constexpr int MR = TY + 2;         // potential rows: y in [j0-1, j0+TY+1); row m <-> field row m+1
    static constexpr int NQ = W / 4;          // float4 per shared row
    static constexpr int NLOAD = CR * NQ;     // float4 loads per field plane
    static constexpr int MPZ = (TZ + 4) / 2;  // 2x2 potential patches per row pair: cols 2..TZ+5
    static constexpr int MPY = MR / 2;
    static constexpr int NMU = MPZ * MPY;     // potential patches per plane
    static constexpr int FIELD = CR * W;      // floats per shared field plane
    static constexpr int POT = MR * W;        // floats per shared potential plane
    static_assert(BX * BY == THREADS, "tile must map to 256 threads");
    static_assert(NLOAD <= 2 * THREADS && NMU <= 2 * THREADS, "at most two loads / patches per thread");
};
using TileWide = Tile<64, 16>;
using TileSquare = Tile<32, 32>;
constexpr int MAX_FIELD = TileWide::FIELD > TileSquare::FIELD ? TileWide::FIELD : TileSquare::FIELD;
constexpr int MAX_POT = TileWide::POT > TileSquare::POT ? TileWide::POT : TileSquare::POT;

// Shared plane rings of the x-streaming tiles: NC field slots and NM potential
// slots, enough for one block barrier per plane (plane i's output, the
// potential of plane i+2 and the store of plane i+4 in one step).
constexpr int NC = 5, NM = 3;
__device__ __forceinline__ int cslot(int p) { return (p + 10) % NC; }   // p >= -5
__device__ __forceinline__ int mslot(int p) { return (p + 9) % NM; }

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void sts2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }
__device__ __forceinline__ void sts4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 clip4(float4 v) {
    return make_float4(clip01(v.x), clip01(v.y), clip01(v.z), clip01(v.w));
}

// Two-lane fp32 arithmetic (sm_100 FADD2 / FMUL2 / FFMA2): each lane rounds
// exactly as the scalar __fadd_rn / __fmul_rn / __fmaf_rn.  sub2 is one
// rounding of a - b (b*(-1) is exact), i.e. the same as __fsub_rn per lane.
// A multiply followed by an add may still be fused by the code generator, so
// the bit-exact kernels use the exact:: variants below.
__device__ __forceinline__ float2 f2s(float s) { return make_float2(s, s); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 mul2(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 fma2(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2s(-1.f), a); }

// Bit-exact two-point arithmetic for the kernels that must round as the
// reference: sums and differences as two-lane .rn PTX instructions, products as
// two scalar roundings.  The code generator may fuse a two-lane multiply into
// a following two-lane add even with explicit rounding modes (and with
// --fmad=false); with scalar products there is no two-lane multiply to fuse,
// and scalar .rn multiplies are never contracted.
namespace exact {
__device__ __forceinline__ unsigned long long f2bits(float2 v) { return *reinterpret_cast<unsigned long long*>(&v); }
__device__ __forceinline__ float2 bits2f(unsigned long long v) { return *reinterpret_cast<float2*>(&v); }
__device__ __forceinline__ float2 add2(float2 a, float2 b) {
    unsigned long long r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bits2f(r);
}
__device__ __forceinline__ float2 sub2(float2 a, float2 b) {
    unsigned long long r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(f2bits(a)), "l"(f2bits(b)));
    return bits2f(r);
}
__device__ __forceinline__ float2 mul2(float2 a, float2 b) {
    return make_float2(__fmul_rn(a.x, b.x), __fmul_rn(a.y, b.y));
}
// A two-lane product for the places where nothing can be fused into it: its
// result feeds only further products, or it is exact (a power of two times x).
__device__ __forceinline__ float2 mul2_nofuse(float2 a, float2 b) { return __fmul2_rn(a, b); }
}  // namespace exact

// Per-thread load plan for one shared field plane (precomputed once per tile).
struct LoadPlan {
    int goff[2];    // in-plane global offset of the float4 (wrapped)
    int soff[2];    // shared offset
    bool valid[2];
    bool own[2];    // inside the tile and the domain (written back in fused mode)
};

template <class T>
__device__ __forceinline__ LoadPlan make_load_plan(int tid, int j0, int k0, int ny, int nz) {
    LoadPlan L;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const int e = tid + s * THREADS;
        L.valid[s] = e < T::NLOAD;
        const int row = L.valid[s] ? e / T::NQ : 0;
        const int q = L.valid[s] ? e - row * T::NQ : 0;
        const int gy = j0 + row - 2, gz = k0 + 4 * q - 4;
        L.own[s] = L.valid[s] && row >= 2 && row < 2 + T::TY && q >= 1 && q < 1 + T::TZ / 4 && gy < ny && gz < nz;
        L.goff[s] = pmod(gy, ny) * nz + pmod(gz, nz);
        L.soff[s] = row * T::W + 4 * q;
    }
    return L;
}

// Grid over (z tiles, y tiles, x chunks) sized to at most one wave of resident blocks.
template <class T>
inline dim3 fast_grid(int nx, int ny, int nz, int blocks_per_sm, int sms, int* LX) {
    const int tz = (nz + T::TZ - 1) / T::TZ, ty = (ny + T::TY - 1) / T::TY;
    const long tiles = (long)tz * ty;
    const long slots = (long)blocks_per_sm * sms;
    long chunks = slots / tiles;                          // no partial second wave
    if (chunks < 1) chunks = 1;
    int lx = (int)((nx + chunks - 1) / chunks);
    if (lx < 8) lx = 8;                                   // keep the x halo overhead bounded
    if (lx > nx) lx = nx;
    *LX = lx;
    return dim3(tz, ty, (nx + lx - 1) / lx);
}

}  // namespace fast

// Fast-path eligibility: periodic grid, nz % 4 == 0, 16-byte aligned fields.
inline bool fast_ok(const evx_grid* g, std::initializer_list<const void*> ptrs) {
    if (g->nz % 4 != 0) return false;
    for (const void* p : ptrs)
        if (p && (reinterpret_cast<uintptr_t>(p) & 15)) return false;
    return true;
}

// Tile variant for a grid: 0 = 16 x 64, 1 = 32 x 32.  Default: the square tile
// when nz is a multiple of 32 but not of 64, else the wide one.
inline int default_tile_variant(int nz) { return (nz % 64 != 0 && nz % 32 == 0) ? 1 : 0; }
int ch_tile_variant(int nz);   // honours evx_set_tile_variant

// exact: the reference's float32 operations in its order (evx_ch_rhs); else the
// fused-product arithmetic of the spectral loops (always for the fused pass)
int ch_rhs_fast_launch(bool fused, bool exact, const float* u, const float* upd, float* u_new, float* r,
                       const evx_grid* g, const Geo& G, const ChP& P, cudaStream_t st);
// Final gradient reduction of the spectral-gradient pullback (grads == 2), done by
// the block that finishes last: the blocks' partial sums (part) and the x-pass
// Parseval partials (xpart: <lam', u'-u>, <K lam', u'-u> per block) in a fixed
// order, dL/dD += t1/D - kappa*A*t2, dL/dkappa += sK - D*A*t2, dL/dw += sW.
// counter must be zero before the launch; the last block resets it.
struct GradSink {
    double* grads;
    const double* xpart;
    int nxpart;
    int* counter;
    double kA, DA, invD;
};

// grads: 0 none, 1 all four partial sums (reads h and u1), 2 the two real-space sums only
// (sink: optional last-block reduction for grads == 2; else part is left for a reduce kernel)
int ch_pullback_fast_launch(int grads, const float* u, const float* g, const float* lam, const float* h,
                            const float* u1, float* lam_out, double* part, int n_part_cap, const evx_grid* grid,
                            const Geo& G, const ChP& P, cudaStream_t st, int* n_part_used,
                            const GradSink* sink = nullptr);
int ch_pullback_fast_blocks(const evx_grid* g);

// ---- batched (persistent) kernels ------------------------------------------------
// One work item = one tile x one x-chunk of one instance.
struct BatchInst {
    int nx, ny, nz, tile;          // tile variant (0 wide, 1 square)
    long long off;                 // field offset (floats) in the packed buffers
    int part0;                     // first work item of this instance (partial sums)
    int orig;                      // the caller's index of this instance
    float ih[3], ih2[3], ih2sum;
    ChP P;
};
struct BatchItem {
    int inst;
    int k0, j0, x0, x1;
    int part;                      // partial-sum slot (items of one instance are consecutive slots)
};
int batch_rhs_launch(bool fused, const float* u, const float* upd, float* u_new, float* r, const BatchInst* insts,
                     const BatchItem* items, int n_items, int* counter, int grid, cudaStream_t st);
// grads: 0 none, 1 the four real-space gradient sums (h and u1 read), 2 the two
// real-space sums of the spectral-gradient path
int batch_pullback_launch(int grads, const float* u, const float* g, const float* lam, const float* h,
                          const float* u1, float* lam_out, double* part, const BatchInst* insts,
                          const BatchItem* items, int n_items, int* counter, int grid, cudaStream_t st);
int batch_rhs_blocks_per_sm();
int batch_pullback_blocks_per_sm(int grads);

}  // namespace evx
