// Tile geometry and helpers shared by the periodic fast-path stencil kernels
// (Cahn-Hilliard rhs and its adjoint pullback).
//
// A block of 32 x 8 threads owns a TY x TZ = 16 x 64 (y, z) tile and streams
// along x.  Every thread owns a 2 x 2 (y, z) patch of outputs, so faces inside
// a patch are evaluated once and the x face of a patch is carried in
// registers from one plane to the next.  Field planes are staged in shared
// memory with a halo of 2 rows in y and 4 columns in z (4 keeps every row
// float4-aligned for nz % 4 == 0); chemical-potential planes cover the tile
// grown by one cell.  Wrap-around (periodic) offsets are computed once per
// block, so the per-plane loads are plain float4 loads.
#pragma once

#include <initializer_list>

#include "evx_ch_plan.cuh"

namespace evx {
namespace fast {

constexpr int TZ = 64, TY = 16;
constexpr int W = TZ + 8;          // shared row width: z in [k0-4, k0+68)
constexpr int CR = TY + 4;         // field rows: y in [j0-2, j0+18)
constexpr int MR = TY + 2;         // potential rows: y in [j0-1, j0+17); row m <-> field row m+1
constexpr int NQ = W / 4;          // float4 per shared row
constexpr int NLOAD = CR * NQ;     // float4 loads per field plane (360)
constexpr int MPZ = (TZ + 4) / 2;  // 2x2 potential patches per row pair: cols 2..69
constexpr int MPY = MR / 2;
constexpr int NMU = MPZ * MPY;     // 306 potential patches per plane
constexpr int THREADS = 256;

__device__ __forceinline__ float4 ldg4(const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); }
__device__ __forceinline__ float2 lds2(const float* p) { return *reinterpret_cast<const float2*>(p); }
__device__ __forceinline__ void sts2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }
__device__ __forceinline__ void sts4(float* p, float4 v) { *reinterpret_cast<float4*>(p) = v; }
__device__ __forceinline__ float4 clip4(float4 v) {
    return make_float4(clip01(v.x), clip01(v.y), clip01(v.z), clip01(v.w));
}

// Per-thread load plan for one shared field plane (precomputed once per block).
struct LoadPlan {
    int goff[2];    // in-plane global offset of the float4 (wrapped)
    int soff[2];    // shared offset
    bool valid[2];
    bool own[2];    // inside the tile and the domain (written back in fused mode)
};

__device__ __forceinline__ LoadPlan make_load_plan(int tid, int j0, int k0, int ny, int nz) {
    LoadPlan L;
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const int e = tid + s * THREADS;
        L.valid[s] = e < NLOAD;
        const int row = L.valid[s] ? e / NQ : 0;
        const int q = L.valid[s] ? e - row * NQ : 0;
        const int gy = j0 + row - 2, gz = k0 + 4 * q - 4;
        L.own[s] = L.valid[s] && row >= 2 && row < 2 + TY && q >= 1 && q < 1 + TZ / 4 && gy < ny && gz < nz;
        L.goff[s] = pmod(gy, ny) * nz + pmod(gz, nz);
        L.soff[s] = row * W + 4 * q;
    }
    return L;
}

// Grid over (z tiles, y tiles, x chunks) sized to about one wave of resident blocks.
inline dim3 fast_grid(int nx, int ny, int nz, int blocks_per_sm, int sms, int* LX) {
    const int tz = (nz + TZ - 1) / TZ, ty = (ny + TY - 1) / TY;
    const long tiles = (long)tz * ty;
    const long slots = (long)blocks_per_sm * sms;
    long chunks = slots / tiles;                         // at most one wave: no partial second wave
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

int ch_rhs_fast_launch(bool fused, const float* u, const float* upd, float* u_new, float* r, const evx_grid* g,
                       const Geo& G, const ChP& P, cudaStream_t st);
int ch_pullback_fast_launch(bool grads, const float* u, const float* g, const float* lam, const float* h,
                            const float* u1, float* lam_out, double* part, int n_part_cap, const evx_grid* grid,
                            const Geo& G, const ChP& P, cudaStream_t st, int* n_part_used);
int ch_pullback_fast_blocks(const evx_grid* g);

}  // namespace evx
