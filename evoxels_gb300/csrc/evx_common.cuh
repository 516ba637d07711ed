// Shared device helpers for libevx (GB300 / sm_103a).
//
// Arithmetic convention: every translation unit is compiled with
// --fmad=false so each add/mul rounds separately, in the order the reference's
// torch elementwise ops round (one op = one rounding).  That makes the stencil
// parts bit-identical to the reference's float32 arithmetic.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <stddef.h>

#include "../../include/evx.h"

namespace evx {

// ---- error plumbing (host) -------------------------------------------------
void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);
int check_cuda(cudaError_t e, const char* where);
int check_launch(const char* where);

inline cudaStream_t as_stream(void* s) { return reinterpret_cast<cudaStream_t>(s); }

// Validate a grid + BC pair; returns EVX_OK or an error code with message set.
int validate_grid(const evx_grid* g);
int validate_bc(const evx_bc* bc);

inline size_t field_elems(const evx_grid* g) {
    return (size_t)g->nx * (size_t)g->ny * (size_t)g->nz;
}

// ---- device helpers ---------------------------------------------------------

// Non-negative modulo for periodic wrap; i may be any small negative/positive.
__device__ __forceinline__ int pmod(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}

// Kernel-side copy of evx_bc plus the grid factors, passed by value.
struct Geo {
    int nx, ny, nz;
    int kind[3];
    float lo[3], hi[3];        // float32(2*v) for Dirichlet axes
    float ih[3], ih2[3], ih2sum;
};

inline Geo make_geo(const evx_grid* g, const evx_bc* bc) {
    Geo o;
    o.nx = g->nx; o.ny = g->ny; o.nz = g->nz;
    for (int a = 0; a < 3; ++a) {
        o.kind[a] = bc ? bc->kind[a] : EVX_BC_PERIODIC;
        o.lo[a] = bc ? bc->two_v_lo[a] : 0.f;
        o.hi[a] = bc ? bc->two_v_hi[a] : 0.f;
        o.ih[a] = g->inv_h[a];
        o.ih2[a] = g->inv_h2[a];
    }
    o.ih2sum = g->inv_h2_sum;
    return o;
}

// Ghost value for a neighbour outside the domain along axis a, given the
// boundary cell's value (evoxels/boundary_conditions.py:47-55):
// Neumann -> the boundary value, Dirichlet -> float32(2v) - boundary value.
__device__ __forceinline__ float ghost_lo(const Geo& G, int a, float boundary) {
    return G.kind[a] == EVX_BC_NEUMANN ? boundary : __fsub_rn(G.lo[a], boundary);
}
__device__ __forceinline__ float ghost_hi(const Geo& G, int a, float boundary) {
    return G.kind[a] == EVX_BC_NEUMANN ? boundary : __fsub_rn(G.hi[a], boundary);
}

// 7-point Laplacian in the reference's association (evoxels/fd_stencils.py:70-74):
// ((R+L)*ih2x + (T+B)*ih2y) + (F+Bk)*ih2z - (2*C)*sum(ih2)
__device__ __forceinline__ float lap7(const Geo& G, float c, float xm, float xp,
                                      float ym, float yp, float zm, float zp) {
    float t = __fmul_rn(__fadd_rn(xp, xm), G.ih2[0]);
    t = __fadd_rn(t, __fmul_rn(__fadd_rn(yp, ym), G.ih2[1]));
    t = __fadd_rn(t, __fmul_rn(__fadd_rn(zp, zm), G.ih2[2]));
    return __fsub_rn(t, __fmul_rn(__fmul_rn(2.f, c), G.ih2sum));
}

// clip(u, 0, 1) as torch.clip: NaN propagates.
__device__ __forceinline__ float clip01(float u) {
    return u != u ? u : fminf(fmaxf(u, 0.f), 1.f);
}

// Default homogeneous chemical potential w*c*(1-c)*(1-2c)
// (evoxels/problem_definition.py:305), left to right as python evaluates it.
__device__ __forceinline__ float mu_hom(float w, float c) {
    float t = __fmul_rn(w, c);
    t = __fmul_rn(t, __fsub_rn(1.f, c));
    return __fmul_rn(t, __fsub_rn(1.f, __fmul_rn(2.f, c)));
}

// Regular-solution chemical potential log(c) - log(1-c) + w*(1-2c), in the
// reference notebook's operation order (docs/notebooks/01-using-solvers.ipynb:
// lib.log(c) - lib.log(1-c) + 3.0*(1-2*c)); CUDA's logf for the logarithms.
__device__ __forceinline__ float mu_regular(float w, float c) {
    const float t = __fsub_rn(logf(c), logf(__fsub_rn(1.f, c)));
    return __fadd_rn(t, __fmul_rn(w, __fsub_rn(1.f, __fmul_rn(2.f, c))));
}

// The bulk term selected by evx_ch_params.bulk.
__device__ __forceinline__ float mu_bulk(int bulk, float w, float c) {
    return bulk == EVX_BULK_REGULAR_SOLUTION ? mu_regular(w, c) : mu_hom(w, c);
}

// Face flux m(cf)*grad: (cf*(1-cf)) * ((mu_hi - mu_lo)*ih), cf = 0.5*(c_hi + c_lo)
// (evoxels/problem_definition.py:356-369, evoxels/fd_stencils.py:20-42).
__device__ __forceinline__ float face_flux(float c_lo, float c_hi, float mu_lo, float mu_hi, float ih) {
    float cf = __fmul_rn(0.5f, __fadd_rn(c_hi, c_lo));
    float m = __fmul_rn(cf, __fsub_rn(1.f, cf));
    return __fmul_rn(m, __fmul_rn(__fsub_rn(mu_hi, mu_lo), ih));
}

}  // namespace evx
