// Two-phase Allen-Cahn right-hand side (evoxels/problem_definition.py:374-447)
// with the compact 19-point normal Laplacian (evoxels/fd_stencils.py:77-103),
// the combination step of the classical Runge-Kutta scheme
// (evoxels/timesteppers.py:46-61) and the stage recursion of the
// Runge-Kutta-Chebyshev schemes (evoxels/timesteppers.py:202-295).  Compiled with --fmad=false: every float32
// operation rounds separately, in the reference's order, so results are
// bit-identical to the reference's torch arithmetic.
//
//   phi = clip(u, 0, 1); pot = w*phi*(1-phi)*(1-2phi)
//   lap = curvature * L(phi); nlap = (1 - curvature) * N(phi)
//   r = M * (gab * ((lap + nlap) - pot/2/eps) + 3/eps*phi*(1-phi)*force)
//   N = [sum_a g_a^2 (f+a - 2f + f-a) ih2_a + sum_(a<b) 0.5 g_a g_b (f++ + f-- - f-+ - f+-) ih_a ih_b] / |g|^2,
//       g_a = 0.5 (f+a - f-a) ih_a, |g|^2 := 1 where |g|^2 <= 1e-7.
//
// Ghost cells.  The reference pads the clipped field periodically and then, axis
// by axis in x, y, z order, overwrites the two ghost slabs of every
// non-periodic axis (Neumann: copy of the adjacent cell, Dirichlet: 2v minus
// it) - whole slabs, ghost rows of the other axes included.  The mixed second
// differences read edge ghosts (two coordinates outside), which that sequence
// makes: value of the interior cell reached by wrapping periodic and clamping
// non-periodic coordinates, then the x, then the y, then the z boundary map of
// each non-periodic axis the point lies outside of.
//
// Tiling: a 32 (z) x 8 (y) block streams along x through a 3-slot ring of
// shared planes, each (8+2) x (32+2) cells of the ghosted field.
#include "evx_common.cuh"
#include "evx_prof.cuh"

namespace evx {
namespace {

constexpr int AZ = 32, AY = 8;              // output tile
constexpr int PZ = AZ + 2, PY = AY + 2;     // plane with halo
constexpr int PLANE = PZ * PY;

struct AcP {
    float w, eps, gab, M, force, three_over_eps, curv, one_minus_curv;
};

// Value of the ghosted (padded) clipped field at (x, y, z), each coordinate in [-1, n].
__device__ __forceinline__ float ghosted(const float* __restrict__ u, const Geo& G, int x, int y, int z) {
    const bool ox = x < 0 || x >= G.nx, oy = y < 0 || y >= G.ny, oz = z < 0 || z >= G.nz;
    auto fix = [](int c, int n, bool per) {
        if (c < 0) return per ? c + n : 0;
        if (c >= n) return per ? c - n : n - 1;
        return c;
    };
    const int xi = fix(x, G.nx, G.kind[0] == EVX_BC_PERIODIC);
    const int yi = fix(y, G.ny, G.kind[1] == EVX_BC_PERIODIC);
    const int zi = fix(z, G.nz, G.kind[2] == EVX_BC_PERIODIC);
    float v = clip01(__ldg(u + ((size_t)xi * G.ny + yi) * G.nz + zi));
    if (ox && G.kind[0] != EVX_BC_PERIODIC) v = x < 0 ? ghost_lo(G, 0, v) : ghost_hi(G, 0, v);
    if (oy && G.kind[1] != EVX_BC_PERIODIC) v = y < 0 ? ghost_lo(G, 1, v) : ghost_hi(G, 1, v);
    if (oz && G.kind[2] != EVX_BC_PERIODIC) v = z < 0 ? ghost_lo(G, 2, v) : ghost_hi(G, 2, v);
    return v;
}

// ((R - 2C) + L)
__device__ __forceinline__ float d2(float R, float C, float L) {
    return __fadd_rn(__fsub_rn(R, __fmul_rn(2.f, C)), L);
}
// ((pp + mm) - mp) - pm
__device__ __forceinline__ float mixed(float pp, float mm, float mp, float pm) {
    return __fsub_rn(__fsub_rn(__fadd_rn(pp, mm), mp), pm);
}

__global__ void __launch_bounds__(AZ * AY)
ac_rhs_kernel(const float* __restrict__ u, float* __restrict__ r, Geo G, AcP P, int LX) {
    __shared__ float ring[3][PLANE];
    const int tz = threadIdx.x, ty = threadIdx.y, tid = ty * AZ + tz;
    const int k0 = blockIdx.x * AZ, j0 = blockIdx.y * AY;
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    if (x0 >= x1) return;   // uniform across the block
    auto load = [&](int x) {
        float* dst = ring[(x + 3) % 3];
        for (int e = tid; e < PLANE; e += AZ * AY) {
            const int py = e / PZ, pz = e - py * PZ;
            const int y = j0 + py - 1, z = k0 + pz - 1;
            // cells beyond the ghost layer are never read by in-domain outputs
            dst[e] = (y <= G.ny && z <= G.nz) ? ghosted(u, G, x, y, z) : 0.f;
        }
    };
    const float dx0 = G.ih[0], dx1 = G.ih[1], dx2 = G.ih[2];
    const float q0 = G.ih2[0], q1 = G.ih2[1], q2 = G.ih2[2];
    const int j = j0 + ty, k = k0 + tz;
    const bool out = j < G.ny && k < G.nz;
    const int c = (ty + 1) * PZ + (tz + 1);
    load(x0 - 1);
    load(x0);
    for (int i = x0; i < x1; ++i) {
        load(i + 1);
        __syncthreads();
        const float* m = ring[(i + 2) % 3];   // plane i-1
        const float* o = ring[i % 3];
        const float* p = ring[(i + 1) % 3];
        if (out) {
            const float C = o[c];
            const float L = m[c], R = p[c];
            const float B = o[c - PZ], T = o[c + PZ];
            const float Bk = o[c - 1], F = o[c + 1];
            const float gx = __fmul_rn(__fmul_rn(0.5f, __fsub_rn(R, L)), dx0);
            const float gy = __fmul_rn(__fmul_rn(0.5f, __fsub_rn(T, B)), dx1);
            const float gz = __fmul_rn(__fmul_rn(0.5f, __fsub_rn(F, Bk)), dx2);
            const float gx2 = __fmul_rn(gx, gx), gy2 = __fmul_rn(gy, gy), gz2 = __fmul_rn(gz, gz);
            float n = __fmul_rn(__fmul_rn(gx2, d2(R, C, L)), q0);
            n = __fadd_rn(n, __fmul_rn(__fmul_rn(gy2, d2(T, C, B)), q1));
            n = __fadd_rn(n, __fmul_rn(__fmul_rn(gz2, d2(F, C, Bk)), q2));
            // 0.5 * g_a * g_b * (f++ + f-- - f-+ - f+-) * ih_a * ih_b, left to right
            auto cross = [](float ga, float gb, float m, float ia, float ib) {
                return __fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(__fmul_rn(0.5f, ga), gb), m), ia), ib);
            };
            n = __fadd_rn(n, cross(gx, gy, mixed(p[c + PZ], m[c - PZ], m[c + PZ], p[c - PZ]), dx0, dx1));   // xy
            n = __fadd_rn(n, cross(gx, gz, mixed(p[c + 1], m[c - 1], m[c + 1], p[c - 1]), dx0, dx2));       // xz
            n = __fadd_rn(n, cross(gy, gz, mixed(o[c + PZ + 1], o[c - PZ - 1], o[c - PZ + 1], o[c + PZ - 1]),
                                   dx1, dx2));                                                              // yz
            float norm2 = __fadd_rn(__fadd_rn(gx2, gy2), gz2);
            if (norm2 <= 1e-7f) norm2 = 1.f;
            const float nlap = __fmul_rn(P.one_minus_curv, __fdiv_rn(n, norm2));
            const float lap = __fmul_rn(P.curv, lap7(G, C, L, R, B, T, Bk, F));
            const float pot = mu_hom(P.w, C);
            const float pot2 = __fdiv_rn(__fdiv_rn(pot, 2.f), P.eps);
            const float df = __fadd_rn(__fmul_rn(P.gab, __fsub_rn(__fadd_rn(lap, nlap), pot2)),
                                       __fmul_rn(__fmul_rn(__fmul_rn(P.three_over_eps, C), __fsub_rn(1.f, C)),
                                                 P.force));
            r[((size_t)i * G.ny + j) * G.nz + k] = __fmul_rn(P.M, df);
        }
        __syncthreads();   // slot (i+2)%3 is reloaded with plane i+2 next
    }
}

// out = u + dt6 * (((k1 + 2 k2) + 2 k3) + k4)   (evoxels/timesteppers.py:61)
__global__ void rk4_combine_kernel(const float* __restrict__ u, const float* __restrict__ k1,
                                   const float* __restrict__ k2, const float* __restrict__ k3,
                                   const float* __restrict__ k4, float dt6, float* __restrict__ out, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
        float s = __fadd_rn(__ldg(k1 + e), __fmul_rn(2.f, __ldg(k2 + e)));
        s = __fadd_rn(s, __fmul_rn(2.f, __ldg(k3 + e)));
        s = __fadd_rn(s, __ldg(k4 + e));
        out[e] = __fadd_rn(__ldg(u + e), __fmul_rn(dt6, s));
    }
}

// RKC stage (evoxels/timesteppers.py:237-243, 286-294), left to right:
//   out = mu0*yc + nu*yp + omn*u + m1dt*r [+ gdt*r0]
template <bool R0>
__global__ void rkc_stage_kernel(const float* __restrict__ u, const float* __restrict__ yc,
                                 const float* __restrict__ yp, const float* __restrict__ r,
                                 const float* __restrict__ r0, float mu0, float nu, float omn, float m1dt, float gdt,
                                 float* __restrict__ out, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
        float s = __fadd_rn(__fmul_rn(mu0, __ldg(yc + e)), __fmul_rn(nu, __ldg(yp + e)));
        s = __fadd_rn(s, __fmul_rn(omn, __ldg(u + e)));
        s = __fadd_rn(s, __fmul_rn(m1dt, __ldg(r + e)));
        if constexpr (R0) s = __fadd_rn(s, __fmul_rn(gdt, __ldg(r0 + e)));
        out[e] = s;
    }
}

}  // namespace
}  // namespace evx

using namespace evx;

extern "C" {

int evx_ac_rhs(const float* u, float* r, const evx_grid* g, const evx_bc* bc, const evx_ac_params* p,
               void* stream) {
    int rc = validate_grid(g);
    if (rc) return rc;
    if ((rc = validate_bc(bc))) return rc;
    if (!p) return fail(EVX_ERR_BAD_ARG, "params are NULL");
    if (!u || !r) return fail(EVX_ERR_BAD_ARG, "NULL field pointer");
    if (u == r) return fail(EVX_ERR_BAD_ARG, "input and output must not alias");
    if (!(p->eps != 0.f) || !std::isfinite(p->eps)) return fail(EVX_ERR_BAD_ARG, "eps must be finite and non-zero");
    const AcP P{p->w, p->eps, p->gab, p->M, p->force, p->three_over_eps, p->curvature, p->one_minus_curvature};
    const Geo G = make_geo(g, bc);
    const int tz = (g->nz + AZ - 1) / AZ, ty = (g->ny + AY - 1) / AY;
    // x chunks: about 8 resident blocks per SM on a 152-SM part, at least 4 planes each
    const long tiles = (long)tz * ty;
    int lx = (int)std::max<long>(4, std::min<long>(g->nx, (long)g->nx * tiles / (8L * 152)));
    lx = std::min(lx, g->nx);
    const dim3 grid(tz, ty, (g->nx + lx - 1) / lx);
    cudaStream_t st = as_stream(stream);
    EVX_TIMED("ac_rhs", st, ac_rhs_kernel<<<grid, dim3(AZ, AY), 0, st>>>(u, r, G, P, lx));
    count_launch();
    return check_launch("ac_rhs_kernel");
}

int evx_rk4_combine(const float* u, const float* k1, const float* k2, const float* k3, const float* k4, float dt6,
                    float* out, size_t n, void* stream) {
    if (!u || !k1 || !k2 || !k3 || !k4 || !out) return fail(EVX_ERR_BAD_ARG, "NULL pointer");
    if (n == 0) return EVX_OK;
    cudaStream_t st = as_stream(stream);
    const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)152 * 16);
    EVX_TIMED("rk4_combine", st, rk4_combine_kernel<<<blocks, 256, 0, st>>>(u, k1, k2, k3, k4, dt6, out, n));
    count_launch();
    return check_launch("rk4_combine_kernel");
}

int evx_rkc_stage(const float* u, const float* y_curr, const float* y_prev, const float* r, const float* r0,
                  const evx_rkc_coeffs* c, float* out, size_t n, void* stream) {
    if (!u || !y_curr || !y_prev || !r || !out || !c) return fail(EVX_ERR_BAD_ARG, "NULL pointer");
    if (n == 0) return EVX_OK;
    cudaStream_t st = as_stream(stream);
    const int blocks = (int)std::min<size_t>((n + 255) / 256, (size_t)152 * 16);
    if (r0)
        EVX_TIMED("rkc2_stage", st, (rkc_stage_kernel<true><<<blocks, 256, 0, st>>>(
                                        u, y_curr, y_prev, r, r0, c->mu0, c->nu, c->one_minus_mu0_nu, c->mu1_dt,
                                        c->gamma_dt, out, n)));
    else
        EVX_TIMED("rkc_stage", st, (rkc_stage_kernel<false><<<blocks, 256, 0, st>>>(
                                        u, y_curr, y_prev, r, nullptr, c->mu0, c->nu, c->one_minus_mu0_nu, c->mu1_dt,
                                        0.f, out, n)));
    count_launch();
    return check_launch("rkc_stage_kernel");
}

}  // extern "C"
