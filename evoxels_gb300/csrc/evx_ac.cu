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
// Tiling: a 64 (z) x 8 (y) block of 256 threads streams along x; each thread
// owns two z-adjacent outputs: sums and differences as two-lane .rn
// instructions, products and divisions as scalar roundings (a two-lane multiply
// may be fused into a following add by the code generator), every lane exactly
// the scalar operation in the reference's order.
// Planes of the ghosted clipped field, (8+2) x (64+2) cells, sit in a 4-slot
// shared ring, so one block barrier per plane suffices (the slot written next
// was last read two planes ago).  The next plane's cells are loaded into
// registers before the current plane is computed.  Per staged cell the
// wrapped/clamped (y, z) offset and its boundary maps are fixed per tile; per
// plane only the x index and the x map change.
#include <algorithm>

#include "evx_ch_fast.cuh"
#include "evx_common.cuh"
#include "evx_prof.cuh"

namespace evx {
namespace {

using fast::f2s;

using fast::exact::add2;
using fast::exact::mul2;
using fast::exact::sub2;
using fast::exact::mul2_nofuse;   // products whose result only feeds products, or exact ones

constexpr int AZ = 64, AY = 8;                // output tile
constexpr int PW = AZ + 4;                    // shared row: z in [k0-2, k0+AZ+2), cell z at z-k0+2
constexpr int PR = AY + 2;                    // rows: y in [j0-1, j0+AY]
constexpr int PLANE = PR * PW;
constexpr int NCELL = PR * (AZ + 2);          // staged cells per plane
constexpr int CPT = (NCELL + 255) / 256;      // staged cells per thread
constexpr int AC_THREADS = 256;

struct AcP {
    float w, eps, gab, M, force, three_over_eps, curv, one_minus_curv;
};

// One staged cell: in-plane offset of its source (wrapped / clamped), shared
// offset, and the y / z boundary maps to apply (0 none, 1 low side, 2 high side).
struct Cell {
    int off, soff, fy, fz;
};

__device__ __forceinline__ float bc_map(const Geo& G, int a, int side, float v) {
    return side == 1 ? ghost_lo(G, a, v) : (side == 2 ? ghost_hi(G, a, v) : v);
}

// ((R - 2C) + L), two lanes
__device__ __forceinline__ float2 d2x2(float2 R, float2 C, float2 L) {
    return add2(sub2(R, mul2_nofuse(f2s(2.f), C)), L);
}
// ((pp + mm) - mp) - pm
__device__ __forceinline__ float2 mixed2(float2 pp, float2 mm, float2 mp, float2 pm) {
    return sub2(sub2(add2(pp, mm), mp), pm);
}
// ((((0.5*ga)*gb)*m)*ia)*ib
__device__ __forceinline__ float2 cross2(float2 ga, float2 gb, float2 m, float2 ia, float2 ib) {
    return mul2(mul2_nofuse(mul2_nofuse(mul2_nofuse(mul2_nofuse(f2s(0.5f), ga), gb), m), ia), ib);
}

__global__ void __launch_bounds__(AC_THREADS)
ac_rhs_kernel(const float* __restrict__ u, const float* __restrict__ kst, float cst, float* __restrict__ r, Geo G,
              AcP P, int LX) {
    __shared__ __align__(16) float ring[4][PLANE];
    const int tid = threadIdx.x;
    const int tx = tid & 31, ty = tid >> 5;
    const int k0 = blockIdx.x * AZ, j0 = blockIdx.y * AY;
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    if (x0 >= x1) return;   // uniform across the block
    const int nx = G.nx, ny = G.ny, nz = G.nz;
    const size_t plane = (size_t)ny * nz;
    const bool perx = G.kind[0] == EVX_BC_PERIODIC, pery = G.kind[1] == EVX_BC_PERIODIC,
               perz = G.kind[2] == EVX_BC_PERIODIC;

    // per-tile staging plan; cells beyond the ghost layer are never read by
    // in-domain outputs and are staged as 0
    Cell cell[CPT];
#pragma unroll
    for (int s = 0; s < CPT; ++s) {
        const int e = tid + s * AC_THREADS;
        Cell c{-1, 0, 0, 0};
        if (e < NCELL) {
            const int row = e / (AZ + 2), col = e - row * (AZ + 2);
            const int y = j0 + row - 1, z = k0 + col - 1;
            c.soff = row * PW + col + 1;
            if (y <= ny && z <= nz) {
                int yi = y, zi = z;
                if (y < 0) { yi = pery ? y + ny : 0; c.fy = pery ? 0 : 1; }
                if (y >= ny) { yi = pery ? y - ny : ny - 1; c.fy = pery ? 0 : 2; }
                if (z < 0) { zi = perz ? z + nz : 0; c.fz = perz ? 0 : 1; }
                if (z >= nz) { zi = perz ? z - nz : nz - 1; c.fz = perz ? 0 : 2; }
                c.off = yi * nz + zi;
            }
        } else {
            c.soff = -1;
        }
        cell[s] = c;
    }
    float pre[CPT];
    auto fetch = [&](int x) {   // raw values of plane x into registers
        const int xi = x < 0 ? (perx ? x + nx : 0) : (x >= nx ? (perx ? x - nx : nx - 1) : x);
        const float* src = u + (size_t)xi * plane;
        if (kst) {   // a Runge-Kutta stage input u + c*k, rounded as evx_fe_update rounds it
            const float* ks = kst + (size_t)xi * plane;
#pragma unroll
            for (int s = 0; s < CPT; ++s)
                pre[s] = cell[s].off >= 0 ? __fadd_rn(__ldg(src + cell[s].off), __fmul_rn(cst, __ldg(ks + cell[s].off)))
                                          : 0.f;
        } else {
#pragma unroll
            for (int s = 0; s < CPT; ++s) pre[s] = cell[s].off >= 0 ? __ldg(src + cell[s].off) : 0.f;
        }
    };
    auto stash = [&](int x) {   // clip, boundary maps in x, y, z order, into the ring
        float* dst = ring[x & 3];
        const int fx = perx ? 0 : (x < 0 ? 1 : (x >= nx ? 2 : 0));
#pragma unroll
        for (int s = 0; s < CPT; ++s) {
            if (cell[s].soff < 0) continue;
            float v = 0.f;
            if (cell[s].off >= 0) {
                v = clip01(pre[s]);
                v = bc_map(G, 0, fx, v);
                v = bc_map(G, 1, cell[s].fy, v);
                v = bc_map(G, 2, cell[s].fz, v);
            }
            dst[cell[s].soff] = v;
        }
    };

    const float2 dx0 = f2s(G.ih[0]), dx1 = f2s(G.ih[1]), dx2 = f2s(G.ih[2]);
    const float2 q0 = f2s(G.ih2[0]), q1 = f2s(G.ih2[1]), q2 = f2s(G.ih2[2]), qs = f2s(G.ih2sum);
    const float2 curv = f2s(P.curv), omc = f2s(P.one_minus_curv), w2 = f2s(P.w), gab = f2s(P.gab),
                 toe = f2s(P.three_over_eps), force = f2s(P.force), M = f2s(P.M);
    const int j = j0 + ty, k = k0 + 2 * tx;
    const bool outA = j < ny && k < nz, outB = j < ny && k + 1 < nz;
    const bool vec = outB && (nz % 2 == 0);
    const int c = (ty + 1) * PW + 2 * tx + 2;

    fetch(x0 - 1);
    stash(x0 - 1);
    fetch(x0);
    stash(x0);
    fetch(x0 + 1);
    for (int i = x0; i < x1; ++i) {
        stash(i + 1);
        if (i + 2 <= x1) fetch(i + 2);
        __syncthreads();
        if (outA) {
            const float* m = ring[(i - 1) & 3];
            const float* o = ring[i & 3];
            const float* p = ring[(i + 1) & 3];
            const float2 C = *reinterpret_cast<const float2*>(o + c);
            const float2 L = *reinterpret_cast<const float2*>(m + c);
            const float2 R = *reinterpret_cast<const float2*>(p + c);
            const float2 B = *reinterpret_cast<const float2*>(o + c - PW);
            const float2 T = *reinterpret_cast<const float2*>(o + c + PW);
            const float2 Bk = make_float2(o[c - 1], C.x), F = make_float2(C.y, o[c + 2]);
            const float2 gx = mul2_nofuse(mul2_nofuse(f2s(0.5f), sub2(R, L)), dx0);
            const float2 gy = mul2_nofuse(mul2_nofuse(f2s(0.5f), sub2(T, B)), dx1);
            const float2 gz = mul2_nofuse(mul2_nofuse(f2s(0.5f), sub2(F, Bk)), dx2);
            const float2 gx2 = mul2(gx, gx), gy2 = mul2(gy, gy), gz2 = mul2(gz, gz);
            float2 n = mul2(mul2_nofuse(gx2, d2x2(R, C, L)), q0);
            n = add2(n, mul2(mul2_nofuse(gy2, d2x2(T, C, B)), q1));
            n = add2(n, mul2(mul2_nofuse(gz2, d2x2(F, C, Bk)), q2));
            {   // xy: f(x+1,y+1) + f(x-1,y-1) - f(x-1,y+1) - f(x+1,y-1)
                const float2 pp = *reinterpret_cast<const float2*>(p + c + PW);
                const float2 mm = *reinterpret_cast<const float2*>(m + c - PW);
                const float2 mp = *reinterpret_cast<const float2*>(m + c + PW);
                const float2 pm = *reinterpret_cast<const float2*>(p + c - PW);
                n = add2(n, cross2(gx, gy, mixed2(pp, mm, mp, pm), dx0, dx1));
            }
            {   // xz
                const float2 pp = make_float2(R.y, p[c + 2]), mm = make_float2(m[c - 1], L.x);
                const float2 mp = make_float2(L.y, m[c + 2]), pm = make_float2(p[c - 1], R.x);
                n = add2(n, cross2(gx, gz, mixed2(pp, mm, mp, pm), dx0, dx2));
            }
            {   // yz
                const float2 pp = make_float2(T.y, o[c + PW + 2]), mm = make_float2(o[c - PW - 1], B.x);
                const float2 mp = make_float2(B.y, o[c - PW + 2]), pm = make_float2(o[c + PW - 1], T.x);
                n = add2(n, cross2(gy, gz, mixed2(pp, mm, mp, pm), dx1, dx2));
            }
            float2 norm2 = add2(add2(gx2, gy2), gz2);
            if (norm2.x <= 1e-7f) norm2.x = 1.f;
            if (norm2.y <= 1e-7f) norm2.y = 1.f;
            const float2 nlap = mul2(omc, make_float2(__fdiv_rn(n.x, norm2.x), __fdiv_rn(n.y, norm2.y)));
            // 7-point Laplacian: ((R+L)*ih2x + (T+B)*ih2y) + (F+Bk)*ih2z - (2C)*sum(ih2)
            float2 t = mul2(add2(R, L), q0);
            t = add2(t, mul2(add2(T, B), q1));
            t = add2(t, mul2(add2(F, Bk), q2));
            const float2 lap = mul2(curv, sub2(t, mul2(mul2_nofuse(f2s(2.f), C), qs)));
            // w*c*(1-c)*(1-2c); pot/2 as pot*0.5 (the same correctly rounded value)
            const float2 omC = sub2(f2s(1.f), C);
            const float2 pot = mul2_nofuse(mul2_nofuse(mul2_nofuse(w2, C), omC),
                                           sub2(f2s(1.f), mul2_nofuse(f2s(2.f), C)));   // feeds *0.5
            const float2 ph = mul2_nofuse(pot, f2s(0.5f));                               // feeds a division
            const float2 pot2 = make_float2(__fdiv_rn(ph.x, P.eps), __fdiv_rn(ph.y, P.eps));
            const float2 df = add2(mul2(gab, sub2(add2(lap, nlap), pot2)),
                                   mul2(mul2_nofuse(mul2_nofuse(toe, C), omC), force));
            const float2 res = mul2_nofuse(M, df);   // stored
            float* dst = r + ((size_t)i * ny + j) * nz + k;
            if (vec) {
                *reinterpret_cast<float2*>(dst) = res;
            } else {
                dst[0] = res.x;
                if (outB) dst[1] = res.y;
            }
        }
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

namespace {
int ac_rhs_launch(const float* u, const float* k, float c, float* r, const evx_grid* g, const evx_bc* bc,
                  const evx_ac_params* p, void* stream) {
    int rc = validate_grid(g);
    if (rc) return rc;
    if ((rc = validate_bc(bc))) return rc;
    if (!p) return fail(EVX_ERR_BAD_ARG, "params are NULL");
    if (!u || !r) return fail(EVX_ERR_BAD_ARG, "NULL field pointer");
    if (u == r || k == r) return fail(EVX_ERR_BAD_ARG, "input and output must not alias");
    if (!(p->eps != 0.f) || !std::isfinite(p->eps)) return fail(EVX_ERR_BAD_ARG, "eps must be finite and non-zero");
    const AcP P{p->w, p->eps, p->gab, p->M, p->force, p->three_over_eps, p->curvature, p->one_minus_curvature};
    const Geo G = make_geo(g, bc);
    static int slots = 0;   // resident blocks on the device
    if (!slots) {
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ac_rhs_kernel, AC_THREADS, 0);
        slots = std::max(1, sms) * std::max(1, per);
    }
    const int tz = (g->nz + AZ - 1) / AZ, ty = (g->ny + AY - 1) / AY;
    // x chunks: one wave of resident blocks, at least 8 planes each (the x halo is 2 planes)
    const long tiles = (long)tz * ty;
    const long chunks = std::max<long>(1, slots / tiles);
    int lx = (int)std::max<long>(8, (g->nx + chunks - 1) / chunks);
    lx = std::min(lx, g->nx);
    const dim3 grid(tz, ty, (g->nx + lx - 1) / lx);
    cudaStream_t st = as_stream(stream);
    EVX_TIMED("ac_rhs", st, ac_rhs_kernel<<<grid, AC_THREADS, 0, st>>>(u, k, c, r, G, P, lx));
    count_launch();
    return check_launch("ac_rhs_kernel");
}
}  // namespace

int evx_ac_rhs(const float* u, float* r, const evx_grid* g, const evx_bc* bc, const evx_ac_params* p,
               void* stream) {
    return ac_rhs_launch(u, nullptr, 0.f, r, g, bc, p, stream);
}

int evx_ac_rhs_stage(const float* u, const float* k, float c, float* r, const evx_grid* g, const evx_bc* bc,
                     const evx_ac_params* p, void* stream) {
    if (!k) return fail(EVX_ERR_BAD_ARG, "NULL stage field");
    return ac_rhs_launch(u, k, c, r, g, bc, p, stream);
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
