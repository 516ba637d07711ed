// Explicit finite-difference path: 7-point Laplacian with in-kernel ghost
// boundaries, advanced by forward Euler (ReactionDiffusion with f = 0).
//
// Reference arithmetic (one rounding per torch op, --fmad=false):
//   lap  = ((R+L)*ih2x + (T+B)*ih2y) + (F+Bk)*ih2z - (2*C)*sum(ih2)   evoxels/fd_stencils.py:70-74
//   rhs  = D*lap + 0                                                   evoxels/problem_definition.py:226-229
//   step = u + dt*rhs                                                  evoxels/timesteppers.py:42-43
// Ghosts (evoxels/boundary_conditions.py:33-59) are substituted on the fly:
// periodic wraps, Neumann repeats the boundary cell, Dirichlet uses 2v - cell.
//
// Kernels stream along x (the slowest axis): each thread owns one (y, z)
// column of a tile, keeps the x-1 / x / x+1 values in registers and reads the
// in-plane neighbours through L1.  A temporally blocked variant advances T
// steps per HBM pass with the intermediate planes held in shared memory.
#include <algorithm>

#include "evx_common.cuh"
#include "evx_prof.cuh"

namespace evx {

namespace {

constexpr int FD_BZ = 32;   // threads along z (one warp = one row segment)
constexpr int FD_BY = 8;    // threads along y

// mode 0: r = D*lap + 0 ; mode 1: u + dt*(D*lap + 0)
template <int MODE>
__global__ void __launch_bounds__(FD_BZ * FD_BY)
fd_stream_kernel(const float* __restrict__ u, float* __restrict__ out, Geo G, float D, float dt, int LX) {
    const int k = blockIdx.x * FD_BZ + threadIdx.x;
    const int j = blockIdx.y * FD_BY + threadIdx.y;
    if (j >= G.ny || k >= G.nz) return;  // no block-level synchronisation below
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    if (x0 >= x1) return;
    const size_t plane = (size_t)G.ny * G.nz;
    const int jk = j * G.nz + k;

    // in-plane neighbour offsets (or ghost flags) for this column
    const bool py = G.kind[1] == EVX_BC_PERIODIC, pz = G.kind[2] == EVX_BC_PERIODIC;
    const bool ylo_g = !py && j == 0, yhi_g = !py && j == G.ny - 1;
    const bool zlo_g = !pz && k == 0, zhi_g = !pz && k == G.nz - 1;
    const int jm = (j == 0 ? G.ny - 1 : j - 1) * G.nz + k;
    const int jp = (j == G.ny - 1 ? 0 : j + 1) * G.nz + k;
    const int km = j * G.nz + (k == 0 ? G.nz - 1 : k - 1);
    const int kp = j * G.nz + (k == G.nz - 1 ? 0 : k + 1);
    const bool px = G.kind[0] == EVX_BC_PERIODIC;

    float c = __ldg(u + (size_t)x0 * plane + jk);
    float xm;
    if (x0 > 0) xm = __ldg(u + (size_t)(x0 - 1) * plane + jk);
    else xm = px ? __ldg(u + (size_t)(G.nx - 1) * plane + jk) : ghost_lo(G, 0, c);

    for (int i = x0; i < x1; ++i) {
        const float* pl = u + (size_t)i * plane;
        float xp;
        if (i + 1 < G.nx) xp = __ldg(pl + plane + jk);
        else xp = px ? __ldg(u + jk) : ghost_hi(G, 0, c);
        const float ym = ylo_g ? ghost_lo(G, 1, c) : __ldg(pl + jm);
        const float yp = yhi_g ? ghost_hi(G, 1, c) : __ldg(pl + jp);
        const float zm = zlo_g ? ghost_lo(G, 2, c) : __ldg(pl + km);
        const float zp = zhi_g ? ghost_hi(G, 2, c) : __ldg(pl + kp);
        const float xm_eff = (i == 0 && !px) ? ghost_lo(G, 0, c) : xm;
        const float lap = lap7(G, c, xm_eff, xp, ym, yp, zm, zp);
        const float r = __fadd_rn(__fmul_rn(D, lap), 0.f);
        float o;
        if (MODE == 0) o = r;
        else o = __fadd_rn(c, __fmul_rn(dt, r));
        out[(size_t)i * plane + jk] = o;
        xm = c;
        c = xp;
    }
}

// ---- temporally blocked forward Euler --------------------------------------
// T steps per pass.  A block owns an (TY x TZ) output tile and streams along x.
// Stage s (s = 1..T) produces u^{s} on plane i - s + 1 over the tile grown by
// T - s cells in y and z, from three u^{s-1} planes kept in a shared ring.
// Periodic/ghost handling in y and z is resolved when stage 0 loads a plane
// (global coordinates are wrapped); ghosts of non-periodic axes are substituted
// from the centre value in every stage, exactly as the single-step kernel does.
constexpr int TB_TZ = 32, TB_TY = 16;

template <int T>
struct TbShape {
    static constexpr int HZ = TB_TZ + 2 * T;
    static constexpr int HY = TB_TY + 2 * T;
    static constexpr int PL = HY * HZ;  // elements per plane buffer
};

template <int T>
__global__ void __launch_bounds__(256)
fd_tblock_kernel(const float* __restrict__ u, float* __restrict__ out, Geo G, float D, float dt, int LX) {
    using S = TbShape<T>;
    extern __shared__ float sm[];
    // ring[s][3][PL]: stage s planes (s = 0 is the loaded input)
    float* ring = sm;
    const int tid = threadIdx.x;
    const int k0 = blockIdx.x * TB_TZ, j0 = blockIdx.y * TB_TY;
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    const size_t plane = (size_t)G.ny * G.nz;
    const bool px = G.kind[0] == EVX_BC_PERIODIC;
    const bool py = G.kind[1] == EVX_BC_PERIODIC, pz = G.kind[2] == EVX_BC_PERIODIC;

    auto slot = [&](int s, int p) -> float* { return ring + ((size_t)s * 3 + (size_t)((p % 3 + 3) % 3)) * S::PL; };

    // Planes needed at stage 0: x0 - T .. x1 - 1 + T.  Stage s plane p needs stage s-1 planes p-1..p+1.
    // Iterate over the input plane index q; after loading q, stage s computes plane q - s.
    const int qbeg = x0 - T, qend = x1 - 1 + T;
    for (int q = qbeg; q <= qend; ++q) {
        // stage 0: load plane q (wrapped for periodic x; skipped outside a non-periodic x domain)
        const bool q_in = px || (q >= 0 && q < G.nx);
        if (q_in) {
            const int gq = pmod(q, G.nx);
            float* dst = slot(0, q);
            for (int e = tid; e < S::PL; e += blockDim.x) {
                const int jj = e / S::HZ, kk = e - jj * S::HZ;
                int gj = j0 + jj - T, gk = k0 + kk - T;
                bool ok = true;
                if (py) gj = pmod(gj, G.ny); else ok = ok && gj >= 0 && gj < G.ny;
                if (pz) gk = pmod(gk, G.nz); else ok = ok && gk >= 0 && gk < G.nz;
                dst[e] = ok ? __ldg(u + (size_t)gq * plane + (size_t)gj * G.nz + gk) : 0.f;
            }
        }
        __syncthreads();
        // stages 1..T
#pragma unroll
        for (int s = 1; s <= T; ++s) {
            const int p = q - s;               // plane produced by this stage
            const bool p_in = px || (p >= 0 && p < G.nx);
            if (p >= x0 - (T - s) && p <= x1 - 1 + (T - s) && p_in) {
                const int gp = pmod(p, G.nx);
                const float* cm = slot(s - 1, p - 1);
                const float* cc = slot(s - 1, p);
                const float* cp = slot(s - 1, p + 1);
                float* dst = slot(s, p);
                const int grow = T - s;        // tile growth at this stage
                const int ny_s = TB_TY + 2 * grow, nz_s = TB_TZ + 2 * grow;
                const bool xlo_g = !px && gp == 0, xhi_g = !px && gp == G.nx - 1;
                for (int e = tid; e < ny_s * nz_s; e += blockDim.x) {
                    const int a = e / nz_s, b = e - a * nz_s;
                    const int jj = a + s, kk = b + s;  // coordinates in the HY x HZ buffer
                    const int gj = j0 + jj - T, gk = k0 + kk - T;
                    const int idx = jj * S::HZ + kk;
                    // points outside a non-periodic y/z domain are never consumed
                    if ((!py && (gj < 0 || gj >= G.ny)) || (!pz && (gk < 0 || gk >= G.nz))) {
                        if (s < T) dst[idx] = 0.f;
                        continue;
                    }
                    const int wj = py ? pmod(gj, G.ny) : gj, wk = pz ? pmod(gk, G.nz) : gk;
                    const float c = cc[idx];
                    const float xm = xlo_g ? ghost_lo(G, 0, c) : cm[idx];
                    const float xp = xhi_g ? ghost_hi(G, 0, c) : cp[idx];
                    const float ym = (!py && wj == 0) ? ghost_lo(G, 1, c) : cc[idx - S::HZ];
                    const float yp = (!py && wj == G.ny - 1) ? ghost_hi(G, 1, c) : cc[idx + S::HZ];
                    const float zm = (!pz && wk == 0) ? ghost_lo(G, 2, c) : cc[idx - 1];
                    const float zp = (!pz && wk == G.nz - 1) ? ghost_hi(G, 2, c) : cc[idx + 1];
                    const float lap = lap7(G, c, xm, xp, ym, yp, zm, zp);
                    const float r = __fadd_rn(__fmul_rn(D, lap), 0.f);
                    const float v = __fadd_rn(c, __fmul_rn(dt, r));
                    if (s == T) {
                        if (p >= x0 && p < x1 && gj >= j0 && gj < j0 + TB_TY && gj < G.ny &&
                            gk >= k0 && gk < k0 + TB_TZ && gk < G.nz && gj >= 0 && gk >= 0)
                            out[(size_t)p * plane + (size_t)gj * G.nz + gk] = v;
                    } else {
                        dst[idx] = v;
                    }
                }
            }
            __syncthreads();
        }
    }
}

__global__ void fe_update_kernel(const float* __restrict__ u, const float* __restrict__ r, float dt,
                                 float* __restrict__ out, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride)
        out[e] = __fadd_rn(__ldg(u + e), __fmul_rn(dt, __ldg(r + e)));
}

int fd_launch_grid(const evx_grid* g, dim3* grid, int* LX) {
    const int tz = (g->nz + FD_BZ - 1) / FD_BZ, ty = (g->ny + FD_BY - 1) / FD_BY;
    long tiles = (long)tz * ty;
    // enough blocks for ~8 per SM on a 152-SM part, but long x-runs for reuse
    long want = 8L * 152;
    int lx = (int)std::max<long>(4, std::min<long>(64, (long)g->nx * tiles / want));
    lx = std::min(lx, g->nx);
    *LX = lx;
    *grid = dim3(tz, ty, (g->nx + lx - 1) / lx);
    return EVX_OK;
}

template <int T>
int fd_tblock_launch(const float* in, float* out, const Geo& G, float D, float dt, cudaStream_t st) {
    using S = TbShape<T>;
    const int tz = (G.nz + TB_TZ - 1) / TB_TZ, ty = (G.ny + TB_TY - 1) / TB_TY;
    long tiles = (long)tz * ty;
    long want = 4L * 152;
    int lx = (int)std::max<long>(8, std::min<long>(128, (long)G.nx * tiles / want));
    lx = std::min(lx, G.nx);
    dim3 grid(tz, ty, (G.nx + lx - 1) / lx);
    size_t smem = (size_t)(T) * 3 * S::PL * sizeof(float);  // stages 0..T-1 are stored
    static bool configured = false;
    if (!configured) {
        cudaFuncSetAttribute(fd_tblock_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, 96 * 1024);
        configured = true;
    }
    EVX_TIMED(T == 2 ? "fd_tblock2" : "fd_tblock4", st, fd_tblock_kernel<T><<<grid, 256, smem, st>>>(in, out, G, D, dt, lx));
    count_launch();
    return check_launch("fd_tblock_kernel");
}

int fd_common_checks(const void* a, const void* b, const evx_grid* g, const evx_bc* bc) {
    int rc = validate_grid(g);
    if (rc) return rc;
    rc = validate_bc(bc);
    if (rc) return rc;
    if (!a || !b) return fail(EVX_ERR_BAD_ARG, "NULL field pointer");
    if (a == b) return fail(EVX_ERR_BAD_ARG, "input and output must not alias");
    return EVX_OK;
}

int fd_run(const float* u_in, float* u_out, float* scratch, const evx_grid* g, const Geo& G,
           float D, float dt, int nsteps, int spp, cudaStream_t st) {
    if (nsteps < 0) return fail(EVX_ERR_BAD_ARG, "nsteps must be >= 0");
    if (spp != 1 && spp != 2 && spp != 4) return fail(EVX_ERR_BAD_ARG, "steps_per_pass must be 1, 2 or 4");
    const size_t n = field_elems(g);
    if (nsteps == 0)
        return check_cuda(cudaMemcpyAsync(u_out, u_in, n * sizeof(float), cudaMemcpyDeviceToDevice, st),
                          "evx_fd_forward copy");
    // number of passes; buffers ping-pong so the last pass writes u_out
    int passes = 0;
    for (int s = 0; s < nsteps;) { int t = std::min(spp, nsteps - s); while (t != 1 && t != 2 && t != 4) --t; s += t; ++passes; }
    if (passes > 1 && (!scratch || scratch == u_in || scratch == u_out))
        return fail(EVX_ERR_WORKSPACE, "scratch field required (distinct from input and output) for more than one pass");
    dim3 grid; int lx;
    fd_launch_grid(g, &grid, &lx);
    const float* src = u_in;
    int pass = 0;
    for (int s = 0; s < nsteps; ++pass) {
        int t = std::min(spp, nsteps - s);
        while (t != 1 && t != 2 && t != 4) --t;
        float* dst = ((passes - 1 - pass) % 2 == 0) ? u_out : scratch;
        int rc;
        if (t == 1) {
            EVX_TIMED("fd_step", st, fd_stream_kernel<1><<<grid, dim3(FD_BZ, FD_BY), 0, st>>>(src, dst, G, D, dt, lx));
            count_launch();
            rc = check_launch("fd_stream_kernel");
        } else if (t == 2) {
            rc = fd_tblock_launch<2>(src, dst, G, D, dt, st);
        } else {
            rc = fd_tblock_launch<4>(src, dst, G, D, dt, st);
        }
        if (rc) return rc;
        src = dst;
        s += t;
    }
    return EVX_OK;
}

}  // namespace

}  // namespace evx

using namespace evx;

extern "C" {

int evx_rd_rhs(const float* u, float* r, const evx_grid* g, const evx_bc* bc, float D, void* stream) {
    int rc = fd_common_checks(u, r, g, bc);
    if (rc) return rc;
    Geo G = make_geo(g, bc);
    dim3 grid; int lx;
    fd_launch_grid(g, &grid, &lx);
    EVX_TIMED("rd_rhs", as_stream(stream), fd_stream_kernel<0><<<grid, dim3(FD_BZ, FD_BY), 0, as_stream(stream)>>>(u, r, G, D, 0.f, lx));
    count_launch();
    return check_launch("evx_rd_rhs");
}

int evx_fe_update(const float* u, const float* r, float dt, float* out, size_t n, void* stream) {
    if (!u || !r || !out) return fail(EVX_ERR_BAD_ARG, "NULL field pointer");
    if (n == 0) return EVX_OK;
    const size_t blocks = std::min<size_t>((n + 255) / 256, (size_t)152 * 16);
    EVX_TIMED("fe_update", as_stream(stream), fe_update_kernel<<<(unsigned)blocks, 256, 0, as_stream(stream)>>>(u, r, dt, out, n));
    count_launch();
    return check_launch("evx_fe_update");
}

int evx_fd_forward(const float* u_in, float* u_out, float* scratch, const evx_grid* g, const evx_bc* bc,
                   float D, float dt, int nsteps, int steps_per_pass, void* stream) {
    int rc = fd_common_checks(u_in, u_out, g, bc);
    if (rc) return rc;
    Geo G = make_geo(g, bc);
    return fd_run(u_in, u_out, scratch, g, G, D, dt, nsteps, steps_per_pass, as_stream(stream));
}

int evx_fd_adjoint(const float* lam_in, float* lam_out, float* scratch, const evx_grid* g, const evx_bc* bc,
                   float D, float dt, int nsteps, void* stream) {
    int rc = fd_common_checks(lam_in, lam_out, g, bc);
    if (rc) return rc;
    // The Jacobian of u + dt*D*lap(pad_bc(u)) is I + dt*D*L0, where L0 is the
    // Laplacian with homogeneous ghosts (Dirichlet values set to 0); L0 is
    // symmetric for periodic, Neumann and Dirichlet ghosts, so the adjoint
    // step is the forward step with the Dirichlet values zeroed.
    evx_bc hb;
    if (bc) hb = *bc; else { for (int a = 0; a < 3; ++a) hb.kind[a] = EVX_BC_PERIODIC; }
    for (int a = 0; a < 3; ++a) { hb.two_v_lo[a] = 0.f; hb.two_v_hi[a] = 0.f; }
    Geo G = make_geo(g, &hb);
    return fd_run(lam_in, lam_out, scratch, g, G, D, dt, nsteps, 1, as_stream(stream));
}

}  // extern "C"
