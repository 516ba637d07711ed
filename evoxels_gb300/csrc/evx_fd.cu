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

// ---- temporally blocked forward Euler (fast path) ------------------------------
// T steps per HBM pass, T in {1, 2, 4}.  A block of 256 threads owns a 16 x 64
// (y, z) output tile and streams along x.  Level 0 holds input planes staged
// in shared memory with a halo of T rows in y and 4 columns in z (4 keeps every
// row float4-aligned); level s (1..T) holds u^{s} on plane q - s, computed from
// three level-(s-1) planes kept in a 3-slot ring.  Level T goes to global
// memory.  Work items are float4 groups along z, so the inner stencil is four
// points wide; ghosts of non-periodic axes are substituted from the centre
// value at every level, exactly as in the single-step kernel, so every T gives
// bit-identical results.  Requires nz % 4 == 0 and 16-byte aligned fields.
constexpr int TB_TZ = 64, TB_TY = 16, TB_W = TB_TZ + 8, TB_NQ = TB_W / 4;

template <int T>
struct TbShape {
    static constexpr int R = TB_TY + 2 * T;     // rows per level plane
    static constexpr int PL = R * TB_W;          // floats per level plane
    static constexpr size_t SMEM = (size_t)T * 3 * PL * sizeof(float);   // levels 0..T-1
};

template <bool UNIT>
__device__ __forceinline__ float fd_point(const Geo& G, float D, float dt, float c, float xm, float xp, float ym,
                                          float yp, float zm, float zp) {
    float lap;
    if (UNIT) {   // all inv_h2 == 1: dropping the multiplications by 1.0f is exact
        float t = __fadd_rn(xp, xm);
        t = __fadd_rn(t, __fadd_rn(yp, ym));
        t = __fadd_rn(t, __fadd_rn(zp, zm));
        lap = __fsub_rn(t, __fmul_rn(__fmul_rn(2.f, c), G.ih2sum));
    } else {
        lap = lap7(G, c, xm, xp, ym, yp, zm, zp);
    }
    return __fadd_rn(c, __fmul_rn(dt, __fadd_rn(__fmul_rn(D, lap), 0.f)));
}

// Per-item constants of one level (plane-independent): shared offset and flags.
struct TbItem {
    int o;       // shared offset of the float4 (row * W + 4q); -1 = no item
    int flags;   // bit0 ylo ghost, bit1 yhi ghost, bit2 zlo ghost, bit3 zhi ghost, bit4 output in domain
    int gofs;    // global in-plane offset of the output float4 (last level only)
};

template <int T, bool UNIT>
__global__ void __launch_bounds__(256)
fd_tb_fast_kernel(const float* __restrict__ u, float* __restrict__ out, Geo G, float D, float dt, int LX) {
    using S = TbShape<T>;
    extern __shared__ __align__(16) float sm[];
    const int tid = threadIdx.x;
    const int k0 = blockIdx.x * TB_TZ, j0 = blockIdx.y * TB_TY;
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    if (x0 >= x1) return;
    const int nx = G.nx, ny = G.ny, nz = G.nz;
    const size_t plane = (size_t)ny * nz;
    const bool px = G.kind[0] == EVX_BC_PERIODIC, py = G.kind[1] == EVX_BC_PERIODIC,
               pz = G.kind[2] == EVX_BC_PERIODIC;
    auto slot = [&](int lev, int p) -> float* { return sm + ((size_t)lev * 3 + (size_t)((p % 3 + 3) % 3)) * S::PL; };

    // level-0 load plan: R rows x 18 float4 groups
    constexpr int NL = S::R * TB_NQ;
    constexpr int LSLOTS = (NL + 255) / 256;
    int goff[LSLOTS], soff[LSLOTS];
#pragma unroll
    for (int t = 0; t < LSLOTS; ++t) {
        const int e = tid + 256 * t;
        const int row = e / TB_NQ, q = e - (e / TB_NQ) * TB_NQ;
        int gy = j0 + row - T, gz = k0 + 4 * q - 4;
        gy = py ? pmod(gy, ny) : min(max(gy, 0), ny - 1);
        gz = pz ? pmod(gz, nz) : min(max(gz, 0), nz - 4);
        goff[t] = e < NL ? gy * nz + gz : -1;
        soff[t] = row * TB_W + 4 * q;
    }
    // per-level item descriptors (at most 2 items per thread per level)
    TbItem it[T][2];
#pragma unroll
    for (int s = 1; s <= T; ++s) {
        const int q0 = (s == T) ? 1 : 0, q1 = (s == T) ? TB_NQ - 1 : TB_NQ;
        const int ng = q1 - q0, rows = S::R - 2 * s;
#pragma unroll
        for (int t = 0; t < 2; ++t) {
            const int e = tid + 256 * t;
            TbItem d{-1, 0, 0};
            if (e < rows * ng) {
                const int rr = e / ng, qq = e - rr * ng;
                const int row = rr + s, q = qq + q0;
                const int gy = j0 + row - T, gz = k0 + 4 * q - 4;
                const int wy = py ? pmod(gy, ny) : gy, wz = pz ? pmod(gz, nz) : gz;
                d.o = row * TB_W + 4 * q;
                d.flags = ((!py && wy == 0) ? 1 : 0) | ((!py && wy == ny - 1) ? 2 : 0) |
                          ((!pz && wz == 0) ? 4 : 0) | ((!pz && wz + 3 == nz - 1) ? 8 : 0) |
                          ((gy >= 0 && gy < ny && gz >= 0 && gz < nz) ? 16 : 0);
                d.gofs = gy * nz + gz;
            }
            it[s - 1][t] = d;
        }
    }

    float4 pf[LSLOTS];
    auto fetch = [&](int qi) {
        if (!(px || (qi >= 0 && qi < nx))) return;
        const size_t base = (size_t)pmod(qi, nx) * plane;
#pragma unroll
        for (int t = 0; t < LSLOTS; ++t)
            if (goff[t] >= 0) pf[t] = __ldg(reinterpret_cast<const float4*>(u + base + goff[t]));
    };
    auto stash = [&](int qi) {
        if (!(px || (qi >= 0 && qi < nx))) return;
        float* dst = slot(0, qi);
#pragma unroll
        for (int t = 0; t < LSLOTS; ++t)
            if (goff[t] >= 0) *reinterpret_cast<float4*>(dst + soff[t]) = pf[t];
    };

    fetch(x0 - T);
    stash(x0 - T);
    for (int qi = x0 - T; qi <= x1 - 1 + T; ++qi) {
        if (qi + 1 <= x1 - 1 + T) fetch(qi + 1);   // in flight while the levels below compute
        __syncthreads();
#pragma unroll
        for (int s = 1; s <= T; ++s) {
            const int p = qi - s;
            if (p >= x0 - (T - s) && p <= x1 - 1 + (T - s) && (px || (p >= 0 && p < nx))) {
                const int gp = pmod(p, nx);
                const bool xlo = !px && gp == 0, xhi = !px && gp == nx - 1;
                const float* cm = slot(s - 1, p - 1);
                const float* cc = slot(s - 1, p);
                const float* cp = slot(s - 1, p + 1);
#pragma unroll
                for (int t = 0; t < 2; ++t) {
                    const TbItem d = it[s - 1][t];
                    if (d.o < 0) continue;
                    const int o = d.o;
                    const float4 c = *reinterpret_cast<const float4*>(cc + o);
                    const float4 xm = *reinterpret_cast<const float4*>(cm + o);
                    const float4 xp = *reinterpret_cast<const float4*>(cp + o);
                    const float4 ym = *reinterpret_cast<const float4*>(cc + o - TB_W);
                    const float4 yp = *reinterpret_cast<const float4*>(cc + o + TB_W);
                    const float zl = (o % TB_W) ? cc[o - 1] : c.x;
                    const float zr = (o % TB_W) != TB_W - 4 ? cc[o + 4] : c.w;
                    const bool ylo = d.flags & 1, yhi = d.flags & 2, zlo = d.flags & 4, zhi = d.flags & 8;
                    auto X = [&](float cv, float m) { return xlo ? ghost_lo(G, 0, cv) : m; };
                    auto XP = [&](float cv, float m) { return xhi ? ghost_hi(G, 0, cv) : m; };
                    auto Y = [&](float cv, float m) { return ylo ? ghost_lo(G, 1, cv) : m; };
                    auto YP = [&](float cv, float m) { return yhi ? ghost_hi(G, 1, cv) : m; };
                    float4 v;
                    v.x = fd_point<UNIT>(G, D, dt, c.x, X(c.x, xm.x), XP(c.x, xp.x), Y(c.x, ym.x), YP(c.x, yp.x),
                                         zlo ? ghost_lo(G, 2, c.x) : zl, c.y);
                    v.y = fd_point<UNIT>(G, D, dt, c.y, X(c.y, xm.y), XP(c.y, xp.y), Y(c.y, ym.y), YP(c.y, yp.y),
                                         c.x, c.z);
                    v.z = fd_point<UNIT>(G, D, dt, c.z, X(c.z, xm.z), XP(c.z, xp.z), Y(c.z, ym.z), YP(c.z, yp.z),
                                         c.y, c.w);
                    v.w = fd_point<UNIT>(G, D, dt, c.w, X(c.w, xm.w), XP(c.w, xp.w), Y(c.w, ym.w), YP(c.w, yp.w),
                                         c.z, zhi ? ghost_hi(G, 2, c.w) : zr);
                    if (s < T) {
                        *reinterpret_cast<float4*>(slot(s, p) + o) = v;
                    } else if (p >= x0 && p < x1 && (d.flags & 16)) {
                        *reinterpret_cast<float4*>(out + (size_t)gp * plane + d.gofs) = v;
                    }
                }
            }
            if (s < T) __syncthreads();
        }
        // the slot of plane qi+1 held plane qi-2, last read by level 1 above
        __syncthreads();
        if (qi + 1 <= x1 - 1 + T) stash(qi + 1);
    }
}

// ---- single step, register streaming ---------------------------------------
// One thread owns a float4 along z at fixed (y, z) and walks its x-chunk with
// x-1 / x / x+1 in registers (next plane prefetched); y neighbours come
// through L1, z neighbours from the adjacent lanes by warp shuffles (the two
// warp-edge values by scalar loads).  No barriers.  nz % 4 == 0, aligned.
template <bool UNIT>
__global__ void __launch_bounds__(128)
fd_step_reg_kernel(const float* __restrict__ u, float* __restrict__ out, Geo G, float D, float dt, int LX) {
    const int lane = threadIdx.x;
    const int nq = G.nz >> 2;
    const int q = blockIdx.x * 32 + lane;
    const int y = blockIdx.y * blockDim.y + threadIdx.y;
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    const bool active = q < nq && y < G.ny;
    if (x0 >= x1 || __all_sync(0xffffffffu, !active)) return;   // whole warp idle (warp-uniform exit)
    const int nx = G.nx, ny = G.ny, nz = G.nz;
    const int plane = ny * nz;   // fields have < 2^31 elements
    const bool px = G.kind[0] == EVX_BC_PERIODIC, py = G.kind[1] == EVX_BC_PERIODIC,
               pz = G.kind[2] == EVX_BC_PERIODIC;
    const int qc = active ? q : 0, yc = active ? y : 0;   // inactive lanes read a valid address
    const int z = 4 * qc;
    const float* col = u + yc * nz + z;                   // this thread's column at plane 0
    const int dym = ((yc == 0 ? ny - 1 : yc - 1) - yc) * nz, dyp = ((yc == ny - 1 ? 0 : yc + 1) - yc) * nz;
    const bool ylo = !py && yc == 0, yhi = !py && yc == ny - 1;   // uniform per warp (one row per warp)
    const bool zlo = !pz && z == 0, zhi = !pz && z + 4 == nz;
    const int dzl = (z == 0 ? nz - 1 : z - 1) - z, dzr = (z + 4 == nz ? 0 : z + 4) - z;
    const bool left_load = lane == 0, right_load = lane == 31 || q + 1 >= nq;
    auto ld4 = [](const float* p) { return __ldg(reinterpret_cast<const float4*>(p)); };
    auto glo4 = [&](int a, float4 c) {
        return make_float4(ghost_lo(G, a, c.x), ghost_lo(G, a, c.y), ghost_lo(G, a, c.z), ghost_lo(G, a, c.w));
    };
    auto ghi4 = [&](int a, float4 c) {
        return make_float4(ghost_hi(G, a, c.x), ghost_hi(G, a, c.y), ghost_hi(G, a, c.z), ghost_hi(G, a, c.w));
    };

    float4 c = ld4(col + x0 * plane);
    float4 xm = ld4(col + (x0 == 0 ? nx - 1 : x0 - 1) * plane);
    int ip = x0 + 1;
    if (ip >= nx) ip -= nx;
    float4 xp = ld4(col + ip * plane);
    // y and z-edge neighbours of the current plane, loaded one plane ahead
    float4 ymn = ld4(col + x0 * plane + dym), ypn = ld4(col + x0 * plane + dyp);
    float eln = left_load ? __ldg(col + x0 * plane + dzl) : 0.f;
    float ern = right_load ? __ldg(col + x0 * plane + dzr) : 0.f;
    for (int i = x0; i < x1; ++i) {
        const float* cp = col + i * plane;
        float4 ym = ymn, yp = ypn;
        const float el = eln, er = ern;
        int in = i + 2;
        while (in >= nx) in -= nx;
        const float4 nxt = ld4(col + in * plane);   // prefetch plane i+2
        if (i + 1 < x1) {                            // neighbours of plane i+1 (i+1 < nx here)
            const float* cn = cp + plane;
            ymn = ld4(cn + dym);
            ypn = ld4(cn + dyp);
            eln = left_load ? __ldg(cn + dzl) : 0.f;
            ern = right_load ? __ldg(cn + dzr) : 0.f;
        }
        float zl = __shfl_up_sync(0xffffffffu, c.w, 1);
        float zr = __shfl_down_sync(0xffffffffu, c.x, 1);
        if (left_load) zl = el;
        if (right_load) zr = er;
        if (zlo) zl = ghost_lo(G, 2, c.x);
        if (zhi) zr = ghost_hi(G, 2, c.w);
        if (ylo) ym = glo4(1, c);
        if (yhi) yp = ghi4(1, c);
        if (!px) {
            if (i == 0) xm = glo4(0, c);
            if (i == nx - 1) xp = ghi4(0, c);
        }
        float4 v;
        v.x = fd_point<UNIT>(G, D, dt, c.x, xm.x, xp.x, ym.x, yp.x, zl, c.y);
        v.y = fd_point<UNIT>(G, D, dt, c.y, xm.y, xp.y, ym.y, yp.y, c.x, c.z);
        v.z = fd_point<UNIT>(G, D, dt, c.z, xm.z, xp.z, ym.z, yp.z, c.y, c.w);
        v.w = fd_point<UNIT>(G, D, dt, c.w, xm.w, xp.w, ym.w, yp.w, c.z, zr);
        if (active) *reinterpret_cast<float4*>(out + (cp - u)) = v;
        xm = c;
        c = xp;
        xp = nxt;
    }
}

int g_fd_sms = 0;

template <int T, bool UNIT>
int fd_tb_fast_launch(const float* in, float* out, const Geo& G, float D, float dt, cudaStream_t st) {
    using S = TbShape<T>;
    static int bps = 0;
    if (!g_fd_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_fd_sms, cudaDevAttrMultiProcessorCount, dev);
    }
    if (!bps) {
        cudaFuncSetAttribute(fd_tb_fast_kernel<T, UNIT>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)S::SMEM);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fd_tb_fast_kernel<T, UNIT>, 256, S::SMEM);
        if (bps < 1) bps = 1;
    }
    const int tz = (G.nz + TB_TZ - 1) / TB_TZ, ty = (G.ny + TB_TY - 1) / TB_TY;
    const long tiles = (long)tz * ty;
    long chunks = (long)bps * g_fd_sms / tiles;
    if (chunks < 1) chunks = 1;
    int lx = (int)((G.nx + chunks - 1) / chunks);
    lx = std::max(lx, std::min(G.nx, 4 * T));   // bound the x halo overhead
    dim3 grid(tz, ty, (G.nx + lx - 1) / lx);
    const char* name = T == 1 ? "fd_step" : (T == 2 ? "fd_tblock2" : "fd_tblock4");
    EVX_TIMED(name, st, fd_tb_fast_kernel<T, UNIT><<<grid, 256, S::SMEM, st>>>(in, out, G, D, dt, lx));
    count_launch();
    return check_launch("fd_tb_fast_kernel");
}

template <bool UNIT>
int fd_step_reg_launch(const float* in, float* out, const Geo& G, float D, float dt, cudaStream_t st) {
    if (!g_fd_sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&g_fd_sms, cudaDevAttrMultiProcessorCount, dev);
    }
    static int bps = 0;   // resident blocks per SM
    if (!bps) {
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, fd_step_reg_kernel<UNIT>, 128, 0);
        if (bps < 1) bps = 1;
    }
    const int nq = G.nz / 4;
    const int bx = (nq + 31) / 32, by = (G.ny + 3) / 4;
    const long cols = (long)bx * by, slots = (long)bps * g_fd_sms;
    // x chunks per column: whole waves of resident blocks (the least idle tail),
    // and among those the longest x-runs (2 halo planes per chunk), at least 8 planes
    long chunks = 1;
    double best = 1e30;
    for (long c = 1; c <= std::max(1, G.nx / 8); ++c) {
        const long blocks = cols * c, waves = (blocks + slots - 1) / slots;
        const double cost = (double)waves * ((double)((G.nx + c - 1) / c) + 2.0);   // time ~ waves x planes per block
        if (cost < best - 1e-9) {
            best = cost;
            chunks = c;
        }
    }
    int lx = (int)((G.nx + chunks - 1) / chunks);
    lx = std::max(lx, std::min(G.nx, 8));
    dim3 grid(bx, by, (G.nx + lx - 1) / lx);
    EVX_TIMED("fd_step", st, fd_step_reg_kernel<UNIT><<<grid, dim3(32, 4), 0, st>>>(in, out, G, D, dt, lx));
    count_launch();
    return check_launch("fd_step_reg_kernel");
}

template <int T>
int fd_tb_dispatch(const float* in, float* out, const Geo& G, float D, float dt, cudaStream_t st) {
    const bool unit = G.ih2[0] == 1.f && G.ih2[1] == 1.f && G.ih2[2] == 1.f;
    if (T == 1) return unit ? fd_step_reg_launch<true>(in, out, G, D, dt, st) : fd_step_reg_launch<false>(in, out, G, D, dt, st);
    return unit ? fd_tb_fast_launch<T, true>(in, out, G, D, dt, st) : fd_tb_fast_launch<T, false>(in, out, G, D, dt, st);
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
    const bool fast = g->nz % 4 == 0 &&
                      ((reinterpret_cast<uintptr_t>(u_in) | reinterpret_cast<uintptr_t>(u_out) |
                        reinterpret_cast<uintptr_t>(scratch)) & 15) == 0;
    if (!fast) spp = 1;   // the generic kernel advances one step per pass
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
        if (!fast) {
            EVX_TIMED("fd_step", st, fd_stream_kernel<1><<<grid, dim3(FD_BZ, FD_BY), 0, st>>>(src, dst, G, D, dt, lx));
            count_launch();
            rc = check_launch("fd_stream_kernel");
        } else if (t == 1) {
            rc = fd_tb_dispatch<1>(src, dst, G, D, dt, st);
        } else if (t == 2) {
            rc = fd_tb_dispatch<2>(src, dst, G, D, dt, st);
        } else {
            rc = fd_tb_dispatch<4>(src, dst, G, D, dt, st);
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

// ---- allocation-free forward Euler --------------------------------------------
// evx_fd_forward needs one caller-allocated scratch field for its ping-pong
// passes.  Some callers cannot provide it: hosts whose device memory is handed
// out only by their own pre-reserved pool (an extra cudaMalloc would fail or
// fragment it), and bindings that pass buffers from a foreign allocator and
// must not allocate at all.  evx_fd_forward_noalloc keeps that scratch in the
// file-scope device array below instead.  It holds EVX_FD_NOALLOC_MAX_VOXELS
// floats (16 MiB) on every GPU that loads this library, until the process
// exits.  All calls share the array: calls that overlap on the GPU (on
// different streams, or from different threads) race on it.  The array keeps
// the last call's contents; nothing in it needs to start at zero, because
// every element a call reads was written earlier in the same call.
#include <mutex>

static __device__ __align__(256) float g_fd_noalloc_scratch[EVX_FD_NOALLOC_MAX_VOXELS];

namespace {

std::mutex g_noalloc_mu;
constexpr int NOALLOC_MAX_DEVICES = 64;
float* g_noalloc_ptr[NOALLOC_MAX_DEVICES] = {};

// Device address of the scratch array on the current device.  The host-side
// symbol is only a stand-in, so the address is looked up with that device
// current.  It is looked up again on every call made outside a stream capture
// (cheap), so a device reset or a new primary context never leaves a stale
// address behind; a call on a capturing stream uses the address of the last
// call outside a capture and fails if there was none on this device.
int noalloc_scratch(float** out, cudaStream_t st) {
    int dev = 0;
    int rc = evx::check_cuda(cudaGetDevice(&dev), "evx_fd_forward_noalloc: cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return evx::fail(EVX_ERR_UNSUPPORTED, "evx_fd_forward_noalloc: device ordinal %d not supported", dev);
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    rc = evx::check_cuda(cudaStreamIsCapturing(st, &cap), "evx_fd_forward_noalloc: cudaStreamIsCapturing");
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        rc = evx::check_cuda(cudaGetSymbolAddress(&p, g_fd_noalloc_scratch),
                             "evx_fd_forward_noalloc: cudaGetSymbolAddress");
        if (rc) return rc;
        g_noalloc_ptr[dev] = static_cast<float*>(p);
    } else if (!g_noalloc_ptr[dev]) {
        return evx::fail(EVX_ERR_BAD_ARG,
                         "evx_fd_forward_noalloc: the first call on device %d must come before any stream capture",
                         dev);
    }
    *out = g_noalloc_ptr[dev];
    return EVX_OK;
}

}  // namespace

extern "C" int evx_fd_forward_noalloc(const float* u_in, float* u_out, const evx_grid* g, const evx_bc* bc,
                                      float D, float dt, int nsteps, int steps_per_pass, void* stream) {
    int rc = fd_common_checks(u_in, u_out, g, bc);
    if (rc) return rc;
    const size_t n = field_elems(g);
    if (n > (size_t)EVX_FD_NOALLOC_MAX_VOXELS)
        return fail(EVX_ERR_TOO_LARGE,
                    "evx_fd_forward_noalloc: grid of %zu voxels exceeds the %u-voxel built-in scratch; "
                    "use evx_fd_forward with a caller-provided scratch field",
                    n, (unsigned)EVX_FD_NOALLOC_MAX_VOXELS);
    float* scratch = nullptr;
    if ((rc = noalloc_scratch(&scratch, as_stream(stream)))) return rc;
    Geo G = make_geo(g, bc);
    return fd_run(u_in, u_out, scratch, g, G, D, dt, nsteps, steps_per_pass, as_stream(stream));
}
