// Periodic fast path of the Cahn-Hilliard right-hand side (tiling in
// evx_ch_fast.cuh).  Same float32 operations, in the same order, as the generic
// kernel and the reference (evoxels/problem_definition.py:350-371); the
// translation unit is compiled with --fmad=false, so results are bit-identical.
//
// Per x-plane i a tile: stores the prefetched field plane i+2 (clipped) into a
// 4-slot shared ring and issues the global loads of plane i+3; computes the
// chemical potential of plane i+1 over the tile grown by one cell (2-slot
// ring); then computes r on plane i.  Two barriers per plane.
//
// The tile body is shared by the single-grid kernel (one block per tile and
// x-chunk) and the batched kernel (persistent blocks pulling instance x tile x
// x-chunk work items from a global counter).
#include "evx_ch_fast.cuh"

namespace evx {
namespace {

using namespace fast;

// mu = w*c*(1-c)*(1-2c) - kappa*lap(c)
__device__ __forceinline__ float mu_at(const Geo& G, const ChP& P, float c, float xm, float xp, float ym, float yp,
                                       float zm, float zp) {
    return __fsub_rn(mu_hom(P.w, c), __fmul_rn(P.kappa, lap7(G, c, xm, xp, ym, yp, zm, zp)));
}

template <class T, bool FUSED>
__device__ __forceinline__ void rhs_tile(const float* __restrict__ u, const float* __restrict__ upd,
                                         float* __restrict__ u_new, float* __restrict__ r, const Geo& G,
                                         const ChP& P, int k0, int j0, int x0, int x1, float* cs, float* ms) {
    const int tid = threadIdx.x;
    const int tx = tid % T::BX, ty = tid / T::BX;
    const int nx = G.nx, ny = G.ny, nz = G.nz;
    const size_t plane = (size_t)ny * nz;
    const LoadPlan LP = make_load_plan<T>(tid, j0, k0, ny, nz);

    // potential patches owned by this thread (at most two)
    int mr[2], mc[2];
    bool mv[2];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int pidx = tid + m * THREADS;
        mv[m] = pidx < T::NMU;
        const int py = mv[m] ? pidx / T::MPZ : 0;
        mr[m] = 1 + 2 * py;                        // field row of the patch's upper row
        mc[m] = 2 + 2 * (pidx - py * T::MPZ);       // field column of the patch's left column
    }
    const int W = T::W;
    const int ra = 2 + 2 * ty, rc = 4 + 2 * tx;    // field row / column in shared memory
    const int gj = j0 + 2 * ty, gk = k0 + 2 * tx;   // global y / z of the patch origin
    const bool wk = gk < nz, wj0 = gj < ny && wk, wj1 = gj + 1 < ny && wk;
    const float ihx = G.ih[0], ihy = G.ih[1], ihz = G.ih[2];

    float4 pf[2];
    auto fetch = [&](int p) {
        const size_t base = (size_t)pmod(p, nx) * plane;
        const bool own_plane = p >= x0 && p < x1;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!LP.valid[s]) continue;
            float4 a = ldg4(u + base + LP.goff[s]);
            if (FUSED) {
                const float4 d = ldg4(upd + base + LP.goff[s]);
                a = make_float4(__fadd_rn(a.x, d.x), __fadd_rn(a.y, d.y), __fadd_rn(a.z, d.z), __fadd_rn(a.w, d.w));
                if (own_plane && LP.own[s]) *reinterpret_cast<float4*>(u_new + base + LP.goff[s]) = a;
            }
            pf[s] = a;
        }
    };
    auto stash = [&](int p) {
        float* dst = cs + (p & 3) * T::FIELD;
#pragma unroll
        for (int s = 0; s < 2; ++s)
            if (LP.valid[s]) sts4(dst + LP.soff[s], clip4(pf[s]));
    };
    auto compute_mu = [&](int p) {
        const float* cc = cs + (p & 3) * T::FIELD;
        const float* cm = cs + ((p - 1) & 3) * T::FIELD;
        const float* cp = cs + ((p + 1) & 3) * T::FIELD;
        float* mo = ms + (p & 1) * T::POT;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            if (!mv[m]) continue;
            const int a = mr[m] * W + mc[m], b = a + W;
            const float2 up = lds2(cc + a - W), A = lds2(cc + a), B = lds2(cc + b), dn = lds2(cc + b + W);
            const float Al = cc[a - 1], Ar = cc[a + 2], Bl = cc[b - 1], Br = cc[b + 2];
            const float2 xmA = lds2(cm + a), xmB = lds2(cm + b), xpA = lds2(cp + a), xpB = lds2(cp + b);
            const float m00 = mu_at(G, P, A.x, xmA.x, xpA.x, up.x, B.x, Al, A.y);
            const float m01 = mu_at(G, P, A.y, xmA.y, xpA.y, up.y, B.y, A.x, Ar);
            const float m10 = mu_at(G, P, B.x, xmB.x, xpB.x, A.x, dn.x, Bl, B.y);
            const float m11 = mu_at(G, P, B.y, xmB.y, xpB.y, A.y, dn.y, B.x, Br);
            sts2(mo + a - W, m00, m01);   // potential row = field row - 1
            sts2(mo + b - W, m10, m11);
        }
    };

    float fxm[4] = {0.f, 0.f, 0.f, 0.f};   // x flux on the face below the current plane
    auto x_faces = [&](int plo, float out[4]) {
        const float* c0 = cs + (plo & 3) * T::FIELD;
        const float* c1 = cs + ((plo + 1) & 3) * T::FIELD;
        const float* m0 = ms + (plo & 1) * T::POT;
        const float* m1 = ms + ((plo + 1) & 1) * T::POT;
        const int a = ra * W + rc, b = a + W;
        const float2 cA0 = lds2(c0 + a), cB0 = lds2(c0 + b), cA1 = lds2(c1 + a), cB1 = lds2(c1 + b);
        const float2 mA0 = lds2(m0 + a - W), mB0 = lds2(m0 + b - W), mA1 = lds2(m1 + a - W), mB1 = lds2(m1 + b - W);
        out[0] = face_flux(cA0.x, cA1.x, mA0.x, mA1.x, ihx);
        out[1] = face_flux(cA0.y, cA1.y, mA0.y, mA1.y, ihx);
        out[2] = face_flux(cB0.x, cB1.x, mB0.x, mB1.x, ihx);
        out[3] = face_flux(cB0.y, cB1.y, mB0.y, mB1.y, ihx);
    };

    auto compute_r = [&](int i) {
        const float* cc = cs + (i & 3) * T::FIELD;
        const float* mm = ms + (i & 1) * T::POT;
        const int a = ra * W + rc, b = a + W;     // field offsets; potential offsets are one row up
        float fxp[4];
        x_faces(i, fxp);
        const float2 up = lds2(cc + a - W), A = lds2(cc + a), B = lds2(cc + b), dn = lds2(cc + b + W);
        const float Al = cc[a - 1], Ar = cc[a + 2], Bl = cc[b - 1], Br = cc[b + 2];
        const float2 mup = lds2(mm + a - 2 * W), MA = lds2(mm + a - W), MB = lds2(mm + b - W), mdn = lds2(mm + b);
        const float MAl = mm[a - W - 1], MAr = mm[a - W + 2], MBl = mm[b - W - 1], MBr = mm[b - W + 2];
        // z faces
        const float za0 = face_flux(Al, A.x, MAl, MA.x, ihz), za1 = face_flux(A.x, A.y, MA.x, MA.y, ihz);
        const float za2 = face_flux(A.y, Ar, MA.y, MAr, ihz);
        const float zb0 = face_flux(Bl, B.x, MBl, MB.x, ihz), zb1 = face_flux(B.x, B.y, MB.x, MB.y, ihz);
        const float zb2 = face_flux(B.y, Br, MB.y, MBr, ihz);
        // y faces
        const float y0x = face_flux(up.x, A.x, mup.x, MA.x, ihy), y1x = face_flux(A.x, B.x, MA.x, MB.x, ihy);
        const float y2x = face_flux(B.x, dn.x, MB.x, mdn.x, ihy);
        const float y0y = face_flux(up.y, A.y, mup.y, MA.y, ihy), y1y = face_flux(A.y, B.y, MA.y, MB.y, ihy);
        const float y2y = face_flux(B.y, dn.y, MB.y, mdn.y, ihy);
        auto divr = [&](float fxp_, float fxm_, float fyp, float fym, float fzp, float fzm) {
            float d = __fmul_rn(__fsub_rn(fxp_, fxm_), ihx);
            d = __fadd_rn(d, __fmul_rn(__fsub_rn(fyp, fym), ihy));
            d = __fadd_rn(d, __fmul_rn(__fsub_rn(fzp, fzm), ihz));
            return __fmul_rn(P.D, d);
        };
        const float r00 = divr(fxp[0], fxm[0], y1x, y0x, za1, za0);
        const float r01 = divr(fxp[1], fxm[1], y1y, y0y, za2, za1);
        const float r10 = divr(fxp[2], fxm[2], y2x, y1x, zb1, zb0);
        const float r11 = divr(fxp[3], fxm[3], y2y, y1y, zb2, zb1);
        const size_t o = (size_t)i * plane + (size_t)gj * nz + gk;
        if (wj0) *reinterpret_cast<float2*>(r + o) = make_float2(r00, r01);
        if (wj1) *reinterpret_cast<float2*>(r + o + nz) = make_float2(r10, r11);
#pragma unroll
        for (int q = 0; q < 4; ++q) fxm[q] = fxp[q];
    };

    // prologue: field planes x0-2 .. x0+1, potentials x0-1 and x0, first x face
    for (int p = x0 - 2; p <= x0 + 1; ++p) {
        fetch(p);
        stash(p);
    }
    fetch(x0 + 2);
    __syncthreads();
    compute_mu(x0 - 1);
    compute_mu(x0);
    __syncthreads();
    x_faces(x0 - 1, fxm);
    for (int i = x0; i < x1; ++i) {
        stash(i + 2);
        if (i + 3 <= x1 + 1) fetch(i + 3);
        __syncthreads();
        compute_mu(i + 1);
        __syncthreads();
        compute_r(i);
    }
}

template <class T, bool FUSED>
__global__ void __launch_bounds__(THREADS, 4)
ch_rhs_fast_kernel(const float* __restrict__ u, const float* __restrict__ upd, float* __restrict__ u_new,
                   float* __restrict__ r, Geo G, ChP P, int LX) {
    __shared__ __align__(16) float cs[4 * T::FIELD];
    __shared__ __align__(16) float ms[2 * T::POT];
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    if (x0 >= x1) return;   // uniform across the block
    rhs_tile<T, FUSED>(u, upd, u_new, r, G, P, blockIdx.x * T::TZ, blockIdx.y * T::TY, x0, x1, cs, ms);
}

__device__ __forceinline__ Geo batch_geo(const BatchInst& B) {
    Geo G;
    G.nx = B.nx; G.ny = B.ny; G.nz = B.nz;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        G.kind[a] = EVX_BC_PERIODIC;
        G.lo[a] = G.hi[a] = 0.f;
        G.ih[a] = B.ih[a];
        G.ih2[a] = B.ih2[a];
    }
    G.ih2sum = B.ih2sum;
    return G;
}

// Persistent batched rhs: blocks pull work items until the list is exhausted.
template <bool FUSED>
__global__ void __launch_bounds__(THREADS, 4)
ch_rhs_batch_kernel(const float* __restrict__ u, const float* __restrict__ upd, float* __restrict__ u_new,
                    float* __restrict__ r, const BatchInst* __restrict__ insts, const BatchItem* __restrict__ items,
                    int n_items, int* __restrict__ counter) {
    __shared__ __align__(16) float cs[4 * MAX_FIELD];
    __shared__ __align__(16) float ms[2 * MAX_POT];
    __shared__ int s_item;
    for (;;) {
        if (threadIdx.x == 0) s_item = atomicAdd(counter, 1);
        __syncthreads();
        const int it = s_item;
        if (it >= n_items) break;
        const BatchItem I = items[it];
        const BatchInst B = insts[I.inst];
        const Geo G = batch_geo(B);
        const size_t o = (size_t)B.off;
        if (B.tile == 0)
            rhs_tile<TileWide, FUSED>(u + o, FUSED ? upd + o : nullptr, FUSED ? u_new + o : nullptr, r + o, G, B.P,
                                      I.k0, I.j0, I.x0, I.x1, cs, ms);
        else
            rhs_tile<TileSquare, FUSED>(u + o, FUSED ? upd + o : nullptr, FUSED ? u_new + o : nullptr, r + o, G,
                                        B.P, I.k0, I.j0, I.x0, I.x1, cs, ms);
        __syncthreads();   // shared memory and s_item are reused by the next item
    }
}

int g_rhs_bps[2] = {0, 0}, g_sms = 0, g_batch_bps = 0;
int g_tile_override = -1;

void init_rhs_occupancy() {
    if (g_sms) return;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_rhs_bps[0], ch_rhs_fast_kernel<TileWide, true>, THREADS, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_rhs_bps[1], ch_rhs_fast_kernel<TileSquare, true>, THREADS, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_batch_bps, ch_rhs_batch_kernel<true>, THREADS, 0);
    for (int* b : {&g_rhs_bps[0], &g_rhs_bps[1], &g_batch_bps})
        if (*b < 1) *b = 1;
}

template <class T>
int rhs_fast_launch_t(bool fused, const float* u, const float* upd, float* u_new, float* r, const evx_grid* g,
                      const Geo& G, const ChP& P, cudaStream_t st, int bps) {
    int lx;
    const dim3 grid = fast_grid<T>(g->nx, g->ny, g->nz, bps, g_sms, &lx);
    if (fused)
        EVX_TIMED("ch_rhs_fused", st, ch_rhs_fast_kernel<T, true><<<grid, THREADS, 0, st>>>(u, upd, u_new, r, G, P, lx));
    else
        EVX_TIMED("ch_rhs", st, ch_rhs_fast_kernel<T, false><<<grid, THREADS, 0, st>>>(u, nullptr, nullptr, r, G, P, lx));
    count_launch();
    return check_launch("ch_rhs_fast_kernel");
}

}  // namespace

int ch_tile_variant(int nz) {
    if (g_tile_override == 0) return 0;
    if (g_tile_override == 1) return 1;
    return default_tile_variant(nz);
}

int ch_rhs_fast_launch(bool fused, const float* u, const float* upd, float* u_new, float* r, const evx_grid* g,
                       const Geo& G, const ChP& P, cudaStream_t st) {
    init_rhs_occupancy();
    if (ch_tile_variant(g->nz) == 1)
        return rhs_fast_launch_t<TileSquare>(fused, u, upd, u_new, r, g, G, P, st, g_rhs_bps[1]);
    return rhs_fast_launch_t<TileWide>(fused, u, upd, u_new, r, g, G, P, st, g_rhs_bps[0]);
}

int batch_rhs_blocks_per_sm() {
    init_rhs_occupancy();
    return g_batch_bps;
}

int batch_rhs_launch(bool fused, const float* u, const float* upd, float* u_new, float* r, const BatchInst* insts,
                     const BatchItem* items, int n_items, int* counter, int grid, cudaStream_t st) {
    int rc = check_cuda(cudaMemsetAsync(counter, 0, sizeof(int), st), "batch rhs counter reset");
    if (rc) return rc;
    if (fused)
        EVX_TIMED("batch_rhs_fused", st,
                  ch_rhs_batch_kernel<true><<<grid, THREADS, 0, st>>>(u, upd, u_new, r, insts, items, n_items, counter));
    else
        EVX_TIMED("batch_rhs", st,
                  ch_rhs_batch_kernel<false><<<grid, THREADS, 0, st>>>(u, nullptr, nullptr, r, insts, items, n_items,
                                                                       counter));
    count_launch();
    return check_launch("ch_rhs_batch_kernel");
}

}  // namespace evx

extern "C" int evx_set_tile_variant(int variant) {
    if (variant < -1 || variant > 1) return evx::fail(EVX_ERR_BAD_ARG, "tile variant must be -1, 0 or 1");
    evx::g_tile_override = variant;
    return EVX_OK;
}
