// Periodic fast path of the Cahn-Hilliard right-hand side (tiling in
// evx_ch_fast.cuh), in two arithmetic forms:
// * ExactMath: the same float32 operations, in the same order, as the generic
//   kernel and the reference (evoxels/problem_definition.py:350-371); the
//   translation unit is compiled with --fmad=false, so evx_ch_rhs is
//   bit-identical to the reference.
// * TolMath: the same formula with the constants folded and products fused
//   (two-lane FFMA2), for the rhs passes inside the spectral loops (IMEX and
//   exponential Euler steps, single and batched), whose FFT already differs
//   from the reference's in the last bits; about 40% fewer instructions.
//
// Per x-plane i a tile: computes r on plane i, the chemical potential of plane
// i+2 over the tile grown by one cell (3-slot ring), stores the prefetched
// field plane i+4 (clipped) into a 5-slot shared ring and issues the global
// loads of plane i+5.  One barrier per plane.
//
// The tile body is shared by the single-grid kernel (one block per tile and
// x-chunk) and the batched kernel (persistent blocks pulling instance x tile x
// x-chunk work items from a global counter).
#include "evx_ch_fast.cuh"
#include "evx_graph.cuh"

namespace evx {
namespace {

using namespace fast;

// Two z-adjacent points at a time (two-lane sums, scalar products); every lane
// performs exactly the scalar operations of lap7 / mu_hom / face_flux
// (evx_common.cuh) in the same order, so results stay bit-identical.
struct ExactMath {
    struct C {   // broadcast constants
        float2 ih2x, ih2y, ih2z, ih2sum, w, kappa, D, ih[3];
        int bulk;
    };
    static __device__ __forceinline__ C make(const Geo& G, const ChP& P) {
        return C{f2s(G.ih2[0]), f2s(G.ih2[1]), f2s(G.ih2[2]), f2s(G.ih2sum), f2s(P.w), f2s(P.kappa), f2s(P.D),
                 {f2s(G.ih[0]), f2s(G.ih[1]), f2s(G.ih[2])}, P.bulk};
    }
    static __device__ __forceinline__ float2 lap(const C& K, float2 c, float2 xm, float2 xp, float2 ym, float2 yp,
                                                 float2 zm, float2 zp) {
        using exact::add2; using exact::sub2; using exact::mul2; using exact::mul2_nofuse;
        float2 t = mul2(add2(xp, xm), K.ih2x);
        t = add2(t, mul2(add2(yp, ym), K.ih2y));
        t = add2(t, mul2(add2(zp, zm), K.ih2z));
        return sub2(t, mul2(mul2_nofuse(f2s(2.f), c), K.ih2sum));
    }
    // mu = w*c*(1-c)*(1-2c) - kappa*lap(c)
    static __device__ __forceinline__ float2 mu(const C& K, float2 c, float2 xm, float2 xp, float2 ym, float2 yp,
                                                float2 zm, float2 zp) {
        using exact::add2; using exact::sub2; using exact::mul2; using exact::mul2_nofuse;
        float2 h;
        if (K.bulk == EVX_BULK_REGULAR_SOLUTION) {
            h = make_float2(mu_regular(K.w.x, c.x), mu_regular(K.w.x, c.y));
        } else {
            h = mul2_nofuse(K.w, c);                              // feeds a product
            h = mul2_nofuse(h, sub2(f2s(1.f), c));                // feeds a product
            h = mul2(h, sub2(f2s(1.f), mul2_nofuse(f2s(2.f), c)));   // 2c exact
        }
        return sub2(h, mul2(K.kappa, lap(K, c, xm, xp, ym, yp, zm, zp)));
    }
    // (cf*(1-cf)) * ((mu_hi - mu_lo)*ih), cf = 0.5*(c_hi + c_lo)
    template <int AX>
    static __device__ __forceinline__ float2 flux(const C& K, float2 clo, float2 chi, float2 mlo, float2 mhi) {
        using exact::add2; using exact::sub2; using exact::mul2; using exact::mul2_nofuse;
        const float2 cf = mul2_nofuse(f2s(0.5f), add2(chi, clo));   // exact
        const float2 m = mul2_nofuse(cf, sub2(f2s(1.f), cf));        // feeds a product
        return mul2(m, mul2_nofuse(sub2(mhi, mlo), K.ih[AX]));       // the inner one feeds a product
    }
    static __device__ __forceinline__ float2 div(const C& K, float2 fxp, float2 fxm, float2 fyp, float2 fym,
                                                 float2 fzp, float2 fzm) {
        using exact::add2; using exact::sub2; using exact::mul2; using exact::mul2_nofuse;
        float2 d = mul2(sub2(fxp, fxm), K.ih[0]);
        d = add2(d, mul2(sub2(fyp, fym), K.ih[1]));
        d = add2(d, mul2(sub2(fzp, fzm), K.ih[2]));
        return mul2_nofuse(K.D, d);   // the result is stored
    }
};

// The same rhs with the constants folded: -kappa into the Laplacian weights,
// D*ih^2 into the divergence weights (the face flux is c(1-c)*(mu_hi - mu_lo)
// with cf(1-cf) = s*(1/2 - s/4), s = c_lo + c_hi), every product fused where
// it feeds a sum.
struct TolMath {
    struct C {
        float2 lx, ly, lz, lc, w, dx, dy, dz;   // -kappa*ih2_a, 2*kappa*sum(ih2), w, D*ih2_a
        int bulk;
    };
    static __device__ __forceinline__ C make(const Geo& G, const ChP& P) {
        return C{f2s(-P.kappa * G.ih2[0]), f2s(-P.kappa * G.ih2[1]), f2s(-P.kappa * G.ih2[2]),
                 f2s(2.f * P.kappa * G.ih2sum), f2s(P.w), f2s(P.D * G.ih2[0]), f2s(P.D * G.ih2[1]),
                 f2s(P.D * G.ih2[2]), P.bulk};
    }
    static __device__ __forceinline__ float2 mu(const C& K, float2 c, float2 xm, float2 xp, float2 ym, float2 yp,
                                                float2 zm, float2 zp) {
        float2 t = mul2(add2(xp, xm), K.lx);
        t = fma2(add2(yp, ym), K.ly, t);
        t = fma2(add2(zp, zm), K.lz, t);
        t = fma2(c, K.lc, t);                                     // -kappa*lap(c)
        if (K.bulk == EVX_BULK_REGULAR_SOLUTION) {                // log(c) - log(1-c) + w*(1-2c)
            const float2 lg = make_float2(logf(c.x) - logf(1.f - c.x), logf(c.y) - logf(1.f - c.y));
            return add2(fma2(K.w, fma2(c, f2s(-2.f), f2s(1.f)), lg), t);
        }
        const float2 h = mul2(mul2(K.w, c), sub2(f2s(1.f), c));  // w*c*(1-c)
        return fma2(h, fma2(c, f2s(-2.f), f2s(1.f)), t);
    }
    template <int AX>
    static __device__ __forceinline__ float2 flux(const C&, float2 clo, float2 chi, float2 mlo, float2 mhi) {
        const float2 sm = add2(clo, chi);
        return mul2(mul2(sm, fma2(sm, f2s(-0.25f), f2s(0.5f))), sub2(mhi, mlo));
    }
    static __device__ __forceinline__ float2 div(const C& K, float2 fxp, float2 fxm, float2 fyp, float2 fym,
                                                 float2 fzp, float2 fzm) {
        float2 d = mul2(sub2(fxp, fxm), K.dx);
        d = fma2(sub2(fyp, fym), K.dy, d);
        return fma2(sub2(fzp, fzm), K.dz, d);
    }
};

// XB: a Neumann or Dirichlet x axis (y and z periodic; the spectral loops' mirrored-x step).  Planes
// outside [0, nx) are still staged (wrapped) but never read: the x neighbours of the boundary planes
// are the ghosts of the boundary values, for c and for mu alike (evoxels pads both).
template <class T, bool FUSED, class M, bool DEFER, bool XB = false>
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
    const typename M::C K = M::make(G, P);

    // The loads of a plane are issued one plane ahead and consumed by its stash.  In the fused pass
    // the update is added (and u_n stored) at the stash with DEFER, so no thread waits on its own
    // prefetch; without DEFER (fewer registers: the persistent batched kernel) right after the loads.
    float4 pf[2], pd[DEFER && FUSED ? 2 : 1];
    auto add_store = [&](int p, size_t base, int s, float4 a, float4 d) {
        const float2 lo = exact::add2(make_float2(a.x, a.y), make_float2(d.x, d.y));
        const float2 hi = exact::add2(make_float2(a.z, a.w), make_float2(d.z, d.w));
        a = make_float4(lo.x, lo.y, hi.x, hi.y);
        if (p >= x0 && p < x1 && LP.own[s]) *reinterpret_cast<float4*>(u_new + base + LP.goff[s]) = a;
        return a;
    };
    auto fetch = [&](int p) {
        const size_t base = (size_t)pmod(p, nx) * plane;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!LP.valid[s]) continue;
            pf[s] = ldg4(u + base + LP.goff[s]);
            if (FUSED) {
                const float4 d = ldg4(upd + base + LP.goff[s]);
                if constexpr (DEFER) pd[s] = d;
                else pf[s] = add_store(p, base, s, pf[s], d);
            }
        }
    };
    auto stash = [&](int p) {
        float* dst = cs + cslot(p) * T::FIELD;
        const size_t base = (size_t)pmod(p, nx) * plane;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!LP.valid[s]) continue;
            float4 a = pf[s];
            if constexpr (FUSED && DEFER) a = add_store(p, base, s, a, pd[s]);
            sts4(dst + LP.soff[s], clip4(a));
        }
    };
    // x ghost of a pair of boundary values: Neumann the values, Dirichlet 2v - values
    auto xghost = [&](float2 v, bool lo) -> float2 {
        if (G.kind[0] == EVX_BC_NEUMANN) return v;
        return sub2(f2s(lo ? G.lo[0] : G.hi[0]), v);
    };
    auto compute_mu = [&](int p) {
        const float* cc = cs + cslot(p) * T::FIELD;
        const float* cm = cs + cslot(p - 1) * T::FIELD;
        const float* cp = cs + cslot(p + 1) * T::FIELD;
        float* mo = ms + mslot(p) * T::POT;
        const bool glo = XB && p == 0, ghi = XB && p == nx - 1;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            if (!mv[m]) continue;
            const int a = mr[m] * W + mc[m], b = a + W;
            const float2 up = lds2(cc + a - W), A = lds2(cc + a), B = lds2(cc + b), dn = lds2(cc + b + W);
            const float2 zmA = make_float2(cc[a - 1], A.x), zpA = make_float2(A.y, cc[a + 2]);
            const float2 zmB = make_float2(cc[b - 1], B.x), zpB = make_float2(B.y, cc[b + 2]);
            const float2 xmA = glo ? xghost(A, true) : lds2(cm + a), xmB = glo ? xghost(B, true) : lds2(cm + b);
            const float2 xpA = ghi ? xghost(A, false) : lds2(cp + a), xpB = ghi ? xghost(B, false) : lds2(cp + b);
            // potential row = field row - 1
            *reinterpret_cast<float2*>(mo + a - W) = M::mu(K, A, xmA, xpA, up, B, zmA, zpA);
            *reinterpret_cast<float2*>(mo + b - W) = M::mu(K, B, xmB, xpB, A, dn, zmB, zpB);
        }
    };

    float2 fxm[2] = {f2s(0.f), f2s(0.f)};   // x flux on the face below the current plane (rows a, b)
    // c and mu of the current plane at the patch points (rows a, b), carried from the x faces of the
    // plane below, where they were the upper side
    float2 cA, cB, mA, mB;
    auto x_faces = [&](int plo, float2 out[2]) {
        const float* c0 = cs + cslot(plo) * T::FIELD;
        const float* c1 = cs + cslot(plo + 1) * T::FIELD;
        const float* m0 = ms + mslot(plo) * T::POT;
        const float* m1 = ms + mslot(plo + 1) * T::POT;
        const int a = ra * W + rc, b = a + W;
        cA = lds2(c1 + a);
        cB = lds2(c1 + b);
        mA = lds2(m1 + a - W);
        mB = lds2(m1 + b - W);
        if (XB && plo == -1) {   // the face below plane 0: the ghosts of plane 0
            out[0] = M::template flux<0>(K, xghost(cA, true), cA, xghost(mA, true), mA);
            out[1] = M::template flux<0>(K, xghost(cB, true), cB, xghost(mB, true), mB);
        } else {
            out[0] = M::template flux<0>(K, lds2(c0 + a), cA, lds2(m0 + a - W), mA);
            out[1] = M::template flux<0>(K, lds2(c0 + b), cB, lds2(m0 + b - W), mB);
        }
    };

    auto compute_r = [&](int i) {
        const float* cc = cs + cslot(i) * T::FIELD;
        const float* mm = ms + mslot(i) * T::POT;
        const float* cx = cs + cslot(i + 1) * T::FIELD;
        const float* mx = ms + mslot(i + 1) * T::POT;
        const int a = ra * W + rc, b = a + W;     // field offsets; potential offsets are one row up
        const float2 A = cA, B = cB, MA = mA, MB = mB;
        cA = lds2(cx + a);
        cB = lds2(cx + b);
        mA = lds2(mx + a - W);
        mB = lds2(mx + b - W);
        float2 fxp[2];
        if (XB && i == nx - 1) {   // the face above the last plane: its ghosts
            fxp[0] = M::template flux<0>(K, A, xghost(A, false), MA, xghost(MA, false));
            fxp[1] = M::template flux<0>(K, B, xghost(B, false), MB, xghost(MB, false));
        } else {
            fxp[0] = M::template flux<0>(K, A, cA, MA, mA);
            fxp[1] = M::template flux<0>(K, B, cB, MB, mB);
        }
        const float2 up = lds2(cc + a - W), dn = lds2(cc + b + W);
        const float2 mup = lds2(mm + a - 2 * W), mdn = lds2(mm + b);
        // z faces (left, mid) and (mid, right) of each row
        const float2 zlA = M::template flux<2>(K, make_float2(cc[a - 1], A.x), A, make_float2(mm[a - W - 1], MA.x), MA);
        const float2 zhA = M::template flux<2>(K, A, make_float2(A.y, cc[a + 2]), MA, make_float2(MA.y, mm[a - W + 2]));
        const float2 zlB = M::template flux<2>(K, make_float2(cc[b - 1], B.x), B, make_float2(mm[b - W - 1], MB.x), MB);
        const float2 zhB = M::template flux<2>(K, B, make_float2(B.y, cc[b + 2]), MB, make_float2(MB.y, mm[b - W + 2]));
        // y faces above, between and below the two rows
        const float2 y0 = M::template flux<1>(K, up, A, mup, MA), y1 = M::template flux<1>(K, A, B, MA, MB);
        const float2 y2 = M::template flux<1>(K, B, dn, MB, mdn);
        const float2 rA = M::div(K, fxp[0], fxm[0], y1, y0, zhA, zlA);
        const float2 rB = M::div(K, fxp[1], fxm[1], y2, y1, zhB, zlB);
        const size_t o = (size_t)i * plane + (size_t)gj * nz + gk;
        if (wj0) *reinterpret_cast<float2*>(r + o) = rA;
        if (wj1) *reinterpret_cast<float2*>(r + o + nz) = rB;
        fxm[0] = fxp[0];
        fxm[1] = fxp[1];
    };

    // prologue: field planes x0-2 .. x0+2, potentials x0-1 .. x0+1, plane x0+3
    // into the slot of x0-2, first x face.  Planes up to x1+1 and potentials up
    // to x1 are needed; every plane is fetched (and, fused, written) once.
    for (int p = x0 - 2; p <= x0 + 2; ++p) {
        fetch(p);
        stash(p);
    }
    fetch(x0 + 3);
    __syncthreads();
    compute_mu(x0 - 1);
    compute_mu(x0);
    compute_mu(x0 + 1);
    __syncthreads();
    if (x0 + 3 <= x1 + 1) stash(x0 + 3);
    if (x0 + 4 <= x1 + 1) fetch(x0 + 4);
    x_faces(x0 - 1, fxm);
    __syncthreads();
    // plane i: r(i) reads potentials i, i+1 and planes i, i+1; mu(i+2) reads
    // planes i+1 .. i+3 and writes the potential slot of i-1; the store of plane
    // i+4 overwrites the slot of plane i-1 - all last read before the barrier
    for (int i = x0; i < x1; ++i) {
        compute_r(i);
        if (i + 2 <= x1) compute_mu(i + 2);
        if (i + 4 <= x1 + 1) stash(i + 4);
        if (i + 5 <= x1 + 1) fetch(i + 5);
        __syncthreads();
    }
}

template <class T, bool FUSED, class M, bool XB = false>
__global__ void __launch_bounds__(THREADS, 4)
ch_rhs_fast_kernel(const float* __restrict__ u, const float* __restrict__ upd, float* __restrict__ u_new,
                   float* __restrict__ r, Geo G, ChP P, int LX) {
    __shared__ __align__(16) float cs[NC * T::FIELD];
    __shared__ __align__(16) float ms[NM * T::POT];
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    if (x0 >= x1) return;   // uniform across the block
    rhs_tile<T, FUSED, M, true, XB>(u, upd, u_new, r, G, P, blockIdx.x * T::TZ, blockIdx.y * T::TY, x0, x1, cs, ms);
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

// Persistent batched rhs: blocks pull work items until the list is exhausted
// (3 blocks per SM: the item loop's state does not fit the 64 registers of 4).
template <bool FUSED>
__global__ void __launch_bounds__(THREADS, 3)
ch_rhs_batch_kernel(const float* __restrict__ u, const float* __restrict__ upd, float* __restrict__ u_new,
                    float* __restrict__ r, const BatchInst* __restrict__ insts, const BatchItem* __restrict__ items,
                    int n_items, int* __restrict__ counter) {
    __shared__ __align__(16) float cs[NC * MAX_FIELD];
    __shared__ __align__(16) float ms[NM * MAX_POT];
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
            rhs_tile<TileWide, FUSED, TolMath, false>(u + o, FUSED ? upd + o : nullptr, FUSED ? u_new + o : nullptr, r + o,
                                               G, B.P, I.k0, I.j0, I.x0, I.x1, cs, ms);
        else
            rhs_tile<TileSquare, FUSED, TolMath, false>(u + o, FUSED ? upd + o : nullptr, FUSED ? u_new + o : nullptr,
                                                 r + o, G, B.P, I.k0, I.j0, I.x0, I.x1, cs, ms);
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
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_rhs_bps[0], ch_rhs_fast_kernel<TileWide, true, TolMath>,
                                                  THREADS, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_rhs_bps[1], ch_rhs_fast_kernel<TileSquare, true, TolMath>,
                                                  THREADS, 0);
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&g_batch_bps, ch_rhs_batch_kernel<true>, THREADS, 0);
    for (int* b : {&g_rhs_bps[0], &g_rhs_bps[1], &g_batch_bps})
        if (*b < 1) *b = 1;
}

template <class T>
int rhs_fast_launch_t(bool fused, bool exact, const float* u, const float* upd, float* u_new, float* r,
                      const evx_grid* g, const Geo& G, const ChP& P, cudaStream_t st, int bps) {
    int lx;
    const dim3 grid = fast_grid<T>(g->nx, g->ny, g->nz, bps, g_sms, &lx);
    if (G.kind[0] != EVX_BC_PERIODIC) {   // mirrored-x step (the caller has y and z periodic)
        if (exact) return fail(EVX_ERR_UNSUPPORTED, "fast rhs: a non-periodic x axis has the spectral loops' arithmetic only");
        if (fused)
            EVX_TIMED("ch_rhs_fused", st,
                      ch_rhs_fast_kernel<T, true, TolMath, true><<<grid, THREADS, 0, st>>>(u, upd, u_new, r, G, P, lx));
        else
            EVX_TIMED("ch_rhs", st,
                      ch_rhs_fast_kernel<T, false, TolMath, true><<<grid, THREADS, 0, st>>>(u, nullptr, nullptr, r, G, P,
                                                                                          lx));
    } else if (fused)
        EVX_TIMED("ch_rhs_fused", st,
                  ch_rhs_fast_kernel<T, true, TolMath><<<grid, THREADS, 0, st>>>(u, upd, u_new, r, G, P, lx));
    else if (exact)
        EVX_TIMED("ch_rhs", st,
                  ch_rhs_fast_kernel<T, false, ExactMath><<<grid, THREADS, 0, st>>>(u, nullptr, nullptr, r, G, P, lx));
    else
        EVX_TIMED("ch_rhs", st,
                  ch_rhs_fast_kernel<T, false, TolMath><<<grid, THREADS, 0, st>>>(u, nullptr, nullptr, r, G, P, lx));
    count_launch();
    return check_launch("ch_rhs_fast_kernel");
}

}  // namespace

int ch_tile_variant(int nz) {
    if (g_tile_override == 0) return 0;
    if (g_tile_override == 1) return 1;
    return default_tile_variant(nz);
}

int ch_rhs_fast_launch(bool fused, bool exact, const float* u, const float* upd, float* u_new, float* r,
                       const evx_grid* g, const Geo& G, const ChP& P, cudaStream_t st) {
    init_rhs_occupancy();
    if (fused && exact) return fail(EVX_ERR_UNSUPPORTED, "the fused rhs pass has the spectral loops' arithmetic only");
    if (ch_tile_variant(g->nz) == 1)
        return rhs_fast_launch_t<TileSquare>(fused, exact, u, upd, u_new, r, g, G, P, st, g_rhs_bps[1]);
    return rhs_fast_launch_t<TileWide>(fused, exact, u, upd, u_new, r, g, G, P, st, g_rhs_bps[0]);
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
    if (evx::g_tile_override != variant) evx::bump_config_epoch();
    evx::g_tile_override = variant;
    return EVX_OK;
}
