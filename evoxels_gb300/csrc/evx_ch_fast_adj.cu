// Periodic fast path of the Cahn-Hilliard adjoint pullback (tiling as in
// evx_ch_fast.cuh; the math is documented in evx_adjoint.cu):
//   lam_s = lam_{s+1} + [0<=u<=1] * ( w*phi'(c)*mub - kappa*L(mub) + sum_faces 0.5*cfb )
//   mub   = sum_a ih_a*(Gb_{-} - Gb_{+}),  Gb_f = ih*D*(g_lo - g_hi) * cf(1-cf)
//   cfb_f = (ih*D*(g_lo - g_hi)) * ((mu_hi - mu_lo)*ih) * (1 - 2cf)
// Per x-plane i a block computes lam on plane i, mu and mub on plane i+2 over
// the tile grown by one cell (3-slot rings) and stores the prefetched planes
// i+4 of c = clip(u_s) and g = P lam_{s+1} (5-slot rings), then loads plane
// i+5 into registers: every phase reads only data finished before the previous
// barrier, so one block barrier per plane suffices.  x faces, the previous
// plane's c and mub at the patch points are carried in registers.  Optional parameter-gradient partial sums are kept in
// float per thread and reduced in double per block: GR = 1 all four sums
// (<lam',u'-u>/D, -<mub,Lc>, <mub,phi(c)>, <h,u'-u>), GR = 2 only the two that
// need real space (the mobility sums then come from the spectral x-pass).
// Compiled with FMA contraction on: no bitwise-parity requirement here.
#include <algorithm>
#include <type_traits>

#include "evx_ch_fast.cuh"

namespace evx {
namespace {

using namespace fast;

// Shared-memory rings of c, g (field planes) and mu, mub (potential planes): one block barrier
// per plane needs NC / NM slots, two barriers per plane 4 / 2 (less shared memory).
template <bool ONEBAR>
struct Rings {
    static constexpr int C = (ONEBAR ? NC : 4) * MAX_FIELD, M = (ONEBAR ? NM : 2) * MAX_POT;
    static constexpr size_t SMEM = (size_t)(2 * C + 2 * M) * sizeof(float) + 4 * 8 * sizeof(double);
};
// Resident blocks per SM the single-grid gradient kernels are built for: 2 (128 registers, one
// barrier per plane) or 3 (80 registers, two barriers per plane, 68 KB of shared memory).
#ifndef EVX_PULLBACK_MIN_BLOCKS
#define EVX_PULLBACK_MIN_BLOCKS 2
#endif
constexpr bool PB_ONEBAR = EVX_PULLBACK_MIN_BLOCKS < 3;
using PbRings = Rings<PB_ONEBAR>;
using BatchRings = Rings<false>;   // the persistent batched kernel: two barriers per plane

// Two points of a patch row (z-adjacent) are processed together with the
// sm_100 two-lane fp32 instructions (FADD2 / FMUL2 / FFMA2).  Constants are
// folded into per-axis weights: with s = c_lo + c_hi on a face (cf = s/2),
//   Gb''  = D*ih2 * cf(1-cf) * (g_lo - g_hi)          = s*(gq2 + gq1*s) * dg
//   cfb'' = 0.5*D*ih2 * (g_lo - g_hi)(mu_hi - mu_lo)(1 - 2cf) = dg*dmu * (hw - hw*s)
// so mub = sum_a (Gb''_minus - Gb''_plus) and the 0.5-weighted cbar face sum is a
// plain sum of cfb''; -kappa is folded into the Laplacian weights.
struct PbK {
    float2 gq1[3], gq2[3];   // -D*ih2_a/4, D*ih2_a/2
    float2 hw[3], nhw[3];    // 0.5*D*ih2_a and its negative
    float2 lk[3], lkc;       // -kappa*ih2_a, 2*kappa*sum(ih2): -kappa*Laplacian
    float2 w, w6, nw6;       // w, 6w, -6w
};
__device__ __forceinline__ PbK make_pbk(const Geo& G, const ChP& P) {
    PbK K;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float dg = P.D * G.ih2[a];
        K.gq1[a] = f2s(-0.25f * dg);
        K.gq2[a] = f2s(0.5f * dg);
        K.hw[a] = f2s(0.5f * dg);
        K.nhw[a] = f2s(-0.5f * dg);
        K.lk[a] = f2s(-P.kappa * G.ih2[a]);
    }
    K.lkc = f2s(2.f * P.kappa * G.ih2sum);
    K.w = f2s(P.w);
    K.w6 = f2s(6.f * P.w);
    K.nw6 = f2s(-6.f * P.w);
    return K;
}
__device__ __forceinline__ float2 phi2(float2 c) {    // c(1-c)(1-2c)
    return mul2(mul2(c, sub2(f2s(1.f), c)), fma2(c, f2s(-2.f), f2s(1.f)));
}
// sum_a wa*(xp_a + xm_a) + c*wc
__device__ __forceinline__ float2 lapw(const float2 (&wa)[3], float2 wc, float2 c, float2 xm, float2 xp, float2 ym,
                                       float2 yp, float2 zm, float2 zp) {
    float2 t = mul2(add2(xp, xm), wa[0]);
    t = fma2(add2(yp, ym), wa[1], t);
    t = fma2(add2(zp, zm), wa[2], t);
    return fma2(c, wc, t);
}
template <int AX>
__device__ __forceinline__ float2 gb2(const PbK& K, float2 clo, float2 chi, float2 glo, float2 ghi) {
    const float2 sm = add2(clo, chi);
    return mul2(mul2(sm, fma2(sm, K.gq1[AX], K.gq2[AX])), sub2(glo, ghi));
}
template <int AX>
__device__ __forceinline__ float2 cfb2(const PbK& K, float2 clo, float2 chi, float2 mlo, float2 mhi, float2 glo,
                                       float2 ghi) {
    const float2 sm = add2(clo, chi);
    return mul2(mul2(sub2(glo, ghi), sub2(mhi, mlo)), fma2(sm, K.nhw[AX], K.hw[AX]));
}
__device__ __forceinline__ float2 sel2(bool px, bool py, float2 v) {
    return make_float2(px ? v.x : 0.f, py ? v.y : 0.f);
}

// Block reduction of four float partial sums into double, written by threads 0..3.
__device__ __forceinline__ void block_reduce4(float a, float b, float c, float d, double* red, double* out) {
    const int tid = threadIdx.x;
    double v[4] = {a, b, c, d};
    __syncthreads();
#pragma unroll
    for (int q = 0; q < 4; ++q) {
        double x = v[q];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
        if ((tid & 31) == 0) red[q * 8 + (tid >> 5)] = x;
    }
    __syncthreads();
    if (tid < 4) {
        double x = 0.0;
        for (int wi = 0; wi < 8; ++wi) x += red[tid * 8 + wi];
        out[tid] = x;
    }
}

// The last block to finish reduces every block's partial sums and the x-pass
// partials in a fixed order (deterministic) and resets the counter.  Partials
// of other blocks are read through L2 (__ldcg) after the counter handshake.
__device__ __noinline__ void last_block_reduce(const double* part, int nblk, const GradSink& sink, double* red) {
    __shared__ int s_last;
    const int tid = threadIdx.x;
    __threadfence();                       // this block's partials before its count
    __syncthreads();
    if (tid == 0) s_last = atomicAdd(sink.counter, 1) == nblk - 1;
    __syncthreads();
    if (!s_last) return;
    __threadfence();
    double a[4] = {0.0, 0.0, 0.0, 0.0};   // sK, sW, t1, t2
    for (int b = tid; b < nblk; b += THREADS) {
        a[0] += __ldcg(part + (size_t)b * 4 + 1);
        a[1] += __ldcg(part + (size_t)b * 4 + 2);
    }
    for (int b = tid; b < sink.nxpart; b += THREADS) {
        a[2] += __ldcg(sink.xpart + (size_t)b * 2);
        a[3] += __ldcg(sink.xpart + (size_t)b * 2 + 1);
    }
#pragma unroll
    for (int q = 0; q < 4; ++q)
        for (int o = 16; o > 0; o >>= 1) a[q] += __shfl_down_sync(0xffffffffu, a[q], o);
    __syncthreads();                       // red was last read by block_reduce4
    if ((tid & 31) == 0)
#pragma unroll
        for (int q = 0; q < 4; ++q) red[q * 8 + (tid >> 5)] = a[q];
    __syncthreads();
    if (tid == 0) {
        double t[4] = {0.0, 0.0, 0.0, 0.0};
        for (int q = 0; q < 4; ++q)
            for (int w = 0; w < THREADS / 32; ++w) t[q] += red[q * 8 + w];
        sink.grads[0] += t[2] * sink.invD - sink.kA * t[3];
        sink.grads[1] += t[0] - sink.DA * t[3];
        sink.grads[2] += t[1];
        *sink.counter = 0;
    }
}

// XB (one-barrier flow only): a Neumann or Dirichlet x axis, y and z periodic (the mirrored-x step).
// As the reference pads c and mu with the ghost a*cell + b (a = 1 Neumann, -1 Dirichlet), the planes
// beyond the grid are staged as the ghosts of the boundary planes with g = 0, the potential of a ghost
// plane is the forward ghost of mu and a*mub of its boundary plane, the boundary plane's outer x face
// enters mub with weight (1 - a) and the cbar face sum with weight (1 + a) (the ghosts' cotangents
// folded back into the boundary cell, as in the generic kernel).
template <class T, int GR, bool ONEBAR = true, bool XB = false>
__device__ __forceinline__ void pullback_tile(const float* __restrict__ u, const float* __restrict__ gfield,
                                              const float* __restrict__ lam, const float* __restrict__ hfield,
                                              const float* __restrict__ u1, float* __restrict__ lam_out,
                                              const Geo& G, const ChP& P, int k0, int j0, int x0, int x1,
                                              float* cs, float* gs, float* ms, float* bs,
                                              float& sD, float& sK, float& sW, float& sH) {
    const int tid = threadIdx.x;
    const int tx = tid % T::BX, ty = tid / T::BX;
    // ring slots: NC / NM slots with one barrier per plane, else 4 / 2 slots and two
    auto cslt = [](int p) { return ONEBAR ? cslot(p) : (p & 3); };
    auto mslt = [](int p) { return ONEBAR ? mslot(p) : (p & 1); };
    const int W = T::W;
    const int nx = G.nx, ny = G.ny, nz = G.nz;
    const size_t plane = (size_t)ny * nz;
    const PbK K = make_pbk(G, P);
    const LoadPlan LP = make_load_plan<T>(tid, j0, k0, ny, nz);
    // Stage-A work (mu and mub over the tile grown by one cell, T::NMU 2x2 patches): patch tid for
    // every thread, and the patches beyond THREADS split into single rows over the first 2*(NMU -
    // THREADS) threads, so the warps that take the extra work carry half a patch more, not a whole one
    // (the block barrier waits for the slowest warp every plane).
    constexpr int NHALF = T::NMU > THREADS ? 2 * (T::NMU - THREADS) : 0;
    static_assert(NHALF <= THREADS, "at most one extra row per thread");
    int mo_[1];   // field offset of this thread's potential patch (upper row, left column)
    bool mv[1];
    mv[0] = tid < T::NMU;
    {
        const int py = mv[0] ? tid / T::MPZ : 0;
        mo_[0] = (1 + 2 * py) * W + 2 + 2 * (tid - py * T::MPZ);
    }
    const bool hv = tid < NHALF;   // this thread's extra row
    int ho;
    {
        const int q = hv ? THREADS + (tid >> 1) : 0;
        const int py = q / T::MPZ;
        ho = (1 + 2 * py + (tid & 1)) * W + 2 + 2 * (q - py * T::MPZ);
    }
    const int ra = 2 + 2 * ty, rc = 4 + 2 * tx;
    const int gj = j0 + 2 * ty, gk = k0 + 2 * tx;
    const bool wk = gk < nz, wj0 = gj < ny && wk, wj1 = gj + 1 < ny && wk;
    const int pa = ra * W + rc, pb = pa + W;   // field offsets of the patch rows
    float2 aD = f2s(0.f), aK = f2s(0.f), aW = f2s(0.f), aH = f2s(0.f);   // gradient partial sums

    static_assert(!XB || ONEBAR, "x boundaries: one-barrier flow only");
    const float ax = (XB && G.kind[0] == EVX_BC_DIRICHLET) ? -1.f : 1.f;
    auto xghost = [&](float2 v, bool lo) -> float2 {   // Neumann the values, Dirichlet 2v - values
        if (G.kind[0] == EVX_BC_NEUMANN) return v;
        return sub2(f2s(lo ? G.lo[0] : G.hi[0]), v);
    };
    float4 pc[2], pg[2];
    auto fetch = [&](int p) {
        const size_t base = (size_t)(XB ? min(max(p, 0), nx - 1) : pmod(p, nx)) * plane;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!LP.valid[s]) continue;
            pc[s] = ldg4(u + base + LP.goff[s]);
            pg[s] = ldg4(gfield + base + LP.goff[s]);
        }
    };
    auto stash = [&](int slot, int p) {
        float* dc = cs + slot * T::FIELD;
        float* dg = gs + slot * T::FIELD;
        const bool ghost = XB && (p < 0 || p >= nx);
#pragma unroll
        for (int s = 0; s < 2; ++s)
            if (LP.valid[s]) {
                float4 c = clip4(pc[s]);
                float4 g = pg[s];
                if (ghost) {   // the boundary plane's ghost, with no cotangent
                    const float2 lo = xghost(make_float2(c.x, c.y), p < 0), hi = xghost(make_float2(c.z, c.w), p < 0);
                    c = make_float4(lo.x, lo.y, hi.x, hi.y);
                    g = make_float4(0.f, 0.f, 0.f, 0.f);
                }
                sts4(dc + LP.soff[s], c);
                sts4(dg + LP.soff[s], g);
            }
    };

    float2 gxm[1][2];   // Gb'' on the x face below the current potential plane, per patch row
    float2 gxh;         // the same for the extra row
    // x faces between field slots c0/g0 (plane p) and c1/g1 (plane p+1) of potential patch m
    auto gx_faces = [&](const float* c0, const float* c1, const float* g0, const float* g1, int m, float2 out[2]) {
        const int a = mo_[m], b = a + W;
        out[0] = gb2<0>(K, lds2(c0 + a), lds2(c1 + a), lds2(g0 + a), lds2(g1 + a));
        out[1] = gb2<0>(K, lds2(c0 + b), lds2(c1 + b), lds2(g0 + b), lds2(g1 + b));
    };

    // mu and mub of plane p: field slots cm (p-1), cc (p), cp (p+1) and g slots gc (p), gp (p+1);
    // writes potential slots mo / bo
    auto compute_mu = [&](const float* cm, const float* cc, const float* cp, const float* gc, const float* gp,
                          float* mo, float* bo, int q) {
        // XB: weights of the boundary plane's outer x face in mub
        const bool wlo = XB && q == 0, whi = XB && q == nx - 1;
        const float2 fw = f2s(1.f - ax);
#pragma unroll
        for (int m = 0; m < 1; ++m) {
            if (!mv[m]) continue;
            const int a = mo_[m], b = a + W;
            const float2 up = lds2(cc + a - W), A = lds2(cc + a), B = lds2(cc + b), dn = lds2(cc + b + W);
            const float2 zmA = make_float2(cc[a - 1], A.x), zpA = make_float2(A.y, cc[a + 2]);
            const float2 zmB = make_float2(cc[b - 1], B.x), zpB = make_float2(B.y, cc[b + 2]);
            // chemical potential w*phi(c) - kappa*L(c) on the 2x2 patch
            const float2 muA = fma2(K.w, phi2(A), lapw(K.lk, K.lkc, A, lds2(cm + a), lds2(cp + a), up, B, zmA, zpA));
            const float2 muB = fma2(K.w, phi2(B), lapw(K.lk, K.lkc, B, lds2(cm + b), lds2(cp + b), A, dn, zmB, zpB));
            *reinterpret_cast<float2*>(mo + a - W) = muA;
            *reinterpret_cast<float2*>(mo + b - W) = muB;
            // mub = sum_faces (Gb''_minus - Gb''_plus)
            float2 gxp[2];
            gx_faces(cc, cp, gc, gp, m, gxp);
            float2 bA, bB;
            if (XB && (wlo || whi)) {
                bA = sub2(wlo ? mul2(fw, gxm[m][0]) : gxm[m][0], whi ? mul2(fw, gxp[0]) : gxp[0]);
                bB = sub2(wlo ? mul2(fw, gxm[m][1]) : gxm[m][1], whi ? mul2(fw, gxp[1]) : gxp[1]);
            } else {
                bA = sub2(gxm[m][0], gxp[0]);
                bB = sub2(gxm[m][1], gxp[1]);
            }
            gxm[m][0] = gxp[0];
            gxm[m][1] = gxp[1];
            const float2 gup = lds2(gc + a - W), gA = lds2(gc + a), gB = lds2(gc + b), gdn = lds2(gc + b + W);
            {   // z faces: (left, mid) and (mid, right) of each row
                const float2 gzmA = make_float2(gc[a - 1], gA.x), gzpA = make_float2(gA.y, gc[a + 2]);
                const float2 gzmB = make_float2(gc[b - 1], gB.x), gzpB = make_float2(gB.y, gc[b + 2]);
                bA = add2(bA, sub2(gb2<2>(K, zmA, A, gzmA, gA), gb2<2>(K, A, zpA, gA, gzpA)));
                bB = add2(bB, sub2(gb2<2>(K, zmB, B, gzmB, gB), gb2<2>(K, B, zpB, gB, gzpB)));
            }
            {   // y faces above, between and below the two rows
                const float2 y0 = gb2<1>(K, up, A, gup, gA), y1 = gb2<1>(K, A, B, gA, gB);
                const float2 y2 = gb2<1>(K, B, dn, gB, gdn);
                bA = add2(bA, sub2(y0, y1));
                bB = add2(bB, sub2(y1, y2));
            }
            *reinterpret_cast<float2*>(bo + a - W) = bA;
            *reinterpret_cast<float2*>(bo + b - W) = bB;
        }
        if (hv) {   // the extra row: the same terms for one row
            const int a = ho;
            const float2 up = lds2(cc + a - W), A = lds2(cc + a), dn = lds2(cc + a + W);
            const float2 zmA = make_float2(cc[a - 1], A.x), zpA = make_float2(A.y, cc[a + 2]);
            *reinterpret_cast<float2*>(mo + a - W) =
                fma2(K.w, phi2(A), lapw(K.lk, K.lkc, A, lds2(cm + a), lds2(cp + a), up, dn, zmA, zpA));
            const float2 gA = lds2(gc + a);
            const float2 gxp = gb2<0>(K, A, lds2(cp + a), gA, lds2(gp + a));
            float2 bA;
            if (XB && (wlo || whi)) bA = sub2(wlo ? mul2(fw, gxh) : gxh, whi ? mul2(fw, gxp) : gxp);
            else bA = sub2(gxh, gxp);
            gxh = gxp;
            const float2 gup = lds2(gc + a - W), gdn = lds2(gc + a + W);
            const float2 gzmA = make_float2(gc[a - 1], gA.x), gzpA = make_float2(gA.y, gc[a + 2]);
            bA = add2(bA, sub2(gb2<2>(K, zmA, A, gzmA, gA), gb2<2>(K, A, zpA, gA, gzpA)));
            bA = add2(bA, sub2(gb2<1>(K, up, A, gup, gA), gb2<1>(K, A, dn, gA, gdn)));
            *reinterpret_cast<float2*>(bo + a - W) = bA;
        }
    };

    // x face cbar'' of the output patch between planes (c0, g0, m0) and (c1, g1, m1)
    float2 cfx_m[2], b_prev[2];
    // c, mu and g of the current output plane at the patch points (rows a, b), carried from the x faces
    // of the plane below, where they were the upper side
    float2 xc[2], xm[2], xg[2];
    auto x_faces_b = [&](const float* c1, const float* g1, const float* m1, float2 out[2]) {
        const float2 c1a = lds2(c1 + pa), c1b = lds2(c1 + pb), m1a = lds2(m1 + pa - W), m1b = lds2(m1 + pb - W);
        const float2 g1a = lds2(g1 + pa), g1b = lds2(g1 + pb);
        out[0] = cfb2<0>(K, xc[0], c1a, xm[0], m1a, xg[0], g1a);
        out[1] = cfb2<0>(K, xc[1], c1b, xm[1], m1b, xg[1], g1b);
        xc[0] = c1a;
        xc[1] = c1b;
        xm[0] = m1a;
        xm[1] = m1b;
        xg[0] = g1a;
        xg[1] = g1b;
    };

    // lam on plane i: field slots cc (i), cx (i+1), g slots gc (i), gx (i+1), potential slots mm / bb (i)
    // and mx / bx (i+1)
    auto compute_lam = [&](int i, const float* cc, const float* cx, const float* gc, const float* gx,
                           const float* mm, const float* mx, const float* bb, const float* bx) {
        // acc: sum of the cbar'' face values around each point
        float2 accA, accB;
        const float2 A = xc[0], B = xc[1], MA = xm[0], MB = xm[1], gA = xg[0], gB = xg[1];
        {
            float2 cfx_p[2];
            x_faces_b(cx, gx, mx, cfx_p);
            if (XB && (i == 0 || i == nx - 1)) {   // the boundary plane's outer face, weight 1 + a
                const float2 fw = f2s(1.f + ax);
                accA = add2(i == 0 ? mul2(fw, cfx_m[0]) : cfx_m[0], i == nx - 1 ? mul2(fw, cfx_p[0]) : cfx_p[0]);
                accB = add2(i == 0 ? mul2(fw, cfx_m[1]) : cfx_m[1], i == nx - 1 ? mul2(fw, cfx_p[1]) : cfx_p[1]);
            } else {
                accA = add2(cfx_m[0], cfx_p[0]);
                accB = add2(cfx_m[1], cfx_p[1]);
            }
            cfx_m[0] = cfx_p[0];
            cfx_m[1] = cfx_p[1];
        }
        const float2 up = lds2(cc + pa - W), dn = lds2(cc + pb + W);
        const float2 zmA = make_float2(cc[pa - 1], A.x), zpA = make_float2(A.y, cc[pa + 2]);
        const float2 zmB = make_float2(cc[pb - 1], B.x), zpB = make_float2(B.y, cc[pb + 2]);
        {   // z faces
            const float2 mzmA = make_float2(mm[pa - W - 1], MA.x), mzpA = make_float2(MA.y, mm[pa - W + 2]);
            const float2 mzmB = make_float2(mm[pb - W - 1], MB.x), mzpB = make_float2(MB.y, mm[pb - W + 2]);
            const float2 gzmA = make_float2(gc[pa - 1], gA.x), gzpA = make_float2(gA.y, gc[pa + 2]);
            const float2 gzmB = make_float2(gc[pb - 1], gB.x), gzpB = make_float2(gB.y, gc[pb + 2]);
            accA = add2(accA, add2(cfb2<2>(K, zmA, A, mzmA, MA, gzmA, gA), cfb2<2>(K, A, zpA, MA, mzpA, gA, gzpA)));
            accB = add2(accB, add2(cfb2<2>(K, zmB, B, mzmB, MB, gzmB, gB), cfb2<2>(K, B, zpB, MB, mzpB, gB, gzpB)));
        }
        {   // y faces
            const float2 mup = lds2(mm + pa - 2 * W), mdn = lds2(mm + pb);
            const float2 gup = lds2(gc + pa - W), gdn = lds2(gc + pb + W);
            const float2 y0 = cfb2<1>(K, up, A, mup, MA, gup, gA), y1 = cfb2<1>(K, A, B, MA, MB, gA, gB);
            const float2 y2 = cfb2<1>(K, B, dn, MB, mdn, gB, gdn);
            accA = add2(accA, add2(y0, y1));
            accB = add2(accB, add2(y1, y2));
        }
        // -kappa*L(mub) + acc
        const float2 bA = lds2(bb + pa - W), bB = lds2(bb + pb - W);
        const float2 tA = add2(accA, lapw(K.lk, K.lkc, bA, b_prev[0], lds2(bx + pa - W), lds2(bb + pa - 2 * W), bB,
                                          make_float2(bb[pa - W - 1], bA.x), make_float2(bA.y, bb[pa - W + 2])));
        const float2 tB = add2(accB, lapw(K.lk, K.lkc, bB, b_prev[1], lds2(bx + pb - W), bA, lds2(bb + pb),
                                          make_float2(bb[pb - W - 1], bB.x), make_float2(bB.y, bb[pb - W + 2])));
        const size_t o = (size_t)i * plane + (size_t)gj * nz + gk;
        const float2 u0 = wj0 ? __ldg(reinterpret_cast<const float2*>(u + o)) : f2s(0.f);
        const float2 u1r = wj1 ? __ldg(reinterpret_cast<const float2*>(u + o + nz)) : f2s(0.f);
        const float2 l0 = wj0 ? __ldg(reinterpret_cast<const float2*>(lam + o)) : f2s(0.f);
        const float2 l1 = wj1 ? __ldg(reinterpret_cast<const float2*>(lam + o + nz)) : f2s(0.f);
        {
            // cbar = w*phi'(c)*mub - kappa*L(mub) + acc, w*phi'(c) = w + c*(6w*c - 6w);
            // lam_s = lam' + [0<=u<=1]*cbar, the mask being clip(u) == u
            const float2 cbA = fma2(fma2(A, fma2(A, K.w6, K.nw6), K.w), bA, tA);
            const float2 cbB = fma2(fma2(B, fma2(B, K.w6, K.nw6), K.w), bB, tB);
            const float2 oA = add2(l0, sel2(A.x == u0.x, A.y == u0.y, cbA));
            const float2 oB = add2(l1, sel2(B.x == u1r.x, B.y == u1r.y, cbB));
            if (wj0) *reinterpret_cast<float2*>(lam_out + o) = oA;
            if (wj1) *reinterpret_cast<float2*>(lam_out + o + nz) = oB;
        }
        if (GR) {
            // -<mub, L(c)> from mu = w*phi(c) - kappa*L(c) at the point: sum mub*mu and sum mub*phi,
            // combined as (sum mub*mu - w*sum mub*phi)/kappa at the end
            if (wj0) {
                aK = fma2(bA, MA, aK);
                aW = fma2(bA, phi2(A), aW);
            }
            if (wj1) {
                aK = fma2(bB, MB, aK);
                aW = fma2(bB, phi2(B), aW);
            }
            if (GR == 1) {
                const float2 invD = f2s(1.f / P.D);
                const float2 h0 = wj0 ? __ldg(reinterpret_cast<const float2*>(hfield + o)) : f2s(0.f);
                const float2 h1 = wj1 ? __ldg(reinterpret_cast<const float2*>(hfield + o + nz)) : f2s(0.f);
                const float2 n0 = wj0 ? __ldg(reinterpret_cast<const float2*>(u1 + o)) : f2s(0.f);
                const float2 n1 = wj1 ? __ldg(reinterpret_cast<const float2*>(u1 + o + nz)) : f2s(0.f);
                // <g, r/D> = <P lam', r>/D = <lam', u' - u>/D  (P is symmetric); zeros where a row is outside
                aD = fma2(mul2(l0, sub2(n0, u0)), invD, aD);
                aD = fma2(mul2(l1, sub2(n1, u1r)), invD, aD);
                aH = fma2(h0, sub2(n0, u0), aH);
                aH = fma2(h1, sub2(n1, u1r), aH);
            }
        }
        b_prev[0] = bA;
        b_prev[1] = bB;
    };

    const float* C = cs;
    const float* Gf = gs;
    auto cf = [&](int slot) { return C + slot * T::FIELD; };
    auto gf = [&](int slot) { return Gf + slot * T::FIELD; };
    auto mp = [&](int slot) { return ms + slot * T::POT; };
    auto bp = [&](int slot) { return bs + slot * T::POT; };
    // XB: the potential of ghost plane p from its boundary plane q at this thread's stage-A points (the
    // thread wrote plane q's values there itself): the forward ghost of mu and a*mub
    auto ghost_pot = [&](int p, int q) {
        const bool lo = p < 0;
        const float* mq = mp(mslt(q));
        const float* bq = bp(mslt(q));
        float* mg = mp(mslt(p));
        float* bg = bp(mslt(p));
        const float2 a2 = f2s(ax);
        auto row = [&](int o) {
            *reinterpret_cast<float2*>(mg + o - W) = xghost(lds2(mq + o - W), lo);
            *reinterpret_cast<float2*>(bg + o - W) = mul2(a2, lds2(bq + o - W));
        };
        if (mv[0]) {
            row(mo_[0]);
            row(mo_[0] + W);
        }
        if (hv) row(ho);
    };
    // potential of plane p from the field slots of p-1, p, p+1
    auto mu_of = [&](int p) {
        if (XB && (p < 0 || p >= nx)) {
            ghost_pot(p, p < 0 ? 0 : nx - 1);
            return;
        }
        const int s0 = cslt(p - 1), s1 = cslt(p), s2 = cslt(p + 1), t = mslt(p);
        compute_mu(cf(s0), cf(s1), cf(s2), gf(s1), gf(s2), mp(t), bp(t), p);
    };

    if (ONEBAR) {
        // prologue: planes x0-2 .. x0+2 staged; potentials x0-1 .. x0+1; plane
        // x0+3 staged into the slot of x0-2; carried x quantities.  Planes up to
        // x1+1 and potentials up to x1 are needed.
        for (int p = x0 - 2; p <= x0 + 2; ++p) {
            fetch(p);
            stash(cslt(p), p);
        }
        fetch(x0 + 3);
        __syncthreads();
        if (XB && x0 == 0) {
            // the face below plane 0 against the staged ghost plane; the ghost plane's potential is
            // derived from plane 0's, so it comes after it
            if (mv[0]) gx_faces(cf(cslt(-1)), cf(cslt(0)), gf(cslt(-1)), gf(cslt(0)), 0, gxm[0]);
            if (hv) gxh = gb2<0>(K, lds2(cf(cslt(-1)) + ho), lds2(cf(cslt(0)) + ho), lds2(gf(cslt(-1)) + ho),
                                 lds2(gf(cslt(0)) + ho));
            mu_of(0);
            mu_of(1);
            mu_of(-1);
        } else {
            if (mv[0]) gx_faces(cf(cslt(x0 - 2)), cf(cslt(x0 - 1)), gf(cslt(x0 - 2)), gf(cslt(x0 - 1)), 0, gxm[0]);
            if (hv) gxh = gb2<0>(K, lds2(cf(cslt(x0 - 2)) + ho), lds2(cf(cslt(x0 - 1)) + ho),
                                 lds2(gf(cslt(x0 - 2)) + ho), lds2(gf(cslt(x0 - 1)) + ho));
            mu_of(x0 - 1);
            mu_of(x0);
            mu_of(x0 + 1);
        }
        __syncthreads();
        if (x0 + 3 <= x1 + 1) stash(cslt(x0 + 3), x0 + 3);
        if (x0 + 4 <= x1 + 1) fetch(x0 + 4);
    } else {
        // prologue: planes x0-2 .. x0+1 staged; potentials x0-1, x0
        for (int p = x0 - 2; p <= x0 + 1; ++p) {
            fetch(p);
            stash(cslt(p), p);
        }
        fetch(x0 + 2);
        __syncthreads();
        if (mv[0]) gx_faces(cf(cslt(x0 - 2)), cf(cslt(x0 - 1)), gf(cslt(x0 - 2)), gf(cslt(x0 - 1)), 0, gxm[0]);
        if (hv) gxh = gb2<0>(K, lds2(cf(cslt(x0 - 2)) + ho), lds2(cf(cslt(x0 - 1)) + ho), lds2(gf(cslt(x0 - 2)) + ho),
                             lds2(gf(cslt(x0 - 1)) + ho));
        mu_of(x0 - 1);
        mu_of(x0);
        __syncthreads();
    }
    {
        const int s0 = cslt(x0 - 1), s1 = cslt(x0), t0 = mslt(x0 - 1), t1 = mslt(x0);
        xc[0] = lds2(cf(s0) + pa);
        xc[1] = lds2(cf(s0) + pb);
        xm[0] = lds2(mp(t0) + pa - W);
        xm[1] = lds2(mp(t0) + pb - W);
        xg[0] = lds2(gf(s0) + pa);
        xg[1] = lds2(gf(s0) + pb);
        x_faces_b(cf(s1), gf(s1), mp(t1), cfx_m);
        b_prev[0] = lds2(bp(t0) + pa - W);
        b_prev[1] = lds2(bp(t0) + pb - W);
    }
    if (ONEBAR) {
        __syncthreads();
        // plane i: lam(i) reads potentials i, i+1 and planes i, i+1; mu(i+2) reads
        // planes i+1 .. i+3 and writes the potential slot of i-1; the stash of
        // plane i+4 overwrites the slot of plane i-1 - all last read before the barrier.
        // Slots of planes i .. i+4 (all five) and potentials i .. i+2 (all three),
        // advanced by one per plane.
        int c0 = cslot(x0), m0 = mslot(x0);
        for (int i = x0; i < x1; ++i) {
            const int c1 = c0 + 1 == NC ? 0 : c0 + 1, c2 = c1 + 1 == NC ? 0 : c1 + 1;
            const int c3 = c2 + 1 == NC ? 0 : c2 + 1, c4 = c3 + 1 == NC ? 0 : c3 + 1;
            const int m1 = m0 + 1 == NM ? 0 : m0 + 1, m2 = m1 + 1 == NM ? 0 : m1 + 1;
            compute_lam(i, cf(c0), cf(c1), gf(c0), gf(c1), mp(m0), mp(m1), bp(m0), bp(m1));
            if (i + 2 <= x1) {
                if (XB && i + 2 >= nx) ghost_pot(i + 2, nx - 1);
                else compute_mu(cf(c1), cf(c2), cf(c3), gf(c2), gf(c3), mp(m2), bp(m2), i + 2);
            }
            if (i + 4 <= x1 + 1) stash(c4, i + 4);
            if (i + 5 <= x1 + 1) fetch(i + 5);
            __syncthreads();
            c0 = c1;
            m0 = m1;
        }
    } else {
        for (int i = x0; i < x1; ++i) {
            stash(cslt(i + 2), i + 2);
            if (i + 3 <= x1 + 1) fetch(i + 3);
            __syncthreads();
            mu_of(i + 1);
            __syncthreads();
            const int s0 = cslt(i), s1 = cslt(i + 1), t0 = mslt(i), t1 = mslt(i + 1);
            compute_lam(i, cf(s0), cf(s1), gf(s0), gf(s1), mp(t0), mp(t1), bp(t0), bp(t1));
        }
    }
    sD += aD.x + aD.y;
    sK += ((aK.x + aK.y) - P.w * (aW.x + aW.y)) / P.kappa;
    sW += aW.x + aW.y;
    sH += aH.x + aH.y;
}

template <class T, int GR, bool XB = false>
__global__ void __launch_bounds__(THREADS, EVX_PULLBACK_MIN_BLOCKS)
ch_pullback_fast_kernel(const float* __restrict__ u, const float* __restrict__ gfield, const float* __restrict__ lam,
                        const float* __restrict__ hfield, const float* __restrict__ u1, float* __restrict__ lam_out,
                        double* __restrict__ part, Geo G, ChP P, int seg, GradSink sink) {
    extern __shared__ __align__(16) float smem[];
    float* cs = smem;
    float* gs = cs + PbRings::C;
    float* ms = gs + PbRings::C;
    float* bs = ms + PbRings::M;
    double* red = reinterpret_cast<double*>(bs + PbRings::M);   // [4][8]
    // block b owns planes [b*seg, b*seg + seg) of the tile-major sequence of
    // (tile, x) planes: one wave of equal segments, a segment that crosses a
    // tile boundary finishes one tile and starts the next
    const int ntz = (G.nz + T::TZ - 1) / T::TZ, nty = (G.ny + T::TY - 1) / T::TY;
    const long total = (long)ntz * nty * G.nx;
    long s0 = (long)blockIdx.x * seg;
    const long s1 = min(s0 + (long)seg, total);
    float sD = 0.f, sK = 0.f, sW = 0.f, sH = 0.f;
    while (s0 < s1) {
        const int t = (int)(s0 / G.nx);
        const int xa = (int)(s0 - (long)t * G.nx);
        const int xb = (int)min((long)G.nx, xa + (s1 - s0));
        pullback_tile<T, GR, PB_ONEBAR, XB>(u, gfield, lam, hfield, u1, lam_out, G, P, (t % ntz) * T::TZ, (t / ntz) * T::TY, xa,
                             xb, cs, gs, ms, bs, sD, sK, sW, sH);
        s0 += xb - xa;   // the tile's last barrier protects the rings from the next tile's prologue
    }
    if (GR) {
        block_reduce4(sD, sK, sW, sH, red, part + (size_t)blockIdx.x * 4);
        if (GR == 2 && sink.counter) last_block_reduce(part, (int)gridDim.x, sink, red);
    }
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

// Persistent batched pullback; with GRADS each work item writes its partial sums
// to part[item*4 .. item*4+3].
// GR as pullback_tile: 0 none, 1 all four gradient sums (reads h and u1), 2 the
// two real-space sums of the spectral-gradient path
template <int GR>
__global__ void __launch_bounds__(THREADS, 2)
ch_pullback_batch_kernel(const float* __restrict__ u, const float* __restrict__ gfield, const float* __restrict__ lam,
                         const float* __restrict__ hfield, const float* __restrict__ u1, float* __restrict__ lam_out,
                         double* __restrict__ part, const BatchInst* __restrict__ insts,
                         const BatchItem* __restrict__ items, int n_items, int* __restrict__ counter) {
    extern __shared__ __align__(16) float smem[];
    float* cs = smem;
    float* gs = cs + BatchRings::C;
    float* ms = gs + BatchRings::C;
    float* bs = ms + BatchRings::M;
    double* red = reinterpret_cast<double*>(bs + BatchRings::M);
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
        float sD = 0.f, sK = 0.f, sW = 0.f, sH = 0.f;
        if (B.tile == 0)
            pullback_tile<TileWide, GR, false>(u + o, gfield + o, lam + o, GR == 1 ? hfield + o : nullptr,
                                               GR == 1 ? u1 + o : nullptr, lam_out + o, G, B.P, I.k0, I.j0, I.x0, I.x1,
                                               cs, gs, ms, bs, sD, sK, sW, sH);
        else
            pullback_tile<TileSquare, GR, false>(u + o, gfield + o, lam + o, GR == 1 ? hfield + o : nullptr,
                                                 GR == 1 ? u1 + o : nullptr, lam_out + o, G, B.P, I.k0, I.j0, I.x0,
                                                 I.x1, cs, gs, ms, bs, sD, sK, sW, sH);
        if (GR) block_reduce4(sD, sK, sW, sH, red, part + (size_t)I.part * 4);
        __syncthreads();   // shared memory and s_item are reused by the next item
    }
}

int g_bps[2][3] = {{0, 0, 0}, {0, 0, 0}};   // [tile variant][gradient mode]
int g_batch_bps[3] = {0, 0, 0};
int g_sms = 0;

void init_occupancy() {
    if (g_sms) return;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    auto setup = [](auto kern, int* out, size_t smem) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, kern, THREADS, smem);
        if (*out < 1) *out = 1;
    };
    setup(ch_pullback_fast_kernel<TileWide, 0>, &g_bps[0][0], PbRings::SMEM);
    setup(ch_pullback_fast_kernel<TileWide, 1>, &g_bps[0][1], PbRings::SMEM);
    setup(ch_pullback_fast_kernel<TileWide, 2>, &g_bps[0][2], PbRings::SMEM);
    setup(ch_pullback_fast_kernel<TileSquare, 0>, &g_bps[1][0], PbRings::SMEM);
    setup(ch_pullback_fast_kernel<TileSquare, 1>, &g_bps[1][1], PbRings::SMEM);
    setup(ch_pullback_fast_kernel<TileSquare, 2>, &g_bps[1][2], PbRings::SMEM);
    int xb_bps = 0;   // the mirrored-x variants: the same resources as their periodic counterparts
    setup(ch_pullback_fast_kernel<TileWide, 0, true>, &xb_bps, PbRings::SMEM);
    setup(ch_pullback_fast_kernel<TileWide, 1, true>, &xb_bps, PbRings::SMEM);
    setup(ch_pullback_fast_kernel<TileSquare, 0, true>, &xb_bps, PbRings::SMEM);
    setup(ch_pullback_fast_kernel<TileSquare, 1, true>, &xb_bps, PbRings::SMEM);
    setup(ch_pullback_batch_kernel<0>, &g_batch_bps[0], BatchRings::SMEM);
    setup(ch_pullback_batch_kernel<1>, &g_batch_bps[1], BatchRings::SMEM);
    setup(ch_pullback_batch_kernel<2>, &g_batch_bps[2], BatchRings::SMEM);
}

// One wave of blocks over equal segments of the tile-major (tile, x) plane
// sequence, at least 8 planes each (the x halo costs 6 plane loads per piece; on small grids
// a shorter piece that fills more of the slots still wins).
template <class T>
dim3 pb_grid(const evx_grid* g, int grads, int* seg) {
    const int v = std::is_same<T, TileWide>::value ? 0 : 1;
    const long tiles = (long)((g->nz + T::TZ - 1) / T::TZ) * ((g->ny + T::TY - 1) / T::TY);
    const long total = tiles * g->nx;
    const long slots = (long)std::max(1, g_bps[v][grads]) * std::max(1, g_sms);
    long len = (total + slots - 1) / slots;
    len = std::max(len, std::min<long>(8, g->nx));
    *seg = (int)len;
    return dim3((unsigned)((total + len - 1) / len));
}

template <class T>
int pb_launch_t(int grads, const float* u, const float* g, const float* lam, const float* h, const float* u1,
                float* lam_out, double* part, int n_part_cap, const evx_grid* grid_, const Geo& G, const ChP& P,
                cudaStream_t st, int* n_part_used, const GradSink* sink) {
    const GradSink none{nullptr, nullptr, 0, nullptr, 0.0, 0.0, 0.0};
    const GradSink S = (grads == 2 && sink) ? *sink : none;
    int seg;
    const dim3 grid = pb_grid<T>(grid_, grads, &seg);
    const int nb = (int)grid.x;
    if (grads && nb > n_part_cap) return fail(EVX_ERR_WORKSPACE, "partial-sum buffer too small (%d > %d)", nb, n_part_cap);
    if (n_part_used) *n_part_used = nb;
    if (G.kind[0] != EVX_BC_PERIODIC) {   // mirrored-x step (y and z periodic): x ghosts, no stored spectra
        if (grads == 2) return fail(EVX_ERR_UNSUPPORTED, "fast pullback: spectral sums need a periodic x axis");
        if (grads == 1)
            EVX_TIMED("ch_pullback_grads", st,
                      ch_pullback_fast_kernel<T, 1, true><<<grid, THREADS, PbRings::SMEM, st>>>(u, g, lam, h, u1, lam_out,
                                                                                         part, G, P, seg, S));
        else
            EVX_TIMED("ch_pullback", st,
                      ch_pullback_fast_kernel<T, 0, true><<<grid, THREADS, PbRings::SMEM, st>>>(u, g, lam, nullptr, nullptr,
                                                                                         lam_out, nullptr, G, P, seg, S));
    } else if (grads == 1)
        EVX_TIMED("ch_pullback_grads", st,
                  ch_pullback_fast_kernel<T, 1><<<grid, THREADS, PbRings::SMEM, st>>>(u, g, lam, h, u1, lam_out, part, G, P, seg, S));
    else if (grads == 2)
        EVX_TIMED("ch_pullback_grads_spec", st,
                  ch_pullback_fast_kernel<T, 2><<<grid, THREADS, PbRings::SMEM, st>>>(u, g, lam, nullptr, nullptr, lam_out, part,
                                                                                 G, P, seg, S));
    else
        EVX_TIMED("ch_pullback", st,
                  ch_pullback_fast_kernel<T, 0><<<grid, THREADS, PbRings::SMEM, st>>>(u, g, lam, nullptr, nullptr, lam_out,
                                                                                 nullptr, G, P, seg, S));
    count_launch();
    return check_launch("ch_pullback_fast_kernel");
}

}  // namespace

int ch_pullback_fast_blocks(const evx_grid* g) {
    init_occupancy();
    int seg, most = 0;
    for (int grads : {0, 1, 2}) {
        dim3 a = pb_grid<TileWide>(g, grads, &seg), b = pb_grid<TileSquare>(g, grads, &seg);
        most = std::max(most, (int)std::max(a.x * a.y * a.z, b.x * b.y * b.z));
    }
    return most;
}

int ch_pullback_fast_launch(int grads, const float* u, const float* g, const float* lam, const float* h,
                            const float* u1, float* lam_out, double* part, int n_part_cap, const evx_grid* grid_,
                            const Geo& G, const ChP& P, cudaStream_t st, int* n_part_used, const GradSink* sink) {
    init_occupancy();
    if (ch_tile_variant(grid_->nz) == 1)
        return pb_launch_t<TileSquare>(grads, u, g, lam, h, u1, lam_out, part, n_part_cap, grid_, G, P, st, n_part_used,
                                       sink);
    return pb_launch_t<TileWide>(grads, u, g, lam, h, u1, lam_out, part, n_part_cap, grid_, G, P, st, n_part_used,
                                 sink);
}

int batch_pullback_blocks_per_sm(int grads) {
    init_occupancy();
    return g_batch_bps[grads < 0 ? 0 : (grads > 2 ? 2 : grads)];
}

int batch_pullback_launch(int grads, const float* u, const float* g, const float* lam, const float* h,
                          const float* u1, float* lam_out, double* part, const BatchInst* insts,
                          const BatchItem* items, int n_items, int* counter, int grid, cudaStream_t st) {
    init_occupancy();
    int rc = check_cuda(cudaMemsetAsync(counter, 0, sizeof(int), st), "batch pullback counter reset");
    if (rc) return rc;
    if (grads == 1)
        EVX_TIMED("batch_pullback_grads", st,
                  ch_pullback_batch_kernel<1><<<grid, THREADS, BatchRings::SMEM, st>>>(u, g, lam, h, u1, lam_out, part, insts,
                                                                               items, n_items, counter));
    else if (grads == 2)
        EVX_TIMED("batch_pullback_grads_spec", st,
                  ch_pullback_batch_kernel<2><<<grid, THREADS, BatchRings::SMEM, st>>>(u, g, lam, nullptr, nullptr, lam_out,
                                                                               part, insts, items, n_items, counter));
    else
        EVX_TIMED("batch_pullback", st,
                  ch_pullback_batch_kernel<0><<<grid, THREADS, BatchRings::SMEM, st>>>(u, g, lam, nullptr, nullptr, lam_out,
                                                                               nullptr, insts, items, n_items, counter));
    count_launch();
    return check_launch("ch_pullback_batch_kernel");
}

}  // namespace evx
