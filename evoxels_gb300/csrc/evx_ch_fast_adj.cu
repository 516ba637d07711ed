// Periodic fast path of the Cahn-Hilliard adjoint pullback (tiling as in
// evx_ch_fast.cuh; the math is documented in evx_adjoint.cu):
//   lam_s = lam_{s+1} + [0<=u<=1] * ( w*phi'(c)*mub - kappa*L(mub) + sum_faces 0.5*cfb )
//   mub   = sum_a ih_a*(Gb_{-} - Gb_{+}),  Gb_f = ih*D*(g_lo - g_hi) * cf(1-cf)
//   cfb_f = (ih*D*(g_lo - g_hi)) * ((mu_hi - mu_lo)*ih) * (1 - 2cf)
// Per x-plane i a block: stores the prefetched planes i+2 of c = clip(u_s) and
// g = P lam_{s+1} (4-slot rings) and prefetches plane i+3; computes mu and mub
// on plane i+1 over the tile grown by one cell (2-slot rings); then lam on
// plane i.  x faces, the previous plane's c and mub at the patch points are
// carried in registers.  Optional parameter-gradient partial sums are kept in
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

constexpr int RING_C = 4 * MAX_FIELD, RING_M = 2 * MAX_POT;
constexpr size_t ADJ_SMEM = (size_t)(2 * RING_C + 2 * RING_M) * sizeof(float) + 4 * 8 * sizeof(double);

__device__ __forceinline__ float phi_c(float c) { return c * (1.f - c) * (1.f - 2.f * c); }
__device__ __forceinline__ float dphi_c(float c) { return 1.f - 6.f * c + 6.f * c * c; }
__device__ __forceinline__ float lap_f(const Geo& G, float c, float xm, float xp, float ym, float yp, float zm,
                                       float zp) {
    return ((xp + xm) * G.ih2[0] + (yp + ym) * G.ih2[1]) + (zp + zm) * G.ih2[2] - (2.f * c) * G.ih2sum;
}
// Gbar on a face: (ih*D*(g_lo - g_hi)) * m(cf)
__device__ __forceinline__ float gbar(float c_lo, float c_hi, float g_lo, float g_hi, float ihD) {
    const float cf = 0.5f * (c_lo + c_hi);
    return ihD * (g_lo - g_hi) * (cf * (1.f - cf));
}
// cbar-face and (optionally) forward flux on a face
struct FaceB {
    float cfb, F;
};
template <bool GRADS>
__device__ __forceinline__ FaceB face_b(float c_lo, float c_hi, float m_lo, float m_hi, float g_lo, float g_hi,
                                        float ih, float ihD) {
    const float cf = 0.5f * (c_lo + c_hi);
    const float Gr = (m_hi - m_lo) * ih;
    const float Fb = ihD * (g_lo - g_hi);
    FaceB o;
    o.cfb = (Fb * Gr) * (1.f - 2.f * cf);
    o.F = GRADS ? (cf * (1.f - cf)) * Gr : 0.f;
    return o;
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

template <class T, int GR>
__device__ __forceinline__ void pullback_tile(const float* __restrict__ u, const float* __restrict__ gfield,
                                              const float* __restrict__ lam, const float* __restrict__ hfield,
                                              const float* __restrict__ u1, float* __restrict__ lam_out,
                                              const Geo& G, const ChP& P, int k0, int j0, int x0, int x1,
                                              float* cs, float* gs, float* ms, float* bs,
                                              float& sD, float& sK, float& sW, float& sH) {
    constexpr bool GRADS = GR != 0;
    const int tid = threadIdx.x;
    const int tx = tid % T::BX, ty = tid / T::BX;
    const int W = T::W;
    const int nx = G.nx, ny = G.ny, nz = G.nz;
    const size_t plane = (size_t)ny * nz;
    const float ihx = G.ih[0], ihy = G.ih[1], ihz = G.ih[2];
    const float ihDx = ihx * P.D, ihDy = ihy * P.D, ihDz = ihz * P.D;
    const float w = P.w, kap = P.kappa;
    const LoadPlan LP = make_load_plan<T>(tid, j0, k0, ny, nz);
    int mr[2], mc[2];
    bool mv[2];
#pragma unroll
    for (int m = 0; m < 2; ++m) {
        const int pidx = tid + m * THREADS;
        mv[m] = pidx < T::NMU;
        const int py = mv[m] ? pidx / T::MPZ : 0;
        mr[m] = 1 + 2 * py;
        mc[m] = 2 + 2 * (pidx - py * T::MPZ);
    }
    const int ra = 2 + 2 * ty, rc = 4 + 2 * tx;
    const int gj = j0 + 2 * ty, gk = k0 + 2 * tx;
    const bool wk = gk < nz, wj0 = gj < ny && wk, wj1 = gj + 1 < ny && wk;
    const int pa = ra * W + rc, pb = pa + W;   // field offsets of the patch rows

    float4 pc[2], pg[2];
    auto fetch = [&](int p) {
        const size_t base = (size_t)pmod(p, nx) * plane;
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            if (!LP.valid[s]) continue;
            pc[s] = ldg4(u + base + LP.goff[s]);
            pg[s] = ldg4(gfield + base + LP.goff[s]);
        }
    };
    auto stash = [&](int p) {
        float* dc = cs + (p & 3) * T::FIELD;
        float* dg = gs + (p & 3) * T::FIELD;
#pragma unroll
        for (int s = 0; s < 2; ++s)
            if (LP.valid[s]) {
                sts4(dc + LP.soff[s], clip4(pc[s]));
                sts4(dg + LP.soff[s], pg[s]);
            }
    };

    float gxm[2][4];   // Gbar on the x face below the current potential plane, per patch point
    auto gx_faces = [&](int plo, int m, float out[4]) {
        const float* c0 = cs + (plo & 3) * T::FIELD;
        const float* c1 = cs + ((plo + 1) & 3) * T::FIELD;
        const float* g0 = gs + (plo & 3) * T::FIELD;
        const float* g1 = gs + ((plo + 1) & 3) * T::FIELD;
        const int a = mr[m] * W + mc[m], b = a + W;
        const float2 cA0 = lds2(c0 + a), cB0 = lds2(c0 + b), cA1 = lds2(c1 + a), cB1 = lds2(c1 + b);
        const float2 gA0 = lds2(g0 + a), gB0 = lds2(g0 + b), gA1 = lds2(g1 + a), gB1 = lds2(g1 + b);
        out[0] = gbar(cA0.x, cA1.x, gA0.x, gA1.x, ihDx);
        out[1] = gbar(cA0.y, cA1.y, gA0.y, gA1.y, ihDx);
        out[2] = gbar(cB0.x, cB1.x, gB0.x, gB1.x, ihDx);
        out[3] = gbar(cB0.y, cB1.y, gB0.y, gB1.y, ihDx);
    };

    auto compute_mu = [&](int p) {
        const float* cc = cs + (p & 3) * T::FIELD;
        const float* cm = cs + ((p - 1) & 3) * T::FIELD;
        const float* cp = cs + ((p + 1) & 3) * T::FIELD;
        const float* gc = gs + (p & 3) * T::FIELD;
        float* mo = ms + (p & 1) * T::POT;
        float* bo = bs + (p & 1) * T::POT;
#pragma unroll
        for (int m = 0; m < 2; ++m) {
            if (!mv[m]) continue;
            const int a = mr[m] * W + mc[m], b = a + W;
            {   // chemical potential on the 2x2 patch
                const float2 up = lds2(cc + a - W), A = lds2(cc + a), B = lds2(cc + b), dn = lds2(cc + b + W);
                const float Al = cc[a - 1], Ar = cc[a + 2], Bl = cc[b - 1], Br = cc[b + 2];
                const float2 xmA = lds2(cm + a), xmB = lds2(cm + b), xpA = lds2(cp + a), xpB = lds2(cp + b);
                const float m00 = w * phi_c(A.x) - kap * lap_f(G, A.x, xmA.x, xpA.x, up.x, B.x, Al, A.y);
                const float m01 = w * phi_c(A.y) - kap * lap_f(G, A.y, xmA.y, xpA.y, up.y, B.y, A.x, Ar);
                const float m10 = w * phi_c(B.x) - kap * lap_f(G, B.x, xmB.x, xpB.x, A.x, dn.x, Bl, B.y);
                const float m11 = w * phi_c(B.y) - kap * lap_f(G, B.y, xmB.y, xpB.y, A.y, dn.y, B.x, Br);
                sts2(mo + a - W, m00, m01);
                sts2(mo + b - W, m10, m11);
            }
            // mub = sum_faces ih*(Gb_minus - Gb_plus), accumulated face by face
            float bq[4];
            {
                float gxp[4];
                gx_faces(p, m, gxp);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    bq[q] = (gxm[m][q] - gxp[q]) * ihx;
                    gxm[m][q] = gxp[q];
                }
            }
            {   // z faces, row a then row b
                const float2 A = lds2(cc + a), gA = lds2(gc + a);
                float f = gbar(cc[a - 1], A.x, gc[a - 1], gA.x, ihDz) * ihz;
                bq[0] += f;
                f = gbar(A.x, A.y, gA.x, gA.y, ihDz) * ihz;
                bq[0] -= f; bq[1] += f;
                bq[1] -= gbar(A.y, cc[a + 2], gA.y, gc[a + 2], ihDz) * ihz;
                const float2 B = lds2(cc + b), gB = lds2(gc + b);
                f = gbar(cc[b - 1], B.x, gc[b - 1], gB.x, ihDz) * ihz;
                bq[2] += f;
                f = gbar(B.x, B.y, gB.x, gB.y, ihDz) * ihz;
                bq[2] -= f; bq[3] += f;
                bq[3] -= gbar(B.y, cc[b + 2], gB.y, gc[b + 2], ihDz) * ihz;
            }
            {   // y faces, both columns at once
                const float2 up = lds2(cc + a - W), A = lds2(cc + a), B = lds2(cc + b), dn = lds2(cc + b + W);
                const float2 gup = lds2(gc + a - W), gA = lds2(gc + a), gB = lds2(gc + b), gdn = lds2(gc + b + W);
                bq[0] += gbar(up.x, A.x, gup.x, gA.x, ihDy) * ihy;
                bq[1] += gbar(up.y, A.y, gup.y, gA.y, ihDy) * ihy;
                float f = gbar(A.x, B.x, gA.x, gB.x, ihDy) * ihy;
                bq[0] -= f; bq[2] += f;
                f = gbar(A.y, B.y, gA.y, gB.y, ihDy) * ihy;
                bq[1] -= f; bq[3] += f;
                bq[2] -= gbar(B.x, dn.x, gB.x, gdn.x, ihDy) * ihy;
                bq[3] -= gbar(B.y, dn.y, gB.y, gdn.y, ihDy) * ihy;
            }
            sts2(bo + a - W, bq[0], bq[1]);
            sts2(bo + b - W, bq[2], bq[3]);
        }
    };

    // x face quantities of the output patch between planes plo and plo+1
    float cfx_m[4], Fx_m[4], c_prev[4], b_prev[4];
    auto x_faces_b = [&](int plo, float cfb[4], float F[4]) {
        const float* c0 = cs + (plo & 3) * T::FIELD;
        const float* c1 = cs + ((plo + 1) & 3) * T::FIELD;
        const float* g0 = gs + (plo & 3) * T::FIELD;
        const float* g1 = gs + ((plo + 1) & 3) * T::FIELD;
        const float* m0 = ms + (plo & 1) * T::POT;
        const float* m1 = ms + ((plo + 1) & 1) * T::POT;
        const float2 cA0 = lds2(c0 + pa), cB0 = lds2(c0 + pb), cA1 = lds2(c1 + pa), cB1 = lds2(c1 + pb);
        const float2 gA0 = lds2(g0 + pa), gB0 = lds2(g0 + pb), gA1 = lds2(g1 + pa), gB1 = lds2(g1 + pb);
        const float2 mA0 = lds2(m0 + pa - W), mB0 = lds2(m0 + pb - W), mA1 = lds2(m1 + pa - W),
                     mB1 = lds2(m1 + pb - W);
        FaceB f;
        f = face_b<GRADS>(cA0.x, cA1.x, mA0.x, mA1.x, gA0.x, gA1.x, ihx, ihDx); cfb[0] = f.cfb; F[0] = f.F;
        f = face_b<GRADS>(cA0.y, cA1.y, mA0.y, mA1.y, gA0.y, gA1.y, ihx, ihDx); cfb[1] = f.cfb; F[1] = f.F;
        f = face_b<GRADS>(cB0.x, cB1.x, mB0.x, mB1.x, gB0.x, gB1.x, ihx, ihDx); cfb[2] = f.cfb; F[2] = f.F;
        f = face_b<GRADS>(cB0.y, cB1.y, mB0.y, mB1.y, gB0.y, gB1.y, ihx, ihDx); cfb[3] = f.cfb; F[3] = f.F;
    };

    auto compute_lam = [&](int i) {
        const float* cc = cs + (i & 3) * T::FIELD;
        const float* gc = gs + (i & 3) * T::FIELD;
        const float* mm = ms + (i & 1) * T::POT;
        const float* bb = bs + (i & 1) * T::POT;
        const float* bp = bs + ((i + 1) & 1) * T::POT;
        // acc: sum of cbar-face values around each point (times 0.5 at the end)
        float acc[4];
        {
            float cfx_p[4], Fx_p[4];
            x_faces_b(i, cfx_p, Fx_p);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                acc[q] = cfx_m[q] + cfx_p[q];
                cfx_m[q] = cfx_p[q];
            }
        }
        auto face = [&](int lo, int hi, float c_lo, float c_hi, float m_lo, float m_hi, float g_lo, float g_hi,
                        float ih, float ihD) {
            const FaceB f = face_b<false>(c_lo, c_hi, m_lo, m_hi, g_lo, g_hi, ih, ihD);
            if (lo >= 0) acc[lo] += f.cfb;
            if (hi >= 0) acc[hi] += f.cfb;
        };
        {   // z faces
            const float2 A = lds2(cc + pa), MA = lds2(mm + pa - W), gA = lds2(gc + pa);
            face(-1, 0, cc[pa - 1], A.x, mm[pa - W - 1], MA.x, gc[pa - 1], gA.x, ihz, ihDz);
            face(0, 1, A.x, A.y, MA.x, MA.y, gA.x, gA.y, ihz, ihDz);
            face(1, -1, A.y, cc[pa + 2], MA.y, mm[pa - W + 2], gA.y, gc[pa + 2], ihz, ihDz);
            const float2 B = lds2(cc + pb), MB = lds2(mm + pb - W), gB = lds2(gc + pb);
            face(-1, 2, cc[pb - 1], B.x, mm[pb - W - 1], MB.x, gc[pb - 1], gB.x, ihz, ihDz);
            face(2, 3, B.x, B.y, MB.x, MB.y, gB.x, gB.y, ihz, ihDz);
            face(3, -1, B.y, cc[pb + 2], MB.y, mm[pb - W + 2], gB.y, gc[pb + 2], ihz, ihDz);
        }
        {   // y faces
            const float2 up = lds2(cc + pa - W), A = lds2(cc + pa), B = lds2(cc + pb), dn = lds2(cc + pb + W);
            const float2 mup = lds2(mm + pa - 2 * W), MA = lds2(mm + pa - W), MB = lds2(mm + pb - W),
                         mdn = lds2(mm + pb);
            const float2 gup = lds2(gc + pa - W), gA = lds2(gc + pa), gB = lds2(gc + pb), gdn = lds2(gc + pb + W);
            face(-1, 0, up.x, A.x, mup.x, MA.x, gup.x, gA.x, ihy, ihDy);
            face(-1, 1, up.y, A.y, mup.y, MA.y, gup.y, gA.y, ihy, ihDy);
            face(0, 2, A.x, B.x, MA.x, MB.x, gA.x, gB.x, ihy, ihDy);
            face(1, 3, A.y, B.y, MA.y, MB.y, gA.y, gB.y, ihy, ihDy);
            face(2, -1, B.x, dn.x, MB.x, mdn.x, gB.x, gdn.x, ihy, ihDy);
            face(3, -1, B.y, dn.y, MB.y, mdn.y, gB.y, gdn.y, ihy, ihDy);
        }
        // Laplacian of mub
        float Lb[4], bpt[4];
        {
            const float2 bup = lds2(bb + pa - 2 * W), bA = lds2(bb + pa - W), bB = lds2(bb + pb - W),
                         bdn = lds2(bb + pb);
            const float2 bxA = lds2(bp + pa - W), bxB = lds2(bp + pb - W);
            Lb[0] = lap_f(G, bA.x, b_prev[0], bxA.x, bup.x, bB.x, bb[pa - W - 1], bA.y);
            Lb[1] = lap_f(G, bA.y, b_prev[1], bxA.y, bup.y, bB.y, bA.x, bb[pa - W + 2]);
            Lb[2] = lap_f(G, bB.x, b_prev[2], bxB.x, bA.x, bdn.x, bb[pb - W - 1], bB.y);
            Lb[3] = lap_f(G, bB.y, b_prev[3], bxB.y, bA.y, bdn.y, bB.x, bb[pb - W + 2]);
            bpt[0] = bA.x; bpt[1] = bA.y; bpt[2] = bB.x; bpt[3] = bB.y;
        }
        const float2 A = lds2(cc + pa), B = lds2(cc + pb);
        const float cpt[4] = {A.x, A.y, B.x, B.y};
        const size_t o = (size_t)i * plane + (size_t)gj * nz + gk;
        float ur[4], lv[4];
        {
            const float2 u0 = wj0 ? __ldg(reinterpret_cast<const float2*>(u + o)) : make_float2(0.f, 0.f);
            const float2 u1r = wj1 ? __ldg(reinterpret_cast<const float2*>(u + o + nz)) : make_float2(0.f, 0.f);
            const float2 l0 = wj0 ? __ldg(reinterpret_cast<const float2*>(lam + o)) : make_float2(0.f, 0.f);
            const float2 l1 = wj1 ? __ldg(reinterpret_cast<const float2*>(lam + o + nz)) : make_float2(0.f, 0.f);
            ur[0] = u0.x; ur[1] = u0.y; ur[2] = u1r.x; ur[3] = u1r.y;
            lv[0] = l0.x; lv[1] = l0.y; lv[2] = l1.x; lv[3] = l1.y;
            float out[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const float cbar = w * dphi_c(cpt[q]) * bpt[q] - kap * Lb[q] + 0.5f * acc[q];
                out[q] = lv[q] + ((ur[q] >= 0.f && ur[q] <= 1.f) ? cbar : 0.f);
            }
            if (wj0) *reinterpret_cast<float2*>(lam_out + o) = make_float2(out[0], out[1]);
            if (wj1) *reinterpret_cast<float2*>(lam_out + o + nz) = make_float2(out[2], out[3]);
        }
        if (GRADS) {
            const float* cx = cs + ((i + 1) & 3) * T::FIELD;
            const float2 up = lds2(cc + pa - W), dn = lds2(cc + pb + W);
            const float2 cxA = lds2(cx + pa), cxB = lds2(cx + pb);
            const float lc[4] = {
                lap_f(G, A.x, c_prev[0], cxA.x, up.x, B.x, cc[pa - 1], A.y),
                lap_f(G, A.y, c_prev[1], cxA.y, up.y, B.y, A.x, cc[pa + 2]),
                lap_f(G, B.x, c_prev[2], cxB.x, A.x, dn.x, cc[pb - 1], B.y),
                lap_f(G, B.y, c_prev[3], cxB.y, A.y, dn.y, B.x, cc[pb + 2])};
            const bool okp[4] = {wj0, wj0, wj1, wj1};
            if (GR == 1) {
                const float2 h0 = wj0 ? __ldg(reinterpret_cast<const float2*>(hfield + o)) : make_float2(0.f, 0.f);
                const float2 h1 = wj1 ? __ldg(reinterpret_cast<const float2*>(hfield + o + nz)) : make_float2(0.f, 0.f);
                const float2 n0 = wj0 ? __ldg(reinterpret_cast<const float2*>(u1 + o)) : make_float2(0.f, 0.f);
                const float2 n1 = wj1 ? __ldg(reinterpret_cast<const float2*>(u1 + o + nz)) : make_float2(0.f, 0.f);
                const float hv[4] = {h0.x, h0.y, h1.x, h1.y}, nv[4] = {n0.x, n0.y, n1.x, n1.y};
                const float invD = 1.f / P.D;
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    if (!okp[q]) continue;
                    // <g, r/D> = <P lam', r>/D = <lam', u' - u>/D  (P is symmetric)
                    sD += lv[q] * (nv[q] - ur[q]) * invD;
                    sH += hv[q] * (nv[q] - ur[q]);
                }
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (!okp[q]) continue;
                sK -= bpt[q] * lc[q];
                sW += bpt[q] * phi_c(cpt[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            c_prev[q] = cpt[q];
            b_prev[q] = bpt[q];
        }
    };

    // prologue: planes x0-2 .. x0+1 staged; potentials x0-1, x0; carried x quantities
    for (int p = x0 - 2; p <= x0 + 1; ++p) {
        fetch(p);
        stash(p);
    }
    fetch(x0 + 2);
    __syncthreads();
#pragma unroll
    for (int m = 0; m < 2; ++m)
        if (mv[m]) gx_faces(x0 - 2, m, gxm[m]);
    compute_mu(x0 - 1);
    compute_mu(x0);
    __syncthreads();
    x_faces_b(x0 - 1, cfx_m, Fx_m);
    {
        const float* cprev = cs + ((x0 - 1) & 3) * T::FIELD;
        const float* bprev = bs + ((x0 - 1) & 1) * T::POT;
        const float2 a = lds2(cprev + pa), b = lds2(cprev + pb);
        const float2 ba = lds2(bprev + pa - W), bbv = lds2(bprev + pb - W);
        c_prev[0] = a.x; c_prev[1] = a.y; c_prev[2] = b.x; c_prev[3] = b.y;
        b_prev[0] = ba.x; b_prev[1] = ba.y; b_prev[2] = bbv.x; b_prev[3] = bbv.y;
    }
    for (int i = x0; i < x1; ++i) {
        stash(i + 2);
        if (i + 3 <= x1 + 1) fetch(i + 3);
        __syncthreads();
        compute_mu(i + 1);
        __syncthreads();
        compute_lam(i);
    }

}

template <class T, int GR>
__global__ void __launch_bounds__(THREADS, GR ? 2 : 3)
ch_pullback_fast_kernel(const float* __restrict__ u, const float* __restrict__ gfield, const float* __restrict__ lam,
                        const float* __restrict__ hfield, const float* __restrict__ u1, float* __restrict__ lam_out,
                        double* __restrict__ part, Geo G, ChP P, int LX) {
    extern __shared__ __align__(16) float smem[];
    float* cs = smem;
    float* gs = cs + RING_C;
    float* ms = gs + RING_C;
    float* bs = ms + RING_M;
    double* red = reinterpret_cast<double*>(bs + RING_M);   // [4][8]
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    float sD = 0.f, sK = 0.f, sW = 0.f, sH = 0.f;
    if (x0 < x1)
        pullback_tile<T, GR>(u, gfield, lam, hfield, u1, lam_out, G, P, blockIdx.x * T::TZ, blockIdx.y * T::TY, x0,
                             x1, cs, gs, ms, bs, sD, sK, sW, sH);
    if (GR) {
        const size_t blk = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
        block_reduce4(sD, sK, sW, sH, red, part + blk * 4);
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
template <bool GRADS>
__global__ void __launch_bounds__(THREADS, 2)
ch_pullback_batch_kernel(const float* __restrict__ u, const float* __restrict__ gfield, const float* __restrict__ lam,
                         const float* __restrict__ hfield, const float* __restrict__ u1, float* __restrict__ lam_out,
                         double* __restrict__ part, const BatchInst* __restrict__ insts,
                         const BatchItem* __restrict__ items, int n_items, int* __restrict__ counter) {
    extern __shared__ __align__(16) float smem[];
    float* cs = smem;
    float* gs = cs + RING_C;
    float* ms = gs + RING_C;
    float* bs = ms + RING_M;
    double* red = reinterpret_cast<double*>(bs + RING_M);
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
            pullback_tile<TileWide, GRADS ? 1 : 0>(u + o, gfield + o, lam + o, GRADS ? hfield + o : nullptr,
                                           GRADS ? u1 + o : nullptr, lam_out + o, G, B.P, I.k0, I.j0, I.x0, I.x1, cs,
                                           gs, ms, bs, sD, sK, sW, sH);
        else
            pullback_tile<TileSquare, GRADS ? 1 : 0>(u + o, gfield + o, lam + o, GRADS ? hfield + o : nullptr,
                                             GRADS ? u1 + o : nullptr, lam_out + o, G, B.P, I.k0, I.j0, I.x0, I.x1,
                                             cs, gs, ms, bs, sD, sK, sW, sH);
        if (GRADS) block_reduce4(sD, sK, sW, sH, red, part + (size_t)I.part * 4);
        __syncthreads();   // shared memory and s_item are reused by the next item
    }
}

int g_bps[2][3] = {{0, 0, 0}, {0, 0, 0}};   // [tile variant][gradient mode]
int g_batch_bps[2] = {0, 0};
int g_sms = 0;

void init_occupancy() {
    if (g_sms) return;
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&g_sms, cudaDevAttrMultiProcessorCount, dev);
    auto setup = [](auto kern, int* out) {
        cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ADJ_SMEM);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(out, kern, THREADS, ADJ_SMEM);
        if (*out < 1) *out = 1;
    };
    setup(ch_pullback_fast_kernel<TileWide, 0>, &g_bps[0][0]);
    setup(ch_pullback_fast_kernel<TileWide, 1>, &g_bps[0][1]);
    setup(ch_pullback_fast_kernel<TileWide, 2>, &g_bps[0][2]);
    setup(ch_pullback_fast_kernel<TileSquare, 0>, &g_bps[1][0]);
    setup(ch_pullback_fast_kernel<TileSquare, 1>, &g_bps[1][1]);
    setup(ch_pullback_fast_kernel<TileSquare, 2>, &g_bps[1][2]);
    setup(ch_pullback_batch_kernel<false>, &g_batch_bps[0]);
    setup(ch_pullback_batch_kernel<true>, &g_batch_bps[1]);
}

template <class T>
dim3 pb_grid(const evx_grid* g, int grads, int* lx) {
    const int v = std::is_same<T, TileWide>::value ? 0 : 1;
    return fast_grid<T>(g->nx, g->ny, g->nz, g_bps[v][grads], g_sms, lx);
}

template <class T>
int pb_launch_t(int grads, const float* u, const float* g, const float* lam, const float* h, const float* u1,
                float* lam_out, double* part, int n_part_cap, const evx_grid* grid_, const Geo& G, const ChP& P,
                cudaStream_t st, int* n_part_used) {
    int lx;
    const dim3 grid = pb_grid<T>(grid_, grads, &lx);
    const int nb = (int)(grid.x * grid.y * grid.z);
    if (grads && nb > n_part_cap) return fail(EVX_ERR_WORKSPACE, "partial-sum buffer too small (%d > %d)", nb, n_part_cap);
    if (n_part_used) *n_part_used = nb;
    if (grads == 1)
        EVX_TIMED("ch_pullback_grads", st,
                  ch_pullback_fast_kernel<T, 1><<<grid, THREADS, ADJ_SMEM, st>>>(u, g, lam, h, u1, lam_out, part, G, P, lx));
    else if (grads == 2)
        EVX_TIMED("ch_pullback_grads_spec", st,
                  ch_pullback_fast_kernel<T, 2><<<grid, THREADS, ADJ_SMEM, st>>>(u, g, lam, nullptr, nullptr, lam_out, part,
                                                                                 G, P, lx));
    else
        EVX_TIMED("ch_pullback", st,
                  ch_pullback_fast_kernel<T, 0><<<grid, THREADS, ADJ_SMEM, st>>>(u, g, lam, nullptr, nullptr, lam_out,
                                                                                 nullptr, G, P, lx));
    count_launch();
    return check_launch("ch_pullback_fast_kernel");
}

}  // namespace

int ch_pullback_fast_blocks(const evx_grid* g) {
    init_occupancy();
    int lx, most = 0;
    for (int grads : {0, 1, 2}) {
        dim3 a = pb_grid<TileWide>(g, grads, &lx), b = pb_grid<TileSquare>(g, grads, &lx);
        most = std::max(most, (int)std::max(a.x * a.y * a.z, b.x * b.y * b.z));
    }
    return most;
}

int ch_pullback_fast_launch(int grads, const float* u, const float* g, const float* lam, const float* h,
                            const float* u1, float* lam_out, double* part, int n_part_cap, const evx_grid* grid_,
                            const Geo& G, const ChP& P, cudaStream_t st, int* n_part_used) {
    init_occupancy();
    if (ch_tile_variant(grid_->nz) == 1)
        return pb_launch_t<TileSquare>(grads, u, g, lam, h, u1, lam_out, part, n_part_cap, grid_, G, P, st, n_part_used);
    return pb_launch_t<TileWide>(grads, u, g, lam, h, u1, lam_out, part, n_part_cap, grid_, G, P, st, n_part_used);
}

int batch_pullback_blocks_per_sm(bool grads) {
    init_occupancy();
    return g_batch_bps[grads ? 1 : 0];
}

int batch_pullback_launch(bool grads, const float* u, const float* g, const float* lam, const float* h,
                          const float* u1, float* lam_out, double* part, const BatchInst* insts,
                          const BatchItem* items, int n_items, int* counter, int grid, cudaStream_t st) {
    init_occupancy();
    int rc = check_cuda(cudaMemsetAsync(counter, 0, sizeof(int), st), "batch pullback counter reset");
    if (rc) return rc;
    if (grads)
        EVX_TIMED("batch_pullback_grads", st,
                  ch_pullback_batch_kernel<true><<<grid, THREADS, ADJ_SMEM, st>>>(u, g, lam, h, u1, lam_out, part, insts,
                                                                                  items, n_items, counter));
    else
        EVX_TIMED("batch_pullback", st,
                  ch_pullback_batch_kernel<false><<<grid, THREADS, ADJ_SMEM, st>>>(u, g, lam, nullptr, nullptr, lam_out,
                                                                                   nullptr, insts, items, n_items, counter));
    count_launch();
    return check_launch("ch_pullback_batch_kernel");
}

}  // namespace evx
