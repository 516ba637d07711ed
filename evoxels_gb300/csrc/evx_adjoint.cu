// Hand-written adjoint of the periodic Cahn-Hilliard IMEX step.
//
// Forward step: u' = u + P r(u), P = irfft . diag(prefac/N) . rfft (real,
// symmetric: prefac depends on |k|^2 only).  Reverse step:
//   g      = P lam'                          (R2C, adjoint k-space multiply, C2R)
//   lam    = lam' + J_r(u)^T g               (pullback kernel)
// with r = D*div(m(cf) grad mu), mu = w*phi(c) - kappa*L c, c = clip(u,0,1),
// phi(c) = c(1-c)(1-2c), m(x) = x(1-x), cf the face average
// (evoxels/problem_definition.py:328-371).  Writing Fb_f = ih*D*(g_i - g_{i+1})
// for the face f = i+1/2 of each axis:
//   mub_i  = sum_a ih_a*(Fb_{i-1/2} m_{i-1/2} - Fb_{i+1/2} m_{i+1/2})
//   cbar_i = w*phi'(c_i)*mub_i - kappa*(L mub)_i
//            + sum_a 0.5*(cfb_{i+1/2} + cfb_{i-1/2}),  cfb_f = (Fb_f*G_f)*(1 - 2cf_f)
//   lam_i  = lam'_i + [0 <= u_i <= 1] * cbar_i       (torch.clip passes the gradient inside [0,1])
// L is the periodic 7-point Laplacian, which is symmetric.
//
// A Neumann or Dirichlet x axis (the mirrored-x step; y and z stay periodic):
// the reference pads c and mu with the same ghost g = a*cell + b (a = 1 Neumann,
// -1 Dirichlet; evoxels/boundary_conditions.py:33-59) and r lives on interior
// cells only.  Folding the ghosts' cotangents back into the boundary cell gives,
// at a boundary cell: g = 0 on the ghost side, the boundary face's Gb term in
// mub weighted by (1 - a), its cfb term weighted by (1 + a)/2 instead of 1/2,
// mub continued by a*mub into the ghost for L(mub), and mu by its forward ghost.
// The spectral operator of the mirrored step is symmetric too (see
// ch_apply_spectral), so g = P lam' is the forward operator applied to lam'.
//
// Parameter gradients (optional): with a = kappa*D*A (fourier_symbol = -a k^4,
// evoxels/problem_definition.py:303) and K = irfft.diag(prefac*k^4/N).rfft,
//   dL/dD     += <g, div>            - kappa*A*<K lam', u' - u>
//   dL/dkappa += -<mub, L c>          - D*A*<K lam', u' - u>
//   dL/dw     += <mub, phi(c)>
// (d prefac/da = -prefac^2 k^4, and P r = u' - u).  Block partial sums are
// written to the workspace and reduced in a fixed order by one block, so the
// gradients are deterministic.  With the increment spectra stored by the
// forward pass (x-pass plans), <g, div> = <lam', u'-u>/D and <K lam', u'-u>
// are Parseval sums formed in the adjoint x-pass instead, which drops the
// inverse transform of K lam' and the reads of u' and K lam' in the pullback.
#include <algorithm>

#include "evx_ch_fast.cuh"

namespace evx {

namespace {

constexpr int CZ = CH_TZ + 4, CY = CH_TY + 4;
constexpr int MZ = CH_TZ + 2, MY = CH_TY + 2;

__device__ __forceinline__ float phi(float c) {
    return c * (1.f - c) * (1.f - 2.f * c);
}
__device__ __forceinline__ float dphi(float c) {   // d/dc c(1-c)(1-2c) = 1 - 6c + 6c^2
    return 1.f - 6.f * c + 6.f * c * c;
}

template <bool GRADS>
__global__ void __launch_bounds__(CH_THREADS)
ch_pullback_kernel(const float* __restrict__ u, const float* __restrict__ g, const float* __restrict__ lam,
                   const float* __restrict__ h, const float* __restrict__ u1, float* __restrict__ lam_out,
                   double* __restrict__ part, Geo G, ChP P, int LX) {
    __shared__ float cs[5][CY][CZ];
    __shared__ float gs[5][CY][CZ];
    __shared__ float ms[3][MY][MZ];
    __shared__ float mb[3][MY][MZ];
    __shared__ double red[4][CH_THREADS / 32];
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int k0 = blockIdx.x * CH_TZ, j0 = blockIdx.y * CH_TY;
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    const size_t plane = (size_t)G.ny * G.nz;
    const float D = P.D, kap = P.kappa, w = P.w;
    const float ihx = G.ih[0], ihy = G.ih[1], ihz = G.ih[2];
    double sD = 0.0, sK = 0.0, sW = 0.0, sH = 0.0;
    const bool xb = G.kind[0] != EVX_BC_PERIODIC;          // ghosts in x (y and z periodic)
    const float ax = G.kind[0] == EVX_BC_DIRICHLET ? -1.f : 1.f;
    auto xin = [&](int p) { return xb ? min(max(p, 0), G.nx - 1) : p; };   // the plane a ghost derives from

    auto load_plane = [&](int p) {
        const bool ghost = xb && (p < 0 || p >= G.nx);
        const int gp = xb ? xin(p) : pmod(p, G.nx);
        const int sl = (p + 10) % 5;
        for (int e = tid; e < CY * CZ; e += CH_THREADS) {
            const int jj = e / CZ, kk = e - jj * CZ;
            const int gj = pmod(j0 + jj - 2, G.ny), gk = pmod(k0 + kk - 2, G.nz);
            const size_t idx = (size_t)gp * plane + (size_t)gj * G.nz + gk;
            const float c = clip01(__ldg(u + idx));
            cs[sl][jj][kk] = ghost ? (p < 0 ? ghost_lo(G, 0, c) : ghost_hi(G, 0, c)) : c;
            gs[sl][jj][kk] = ghost ? 0.f : __ldg(g + idx);
        }
    };

    // mu and mub on plane p over the tile grown by one cell; a ghost plane holds the forward
    // ghost of mu and a*mub of the boundary plane it derives from
    auto compute_mu = [&](int p) {
        const int q = xin(p);
        const int s0 = (q + 10) % 5, sm = (q + 9) % 5, sp = (q + 11) % 5;
        const int sl = (p + 9) % 3;
        const float fm = (xb && q == 0) ? 1.f - ax : 1.f, fp = (xb && q == G.nx - 1) ? 1.f - ax : 1.f;
        for (int e = tid; e < MY * MZ; e += CH_THREADS) {
            const int a = e / MZ, b = e - a * MZ;
            const int jj = a + 1, kk = b + 1;
            const float c = cs[s0][jj][kk];
            const float cxm = cs[sm][jj][kk], cxp = cs[sp][jj][kk];
            const float cym = cs[s0][jj - 1][kk], cyp = cs[s0][jj + 1][kk];
            const float czm = cs[s0][jj][kk - 1], czp = cs[s0][jj][kk + 1];
            const float lap = lap7(G, c, cxm, cxp, cym, cyp, czm, czp);
            float mu = __fsub_rn(mu_hom(w, c), __fmul_rn(kap, lap));
            const float gc = gs[s0][jj][kk];
            // Gbar on the faces: Fb * m(cf)
            auto gb = [&](float c_lo, float c_hi, float g_lo, float g_hi, float ih) {
                const float cf = 0.5f * (c_lo + c_hi);
                return ih * D * (g_lo - g_hi) * (cf * (1.f - cf));
            };
            float v = ihx * (fm * gb(cxm, c, gs[sm][jj][kk], gc, ihx) - fp * gb(c, cxp, gc, gs[sp][jj][kk], ihx));
            v += ihy * (gb(cym, c, gs[s0][jj - 1][kk], gc, ihy) - gb(c, cyp, gc, gs[s0][jj + 1][kk], ihy));
            v += ihz * (gb(czm, c, gs[s0][jj][kk - 1], gc, ihz) - gb(c, czp, gc, gs[s0][jj][kk + 1], ihz));
            if (p != q) {
                mu = p < 0 ? ghost_lo(G, 0, mu) : ghost_hi(G, 0, mu);
                v *= ax;
            }
            ms[sl][a][b] = mu;
            mb[sl][a][b] = v;
        }
    };

    auto compute_lam = [&](int i) {
        const int s0 = (i + 10) % 5, sm = (i + 9) % 5, sp = (i + 11) % 5;
        const int m0 = (i + 9) % 3, mm = (i + 8) % 3, mp = (i + 10) % 3;
        for (int e = tid; e < CH_TY * CH_TZ; e += CH_THREADS) {
            const int a = e / CH_TZ, b = e - a * CH_TZ;
            const int gj = j0 + a, gk = k0 + b;
            if (gj >= G.ny || gk >= G.nz) continue;
            const int jj = a + 2, kk = b + 2, ja = a + 1, kb = b + 1;
            const float c = cs[s0][jj][kk], mu = ms[m0][ja][kb], mub = mb[m0][ja][kb], gc = gs[s0][jj][kk];
            float acc = 0.f, div = 0.f;
            // one axis: neighbours (lo, hi) of c, mu, g; wlo / whi weight the faces' cbar terms
            auto axis = [&](float c_lo, float c_hi, float m_lo, float m_hi, float g_lo, float g_hi, float ih,
                            float wlo = 1.f, float whi = 1.f) {
                // + face (c, c_hi)
                const float cfp = 0.5f * (c + c_hi);
                const float Gp = (m_hi - mu) * ih;
                const float Fbp = ih * D * (gc - g_hi);
                // - face (c_lo, c)
                const float cfm = 0.5f * (c_lo + c);
                const float Gm = (mu - m_lo) * ih;
                const float Fbm = ih * D * (g_lo - gc);
                acc += 0.5f * (whi * ((Fbp * Gp) * (1.f - 2.f * cfp)) + wlo * ((Fbm * Gm) * (1.f - 2.f * cfm)));
                if (GRADS) div += ((cfp * (1.f - cfp)) * Gp - (cfm * (1.f - cfm)) * Gm) * ih;
            };
            const float cxm = cs[sm][jj][kk], cxp = cs[sp][jj][kk];
            const float cym = cs[s0][jj - 1][kk], cyp = cs[s0][jj + 1][kk];
            const float czm = cs[s0][jj][kk - 1], czp = cs[s0][jj][kk + 1];
            axis(cxm, cxp, ms[mm][ja][kb], ms[mp][ja][kb], gs[sm][jj][kk], gs[sp][jj][kk], ihx,
                 (xb && i == 0) ? 1.f + ax : 1.f, (xb && i == G.nx - 1) ? 1.f + ax : 1.f);
            axis(cym, cyp, ms[m0][ja - 1][kb], ms[m0][ja + 1][kb], gs[s0][jj - 1][kk], gs[s0][jj + 1][kk], ihy);
            axis(czm, czp, ms[m0][ja][kb - 1], ms[m0][ja][kb + 1], gs[s0][jj][kk - 1], gs[s0][jj][kk + 1], ihz);
            const float lmb = lap7(G, mub, mb[mm][ja][kb], mb[mp][ja][kb], mb[m0][ja - 1][kb], mb[m0][ja + 1][kb],
                                   mb[m0][ja][kb - 1], mb[m0][ja][kb + 1]);
            const float cbar = w * dphi(c) * mub - kap * lmb + acc;
            const size_t idx = (size_t)i * plane + (size_t)gj * G.nz + gk;
            const float ur = __ldg(u + idx);
            const bool pass = ur >= 0.f && ur <= 1.f;
            lam_out[idx] = __ldg(lam + idx) + (pass ? cbar : 0.f);
            if (GRADS) {
                const float lapc = lap7(G, c, cxm, cxp, cym, cyp, czm, czp);
                sK -= (double)mub * (double)lapc;
                sW += (double)mub * (double)phi(c);
                if (h) {   // without h the mobility sums come from the spectral x-pass
                    sD += (double)gc * (double)div;
                    sH += (double)__ldg(h + idx) * ((double)__ldg(u1 + idx) - (double)ur);
                }
            }
        }
    };

    if (x0 < x1) {
        for (int p = x0 - 2; p <= x0 + 1; ++p) load_plane(p);
        __syncthreads();
        compute_mu(x0 - 1);
        compute_mu(x0);
        for (int i = x0; i < x1; ++i) {
            load_plane(i + 2);
            __syncthreads();
            compute_mu(i + 1);
            __syncthreads();
            compute_lam(i);
        }
    }
    if (GRADS) {
        double v[4] = {sD, sK, sW, sH};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            double x = v[q];
            for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(0xffffffffu, x, o);
            if ((tid & 31) == 0) red[q][tid >> 5] = x;
        }
        __syncthreads();
        if (tid < 4) {
            double x = 0.0;
            for (int wi = 0; wi < CH_THREADS / 32; ++wi) x += red[tid][wi];
            const size_t blk = ((size_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
            part[blk * 4 + tid] = x;
        }
    }
}

// g_hat = lam_hat * (prefac/N); optionally h_hat = lam_hat * (prefac*k^4/N).
__global__ void ch_kspace_adj_kernel(float2* __restrict__ spec, float2* __restrict__ spec_h, int ny, int nzh,
                                     size_t total, const float* __restrict__ kx2, const float* __restrict__ ky2,
                                     const float* __restrict__ kz2, float sym_coef, float dt, float invN) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        int i, j, k;
        spec_ijk(e, ny, nzh, i, j, k);
        const float k2 = (__ldg(kx2 + i) + __ldg(ky2 + j)) + __ldg(kz2 + k);
        const float k4 = k2 * k2;
        const float pre = dt / (1.f - dt * (sym_coef * k4));
        const float sg = pre * invN;
        float2 v = spec[e];
        spec[e] = make_float2(v.x * sg, v.y * sg);
        if (spec_h) {
            const float sh = sg * k4;
            spec_h[e] = make_float2(v.x * sh, v.y * sh);
        }
    }
}

// Fixed-order reduction of the per-block partial sums into the gradients.
__global__ void ch_grad_reduce_kernel(const double* __restrict__ part, int nblk, double* __restrict__ grads,
                                      double kA, double DA) {
    __shared__ double s[4][256];
    const int t = threadIdx.x;
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = t; b < nblk; b += 256)
        for (int q = 0; q < 4; ++q) a[q] += part[(size_t)b * 4 + q];
    for (int q = 0; q < 4; ++q) s[q][t] = a[q];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o)
            for (int q = 0; q < 4; ++q) s[q][t] += s[q][t + o];
        __syncthreads();
    }
    if (t == 0) {
        grads[0] += s[0][0] - kA * s[3][0];
        grads[1] += s[1][0] - DA * s[3][0];
        grads[2] += s[2][0];
    }
}

// Same, with the two mobility sums from the x-pass partials (xpart: t1 =
// <lam', u'-u>, t2 = <K lam', u'-u> per block) instead of part's slots 0 and 3.
__global__ void ch_grad_reduce_spec_kernel(const double* __restrict__ part, int nblk, const double* __restrict__ xpart,
                                           int nxblk, double* __restrict__ grads, double kA, double DA, double invD) {
    __shared__ double s[4][256];
    const int t = threadIdx.x;
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = t; b < nblk; b += 256) {
        a[0] += part[(size_t)b * 4 + 1];
        a[1] += part[(size_t)b * 4 + 2];
    }
    for (int b = t; b < nxblk; b += 256) {
        a[2] += xpart[(size_t)b * 2];
        a[3] += xpart[(size_t)b * 2 + 1];
    }
    for (int q = 0; q < 4; ++q) s[q][t] = a[q];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o)
            for (int q = 0; q < 4; ++q) s[q][t] += s[q][t + o];
        __syncthreads();
    }
    if (t == 0) {
        grads[0] += s[2][0] * invD - kA * s[3][0];
        grads[1] += s[0][0] - DA * s[3][0];
        grads[2] += s[1][0];
    }
}

int elementwise_grid(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)std::min<size_t>(b, (size_t)152 * 16);
}

}  // namespace

}  // namespace evx

using namespace evx;

extern "C" {

int evx_ch_adjoint(evx_ch_plan* plan, const float* states, int nsteps, const float* lam_in, float* lam_out,
                   const evx_ch_params* prm, double* grads, void* workspace, void* stream) {
    return evx_ch_adjoint_spectra(plan, states, nullptr, nsteps, lam_in, lam_out, prm, grads, workspace, stream);
}

int evx_ch_adjoint_spectra(evx_ch_plan* plan, const float* states, const float* spectra, int nsteps,
                           const float* lam_in, float* lam_out, const evx_ch_params* prm, double* grads,
                           void* workspace, void* stream) {
    if (!plan) return fail(EVX_ERR_BAD_ARG, "plan is NULL");
    int rc = ch_validate_params(prm);
    if (rc) return rc;
    if (!lam_in || !lam_out || (!states && nsteps > 0)) return fail(EVX_ERR_BAD_ARG, "NULL field pointer");
    if (lam_in == lam_out) return fail(EVX_ERR_BAD_ARG, "lam_in and lam_out must not alias");
    // lam buffers are cuFFT R2C inputs, which must be aligned
    if ((reinterpret_cast<uintptr_t>(lam_in) | reinterpret_cast<uintptr_t>(lam_out)) & 15)
        return fail(EVX_ERR_BAD_ARG, "lam_in and lam_out must be 16-byte aligned");
    if (nsteps < 0) return fail(EVX_ERR_BAD_ARG, "nsteps must be >= 0");
    if (plan->xext && spectra)
        return fail(EVX_ERR_UNSUPPORTED, "stored increment spectra need a periodic x-pass plan");
    if (prm->bulk != EVX_BULK_DOUBLE_WELL)
        return fail(EVX_ERR_UNSUPPORTED, "the adjoint is built for the double-well bulk term w*c(1-c)(1-2c)");
    const bool want = grads != nullptr;
    const bool spectral = want && spectra != nullptr;
    if (spectral) {
        if (!plan->spec_floats) return fail(EVX_ERR_UNSUPPORTED, "stored spectra need an x-pass plan (power-of-two nx)");
        if (reinterpret_cast<uintptr_t>(spectra) & 15) return fail(EVX_ERR_BAD_ARG, "spectra must be 16-byte aligned");
    }
    const size_t N = plan->n;
    if (nsteps == 0)
        return check_cuda(cudaMemcpyAsync(lam_out, lam_in, N * sizeof(float), cudaMemcpyDeviceToDevice,
                                          as_stream(stream)), "evx_ch_adjoint copy");
    const GraphKey key{2, key_p(states), key_p(spectra), (uint64_t)nsteps, key_p(lam_in), key_p(lam_out),
                       key_p(grads), key_p(workspace), key_f(prm->D), key_f(prm->kappa), key_f(prm->w),
                       key_f(prm->A), key_f(prm->sym_coef), key_f(prm->dt), (uint64_t)prm->bulk};
    return plan->graphs.run(key, as_stream(stream), [&](cudaStream_t st) -> int {
    int rc;
    if ((rc = ch_plan_bind(plan, workspace, st, want && !spectral && !plan->xext))) return rc;
    const evx_grid* g = &plan->g;
    const Geo G = make_geo(g, nullptr);
    const ChP P = make_chp(prm);
    float* gbuf = reinterpret_cast<float*>(ws_at(workspace, plan->off_r));
    float* hbuf = gbuf + N;
    float2* spec = reinterpret_cast<float2*>(ws_at(workspace, plan->off_spec));
    float2* spec_h = spec + plan->nspec;
    float* lbuf = reinterpret_cast<float*>(ws_at(workspace, plan->off_lam));
    double* part = reinterpret_cast<double*>(ws_at(workspace, plan->off_part));
    double* xpart = reinterpret_cast<double*>(ws_at(workspace, plan->off_xpart));
    const float invN = (float)(1.0 / (double)N);
    dim3 sg; int lx;
    ch_stencil_grid(g, &sg, &lx);
    const double kA = (double)prm->kappa * prm->A, DA = (double)prm->D * prm->A, invD = 1.0 / (double)prm->D;
    const int gmode = spectral ? 2 : (want ? 1 : 0);
    // spectral gradients on the fast path: the pullback's last block reduces (no reduce launch)
    int* counter = reinterpret_cast<int*>(part + plan->n_part * 4);
    if (spectral && (rc = check_cuda(cudaMemsetAsync(counter, 0, sizeof(int), st), "reduction counter"))) return rc;
    const float* lam = lam_in;
    if (plan->xext) {   // mirrored x: pullback with x ghosts (the tile kernel where the fields allow it)
        const Geo Gb = make_geo(g, &plan->bc);
        float* gout = reinterpret_cast<float*>(ws_at(workspace, plan->off_upd));
        const float invNe = (float)(1.0 / ((double)plan->nxe * g->ny * g->nz));
        for (int s = nsteps - 1; s >= 0; --s) {
            float* dst = (s % 2 == 0) ? lam_out : lbuf;
            const float* us = states + (size_t)s * N;
            if (!want) {   // g = P lam' by the (symmetric) forward operator
                if ((rc = ch_apply_spectral(plan, lam, gbuf, gout, spec, P, st))) return rc;
                if (fast_ok(g, {us, gout, lam, dst})) {   // the tile kernel with x ghosts
                    int nbx = 0;
                    if ((rc = ch_pullback_fast_launch(0, us, gout, lam, nullptr, nullptr, dst, part, plan->n_part, g, Gb,
                                                      P, st, &nbx, nullptr)))
                        return rc;
                    lam = dst;
                    continue;
                }
                EVX_TIMED("ch_pullback", st,
                          ch_pullback_kernel<false><<<sg, dim3(32, 8), 0, st>>>(us, gout, lam, nullptr, nullptr, dst,
                                                                                 nullptr, Gb, P, lx));
                count_launch();
                if ((rc = check_launch("ch_pullback_kernel"))) return rc;
                lam = dst;
                continue;
            }
            // g = P lam' and h = K lam' (K: prefac*k^4/N), both symmetric on the extended grid as well
            float* hout = gbuf;   // the extension scratch is consumed by the R2C before h is written
            if (plan->xmode) {
                if ((rc = ch_r2c(plan, lam, spec, st))) return rc;
                XpassArgs a = xpass_args(plan, 2, spec, P);
                a.spec_h = spec_h;
                if ((rc = xpass_launch(a, st))) return rc;
            } else {
                if ((rc = check_cuda(cudaMemcpyAsync(gbuf, lam, N * sizeof(float), cudaMemcpyDeviceToDevice, st),
                                     "mirror extension copy")))
                    return rc;
                if ((rc = ch_mirror_x(plan, gbuf, st))) return rc;
                if ((rc = ch_r2c(plan, gbuf, spec, st))) return rc;
                EVX_TIMED("ch_kspace_adj", st, ch_kspace_adj_kernel<<<elementwise_grid(plan->nspec), 256, 0, st>>>(
                    spec, spec_h, g->ny, plan->nzh, plan->nspec, plan->kx2, plan->ky2, plan->kz2, P.sym_coef, P.dt,
                    invNe));
                count_launch();
                if ((rc = check_launch("ch_kspace_adj_kernel"))) return rc;
            }
            if ((rc = ch_c2r(plan, spec, gout, false, st))) return rc;
            if ((rc = ch_c2r(plan, spec_h, hout, false, st))) return rc;
            int nbx = (int)(sg.x * sg.y * sg.z);   // partial sums of the generic kernel; the fast launcher sets its own
            if (fast_ok(g, {us, gout, lam, hout, us + N, dst})) {   // the tile kernel with x ghosts
                if ((rc = ch_pullback_fast_launch(1, us, gout, lam, hout, us + N, dst, part, plan->n_part, g, Gb, P, st,
                                                  &nbx, nullptr)))
                    return rc;
            } else {
                EVX_TIMED("ch_pullback_grads", st,
                          ch_pullback_kernel<true><<<sg, dim3(32, 8), 0, st>>>(us, gout, lam, hout, us + N, dst, part, Gb,
                                                                                P, lx));
                count_launch();
                if ((rc = check_launch("ch_pullback_kernel"))) return rc;
            }
            EVX_TIMED("ch_grad_reduce", st, ch_grad_reduce_kernel<<<1, 256, 0, st>>>(
                part, nbx, grads, kA, DA));
            count_launch();
            if ((rc = check_launch("ch_grad_reduce_kernel"))) return rc;
            lam = dst;
        }
        return EVX_OK;
    }
    for (int s = nsteps - 1; s >= 0; --s) {
        float* dst = (s % 2 == 0) ? lam_out : lbuf;
        int nxp = 0;   // x-pass partial-sum slots of this step
        if ((rc = ch_r2c(plan, lam, spec, st))) return rc;
        if (plan->xmode) {
            XpassArgs a = xpass_args(plan, spectral ? 3 : (want ? 2 : 1), spec, P);
            if (spectral) {
                a.dspec = const_cast<float2*>(reinterpret_cast<const float2*>(spectra + (size_t)s * plan->spec_floats));
                a.xpart = xpart;
                a.n_xpart_out = &nxp;
            } else if (want) {
                a.spec_h = spec_h;
            }
            if ((rc = xpass_launch(a, st))) return rc;
        } else {
            EVX_TIMED("ch_kspace_adj", st, ch_kspace_adj_kernel<<<elementwise_grid(plan->nspec), 256, 0, st>>>(
                spec, want ? spec_h : nullptr, g->ny, plan->nzh, plan->nspec, plan->kx2, plan->ky2, plan->kz2,
                P.sym_coef, P.dt, invN));
            count_launch();
            if ((rc = check_launch("ch_kspace_adj_kernel"))) return rc;
        }
        if ((rc = ch_c2r(plan, spec, gbuf, want && !spectral, st))) return rc;
        const float* us = states + (size_t)s * N;
        const float* hb = gmode == 1 ? hbuf : nullptr;
        const float* u1 = gmode == 1 ? us + N : nullptr;
        int nb = (int)(sg.x * sg.y * sg.z);   // generic kernel's partial sums; the fast launcher sets its own
        bool reduced = false;
        if (fast_ok(g, {us, gbuf, lam, hb, u1, dst})) {
            const GradSink sink{grads, xpart, nxp, counter, kA, DA, invD};
            if ((rc = ch_pullback_fast_launch(gmode, us, gbuf, lam, hb, u1, dst, part, plan->n_part, g, G, P, st, &nb,
                                              spectral ? &sink : nullptr)))
                return rc;
            reduced = spectral;
        } else if (want) {
            EVX_TIMED("ch_pullback_grads", st,
                      ch_pullback_kernel<true><<<sg, dim3(32, 8), 0, st>>>(us, gbuf, lam, hb, u1, dst, part, G, P, lx));
            count_launch();
            if ((rc = check_launch("ch_pullback_kernel"))) return rc;
        } else {
            EVX_TIMED("ch_pullback", st,
                      ch_pullback_kernel<false><<<sg, dim3(32, 8), 0, st>>>(us, gbuf, lam, nullptr, nullptr, dst, nullptr,
                                                                             G, P, lx));
            count_launch();
            if ((rc = check_launch("ch_pullback_kernel"))) return rc;
        }
        if (spectral) {
            if (!reduced) {
                EVX_TIMED("ch_grad_reduce", st, ch_grad_reduce_spec_kernel<<<1, 256, 0, st>>>(
                    part, nb, xpart, nxp, grads, kA, DA, invD));
                count_launch();
                if ((rc = check_launch("ch_grad_reduce_spec_kernel"))) return rc;
            }
        } else if (want) {
            EVX_TIMED("ch_grad_reduce", st, ch_grad_reduce_kernel<<<1, 256, 0, st>>>(part, nb, grads, kA, DA));
            count_launch();
            if ((rc = check_launch("ch_grad_reduce_kernel"))) return rc;
        }
        lam = dst;
    }
    return EVX_OK;
    });
}

}  // extern "C"
