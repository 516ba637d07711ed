// Cahn-Hilliard forward path: fused right-hand-side stencil kernel, k-space
// multiply between cuFFT R2C/C2R, and the plan / step / multi-step drivers.
//
// rhs (evoxels/problem_definition.py:328-371), one rounding per torch op:
//   c   = clip(u, 0, 1)
//   mu  = w*c*(1-c)*(1-2c) - kappa*lap(pad_bc(c))          kappa = 2*eps, w = 18/eps
//   F_a = (cf*(1-cf)) * ((mu_+ - mu)*ih_a),  cf = 0.5*(c_+ + c)   on every face
//   r   = D * ((divx + divy) + divz),  div_a = (F_a(+) - F_a(-))*ih_a
// IMEX step (evoxels/timesteppers.py:85-89):
//   u' = u + irfftn(prefac * rfftn(r)),  prefac = dt * (1/(1 - dt*sym_coef*(k^2)^2))
//
// The rhs kernel streams along x.  A block owns a CH_TY x CH_TZ tile of (y, z)
// and keeps a 5-plane ring of clipped c (halo 2) and a 3-plane ring of mu
// (halo 1) in shared memory: per x-plane it loads one c plane, computes one mu
// plane and emits one r plane (two barriers per plane).  In fused mode the
// previous step's update is added while loading (u_n = u_{n-1} + upd), u_n is
// written out and the rhs of u_n is produced in the same pass.
#include <algorithm>
#include <cmath>
#include <vector>

#include "evx_ch_fast.cuh"

namespace evx {

namespace {

constexpr int CZ = CH_TZ + 4, CY = CH_TY + 4;   // c tile (halo 2)
constexpr int MZ = CH_TZ + 2, MY = CH_TY + 2;   // mu tile (halo 1)

template <bool FUSED>
__global__ void __launch_bounds__(CH_THREADS)
ch_rhs_kernel(const float* __restrict__ u, const float* __restrict__ upd, float* __restrict__ u_new,
              float* __restrict__ r, Geo G, ChP P, int LX) {
    __shared__ float cs[5][CY][CZ];
    __shared__ float ms[3][MY][MZ];
    const int tid = threadIdx.y * 32 + threadIdx.x;
    const int k0 = blockIdx.x * CH_TZ, j0 = blockIdx.y * CH_TY;
    const int x0 = blockIdx.z * LX;
    const int x1 = min(x0 + LX, G.nx);
    const size_t plane = (size_t)G.ny * G.nz;
    const bool px = G.kind[0] == EVX_BC_PERIODIC;
    const bool py = G.kind[1] == EVX_BC_PERIODIC, pz = G.kind[2] == EVX_BC_PERIODIC;

    auto load_plane = [&](int p) {
        if (!px && (p < 0 || p >= G.nx)) return;   // ghost plane: substituted by consumers
        const int gp = pmod(p, G.nx);
        const int sl = (p + 10) % 5;
        const bool own = FUSED && p >= x0 && p < x1;
        for (int e = tid; e < CY * CZ; e += CH_THREADS) {
            const int jj = e / CZ, kk = e - jj * CZ;
            int gj = j0 + jj - 2, gk = k0 + kk - 2;
            const bool inj = gj >= 0 && gj < G.ny, ink = gk >= 0 && gk < G.nz;
            bool ok = true;
            if (py) gj = pmod(gj, G.ny); else ok = ok && inj;
            if (pz) gk = pmod(gk, G.nz); else ok = ok && ink;
            float v = 0.f;
            if (ok) {
                const size_t idx = (size_t)gp * plane + (size_t)gj * G.nz + gk;
                v = __ldg(u + idx);
                if (FUSED) {
                    v = __fadd_rn(v, __ldg(upd + idx));
                    if (own && jj >= 2 && jj < 2 + CH_TY && kk >= 2 && kk < 2 + CH_TZ && inj && ink)
                        u_new[idx] = v;
                }
                v = clip01(v);
            }
            cs[sl][jj][kk] = v;
        }
    };

    auto compute_mu = [&](int p) {
        if (!px && (p < 0 || p >= G.nx)) return;
        const int gp = pmod(p, G.nx);
        const int s0 = (p + 10) % 5, sm = (p + 9) % 5, sp = (p + 11) % 5;
        const bool xlo = !px && gp == 0, xhi = !px && gp == G.nx - 1;
        const int ms_sl = (p + 9) % 3;
        for (int e = tid; e < MY * MZ; e += CH_THREADS) {
            const int a = e / MZ, b = e - a * MZ;
            const int gj = j0 + a - 1, gk = k0 + b - 1;
            if ((!py && (gj < 0 || gj >= G.ny)) || (!pz && (gk < 0 || gk >= G.nz))) {
                ms[ms_sl][a][b] = 0.f;
                continue;
            }
            const int jj = a + 1, kk = b + 1;
            const float c = cs[s0][jj][kk];
            const float xm = xlo ? ghost_lo(G, 0, c) : cs[sm][jj][kk];
            const float xp = xhi ? ghost_hi(G, 0, c) : cs[sp][jj][kk];
            const float ym = (!py && gj == 0) ? ghost_lo(G, 1, c) : cs[s0][jj - 1][kk];
            const float yp = (!py && gj == G.ny - 1) ? ghost_hi(G, 1, c) : cs[s0][jj + 1][kk];
            const float zm = (!pz && gk == 0) ? ghost_lo(G, 2, c) : cs[s0][jj][kk - 1];
            const float zp = (!pz && gk == G.nz - 1) ? ghost_hi(G, 2, c) : cs[s0][jj][kk + 1];
            const float lap = lap7(G, c, xm, xp, ym, yp, zm, zp);
            ms[ms_sl][a][b] = __fsub_rn(mu_bulk(P.bulk, P.w, c), __fmul_rn(P.kappa, lap));
        }
    };

    auto compute_r = [&](int i) {
        const int s0 = (i + 10) % 5, sm = (i + 9) % 5, sp = (i + 11) % 5;
        const int m0 = (i + 9) % 3, mm = (i + 8) % 3, mp = (i + 10) % 3;
        const bool xlo = !px && i == 0, xhi = !px && i == G.nx - 1;
        for (int e = tid; e < CH_TY * CH_TZ; e += CH_THREADS) {
            const int a = e / CH_TZ, b = e - a * CH_TZ;
            const int gj = j0 + a, gk = k0 + b;
            if (gj >= G.ny || gk >= G.nz) continue;
            const int jj = a + 2, kk = b + 2, ja = a + 1, kb = b + 1;
            const float c = cs[s0][jj][kk];
            const float mu = ms[m0][ja][kb];
            // x faces
            const float cxm = xlo ? ghost_lo(G, 0, c) : cs[sm][jj][kk];
            const float cxp = xhi ? ghost_hi(G, 0, c) : cs[sp][jj][kk];
            const float mxm = xlo ? ghost_lo(G, 0, mu) : ms[mm][ja][kb];
            const float mxp = xhi ? ghost_hi(G, 0, mu) : ms[mp][ja][kb];
            const float dx = __fmul_rn(__fsub_rn(face_flux(c, cxp, mu, mxp, G.ih[0]),
                                                 face_flux(cxm, c, mxm, mu, G.ih[0])), G.ih[0]);
            // y faces
            const bool ylo = !py && gj == 0, yhi = !py && gj == G.ny - 1;
            const float cym = ylo ? ghost_lo(G, 1, c) : cs[s0][jj - 1][kk];
            const float cyp = yhi ? ghost_hi(G, 1, c) : cs[s0][jj + 1][kk];
            const float mym = ylo ? ghost_lo(G, 1, mu) : ms[m0][ja - 1][kb];
            const float myp = yhi ? ghost_hi(G, 1, mu) : ms[m0][ja + 1][kb];
            const float dy = __fmul_rn(__fsub_rn(face_flux(c, cyp, mu, myp, G.ih[1]),
                                                 face_flux(cym, c, mym, mu, G.ih[1])), G.ih[1]);
            // z faces
            const bool zlo = !pz && gk == 0, zhi = !pz && gk == G.nz - 1;
            const float czm = zlo ? ghost_lo(G, 2, c) : cs[s0][jj][kk - 1];
            const float czp = zhi ? ghost_hi(G, 2, c) : cs[s0][jj][kk + 1];
            const float mzm = zlo ? ghost_lo(G, 2, mu) : ms[m0][ja][kb - 1];
            const float mzp = zhi ? ghost_hi(G, 2, mu) : ms[m0][ja][kb + 1];
            const float dz = __fmul_rn(__fsub_rn(face_flux(c, czp, mu, mzp, G.ih[2]),
                                                 face_flux(czm, c, mzm, mu, G.ih[2])), G.ih[2]);
            const float div = __fadd_rn(__fadd_rn(dx, dy), dz);
            r[(size_t)i * plane + (size_t)gj * G.nz + gk] = __fmul_rn(P.D, div);
        }
    };

    if (x0 >= x1) return;
    for (int p = x0 - 2; p <= x0 + 1; ++p) load_plane(p);
    __syncthreads();
    compute_mu(x0 - 1);
    compute_mu(x0);
    for (int i = x0; i < x1; ++i) {
        load_plane(i + 2);
        __syncthreads();
        compute_mu(i + 1);
        __syncthreads();
        compute_r(i);
    }
}

// u_out = u + upd (the IMEX update, evoxels/timesteppers.py:89); optional second
// destination and non-finite flag.
__global__ void ch_axpy_kernel(const float* __restrict__ u, const float* __restrict__ upd,
                               float* __restrict__ out, float* __restrict__ out2, size_t n, int* nonfinite) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    bool bad = false;
    const size_t n4 = n / 4;
    const bool vec = ((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(upd) |
                       reinterpret_cast<uintptr_t>(out) | reinterpret_cast<uintptr_t>(out2)) & 15) == 0;
    size_t tail0 = 0;
    if (vec) {
        const float4* u4 = reinterpret_cast<const float4*>(u);
        const float4* d4 = reinterpret_cast<const float4*>(upd);
        float4* o4 = reinterpret_cast<float4*>(out);
        float4* p4 = reinterpret_cast<float4*>(out2);
        for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n4; e += stride) {
            float4 a = __ldg(u4 + e), b = __ldg(d4 + e), v;
            v.x = __fadd_rn(a.x, b.x); v.y = __fadd_rn(a.y, b.y);
            v.z = __fadd_rn(a.z, b.z); v.w = __fadd_rn(a.w, b.w);
            o4[e] = v;
            if (out2) p4[e] = v;
            bad |= !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z) || !isfinite(v.w);
        }
        tail0 = n4 * 4;
    }
    for (size_t e = tail0 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
        float v = __fadd_rn(__ldg(u + e), __ldg(upd + e));
        out[e] = v;
        if (out2) out2[e] = v;
        bad |= !isfinite(v);
    }
    if (nonfinite && __any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(nonfinite, 1);
}

// Mirror extension along x of the rhs (evoxels/boundary_conditions.py:64-70):
// r[nx + j] = sign * r[nx - 1 - j] for j in [0, nx), sign +1 (Neumann) or -1
// (Dirichlet); r holds 2*nx planes of `plane` floats.
__global__ void ch_mirror_x_kernel(float* __restrict__ r, int nx, size_t plane, float sign) {
    const size_t half = (size_t)nx * plane, stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < half; e += stride) {
        const size_t j = e / plane, yz = e - j * plane;
        r[half + e] = sign * r[((size_t)nx - 1 - j) * plane + yz];
    }
}

// dst = [src, sign * src mirrored along x]: the x extension of a field of nx
// planes into 2*nx planes (evoxels/boundary_conditions.py:64-70).
__global__ void mirror_copy_x_kernel(const float* __restrict__ src, float* __restrict__ dst, int nx, size_t plane,
                                     float sign) {
    const size_t half = (size_t)nx * plane, stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < half; e += stride) {
        const size_t j = e / plane, yz = e - j * plane;
        dst[e] = __ldg(src + e);
        dst[half + e] = sign * __ldg(src + ((size_t)nx - 1 - j) * plane + yz);
    }
}

// spec[i] = (spec[i] * mult[i]) * invN: a real multiplier table on the spectrum
// (evoxels/timesteppers.py:197) and the 1/N of torch's "backward" irfftn.
__global__ void spec_mult_kernel(float2* __restrict__ spec, const float* __restrict__ mult, float invN, size_t n) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
        const float2 a = spec[e];
        const float m = __ldg(mult + e);
        spec[e] = make_float2(__fmul_rn(__fmul_rn(a.x, m), invN), __fmul_rn(__fmul_rn(a.y, m), invN));
    }
}

// spec[i,j,k] = (spec * prefac) * invN, prefac = dt * (1/(1 - dt*(sym_coef*k4)))
// (evoxels/timesteppers.py:77,87 and torch's 1/N "backward" irfftn scaling).
__global__ void ch_kspace_fwd_kernel(float2* __restrict__ spec, int ny, int nzh, size_t total,
                                     const float* __restrict__ kx2, const float* __restrict__ ky2,
                                     const float* __restrict__ kz2, float sym_coef, float dt, float invN) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        int i, j, k;
        spec_ijk(e, ny, nzh, i, j, k);
        const float k2 = __fadd_rn(__fadd_rn(__ldg(kx2 + i), __ldg(ky2 + j)), __ldg(kz2 + k));
        const float k4 = __fmul_rn(k2, k2);
        const float den = __fsub_rn(1.f, __fmul_rn(dt, __fmul_rn(sym_coef, k4)));
        const float pre = __fmul_rn(__frcp_rn(den), dt);
        float2 v = spec[e];
        v.x = __fmul_rn(__fmul_rn(v.x, pre), invN);
        v.y = __fmul_rn(__fmul_rn(v.y, pre), invN);
        spec[e] = v;
    }
}

int elementwise_grid(size_t n) {
    size_t b = (n + 255) / 256;
    return (int)std::min<size_t>(b, (size_t)152 * 16);
}

}  // namespace

int ch_stencil_grid(const evx_grid* g, dim3* grid, int* LX) {
    const int tz = (g->nz + CH_TZ - 1) / CH_TZ, ty = (g->ny + CH_TY - 1) / CH_TY;
    const long tiles = (long)tz * ty;
    const long want = 6L * 152;   // ~6 resident blocks per SM on 152 SMs
    int lx = (int)std::max<long>(4, std::min<long>(64, (long)g->nx * tiles / want));
    lx = std::min(lx, g->nx);
    *LX = lx;
    *grid = dim3(tz, ty, (g->nx + lx - 1) / lx);
    return EVX_OK;
}

int check_cufft(cufftResult r, const char* where) {
    if (r == CUFFT_SUCCESS) return EVX_OK;
    return fail(EVX_ERR_CUFFT, "%s: cuFFT error %d", where, (int)r);
}

int ch_validate_params(const evx_ch_params* p) {
    if (!p) return fail(EVX_ERR_BAD_ARG, "params is NULL");
    const float v[6] = {p->D, p->kappa, p->w, p->A, p->sym_coef, p->dt};
    for (float x : v)
        if (!std::isfinite(x)) return fail(EVX_ERR_BAD_ARG, "Cahn-Hilliard parameters must be finite");
    if (p->bulk != EVX_BULK_DOUBLE_WELL && p->bulk != EVX_BULK_REGULAR_SOLUTION)
        return fail(EVX_ERR_BAD_ARG, "unknown bulk potential form %d", (int)p->bulk);
    return EVX_OK;
}

int ch_plan_bind(evx_ch_plan* plan, void* workspace, cudaStream_t st, bool need_c2r2) {
    if (!workspace) return fail(EVX_ERR_WORKSPACE, "workspace is NULL");
    if (reinterpret_cast<uintptr_t>(workspace) & 255)
        return fail(EVX_ERR_WORKSPACE, "workspace must be 256-byte aligned");
    void* fw = ws_at(workspace, plan->off_fft);
    int rc;
    if ((rc = check_cufft(cufftSetWorkArea(plan->r2c, fw), "cufftSetWorkArea"))) return rc;
    if ((rc = check_cufft(cufftSetWorkArea(plan->c2r, fw), "cufftSetWorkArea"))) return rc;
    if ((rc = check_cufft(cufftSetStream(plan->r2c, st), "cufftSetStream"))) return rc;
    if ((rc = check_cufft(cufftSetStream(plan->c2r, st), "cufftSetStream"))) return rc;
    if (plan->yc2c) {
        if ((rc = check_cufft(cufftSetWorkArea(plan->yc2c, fw), "cufftSetWorkArea"))) return rc;
        if ((rc = check_cufft(cufftSetStream(plan->yc2c, st), "cufftSetStream"))) return rc;
    }
    if (plan->yc2c2) {
        if ((rc = check_cufft(cufftSetWorkArea(plan->yc2c2, fw), "cufftSetWorkArea"))) return rc;
        if ((rc = check_cufft(cufftSetStream(plan->yc2c2, st), "cufftSetStream"))) return rc;
    }
    if (need_c2r2) {
        if (!plan->has_c2r2) return fail(EVX_ERR_BAD_ARG, "parameter gradients need a plan created with flags bit 0");
        if ((rc = check_cufft(cufftSetWorkArea(plan->c2r2, fw), "cufftSetWorkArea"))) return rc;
        if ((rc = check_cufft(cufftSetStream(plan->c2r2, st), "cufftSetStream"))) return rc;
    }
    return EVX_OK;
}

int ch_r2c(evx_ch_plan* plan, const float* in, float2* out, cudaStream_t st) {
    if (plan->yzmode) return fft_yz_r2c(plan->g.nx, plan->g.ny, plan->g.nz, in, out, st);
    if (plan->ztmode) {   // z pass into [x][kz][y], then the contiguous y transform in place
        int rc = fft_zt_r2c(plan->g.nx, plan->g.ny, plan->g.nz, in, out, st);
        if (rc) return rc;
        cufftResult r;
        cufftComplex* s = reinterpret_cast<cufftComplex*>(out);
        EVX_TIMED("cufft_c2c_y", st, r = cufftExecC2C(plan->yc2c, s, s, CUFFT_FORWARD));
        return check_cufft(r, "cufftExecC2C (y)");
    }
    cufftResult r;
    EVX_TIMED("cufft_r2c", st, r = cufftExecR2C(plan->r2c, const_cast<cufftReal*>(in), reinterpret_cast<cufftComplex*>(out)));
    return check_cufft(r, "cufftExecR2C");
}

int ch_c2r(evx_ch_plan* plan, float2* in, float* out, bool batch2, cudaStream_t st) {
    if (plan->yzmode) {
        const evx_grid& g = plan->g;
        int rc = fft_yz_c2r(g.nx, g.ny, g.nz, in, out, st);
        if (!rc && batch2) rc = fft_yz_c2r(g.nx, g.ny, g.nz, in + plan->nspec, out + plan->n, st);
        return rc;
    }
    if (plan->ztmode) {   // inverse y transform in place (the input is consumed, as by a C2R), then z
        const evx_grid& g = plan->g;
        if (batch2 && !plan->yc2c2) return fail(EVX_ERR_BAD_ARG, "parameter gradients need a plan created with flags bit 0");
        cufftResult r;
        cufftComplex* s = reinterpret_cast<cufftComplex*>(in);
        EVX_TIMED(batch2 ? "cufft_c2c_y_x2" : "cufft_c2c_y", st,
                  r = cufftExecC2C(batch2 ? plan->yc2c2 : plan->yc2c, s, s, CUFFT_INVERSE));
        int rc = check_cufft(r, "cufftExecC2C (y)");
        if (rc) return rc;
        return fft_zt_c2r(batch2 ? 2 * g.nx : g.nx, g.ny, g.nz, in, out, st);   // two spectra: 2*nx planes
    }
    cufftResult r;
    EVX_TIMED(batch2 ? "cufft_c2r_x2" : "cufft_c2r", st,
              r = cufftExecC2R(batch2 ? plan->c2r2 : plan->c2r, reinterpret_cast<cufftComplex*>(in), out));
    return check_cufft(r, "cufftExecC2R");
}

int ch_kspace_forward(evx_ch_plan* plan, float2* spec, const ChP& P, cudaStream_t st, float2* dspec) {
    const float invN = (float)(1.0 / ((double)plan->nxe * plan->g.ny * plan->g.nz));
    if (plan->xmode) {
        XpassArgs a = xpass_args(plan, 0, spec, P);
        a.dspec = dspec;
        return xpass_launch(a, st);
    }
    if (dspec) return fail(EVX_ERR_UNSUPPORTED, "stored spectra need an x-pass plan");
    EVX_TIMED("ch_kspace_fwd", st, ch_kspace_fwd_kernel<<<elementwise_grid(plan->nspec), 256, 0, st>>>(
        spec, plan->g.ny, plan->nzh, plan->nspec, plan->kx2, plan->ky2, plan->kz2, P.sym_coef, P.dt, invN));
    count_launch();
    return check_launch("ch_kspace_fwd_kernel");
}

// The x mirror extension of a field of nx planes held in a buffer of 2*nx planes (in place).
int ch_mirror_x(const evx_ch_plan* plan, float* buf, cudaStream_t st) {
    EVX_TIMED("ch_mirror_x", st, ch_mirror_x_kernel<<<elementwise_grid(plan->n), 256, 0, st>>>(
        buf, plan->g.nx, (size_t)plan->g.ny * plan->g.nz, plan->xext == 2 ? -1.f : 1.f));
    count_launch();
    return check_launch("ch_mirror_x_kernel");
}

// out = P in, the step's spectral operator irfft . diag(prefac/N) . rfft with the x mirror
// extension of a non-periodic x axis (evoxels/timesteppers.py:85-89, boundary_conditions.py:64-70).
// P is symmetric (prefac depends on k^2 only, and the extension, the multiply and the restriction
// to the first nx planes commute with the reflection), so this is also its adjoint.  ext: 2*n floats
// of scratch for the cuFFT 3-D mirror path; out: 2*n floats on that path, n otherwise.
int ch_apply_spectral(evx_ch_plan* plan, const float* in, float* ext, float* out, float2* spec, const ChP& P,
                      cudaStream_t st) {
    int rc;
    const float* src = in;
    if (plan->xext && !plan->xmode) {
        const size_t N = plan->n;
        if ((rc = check_cuda(cudaMemcpyAsync(ext, in, N * sizeof(float), cudaMemcpyDeviceToDevice, st),
                             "mirror extension copy")))
            return rc;
        if ((rc = ch_mirror_x(plan, ext, st))) return rc;
        src = ext;
    }
    if ((rc = ch_r2c(plan, src, spec, st))) return rc;
    if ((rc = ch_kspace_forward(plan, spec, P, st))) return rc;
    return ch_c2r(plan, spec, out, false, st);
}

}  // namespace evx

using namespace evx;

namespace {

bool all_periodic(const Geo& G) {
    return G.kind[0] == EVX_BC_PERIODIC && G.kind[1] == EVX_BC_PERIODIC && G.kind[2] == EVX_BC_PERIODIC;
}

// exact: the reference's float32 operations (evx_ch_rhs); the spectral loops pass
// false, which lets the periodic fast path fuse its products
int ch_rhs_launch(bool fused, bool exact, const float* u, const float* upd, float* u_new, float* r,
                  const evx_grid* g, const Geo& G, const ChP& P, cudaStream_t st) {
    // the tile kernels: periodic grids, and (spectral loops only) a Neumann or Dirichlet x axis
    const bool yz_periodic = G.kind[1] == EVX_BC_PERIODIC && G.kind[2] == EVX_BC_PERIODIC;
    if ((all_periodic(G) || (!exact && yz_periodic)) && fast_ok(g, {u, upd, u_new, r}))
        return ch_rhs_fast_launch(fused, exact, u, upd, u_new, r, g, G, P, st);
    dim3 grid; int lx;
    ch_stencil_grid(g, &grid, &lx);
    if (fused) EVX_TIMED("ch_rhs_fused", st, ch_rhs_kernel<true><<<grid, dim3(32, 8), 0, st>>>(u, upd, u_new, r, G, P, lx));
    else EVX_TIMED("ch_rhs", st, ch_rhs_kernel<false><<<grid, dim3(32, 8), 0, st>>>(u, nullptr, nullptr, r, G, P, lx));
    count_launch();
    return check_launch("ch_rhs_kernel");
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

extern "C" {

int evx_ch_rhs(const float* u, float* r, const evx_grid* g, const evx_bc* bc, const evx_ch_params* p,
               void* stream) {
    int rc = validate_grid(g);
    if (rc) return rc;
    if ((rc = validate_bc(bc))) return rc;
    if ((rc = ch_validate_params(p))) return rc;
    if (!u || !r) return fail(EVX_ERR_BAD_ARG, "NULL field pointer");
    if (u == r) return fail(EVX_ERR_BAD_ARG, "input and output must not alias");
    return ch_rhs_launch(false, true, u, nullptr, nullptr, r, g, make_geo(g, bc), make_chp(p), as_stream(stream));
}

int evx_ch_plan_create(evx_ch_plan** out, const evx_grid* g, int flags) {
    return evx_ch_plan_create_bc(out, g, nullptr, flags);
}

int evx_ch_plan_create_bc(evx_ch_plan** out, const evx_grid* g, const evx_bc* bc, int flags) {
    if (!out) return fail(EVX_ERR_BAD_ARG, "plan pointer is NULL");
    *out = nullptr;
    int rc = validate_grid(g);
    if (rc) return rc;
    int xext = 0;
    if (bc) {
        if ((rc = validate_bc(bc))) return rc;
        const int nonper = (bc->kind[0] != EVX_BC_PERIODIC) + (bc->kind[1] != EVX_BC_PERIODIC) +
                           (bc->kind[2] != EVX_BC_PERIODIC);
        if (nonper > 1)
            return fail(EVX_ERR_BAD_BC, "FFT-based timesteppers currently support at most one non-periodic axis");
        if (nonper == 1 && bc->kind[0] == EVX_BC_PERIODIC)
            return fail(EVX_ERR_UNSUPPORTED, "FFT-based timesteppers currently only implement the single "
                                             "non-periodic axis case for x");
        xext = bc->kind[0] == EVX_BC_NEUMANN ? 1 : (bc->kind[0] == EVX_BC_DIRICHLET ? 2 : 0);
    }
    evx_ch_plan* p = new evx_ch_plan();
    p->g = *g;
    p->xext = xext;
    p->nxe = xext ? 2 * g->nx : g->nx;
    if (bc) p->bc = *bc;
    else for (int a = 0; a < 3; ++a) { p->bc.kind[a] = EVX_BC_PERIODIC; p->bc.two_v_lo[a] = p->bc.two_v_hi[a] = 0.f; }
    p->nzh = g->nz / 2 + 1;
    p->n = field_elems(g);
    // the x-pass keeps nx planes of the (y, z) spectrum; cuFFT's 3-D transform all nxe
    const bool xmode = xpass_supported(p->nxe) && !(flags & 2);
    p->nspec = (size_t)(xmode ? g->nx : p->nxe) * g->ny * p->nzh;
    size_t w1 = 0, w2 = 0, w3 = 0;
    auto cleanup = [&](int code) {
        if (p->r2c) cufftDestroy(p->r2c);
        if (p->c2r) cufftDestroy(p->c2r);
        if (p->c2r2) cufftDestroy(p->c2r2);
        if (p->yc2c) cufftDestroy(p->yc2c);
        if (p->yc2c2) cufftDestroy(p->yc2c2);
        if (p->kx2) cudaFree(p->kx2);
        delete p;
        return code;
    };
    if (p->nspec > 2147483647ull || 2 * p->n > 2147483647ull)
        return cleanup(fail(EVX_ERR_TOO_LARGE, "grid too large for 32-bit cuFFT plans"));
    if (xext && (flags & 1))
        return cleanup(fail(EVX_ERR_UNSUPPORTED, "parameter gradients of the mirrored-x spectral step are not built"));
    if ((rc = check_cufft(cufftCreate(&p->r2c), "cufftCreate"))) return cleanup(rc);
    if ((rc = check_cufft(cufftCreate(&p->c2r), "cufftCreate"))) return cleanup(rc);
    cufftSetAutoAllocation(p->r2c, 0);
    cufftSetAutoAllocation(p->c2r, 0);
    // power-of-two nx: cuFFT transforms (y, z) for every x plane and the fused x-pass does the rest
    p->xmode = xmode;
    p->yzmode = p->xmode && yz_supported(g->ny, g->nz) && (flags & 4);
    // z pass of our own with a y-contiguous spectrum: by default for nz = 256 (faster than cuFFT's
    // 2-D plans there; not below), flags bit 4 for every supported nz, flags bit 3 never
    p->ztmode = p->xmode && !p->yzmode && zt_supported(g->nz) && !(flags & 8) && ((flags & 16) || g->nz == 256);
    size_t w4 = 0, w5 = 0;
    if (p->ztmode) {
        int ny1[1] = {g->ny};
        const int cols = g->nx * p->nzh;
        if ((rc = check_cufft(cufftCreate(&p->yc2c), "cufftCreate"))) return cleanup(rc);
        cufftSetAutoAllocation(p->yc2c, 0);
        if ((rc = check_cufft(cufftMakePlanMany(p->yc2c, 1, ny1, nullptr, 1, g->ny, nullptr, 1, g->ny, CUFFT_C2C,
                                                cols, &w4), "cufftMakePlanMany C2C (y)")))
            return cleanup(rc);
        if (flags & 1) {
            if ((rc = check_cufft(cufftCreate(&p->yc2c2), "cufftCreate"))) return cleanup(rc);
            cufftSetAutoAllocation(p->yc2c2, 0);
            if ((rc = check_cufft(cufftMakePlanMany(p->yc2c2, 1, ny1, nullptr, 1, g->ny, nullptr, 1, g->ny, CUFFT_C2C,
                                                    2 * cols, &w5), "cufftMakePlanMany C2C (y) x2")))
                return cleanup(rc);
        }
    }
    if (p->xmode) {
        int d2[2] = {g->ny, g->nz};
        const int pr = g->ny * g->nz, ps = g->ny * p->nzh;
        if ((rc = check_cufft(cufftMakePlanMany(p->r2c, 2, d2, nullptr, 1, pr, nullptr, 1, ps, CUFFT_R2C, g->nx, &w1),
                              "cufftMakePlanMany R2C (y,z)")))
            return cleanup(rc);
        if ((rc = check_cufft(cufftMakePlanMany(p->c2r, 2, d2, nullptr, 1, ps, nullptr, 1, pr, CUFFT_C2R, g->nx, &w2),
                              "cufftMakePlanMany C2R (y,z)")))
            return cleanup(rc);
    } else {
        if ((rc = check_cufft(cufftMakePlan3d(p->r2c, p->nxe, g->ny, g->nz, CUFFT_R2C, &w1), "cufftMakePlan3d R2C")))
            return cleanup(rc);
        if ((rc = check_cufft(cufftMakePlan3d(p->c2r, p->nxe, g->ny, g->nz, CUFFT_C2R, &w2), "cufftMakePlan3d C2R")))
            return cleanup(rc);
    }
    if (flags & 1) {
        if ((rc = check_cufft(cufftCreate(&p->c2r2), "cufftCreate"))) return cleanup(rc);
        cufftSetAutoAllocation(p->c2r2, 0);
        if (p->xmode) {
            int d2[2] = {g->ny, g->nz};
            const int pr = g->ny * g->nz, ps = g->ny * p->nzh;
            if ((rc = check_cufft(cufftMakePlanMany(p->c2r2, 2, d2, nullptr, 1, ps, nullptr, 1, pr, CUFFT_C2R,
                                                    2 * g->nx, &w3), "cufftMakePlanMany C2R (y,z) x2")))
                return cleanup(rc);
        } else {
            int dims[3] = {g->nx, g->ny, g->nz};
            if ((rc = check_cufft(cufftMakePlanMany(p->c2r2, 3, dims, nullptr, 1, (int)p->nspec, nullptr, 1,
                                                    (int)p->n, CUFFT_C2R, 2, &w3), "cufftMakePlanMany C2R x2")))
                return cleanup(rc);
        }
        p->has_c2r2 = true;
    }
    p->ws_fft = std::max(std::max(w1, std::max(w2, w3)), std::max(w4, w5));
    // k^2 tables, bit-identical to the reference's float32 k-grid (2*nx x points when mirrored)
    const size_t nt = (size_t)p->nxe + g->ny + p->nzh;
    float* host = new float[nt];
    rc = evx_k2_tables_host(p->nxe, g->ny, g->nz, g->h[0], g->h[1], g->h[2], host, host + p->nxe,
                            host + p->nxe + g->ny);
    if (rc) { delete[] host; return cleanup(rc); }
    if ((rc = check_cuda(cudaMalloc(&p->kx2, nt * sizeof(float)), "cudaMalloc k2 tables"))) {
        delete[] host;
        return cleanup(rc);
    }
    rc = check_cuda(cudaMemcpy(p->kx2, host, nt * sizeof(float), cudaMemcpyHostToDevice), "cudaMemcpy k2 tables");
    delete[] host;
    if (rc) return cleanup(rc);
    p->ky2 = p->kx2 + p->nxe;
    p->kz2 = p->ky2 + g->ny;
    // workspace layout
    dim3 sg; int lx;
    ch_stencil_grid(g, &sg, &lx);
    p->n_part = std::max((int)(sg.x * sg.y * sg.z), ch_pullback_fast_blocks(g));
    size_t off = 0;
    p->off_fft = off;  off += align256(p->ws_fft);
    // r: 2 fields (rhs extended to 2*nx planes; g and h in the adjoint); update: the
    // whole 2*nx-plane inverse transform on the cuFFT 3-D mirrored path
    const size_t upd_fields = (xext && !xmode) ? 2 : 1;
    p->off_r = off;    off += align256(2 * p->n * sizeof(float));
    p->off_upd = off;  off += align256(upd_fields * p->n * sizeof(float));
    p->off_spec = off; off += align256(2 * p->nspec * sizeof(float2));
    p->off_u = off;    off += align256(p->n * sizeof(float));
    p->off_lam = off;  off += align256(p->n * sizeof(float));
    p->off_part = off; off += align256((size_t)p->n_part * 4 * sizeof(double) + 16);   // + reduction counter
    p->n_xpart = p->xmode && !xext ? xpass_blocks(g->nx, g->ny * p->nzh) : 0;
    p->spec_floats = p->xmode && !xext ? xpass_spectrum_floats(g->nx, g->ny * p->nzh) : 0;
    p->off_xpart = off; off += align256(p->n_xpart * 2 * sizeof(double));
    p->total = off;
    *out = p;
    return EVX_OK;
}

int evx_ch_plan_destroy(evx_ch_plan* p) {
    if (!p) return EVX_OK;
    if (p->r2c) cufftDestroy(p->r2c);
    if (p->c2r) cufftDestroy(p->c2r);
    if (p->c2r2) cufftDestroy(p->c2r2);
    if (p->yc2c) cufftDestroy(p->yc2c);
    if (p->yc2c2) cufftDestroy(p->yc2c2);
    if (p->kx2) cudaFree(p->kx2);
    delete p;
    return EVX_OK;
}

size_t evx_ch_workspace_bytes(const evx_ch_plan* p) { return p ? p->total : 0; }

int evx_spectral_update(evx_ch_plan* plan, const float* u, const float* r, const float* mult, float* out,
                        void* workspace, void* stream) {
    if (!plan) return fail(EVX_ERR_BAD_ARG, "plan is NULL");
    if (!u || !r || !mult || !out) return fail(EVX_ERR_BAD_ARG, "NULL pointer");
    if (r == out || mult == out) return fail(EVX_ERR_BAD_ARG, "rhs and multiplier must not alias the output");
    cudaStream_t st = as_stream(stream);
    int rc = ch_plan_bind(plan, workspace, st, false);
    if (rc) return rc;
    const evx_grid* g = &plan->g;
    const size_t N = plan->n;
    float* rbuf = reinterpret_cast<float*>(ws_at(workspace, plan->off_r));
    float* upd = reinterpret_cast<float*>(ws_at(workspace, plan->off_upd));
    float2* spec = reinterpret_cast<float2*>(ws_at(workspace, plan->off_spec));
    const float invN = (float)(1.0 / ((double)plan->nxe * g->ny * g->nz));
    if (plan->xmode) {   // (y, z) transforms of the nx planes; the x-pass extends, transforms, multiplies
        if ((rc = ch_r2c(plan, r, spec, st))) return rc;
        const ChP P{};
        XpassArgs a = xpass_args(plan, 4, spec, P);
        a.mult = mult;
        if ((rc = xpass_launch(a, st))) return rc;
    } else {
        const float* src = r;
        if (plan->xext) {
            EVX_TIMED("mirror_copy_x", st, mirror_copy_x_kernel<<<elementwise_grid(N), 256, 0, st>>>(
                r, rbuf, g->nx, (size_t)g->ny * g->nz, plan->xext == 2 ? -1.f : 1.f));
            count_launch();
            if ((rc = check_launch("mirror_copy_x_kernel"))) return rc;
            src = rbuf;
        }
        if ((rc = ch_r2c(plan, src, spec, st))) return rc;
        EVX_TIMED("spec_mult", st, spec_mult_kernel<<<elementwise_grid(plan->nspec), 256, 0, st>>>(
            spec, mult, invN, plan->nspec));
        count_launch();
        if ((rc = check_launch("spec_mult_kernel"))) return rc;
    }
    if ((rc = ch_c2r(plan, spec, upd, false, st))) return rc;
    // the first nx planes of the (extended) inverse transform: u + update[:, :nx]
    EVX_TIMED("ch_axpy", st, ch_axpy_kernel<<<elementwise_grid(N / 4 + 1), 256, 0, st>>>(
        u, upd, out, nullptr, N, nullptr));
    count_launch();
    return check_launch("ch_axpy_kernel");
}

size_t evx_ch_spectrum_floats(const evx_ch_plan* p) { return p ? p->spec_floats : 0; }

int evx_ch_mult_layout(const evx_ch_plan* p) { return p ? (p->ztmode ? 1 : 0) : -1; }

int evx_ch_forward(evx_ch_plan* plan, const float* u_in, float* u_out, int nsteps, float* traj,
                   const evx_ch_params* prm, int* nonfinite, void* workspace, void* stream) {
    return evx_ch_forward_spectra(plan, u_in, u_out, nsteps, traj, nullptr, prm, nonfinite, workspace, stream);
}

namespace {
// The forward loop of evx_ch_forward_spectra; mult != NULL replaces the IMEX
// multiplier by a table (the ExponentialEuler step of evx_ch_forward_mult).
int ch_forward_impl(evx_ch_plan* plan, const float* u_in, float* u_out, int nsteps, float* traj, float* spectra,
                    const float* mult, const evx_ch_params* prm, int* nonfinite, void* workspace, void* stream);
}  // namespace

int evx_ch_forward_spectra(evx_ch_plan* plan, const float* u_in, float* u_out, int nsteps, float* traj,
                           float* spectra, const evx_ch_params* prm, int* nonfinite, void* workspace, void* stream) {
    return ch_forward_impl(plan, u_in, u_out, nsteps, traj, spectra, nullptr, prm, nonfinite, workspace, stream);
}

int evx_ch_forward_mult(evx_ch_plan* plan, const float* u_in, float* u_out, int nsteps, const float* mult,
                        const evx_ch_params* prm, int* nonfinite, void* workspace, void* stream) {
    if (!mult) return fail(EVX_ERR_BAD_ARG, "NULL multiplier table");
    return ch_forward_impl(plan, u_in, u_out, nsteps, nullptr, nullptr, mult, prm, nonfinite, workspace, stream);
}

namespace {
int ch_forward_impl(evx_ch_plan* plan, const float* u_in, float* u_out, int nsteps, float* traj, float* spectra,
                    const float* mult, const evx_ch_params* prm, int* nonfinite, void* workspace, void* stream) {
    if (!plan) return fail(EVX_ERR_BAD_ARG, "plan is NULL");
    int rc = ch_validate_params(prm);
    if (rc) return rc;
    if (!u_in || !u_out) return fail(EVX_ERR_BAD_ARG, "NULL field pointer");
    if (u_in == u_out) return fail(EVX_ERR_BAD_ARG, "input and output must not alias");
    if (nsteps < 0) return fail(EVX_ERR_BAD_ARG, "nsteps must be >= 0");
    if (spectra) {
        if (!plan->spec_floats) return fail(EVX_ERR_UNSUPPORTED, "stored spectra need an x-pass plan (power-of-two nx)");
        if (reinterpret_cast<uintptr_t>(spectra) & 15) return fail(EVX_ERR_BAD_ARG, "spectra must be 16-byte aligned");
    }
    const size_t N = plan->n;
    if (nsteps == 0)
        return check_cuda(cudaMemcpyAsync(u_out, u_in, N * sizeof(float), cudaMemcpyDeviceToDevice, as_stream(stream)),
                          "evx_ch_forward copy");
    const GraphKey key{1, key_p(u_in), key_p(u_out), (uint64_t)nsteps, key_p(traj), key_p(spectra), key_p(mult),
                       key_p(nonfinite), key_p(workspace), key_f(prm->D), key_f(prm->kappa), key_f(prm->w),
                       key_f(prm->A), key_f(prm->sym_coef), key_f(prm->dt), (uint64_t)prm->bulk};
    return plan->graphs.run(key, as_stream(stream), [&](cudaStream_t st) -> int {
    int rc;
    if ((rc = ch_plan_bind(plan, workspace, st, false))) return rc;
    const evx_grid* g = &plan->g;
    const Geo G = make_geo(g, &plan->bc);
    const ChP P = make_chp(prm);
    float* r = reinterpret_cast<float*>(ws_at(workspace, plan->off_r));
    float* upd = reinterpret_cast<float*>(ws_at(workspace, plan->off_upd));
    float2* spec = reinterpret_cast<float2*>(ws_at(workspace, plan->off_spec));
    float* ubuf = reinterpret_cast<float*>(ws_at(workspace, plan->off_u));
    const float* src = u_in;
    for (int s = 0; s < nsteps; ++s) {
        if (s == 0) {
            rc = ch_rhs_launch(false, false, src, nullptr, nullptr, r, g, G, P, st);
        } else {
            float* dst = traj ? traj + (size_t)(s - 1) * N : (((nsteps - 1 - s) % 2 == 0) ? ubuf : u_out);
            rc = ch_rhs_launch(true, false, src, upd, dst, r, g, G, P, st);
            src = dst;
        }
        if (rc) return rc;
        if (plan->xext && !plan->xmode) {   // cuFFT 3-D path: extend the rhs to 2*nx planes
            EVX_TIMED("ch_mirror_x", st, ch_mirror_x_kernel<<<elementwise_grid(N), 256, 0, st>>>(
                r, g->nx, (size_t)g->ny * g->nz, plan->xext == 2 ? -1.f : 1.f));
            count_launch();
            if ((rc = check_launch("ch_mirror_x_kernel"))) return rc;
        }
        if ((rc = ch_r2c(plan, r, spec, st))) return rc;
        if (mult) {   // table multiplier (exponential Euler)
            if (plan->xmode) {
                XpassArgs a = xpass_args(plan, 4, spec, P);
                a.mult = mult;
                if ((rc = xpass_launch(a, st))) return rc;
            } else {
                const float invN = (float)(1.0 / ((double)plan->nxe * g->ny * g->nz));
                EVX_TIMED("spec_mult", st, spec_mult_kernel<<<elementwise_grid(plan->nspec), 256, 0, st>>>(
                    spec, mult, invN, plan->nspec));
                count_launch();
                if ((rc = check_launch("spec_mult_kernel"))) return rc;
            }
        } else {
            float2* ds = spectra ? reinterpret_cast<float2*>(spectra + (size_t)s * plan->spec_floats) : nullptr;
            if ((rc = ch_kspace_forward(plan, spec, P, st, ds))) return rc;
        }
        if ((rc = ch_c2r(plan, spec, upd, false, st))) return rc;
    }
    EVX_TIMED("ch_axpy", st, ch_axpy_kernel<<<elementwise_grid(N / 4 + 1), 256, 0, st>>>(
        src, upd, u_out, traj ? traj + (size_t)(nsteps - 1) * N : nullptr, N, nonfinite));
    count_launch();
    return check_launch("ch_axpy_kernel");
    });
}
}  // namespace

int evx_ch_step(evx_ch_plan* plan, const float* u_in, float* u_out, const evx_ch_params* p, void* workspace,
                void* stream) {
    return evx_ch_forward(plan, u_in, u_out, 1, nullptr, p, nullptr, workspace, stream);
}

}  // extern "C"
