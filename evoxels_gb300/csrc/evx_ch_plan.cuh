// Internal definition of evx_ch_plan, shared by the forward and adjoint units.
#pragma once

#include <cufft.h>

#include "evx_common.cuh"
#include "evx_graph.cuh"
#include "evx_prof.cuh"

struct evx_ch_plan {
    evx_grid g;
    evx_bc bc;               // the problem's BCs (y, z periodic; x periodic, Neumann or Dirichlet)
    int xext = 0;            // x mirror extension of the spectral step: 0 none, 1 even (Neumann), 2 odd (Dirichlet)
    int nxe;                 // transform length along x (2*nx with the extension)
    int nzh;                 // nz/2 + 1
    size_t n;                // nx*ny*nz
    size_t nspec;            // complex values of the spectrum buffer (nxe*ny*nzh; nx*ny*nzh with the x-pass)
    cufftHandle r2c = 0, c2r = 0, c2r2 = 0;
    bool has_c2r2 = false;
    bool xmode = false;      // (y, z) transforms batched over x + fused x-pass (power-of-two nx)
    bool yzmode = false;     // the (y, z) transforms by evx_fftyz.cu instead of cuFFT
    bool ztmode = false;     // z pass by evx_fftz.cu (spectrum [x][kz][y]) + cuFFT contiguous C2C along y
    cufftHandle yc2c = 0, yc2c2 = 0;   // ztmode: 1-D C2C along y over nx*(nz/2+1) columns (x2: two spectra)
    size_t ws_fft = 0;       // cuFFT work area (max over plans)
    float* kx2 = nullptr;    // device k^2 tables
    float* ky2 = nullptr;
    float* kz2 = nullptr;
    // workspace layout (byte offsets)
    size_t off_fft, off_r, off_upd, off_spec, off_u, off_lam, off_part, off_xpart, total;
    int n_part;              // capacity of the partial-sum array (blocks)
    size_t n_xpart;          // x-pass blocks (Parseval partial sums, 2 doubles each); 0 without x-pass
    size_t spec_floats;      // floats per stored increment spectrum; 0 without x-pass
    evx::GraphCache graphs;  // replays of repeated forward / adjoint calls
};

namespace evx {

// Kernel-side Cahn-Hilliard parameters.
struct ChP {
    float D, kappa, w, A, sym_coef, dt;
    int bulk;   // EVX_BULK_*
};

inline ChP make_chp(const evx_ch_params* p) {
    ChP o;
    o.D = p->D; o.kappa = p->kappa; o.w = p->w; o.A = p->A; o.sym_coef = p->sym_coef; o.dt = p->dt;
    o.bulk = p->bulk;
    return o;
}

inline char* ws_at(void* ws, size_t off) { return static_cast<char*>(ws) + off; }

int check_cufft(cufftResult r, const char* where);
int ch_validate_params(const evx_ch_params* p);
int ch_plan_bind(evx_ch_plan* plan, void* workspace, cudaStream_t st, bool need_c2r2);

// FFT helpers (stream already bound by ch_plan_bind)
int ch_r2c(evx_ch_plan* plan, const float* in, float2* out, cudaStream_t st);
int ch_c2r(evx_ch_plan* plan, float2* in, float* out, bool batch2, cudaStream_t st);

// (i, j, k) of element e of an [nx][ny][nzh] spectrum: 32-bit divisions while e fits in 32 bits
// (every half spectrum up to 1024^3), 64-bit beyond.
__device__ __forceinline__ void spec_ijk(size_t e, int ny, int nzh, int& i, int& j, int& k) {
    if (e < (size_t(1) << 32)) {
        const unsigned u = (unsigned)e, t = u / (unsigned)nzh, ii = t / (unsigned)ny;
        k = (int)(u - t * (unsigned)nzh);
        j = (int)(t - ii * (unsigned)ny);
        i = (int)ii;
    } else {
        const size_t t = e / (size_t)nzh;
        k = (int)(e - t * (size_t)nzh);
        j = (int)(t % (size_t)ny);
        i = (int)(t / (size_t)ny);
    }
}

// IMEX prefactor dt * (1/(1 - dt*(sym_coef*k4))) with k4 = (k^2)^2, in the
// reference's float32 operation order (evoxels/timesteppers.py:77).
__device__ __forceinline__ float imex_prefac(float k2, float sym_coef, float dt) {
    const float k4 = __fmul_rn(k2, k2);
    const float den = __fsub_rn(1.f, __fmul_rn(dt, __fmul_rn(sym_coef, k4)));
    return __fmul_rn(__frcp_rn(den), dt);
}

// Forward k-space multiply: spec *= prefac(k) then * invN (in that order);
// with dspec (x-pass plans only) the product is also stored there.
int ch_kspace_forward(evx_ch_plan* plan, float2* spec, const ChP& P, cudaStream_t st, float2* dspec = nullptr);
// The x mirror extension (even / odd by the plan's x BC) of nx planes into 2*nx planes, in place.
int ch_mirror_x(const evx_ch_plan* plan, float* buf, cudaStream_t st);
// out = P in, the step's (symmetric) spectral operator, x mirror extension included; ext: 2*n
// floats of scratch and out 2*n floats on a cuFFT 3-D mirror plan, out n floats otherwise.
int ch_apply_spectral(evx_ch_plan* plan, const float* in, float* ext, float* out, float2* spec, const ChP& P,
                      cudaStream_t st);

// Fused spectral x-pass (evx_fftx.cu): mode 0 forward multiply (and optional
// store of the increment spectrum into dspec), 1 adjoint g, 2 adjoint g and h
// (h into spec_h), 3 adjoint g plus Parseval sums against dspec into xpart.
struct XpassArgs {
    int mode, nx, M, nzh, nz;          // M = ny*nzh pencils
    float2* spec;
    float2* spec_h;
    float2* dspec;
    double* xpart;
    const float *kx2, *ky2, *kz2;
    float sym, dt, invN;
    int* n_xpart_out;                  // optional: partial-sum slots written (mode 3)
    int ext;                           // x mirror extension (mode 0 / 4): 1 even, 2 odd; nx = transform length
    const float* mult;                 // mode 4: multiplier table [kx < nx][ky][kz]
    int nyk;                           // 0: pencil m = ky*nzh + kz; ny: m = kz*ny + ky (y-contiguous spectrum)
};
// Batched x-pass (one launch per shape group of the batched path): per-instance
// spectrum offset and IMEX constants, indexed by blockIdx.y.
struct XBatchInst {
    long long soff;    // complex values
    float sym, dt, invN;
    int xoff;          // first partial-sum slot (pairs of doubles) of the instance's blocks
    long long doff;    // stored increment spectrum offset (complex values)
};
bool xpass_supported(int nx);
// mode 0 forward (optional store of the increment spectra to dspec), 1 adjoint g,
// 2 adjoint g and h (spec_h, same offsets), 3 adjoint g with the Parseval sums
// against dspec into xpart; per-tile kernel, per-instance offsets from xb
int xpass_batch_launch(int mode, int nx, float2* spec, float2* spec_h, const XBatchInst* xb, int count, int M,
                       int nzh, int nz, const float* kx2, const float* ky2, const float* kz2, cudaStream_t st,
                       int nyk = 0, float2* dspec = nullptr, double* xpart = nullptr);
size_t xpass_blocks(int nx, int M);
size_t xpass_spectrum_floats(int nx, int M);
int xpass_launch(const XpassArgs& a, cudaStream_t st);
inline XpassArgs xpass_args(const evx_ch_plan* plan, int mode, float2* spec, const ChP& P) {
    XpassArgs a{};
    a.mode = mode; a.nx = plan->nxe; a.M = plan->g.ny * plan->nzh; a.nzh = plan->nzh; a.nz = plan->g.nz;
    a.spec = spec;
    a.kx2 = plan->kx2; a.ky2 = plan->ky2; a.kz2 = plan->kz2;
    a.sym = P.sym_coef; a.dt = P.dt;
    a.invN = (float)(1.0 / ((double)plan->nxe * plan->g.ny * plan->g.nz));
    a.ext = plan->xext;
    a.nyk = plan->ztmode ? plan->g.ny : 0;
    return a;
}

// Fused (y, z) R2C / C2R of all x planes (evx_fftyz.cu), cuFFT's layout and scaling.
bool yz_supported(int ny, int nz);
// Real transforms along z with a y-contiguous half spectrum (evx_fftz.cu).
bool zt_supported(int nz);
int fft_zt_r2c(int nx, int ny, int nz, const float* in, float2* out, cudaStream_t st);
int fft_zt_c2r(int nx, int ny, int nz, const float2* in, float* out, cudaStream_t st);
int fft_yz_r2c(int nx, int ny, int nz, const float* in, float2* out, cudaStream_t st);
int fft_yz_c2r(int nx, int ny, int nz, const float2* in, float* out, cudaStream_t st);

// Tile shape shared by the rhs and pullback stencil kernels.
constexpr int CH_TZ = 32;           // tile extent along z (= warp width)
constexpr int CH_TY = 16;           // tile extent along y
constexpr int CH_THREADS = 256;     // 32 x 8 threads
int ch_stencil_grid(const evx_grid* g, dim3* grid, int* LX);

}  // namespace evx
