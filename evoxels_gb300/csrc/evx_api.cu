// Library-wide C ABI helpers: error strings, version, validation, k^2 tables.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>

#include "evx_common.cuh"

namespace evx {

static thread_local char g_err[512] = "";

void set_error(const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int fail(int code, const char* fmt, ...) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
    return code;
}

int check_cuda(cudaError_t e, const char* where) {
    if (e == cudaSuccess) return EVX_OK;
    return fail(EVX_ERR_CUDA, "%s: %s", where, cudaGetErrorString(e));
}

int check_launch(const char* where) { return check_cuda(cudaGetLastError(), where); }

int validate_grid(const evx_grid* g) {
    if (!g) return fail(EVX_ERR_BAD_ARG, "grid is NULL");
    if (g->nx < 1 || g->ny < 1 || g->nz < 1)
        return fail(EVX_ERR_BAD_SHAPE, "grid shape (%d, %d, %d) must be positive", g->nx, g->ny, g->nz);
    // 2^31 elements per field keeps 32-bit in-plane and 64-bit plane offsets safe.
    if ((double)g->nx * g->ny * g->nz > 2147483647.0)
        return fail(EVX_ERR_TOO_LARGE, "grid (%d, %d, %d) exceeds 2^31-1 voxels", g->nx, g->ny, g->nz);
    for (int a = 0; a < 3; ++a)
        if (!(g->inv_h[a] > 0.f) || !(g->inv_h2[a] > 0.f) || !std::isfinite(g->inv_h[a]))
            return fail(EVX_ERR_BAD_ARG, "grid spacing factors must be positive and finite");
    return EVX_OK;
}

int validate_bc(const evx_bc* bc) {
    if (!bc) return EVX_OK;  // NULL = fully periodic
    for (int a = 0; a < 3; ++a) {
        int k = bc->kind[a];
        if (k != EVX_BC_PERIODIC && k != EVX_BC_NEUMANN && k != EVX_BC_DIRICHLET)
            return fail(EVX_ERR_BAD_BC, "Unsupported BC type code %d on axis %d", k, a);
    }
    return EVX_OK;
}

}  // namespace evx

extern "C" {

const char* evx_last_error(void) { return evx::g_err; }

int evx_version(void) { return 10000; }  // 1.0.0

// float32 k^2 tables, computed with the same float operations torch performs in
// fftfreq / rfftfreq (arange(n) * float32(1/(n*d))), then float32(2*pi) * f and
// the square (evoxels/voxelgrid.py:84-90,110-114).
int evx_k2_tables_host(int nx, int ny, int nz, double hx, double hy, double hz,
                       float* kx2, float* ky2, float* kz2) {
    if (nx < 1 || ny < 1 || nz < 1) return evx::fail(EVX_ERR_BAD_SHAPE, "bad shape");
    if (!(hx > 0) || !(hy > 0) || !(hz > 0)) return evx::fail(EVX_ERR_BAD_ARG, "bad spacing");
    if (!kx2 || !ky2 || !kz2) return evx::fail(EVX_ERR_BAD_ARG, "NULL table");
    const volatile float two_pi = (float)(2.0 * M_PI);
    auto fill = [&](int n, double h, float* out) {
        const volatile float scale = (float)(1.0 / ((double)n * h));
        for (int i = 0; i < n; ++i) {
            int f = i < (n + 1) / 2 ? i : i - n;   // fftfreq ordering
            volatile float v = (float)f * scale;
            volatile float k = two_pi * v;
            out[i] = k * k;
        }
    };
    fill(nx, hx, kx2);
    fill(ny, hy, ky2);
    const volatile float sz = (float)(1.0 / ((double)nz * hz));
    for (int i = 0; i < nz / 2 + 1; ++i) {   // rfftfreq: 0 .. n/2
        volatile float v = (float)i * sz;
        volatile float k = two_pi * v;
        kz2[i] = k * k;
    }
    return EVX_OK;
}

}  // extern "C"
