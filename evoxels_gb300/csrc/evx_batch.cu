// Batched uneven Cahn-Hilliard instances: many independent periodic grids of
// different sizes advanced together (the role jax.vmap plays for the
// reference's parameter estimation, evoxels/inversion.py:105-124, here for
// grids of different shapes).
//
// Layout: instances are packed into one field buffer, grouped by shape
// (largest first), consecutive within a group so that one cuFFT plan with
// batch = group size transforms the whole group.  Half spectra are packed the
// same way.  One IMEX step of the whole batch is
//   batched rhs (one persistent launch over instance x tile x x-chunk work
//   items, largest items first, pulled from a global counter)
//   -> R2C per shape group -> k-space multiply -> C2R per shape group,
// where a group with a power-of-two nx uses cuFFT's 2-D (y, z) transforms over
// all its instances' x planes and one batched x-pass launch (FFT along x,
// multiply, inverse FFT along x; the single-grid kernel of evx_fftx.cu with a
// per-instance table), and the other groups cuFFT 3-D and one batched k-space
// launch,
// with the update fused into the next step's rhs pass as in the single-grid
// path.  Runs of steps without a stored trajectory are captured once into a
// CUDA graph on an internal stream and replayed.  The adjoint runs the same
// way with the batched pullback, and reduces parameter-gradient partial sums
// per instance in a fixed order.
#include <algorithm>
#include <cmath>
#include <map>
#include <vector>

#include "evx_ch_fast.cuh"

namespace evx {
namespace {

struct KInst {          // k-space descriptor of one instance
    long long soff;     // spectrum offset (complex values)
    long long doff;     // stored increment spectrum offset (complex values)
    int nx, ny, nzh, nz;
    int kx, ky, kz;     // offsets of the k^2 tables
    float sym_coef, dt, invN;
    int xmode;          // 1: its group's multiply is done by the x-pass
    int xoff;           // first partial-sum slot of the spectral adjoint's blocks
};

struct RInst {          // gradient-reduction descriptor of one instance
    int part0, nparts, orig, xpart0, nxpart, pad;
    double kA, DA, invD;   // kappa*A, D*A, 1/D
};

// With dspec the multiplied spectrum (the step's increment spectrum) is also
// stored there, at the instance's doff.
__global__ void batch_kspace_fwd_kernel(float2* __restrict__ spec, const KInst* __restrict__ ki,
                                        const float* __restrict__ k2, float2* __restrict__ dspec) {
    const KInst K = ki[blockIdx.y];
    if (K.xmode) return;   // uniform in the block
    const size_t total = (size_t)K.nx * K.ny * K.nzh;
    float2* s = spec + K.soff;
    float2* ds = dspec ? dspec + K.doff : nullptr;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        int i, j, k;
        spec_ijk(e, K.ny, K.nzh, i, j, k);
        const float kk = __fadd_rn(__fadd_rn(__ldg(k2 + K.kx + i), __ldg(k2 + K.ky + j)), __ldg(k2 + K.kz + k));
        const float pre = imex_prefac(kk, K.sym_coef, K.dt);
        float2 v = s[e];
        v.x = __fmul_rn(__fmul_rn(v.x, pre), K.invN);
        v.y = __fmul_rn(__fmul_rn(v.y, pre), K.invN);
        s[e] = v;
        if (ds) ds[e] = v;
    }
}

// Spectral adjoint of the k-space groups: g-hat = prefac/N * lam-hat, and the
// Parseval sums t1 = sum wz Re(lam-hat conj dU), t2 = sum wz prefac k^4 Re(...)
// against the stored increment spectrum dU (wz = 1 on the kz = 0 and nz/2
// planes, 2 elsewhere), per block in double into xpart[2*(xoff + block)].
__global__ void batch_kspace_adj_spec_kernel(float2* __restrict__ spec, const float2* __restrict__ dspec,
                                             double* __restrict__ xpart, const KInst* __restrict__ ki,
                                             const float* __restrict__ k2) {
    __shared__ double red[2][8];
    const KInst K = ki[blockIdx.y];
    if (K.xmode) return;   // uniform in the block
    const size_t total = (size_t)K.nx * K.ny * K.nzh;
    float2* s = spec + K.soff;
    const float2* ds = dspec + K.doff;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    float t1 = 0.f, t2 = 0.f;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        int i, j, k;
        spec_ijk(e, K.ny, K.nzh, i, j, k);
        const float kk = (__ldg(k2 + K.kx + i) + __ldg(k2 + K.ky + j)) + __ldg(k2 + K.kz + k);
        const float k4 = kk * kk;
        const float pre = K.dt / (1.f - K.dt * (K.sym_coef * k4));
        const float sg = pre * K.invN;
        const float2 v = s[e], d = __ldg(ds + e);
        const float wz = (k == 0 || 2 * k == K.nz) ? 1.f : 2.f;
        const float re = wz * (v.x * d.x + v.y * d.y);
        t1 += re;
        t2 += re * (pre * k4);
        s[e] = make_float2(v.x * sg, v.y * sg);
    }
    double a = t1, b = t2;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xffffffffu, a, o);
        b += __shfl_down_sync(0xffffffffu, b, o);
    }
    const int w = threadIdx.x >> 5;
    if ((threadIdx.x & 31) == 0) { red[0][w] = a; red[1][w] = b; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double sa = 0.0, sb = 0.0;
        for (int q = 0; q < (int)(blockDim.x >> 5); ++q) { sa += red[0][q]; sb += red[1][q]; }
        double* o = xpart + (size_t)(K.xoff + blockIdx.x) * 2;
        o[0] = sa;
        o[1] = sb;
    }
}

__global__ void batch_kspace_adj_kernel(float2* __restrict__ spec, float2* __restrict__ spec_h,
                                        const KInst* __restrict__ ki, const float* __restrict__ k2) {
    const KInst K = ki[blockIdx.y];
    if (K.xmode) return;   // uniform in the block
    const size_t total = (size_t)K.nx * K.ny * K.nzh;
    float2* s = spec + K.soff;
    float2* sh = spec_h ? spec_h + K.soff : nullptr;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < total; e += stride) {
        int i, j, k;
        spec_ijk(e, K.ny, K.nzh, i, j, k);
        const float kk = (__ldg(k2 + K.kx + i) + __ldg(k2 + K.ky + j)) + __ldg(k2 + K.kz + k);
        const float k4 = kk * kk;
        const float sg = (K.dt / (1.f - K.dt * (K.sym_coef * k4))) * K.invN;
        const float2 v = s[e];
        s[e] = make_float2(v.x * sg, v.y * sg);
        if (sh) sh[e] = make_float2(v.x * (sg * k4), v.y * (sg * k4));
    }
}

__global__ void batch_axpy_kernel(const float* __restrict__ u, const float* __restrict__ upd, float* __restrict__ out,
                                  float* __restrict__ out2, size_t n4, int* nonfinite) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    bool bad = false;
    const float4* u4 = reinterpret_cast<const float4*>(u);
    const float4* d4 = reinterpret_cast<const float4*>(upd);
    for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n4; e += stride) {
        const float4 a = __ldg(u4 + e), b = __ldg(d4 + e);
        const float4 v = make_float4(__fadd_rn(a.x, b.x), __fadd_rn(a.y, b.y), __fadd_rn(a.z, b.z), __fadd_rn(a.w, b.w));
        reinterpret_cast<float4*>(out)[e] = v;
        if (out2) reinterpret_cast<float4*>(out2)[e] = v;
        bad |= !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z) || !isfinite(v.w);
    }
    if (nonfinite && __any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(nonfinite, 1);
}

// grads[orig*3 + 0..2] += per-instance reduction of the work items' partial sums
__global__ void batch_grad_reduce_kernel(const double* __restrict__ part, const RInst* __restrict__ ri,
                                         double* __restrict__ grads) {
    __shared__ double s[4][256];
    const RInst R = ri[blockIdx.x];
    const int t = threadIdx.x;
    double a[4] = {0.0, 0.0, 0.0, 0.0};
    for (int b = t; b < R.nparts; b += 256)
        for (int q = 0; q < 4; ++q) a[q] += part[(size_t)(R.part0 + b) * 4 + q];
    for (int q = 0; q < 4; ++q) s[q][t] = a[q];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o)
            for (int q = 0; q < 4; ++q) s[q][t] += s[q][t + o];
        __syncthreads();
    }
    if (t == 0) {
        double* g = grads + (size_t)R.orig * 3;
        g[0] += s[0][0] - R.kA * s[3][0];
        g[1] += s[1][0] - R.DA * s[3][0];
        g[2] += s[2][0];
    }
}

// Spectral variant: the pullback's two real-space sums (slots 1, 2 of each
// work item) and the Parseval sums t1, t2 of the instance's x-pass or k-space
// blocks: dL/dD += t1/D - kappa*A*t2, dL/dkappa += sK - D*A*t2, dL/dw += sW.
__global__ void batch_grad_reduce_spec_kernel(const double* __restrict__ part, const double* __restrict__ xpart,
                                              const RInst* __restrict__ ri, double* __restrict__ grads) {
    __shared__ double s[4][256];
    const RInst R = ri[blockIdx.x];
    const int t = threadIdx.x;
    double a[4] = {0.0, 0.0, 0.0, 0.0};   // sK, sW, t1, t2
    for (int b = t; b < R.nparts; b += 256) {
        a[0] += part[(size_t)(R.part0 + b) * 4 + 1];
        a[1] += part[(size_t)(R.part0 + b) * 4 + 2];
    }
    for (int b = t; b < R.nxpart; b += 256) {
        a[2] += xpart[(size_t)(R.xpart0 + b) * 2];
        a[3] += xpart[(size_t)(R.xpart0 + b) * 2 + 1];
    }
    for (int q = 0; q < 4; ++q) s[q][t] = a[q];
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (t < o)
            for (int q = 0; q < 4; ++q) s[q][t] += s[q][t + o];
        __syncthreads();
    }
    if (t == 0) {
        double* g = grads + (size_t)R.orig * 3;
        g[0] += s[2][0] * R.invD - R.kA * s[3][0];
        g[1] += s[0][0] - R.DA * s[3][0];
        g[2] += s[1][0];
    }
}

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace
}  // namespace evx

using namespace evx;

struct evx_batch {
    struct Plan {
        cufftHandle r2c = 0, c2r = 0;
        int first = 0, count = 0;   // instances (internal order) transformed by this plan pair
    };
    struct Group {
        int nx, ny, nz, nzh;
        long long off = 0, soff = 0;   // packed offsets of the group's first instance
        size_t n = 0, nspec = 0;       // per instance
        int first = 0, count = 0;      // internal instance range
        bool xmode = false;            // cuFFT (y, z) plans + batched x-pass
        bool zt = false;               // xmode with the library's z pass: spectrum [x][kz][y], plans' r2c = C2C along y
        int k2x = 0, k2y = 0, k2z = 0; // offsets of the group's k^2 tables
        std::vector<Plan> plans;
    };
    int n = 0;
    std::vector<evx_batch_instance> in;    // caller order
    std::vector<int> order;                // internal -> caller index
    std::vector<long long> off;            // caller index -> packed field offset (floats)
    size_t total = 0, total_spec = 0;
    std::vector<Group> groups;
    evx_batch_tuning tune{};
    int n_items = 0;
    void* dev = nullptr;                   // device tables
    BatchInst* d_inst = nullptr;
    BatchItem* d_items = nullptr;
    KInst* d_kinst = nullptr;
    RInst* d_rinst = nullptr;
    XBatchInst* d_xb = nullptr;
    bool any_kspace = true;                // a group still uses the k-space kernels
    float* d_k2 = nullptr;
    size_t ws_fft = 0;
    size_t off_fft = 0, off_r = 0, off_upd = 0, off_spec = 0, off_ua = 0, off_ub = 0, off_lam = 0, off_part = 0,
           off_xpart = 0, off_cnt = 0, total_ws = 0;
    int grid_rhs = 0, grid_pb[3] = {0, 0, 0};
    size_t spec_floats = 0;                // floats of one step's stored increment spectra (all instances)
    size_t n_xpart = 0;                    // Parseval partial-sum slots of the spectral adjoint
    cudaStream_t cap = nullptr;
    cudaGraphExec_t gexec = nullptr;
    const void* gexec_ws = nullptr;
    int gexec_steps = 0;
    unsigned long long gexec_launches = 0;
    int kspace_blocks = 0;
    evx::GraphCache graphs;                // replays of repeated forward / adjoint calls
};

namespace {

void batch_free(evx_batch* b) {
    for (auto& g : b->groups)
        for (auto& p : g.plans) {
            if (p.r2c) cufftDestroy(p.r2c);
            if (p.c2r) cufftDestroy(p.c2r);
        }
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    if (b->cap) cudaStreamDestroy(b->cap);
    if (b->dev) cudaFree(b->dev);
    delete b;
}

int bind_plans(evx_batch* b, void* ws, cudaStream_t st) {
    void* fw = ws_at(ws, b->off_fft);
    for (auto& g : b->groups)
        for (auto& p : g.plans) {
            int rc;
            if ((rc = check_cufft(cufftSetWorkArea(p.r2c, fw), "cufftSetWorkArea"))) return rc;
            if ((rc = check_cufft(cufftSetWorkArea(p.c2r, fw), "cufftSetWorkArea"))) return rc;
            if ((rc = check_cufft(cufftSetStream(p.r2c, st), "cufftSetStream"))) return rc;
            if ((rc = check_cufft(cufftSetStream(p.c2r, st), "cufftSetStream"))) return rc;
        }
    return EVX_OK;
}

int batch_r2c(evx_batch* b, const float* in, float2* out, cudaStream_t st) {
    for (auto& g : b->groups)
        for (auto& p : g.plans) {
            const long long fo = g.off + (long long)(p.first - g.first) * (long long)g.n;
            const long long so = g.soff + (long long)(p.first - g.first) * (long long)g.nspec;
            cufftResult r;
            if (g.zt) {   // z pass, then the contiguous y transform in place
                int rc = fft_zt_r2c(p.count * g.nx, g.ny, g.nz, in + fo, out + so, st);
                if (rc) return rc;
                cufftComplex* sp = reinterpret_cast<cufftComplex*>(out + so);
                EVX_TIMED("batch_cufft_c2c_y", st, r = cufftExecC2C(p.r2c, sp, sp, CUFFT_FORWARD));
                if ((rc = check_cufft(r, "cufftExecC2C (y) (batch)"))) return rc;
                continue;
            }
            EVX_TIMED("batch_cufft_r2c", st,
                      r = cufftExecR2C(p.r2c, const_cast<cufftReal*>(in + fo), reinterpret_cast<cufftComplex*>(out + so)));
            int rc = check_cufft(r, "cufftExecR2C (batch)");
            if (rc) return rc;
        }
    return EVX_OK;
}

int batch_c2r(evx_batch* b, float2* in, float* out, cudaStream_t st) {
    for (auto& g : b->groups)
        for (auto& p : g.plans) {
            const long long fo = g.off + (long long)(p.first - g.first) * (long long)g.n;
            const long long so = g.soff + (long long)(p.first - g.first) * (long long)g.nspec;
            cufftResult r;
            if (g.zt) {   // inverse y transform in place (the input is consumed), then z
                cufftComplex* sp = reinterpret_cast<cufftComplex*>(in + so);
                EVX_TIMED("batch_cufft_c2c_y", st, r = cufftExecC2C(p.r2c, sp, sp, CUFFT_INVERSE));
                int rc = check_cufft(r, "cufftExecC2C (y) (batch)");
                if (!rc) rc = fft_zt_c2r(p.count * g.nx, g.ny, g.nz, in + so, out + fo, st);
                if (rc) return rc;
                continue;
            }
            EVX_TIMED("batch_cufft_c2r", st,
                      r = cufftExecC2R(p.c2r, reinterpret_cast<cufftComplex*>(in + so), out + fo));
            int rc = check_cufft(r, "cufftExecC2R (batch)");
            if (rc) return rc;
        }
    return EVX_OK;
}

// x-pass of every power-of-two group: mode 0 forward (dspec: store the increment
// spectra), 1 adjoint g, 2 adjoint g and h, 3 adjoint g with the Parseval sums
int batch_xpass(evx_batch* b, int mode, float2* spec, float2* spec_h, cudaStream_t st, float2* dspec = nullptr,
                double* xpart = nullptr) {
    for (auto& g : b->groups) {
        if (!g.xmode) continue;
        int rc = xpass_batch_launch(mode, g.nx, spec, spec_h, b->d_xb + g.first, g.count, g.ny * g.nzh, g.nzh, g.nz,
                                    b->d_k2 + g.k2x, b->d_k2 + g.k2y, b->d_k2 + g.k2z, st, g.zt ? g.ny : 0, dspec,
                                    xpart);
        if (rc) return rc;
    }
    return EVX_OK;
}

// One IMEX step's spectral part: r -> upd; dspec (optional) receives the step's
// increment spectra
int batch_spectral(evx_batch* b, float* r, float2* spec, float* upd, cudaStream_t st, float2* dspec = nullptr) {
    int rc;
    if ((rc = batch_r2c(b, r, spec, st))) return rc;
    if (b->any_kspace) {
        EVX_TIMED("batch_kspace_fwd", st,
                  batch_kspace_fwd_kernel<<<dim3(b->kspace_blocks, b->n), 256, 0, st>>>(spec, b->d_kinst, b->d_k2,
                                                                                      dspec));
        count_launch();
        if ((rc = check_launch("batch_kspace_fwd_kernel"))) return rc;
    }
    if ((rc = batch_xpass(b, 0, spec, nullptr, st, dspec))) return rc;
    return batch_c2r(b, spec, upd, st);
}

struct Bufs {
    float *r, *upd, *ua, *ub, *lam;
    float2* spec;
    double *part, *xpart;
    int* cnt;
};

Bufs bufs(evx_batch* b, void* ws) {
    Bufs o;
    o.r = reinterpret_cast<float*>(ws_at(ws, b->off_r));
    o.upd = reinterpret_cast<float*>(ws_at(ws, b->off_upd));
    o.spec = reinterpret_cast<float2*>(ws_at(ws, b->off_spec));
    o.ua = reinterpret_cast<float*>(ws_at(ws, b->off_ua));
    o.ub = reinterpret_cast<float*>(ws_at(ws, b->off_ub));
    o.lam = reinterpret_cast<float*>(ws_at(ws, b->off_lam));
    o.part = reinterpret_cast<double*>(ws_at(ws, b->off_part));
    o.xpart = reinterpret_cast<double*>(ws_at(ws, b->off_xpart));
    o.cnt = reinterpret_cast<int*>(ws_at(ws, b->off_cnt));
    return o;
}

int fused_step(evx_batch* b, const Bufs& B, const float* src, float* dst, cudaStream_t st, float2* dspec = nullptr) {
    int rc = batch_rhs_launch(true, src, B.upd, dst, B.r, b->d_inst, b->d_items, b->n_items, B.cnt, b->grid_rhs, st);
    if (rc) return rc;
    return batch_spectral(b, B.r, B.spec, B.upd, st, dspec);
}

// Capture `steps` (even) fused steps A->B->A... on the internal stream.
int capture_chunk(evx_batch* b, void* ws, int steps) {
    if (b->gexec) {
        cudaGraphExecDestroy(b->gexec);
        b->gexec = nullptr;
    }
    int rc;
    if (!b->cap && (rc = check_cuda(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking), "capture stream")))
        return rc;
    if ((rc = bind_plans(b, ws, b->cap))) return rc;
    const Bufs B = bufs(b, ws);
    if ((rc = check_cuda(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal), "begin capture"))) return rc;
    const unsigned long long c0 = launch_counter();
    int rc2 = EVX_OK;
    for (int s = 0; s < steps && !rc2; ++s)
        rc2 = (s % 2 == 0) ? fused_step(b, B, B.ua, B.ub, b->cap) : fused_step(b, B, B.ub, B.ua, b->cap);
    cudaGraph_t graph = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->cap, &graph);
    b->gexec_launches = launch_counter() - c0;   // counted per replay instead
    uncount_launch(b->gexec_launches);
    if (rc2) {
        if (graph) cudaGraphDestroy(graph);
        return rc2;
    }
    if ((rc = check_cuda(e, "end capture"))) return rc;
    e = cudaGraphInstantiate(&b->gexec, graph, 0);
    cudaGraphDestroy(graph);
    if ((rc = check_cuda(e, "graph instantiate"))) return rc;
    b->gexec_ws = ws;
    b->gexec_steps = steps;
    return EVX_OK;
}

}  // namespace

namespace evx {
namespace {
// Every offset the batched kernels derive from the descriptors, checked against
// the buffers they index before anything is uploaded: each instance's field
// slice (16-byte aligned, disjoint, inside the packed field), every work item
// inside its instance with the tiles of an instance covering it exactly once,
// the spectrum, stored-spectrum and partial-sum ranges of every instance, and
// the k^2 table offsets.  A failure is a bug in the layout code.
int validate_layout(const evx_batch* b, const std::vector<BatchInst>& hinst, const std::vector<BatchItem>& items,
                    const std::vector<KInst>& hk, const std::vector<RInst>& hr, const std::vector<XBatchInst>& hxb,
                    size_t k2_len) {
    auto bad = [](const char* what, int i) {
        return fail(EVX_ERR_BAD_ARG, "batched layout check failed (internal error): %s, instance %d", what, i);
    };
    const int n = b->n;
    std::vector<std::pair<long long, long long>> spans;
    std::vector<long long> covered(n, 0);
    for (int ii = 0; ii < n; ++ii) {
        const BatchInst& B = hinst[ii];
        const long long ni = (long long)B.nx * B.ny * B.nz, nsi = (long long)B.nx * B.ny * (B.nz / 2 + 1);
        if (B.off < 0 || B.off % 4 || B.off + ni > (long long)b->total) return bad("field slice", ii);
        if (B.tile != 0 && B.tile != 1) return bad("tile variant", ii);
        spans.emplace_back(B.off, B.off + ni);
        const KInst& K = hk[ii];
        if (K.soff < 0 || K.soff + nsi > (long long)b->total_spec) return bad("spectrum slice", ii);
        if (K.nx != B.nx || K.ny != B.ny || K.nzh != B.nz / 2 + 1) return bad("k-space shape", ii);
        if (K.kx < 0 || K.ky != K.kx + B.nx || K.kz != K.ky + B.ny || (size_t)K.kz + K.nzh > k2_len)
            return bad("k^2 tables", ii);
        const int Mx = B.ny * (B.nz / 2 + 1);
        const long long dsz = K.xmode ? (long long)xpass_spectrum_floats(B.nx, Mx) / 2 : nsi;
        if (K.doff < 0 || 2 * (K.doff + dsz) > (long long)b->spec_floats) return bad("stored spectrum", ii);
        if (hxb[ii].soff != K.soff || hxb[ii].doff != K.doff || hxb[ii].xoff != K.xoff) return bad("x-pass descriptor", ii);
        const RInst& R = hr[ii];
        if (R.xpart0 != K.xoff || R.nxpart < 1 || (size_t)R.xpart0 + R.nxpart > std::max<size_t>(1, b->n_xpart))
            return bad("partial-sum slots", ii);
        if (R.part0 < 0 || R.nparts < 1 || R.part0 + R.nparts > (int)items.size()) return bad("work-item slots", ii);
    }
    std::sort(spans.begin(), spans.end());
    for (size_t i = 1; i < spans.size(); ++i)
        if (spans[i].first < spans[i - 1].second) return bad("overlapping field slices", (int)i);
    for (const BatchItem& it : items) {
        if (it.inst < 0 || it.inst >= n) return bad("work item instance", it.inst);
        const BatchInst& B = hinst[it.inst];
        const int TZ = B.tile ? 32 : 64, TY = B.tile ? 32 : 16;
        if (it.x0 < 0 || it.x0 >= it.x1 || it.x1 > B.nx || it.k0 < 0 || it.k0 >= B.nz || it.k0 % TZ ||
            it.j0 < 0 || it.j0 >= B.ny || it.j0 % TY)
            return bad("work item bounds", it.inst);
        if (it.part < hr[it.inst].part0 || it.part >= hr[it.inst].part0 + hr[it.inst].nparts)
            return bad("work item slot", it.inst);
        covered[it.inst] += (long long)(it.x1 - it.x0) * std::min(TZ, B.nz - it.k0) * std::min(TY, B.ny - it.j0);
    }
    for (int ii = 0; ii < n; ++ii)
        if (covered[ii] != (long long)hinst[ii].nx * hinst[ii].ny * hinst[ii].nz) return bad("tile cover", ii);
    return EVX_OK;
}
}  // namespace
}  // namespace evx

extern "C" {

int evx_batch_create(evx_batch** out, const evx_batch_instance* inst, int n, const evx_batch_tuning* tune, int flags) {
    if (!out) return fail(EVX_ERR_BAD_ARG, "batch pointer is NULL");
    *out = nullptr;
    if (!inst || n < 1) return fail(EVX_ERR_BAD_ARG, "need at least one instance");
    for (int i = 0; i < n; ++i) {
        evx_grid g;
        g.nx = inst[i].nx; g.ny = inst[i].ny; g.nz = inst[i].nz;
        for (int a = 0; a < 3; ++a) { g.h[a] = inst[i].h[a]; g.inv_h[a] = inst[i].inv_h[a]; g.inv_h2[a] = inst[i].inv_h2[a]; }
        g.inv_h2_sum = inst[i].inv_h2_sum;
        int rc = validate_grid(&g);
        if (rc) return rc;
        if (inst[i].nz % 4) return fail(EVX_ERR_UNSUPPORTED, "batched instances need nz %% 4 == 0 (instance %d)", i);
        if ((rc = ch_validate_params(&inst[i].params))) return rc;
        if (inst[i].params.bulk != EVX_BULK_DOUBLE_WELL)
            return fail(EVX_ERR_UNSUPPORTED, "batched instances take the double-well bulk term only");
    }
    evx_batch* b = new evx_batch();
    b->n = n;
    b->in.assign(inst, inst + n);
    if (tune) b->tune = *tune;
    else { b->tune.tile_variant = -1; b->tune.x_chunk = 0; b->tune.blocks_per_sm = 0; b->tune.fft_group_max = 0; b->tune.graph_steps = 20; }
    // internal order: group by shape and spacing, largest first; stable within a group
    b->order.resize(n);
    for (int i = 0; i < n; ++i) b->order[i] = i;
    auto key = [&](int i) {
        const auto& s = b->in[i];
        return std::make_tuple(-(long long)s.nx * s.ny * s.nz, s.nx, s.ny, s.nz, s.h[0], s.h[1], s.h[2]);
    };
    std::stable_sort(b->order.begin(), b->order.end(), [&](int a, int c) { return key(a) < key(c); });
    b->off.assign(n, 0);
    size_t foff = 0, soff = 0;
    std::vector<long long> soff_of(n);
    for (int ii = 0; ii < n; ++ii) {
        const int i = b->order[ii];
        const auto& s = b->in[i];
        const bool new_group = b->groups.empty() || key(b->order[b->groups.back().first]) != key(i);
        const size_t ni = (size_t)s.nx * s.ny * s.nz, nsi = (size_t)s.nx * s.ny * (s.nz / 2 + 1);
        if (new_group) {
            foff = al256(foff * 4) / 4;   // group starts 256-byte aligned
            soff = al256(soff * 8) / 8;
            evx_batch::Group g;
            g.nx = s.nx; g.ny = s.ny; g.nz = s.nz; g.nzh = s.nz / 2 + 1;
            g.off = (long long)foff; g.soff = (long long)soff;
            g.n = ni; g.nspec = nsi; g.first = ii; g.count = 0;
            b->groups.push_back(g);
        }
        b->groups.back().count++;
        b->off[i] = (long long)foff;
        soff_of[ii] = (long long)soff;
        foff += ni;
        soff += nsi;
    }
    b->total = al256(foff * 4) / 4;
    b->total_spec = al256(soff * 8) / 8;
    auto cleanup = [&](int code) { batch_free(b); return code; };
    // cuFFT plans per group (split by fft_group_max)
    size_t wmax = 0;
    b->any_kspace = false;
    for (auto& g : b->groups) {
        // flags bit 1: cuFFT's 3-D transforms for every group (as evx_ch_plan_create)
        g.xmode = xpass_supported(g.nx) && !(flags & 2) && (size_t)g.count * g.nx <= 2147483647ull;
        if (!g.xmode) b->any_kspace = true;
        // the z pass as in evx_ch_plan_create_bc: nz = 256 by default, flags bit 4 always, bit 3 never
        g.zt = g.xmode && zt_supported(g.nz) && !(flags & 8) && ((flags & 16) || g.nz == 256);
        const int gm = b->tune.fft_group_max > 0 ? b->tune.fft_group_max : g.count;
        for (int f = 0; f < g.count; f += gm) {
            evx_batch::Plan p;
            p.first = g.first + f;
            p.count = std::min(gm, g.count - f);
            size_t w1 = 0, w2 = 0;
            int rc;
            if ((rc = check_cufft(cufftCreate(&p.r2c), "cufftCreate"))) return cleanup(rc);
            if ((rc = check_cufft(cufftCreate(&p.c2r), "cufftCreate"))) { cufftDestroy(p.r2c); return cleanup(rc); }
            cufftSetAutoAllocation(p.r2c, 0);
            cufftSetAutoAllocation(p.c2r, 0);
            g.plans.push_back(p);
            if (g.zt) {      // 1-D C2C along the contiguous y of every (x, kz) column, both directions
                int ny1[1] = {g.ny};
                if ((rc = check_cufft(cufftMakePlanMany(p.r2c, 1, ny1, nullptr, 1, g.ny, nullptr, 1, g.ny, CUFFT_C2C,
                                                        p.count * g.nx * g.nzh, &w1), "cufftMakePlanMany C2C (y) (batch)")))
                    return cleanup(rc);
            } else if (g.xmode) {   // 2-D (y, z) over every x plane of the plan's instances
                int d2[2] = {g.ny, g.nz};
                const int pr = g.ny * g.nz, ps = g.ny * g.nzh;
                if ((rc = check_cufft(cufftMakePlanMany(p.r2c, 2, d2, nullptr, 1, pr, nullptr, 1, ps, CUFFT_R2C,
                                                        p.count * g.nx, &w1), "cufftMakePlanMany R2C (y,z) (batch)")))
                    return cleanup(rc);
                if ((rc = check_cufft(cufftMakePlanMany(p.c2r, 2, d2, nullptr, 1, ps, nullptr, 1, pr, CUFFT_C2R,
                                                        p.count * g.nx, &w2), "cufftMakePlanMany C2R (y,z) (batch)")))
                    return cleanup(rc);
            } else {
                int dims[3] = {g.nx, g.ny, g.nz};
                if ((rc = check_cufft(cufftMakePlanMany(p.r2c, 3, dims, nullptr, 1, (int)g.n, nullptr, 1,
                                                        (int)g.nspec, CUFFT_R2C, p.count, &w1),
                                      "cufftMakePlanMany R2C (batch)")))
                    return cleanup(rc);
                if ((rc = check_cufft(cufftMakePlanMany(p.c2r, 3, dims, nullptr, 1, (int)g.nspec, nullptr, 1,
                                                        (int)g.n, CUFFT_C2R, p.count, &w2),
                                      "cufftMakePlanMany C2R (batch)")))
                    return cleanup(rc);
            }
            wmax = std::max(wmax, std::max(w1, w2));
        }
    }
    b->ws_fft = wmax;
    size_t maxspec = 0;
    for (auto& g : b->groups) maxspec = std::max(maxspec, g.nspec);
    b->kspace_blocks = (int)std::max<size_t>(1, std::min<size_t>(256, (maxspec + 2047) / 2048));
    // work items, k-space and reduction descriptors, k^2 tables
    std::vector<BatchInst> hinst(n);
    std::vector<KInst> hk(n);
    std::vector<RInst> hr(n);
    std::vector<XBatchInst> hxb(n);
    std::vector<int> group_of(n);
    for (size_t gi = 0; gi < b->groups.size(); ++gi)
        for (int k = 0; k < b->groups[gi].count; ++k) group_of[b->groups[gi].first + k] = (int)gi;
    std::vector<BatchItem> items;
    std::vector<float> k2;
    size_t doff = 0, xoff = 0;   // stored-spectrum offsets (complex) and partial-sum slots, internal order
    std::map<std::tuple<int, int, int, double, double, double>, int> k2pos;
    for (int ii = 0; ii < n; ++ii) {
        const int i = b->order[ii];
        const auto& s = b->in[i];
        BatchInst& B = hinst[ii];
        B.nx = s.nx; B.ny = s.ny; B.nz = s.nz;
        B.tile = b->tune.tile_variant >= 0 ? b->tune.tile_variant : default_tile_variant(s.nz);
        B.off = b->off[i];
        B.orig = i;
        for (int a = 0; a < 3; ++a) { B.ih[a] = s.inv_h[a]; B.ih2[a] = s.inv_h2[a]; }
        B.ih2sum = s.inv_h2_sum;
        B.P = make_chp(&s.params);
        const int TZ = B.tile ? 32 : 64, TY = B.tile ? 32 : 16;
        const int lx = b->tune.x_chunk > 0 ? std::min(b->tune.x_chunk, s.nx) : std::min(16, s.nx);
        B.part0 = (int)items.size();
        for (int k0 = 0; k0 < s.nz; k0 += TZ)
            for (int j0 = 0; j0 < s.ny; j0 += TY)
                for (int x0 = 0; x0 < s.nx; x0 += lx) {
                    BatchItem it;
                    it.inst = ii; it.k0 = k0; it.j0 = j0; it.x0 = x0; it.x1 = std::min(x0 + lx, s.nx);
                    it.part = (int)items.size();
                    items.push_back(it);
                }
        hr[ii].part0 = B.part0;
        hr[ii].nparts = (int)items.size() - B.part0;
        hr[ii].orig = i;
        hr[ii].kA = (double)s.params.kappa * s.params.A;
        hr[ii].DA = (double)s.params.D * s.params.A;
        hr[ii].invD = 1.0 / (double)s.params.D;
        hr[ii].pad = 0;
        const auto kk = std::make_tuple(s.nx, s.ny, s.nz, s.h[0], s.h[1], s.h[2]);
        if (!k2pos.count(kk)) {
            k2pos[kk] = (int)k2.size();
            const size_t base = k2.size();
            k2.resize(base + s.nx + s.ny + s.nz / 2 + 1);
            int rc = evx_k2_tables_host(s.nx, s.ny, s.nz, s.h[0], s.h[1], s.h[2], &k2[base], &k2[base + s.nx],
                                        &k2[base + s.nx + s.ny]);
            if (rc) return cleanup(rc);
        }
        const int kb = k2pos[kk];
        hk[ii].soff = soff_of[ii];
        hk[ii].nx = s.nx; hk[ii].ny = s.ny; hk[ii].nzh = s.nz / 2 + 1;
        hk[ii].kx = kb; hk[ii].ky = kb + s.nx; hk[ii].kz = kb + s.nx + s.ny;
        hk[ii].sym_coef = s.params.sym_coef;
        hk[ii].dt = s.params.dt;
        hk[ii].invN = (float)(1.0 / ((double)s.nx * s.ny * s.nz));
        evx_batch::Group& grp = b->groups[group_of[ii]];
        hk[ii].xmode = grp.xmode ? 1 : 0;
        hk[ii].nz = s.nz;
        grp.k2x = hk[ii].kx; grp.k2y = hk[ii].ky; grp.k2z = hk[ii].kz;
        hxb[ii].soff = soff_of[ii];
        hxb[ii].sym = s.params.sym_coef;
        hxb[ii].dt = s.params.dt;
        hxb[ii].invN = hk[ii].invN;
        // the stored spectrum: the x-pass tile layout ([tile][element][thread]) or the k-space layout
        const int Mx = s.ny * (s.nz / 2 + 1);
        const size_t dsz = grp.xmode ? xpass_spectrum_floats(s.nx, Mx) / 2 : (size_t)s.nx * s.ny * (s.nz / 2 + 1);
        const size_t xsl = grp.xmode ? xpass_blocks(s.nx, Mx) : (size_t)b->kspace_blocks;
        hxb[ii].doff = hk[ii].doff = (long long)doff;
        hxb[ii].xoff = hk[ii].xoff = (int)xoff;
        hr[ii].xpart0 = (int)xoff;
        hr[ii].nxpart = (int)xsl;
        doff += (dsz + 1) & ~(size_t)1;   // 16-byte aligned starts
        xoff += xsl;
    }
    b->spec_floats = 2 * doff;
    b->n_xpart = xoff;
    int rc0;
    // largest work items first (longest-processing-time order for the persistent blocks)
    std::stable_sort(items.begin(), items.end(), [&](const BatchItem& a, const BatchItem& c) {
        auto cost = [&](const BatchItem& x) {
            const BatchInst& B = hinst[x.inst];
            return (long long)(B.tile ? 32 * 32 : 64 * 16) * (x.x1 - x.x0 + 4);
        };
        return cost(a) > cost(c);
    });
    b->n_items = (int)items.size();
    if ((rc0 = validate_layout(b, hinst, items, hk, hr, hxb, k2.size()))) return cleanup(rc0);
    // one device allocation for the tables
    const size_t s_inst = al256(sizeof(BatchInst) * n), s_items = al256(sizeof(BatchItem) * items.size());
    const size_t s_k = al256(sizeof(KInst) * n), s_r = al256(sizeof(RInst) * n), s_k2 = al256(sizeof(float) * k2.size());
    const size_t s_xb = al256(sizeof(XBatchInst) * n);
    int rc;
    if ((rc = check_cuda(cudaMalloc(&b->dev, s_inst + s_items + s_k + s_r + s_k2 + s_xb), "cudaMalloc batch tables")))
        return cleanup(rc);
    char* d = static_cast<char*>(b->dev);
    b->d_inst = reinterpret_cast<BatchInst*>(d);
    b->d_items = reinterpret_cast<BatchItem*>(d + s_inst);
    b->d_kinst = reinterpret_cast<KInst*>(d + s_inst + s_items);
    b->d_rinst = reinterpret_cast<RInst*>(d + s_inst + s_items + s_k);
    b->d_k2 = reinterpret_cast<float*>(d + s_inst + s_items + s_k + s_r);
    b->d_xb = reinterpret_cast<XBatchInst*>(d + s_inst + s_items + s_k + s_r + s_k2);
    if ((rc = check_cuda(cudaMemcpy(b->d_inst, hinst.data(), sizeof(BatchInst) * n, cudaMemcpyHostToDevice), "copy")) ||
        (rc = check_cuda(cudaMemcpy(b->d_items, items.data(), sizeof(BatchItem) * items.size(), cudaMemcpyHostToDevice),
                         "copy")) ||
        (rc = check_cuda(cudaMemcpy(b->d_kinst, hk.data(), sizeof(KInst) * n, cudaMemcpyHostToDevice), "copy")) ||
        (rc = check_cuda(cudaMemcpy(b->d_rinst, hr.data(), sizeof(RInst) * n, cudaMemcpyHostToDevice), "copy")) ||
        (rc = check_cuda(cudaMemcpy(b->d_k2, k2.data(), sizeof(float) * k2.size(), cudaMemcpyHostToDevice), "copy")) ||
        (rc = check_cuda(cudaMemcpy(b->d_xb, hxb.data(), sizeof(XBatchInst) * n, cudaMemcpyHostToDevice), "copy")))
        return cleanup(rc);
    // persistent grids
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    auto bps = [&](int occ) { return b->tune.blocks_per_sm > 0 ? std::min(b->tune.blocks_per_sm, occ) : occ; };
    b->grid_rhs = bps(batch_rhs_blocks_per_sm()) * sms;
    for (int gr = 0; gr < 3; ++gr) b->grid_pb[gr] = bps(batch_pullback_blocks_per_sm(gr)) * sms;
    // workspace layout
    size_t o = 0;
    b->off_fft = o;  o += al256(b->ws_fft);
    b->off_r = o;    o += al256(2 * b->total * sizeof(float));
    b->off_upd = o;  o += al256(b->total * sizeof(float));
    b->off_spec = o; o += al256(2 * b->total_spec * sizeof(float2));
    b->off_ua = o;   o += al256(b->total * sizeof(float));
    b->off_ub = o;   o += al256(b->total * sizeof(float));
    b->off_lam = o;  o += al256(b->total * sizeof(float));
    b->off_part = o; o += al256((size_t)b->n_items * 4 * sizeof(double));
    b->off_xpart = o; o += al256(std::max<size_t>(1, b->n_xpart) * 2 * sizeof(double));
    b->off_cnt = o;  o += 256;
    b->total_ws = o;
    *out = b;
    return EVX_OK;
}

int evx_batch_destroy(evx_batch* b) {
    if (b) batch_free(b);
    return EVX_OK;
}

size_t evx_batch_field_floats(const evx_batch* b) { return b ? b->total : 0; }
size_t evx_batch_workspace_bytes(const evx_batch* b) { return b ? b->total_ws : 0; }
int evx_batch_work_items(const evx_batch* b) { return b ? b->n_items : 0; }

int evx_batch_offsets(const evx_batch* b, int64_t* offsets) {
    if (!b || !offsets) return fail(EVX_ERR_BAD_ARG, "NULL argument");
    for (int i = 0; i < b->n; ++i) offsets[i] = b->off[i];
    return EVX_OK;
}

size_t evx_batch_spectrum_floats(const evx_batch* b) { return b ? b->spec_floats : 0; }

int evx_batch_forward(evx_batch* b, const float* u_in, float* u_out, int nsteps, float* traj, int* nonfinite,
                      void* ws, void* stream) {
    return evx_batch_forward_spectra(b, u_in, u_out, nsteps, traj, nullptr, nonfinite, ws, stream);
}

int evx_batch_forward_spectra(evx_batch* b, const float* u_in, float* u_out, int nsteps, float* traj, float* spectra,
                              int* nonfinite, void* ws, void* stream) {
    if (!b) return fail(EVX_ERR_BAD_ARG, "batch is NULL");
    if (!u_in || !u_out || !ws) return fail(EVX_ERR_BAD_ARG, "NULL buffer");
    if (u_in == u_out) return fail(EVX_ERR_BAD_ARG, "input and output must not alias");
    if (((reinterpret_cast<uintptr_t>(u_in) | reinterpret_cast<uintptr_t>(u_out) | reinterpret_cast<uintptr_t>(traj) |
          reinterpret_cast<uintptr_t>(spectra)) & 15) || (reinterpret_cast<uintptr_t>(ws) & 255))
        return fail(EVX_ERR_BAD_ARG, "buffers must be 16-byte aligned (workspace 256-byte)");
    if (nsteps < 0) return fail(EVX_ERR_BAD_ARG, "nsteps must be >= 0");
    if (spectra && !traj) return fail(EVX_ERR_BAD_ARG, "stored spectra are kept with the trajectory only");
    const size_t T = b->total;
    if (nsteps == 0)
        return check_cuda(cudaMemcpyAsync(u_out, u_in, T * sizeof(float), cudaMemcpyDeviceToDevice, as_stream(stream)),
                          "copy");
    const GraphKey key{3, key_p(u_in), key_p(u_out), (uint64_t)nsteps, key_p(traj), key_p(spectra), key_p(nonfinite),
                       key_p(ws)};
    return b->graphs.run(key, as_stream(stream), [&](cudaStream_t st) -> int {
    int rc;
    if ((rc = bind_plans(b, ws, st))) return rc;
    const Bufs B = bufs(b, ws);
    const float* src = u_in;
    auto dspec = [&](int s) {
        return spectra ? reinterpret_cast<float2*>(spectra + (size_t)s * b->spec_floats) : nullptr;
    };
    // step 0 from the input
    if ((rc = batch_rhs_launch(false, u_in, nullptr, nullptr, B.r, b->d_inst, b->d_items, b->n_items, B.cnt,
                               b->grid_rhs, st)))
        return rc;
    if ((rc = batch_spectral(b, B.r, B.spec, B.upd, st, dspec(0)))) return rc;
    int s = 1;
    if (traj) {
        for (; s < nsteps; ++s) {
            float* dst = traj + (size_t)(s - 1) * T;
            if ((rc = fused_step(b, B, src, dst, st, dspec(s)))) return rc;
            src = dst;
        }
    } else {
        if (s < nsteps) {   // u_in -> A
            if ((rc = fused_step(b, B, src, B.ua, st))) return rc;
            src = B.ua;
            ++s;
        }
        const int chunk = (b->tune.graph_steps / 2) * 2;
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;   // inside a capture of the whole call: no chunk graph
        if ((rc = check_cuda(cudaStreamIsCapturing(st, &cs), "cudaStreamIsCapturing"))) return rc;
        if (chunk >= 2 && nsteps - s >= chunk && cs == cudaStreamCaptureStatusNone) {
            if (!b->gexec || b->gexec_ws != ws || b->gexec_steps != chunk) {
                if ((rc = capture_chunk(b, ws, chunk))) return rc;
                if ((rc = bind_plans(b, ws, st))) return rc;
            }
            while (nsteps - s >= chunk) {
                EVX_TIMED("batch_graph_chunk", st, rc = check_cuda(cudaGraphLaunch(b->gexec, st), "cudaGraphLaunch"));
                if (rc) return rc;
                count_launch((unsigned)b->gexec_launches);
                s += chunk;
            }
        }
        for (; s < nsteps; ++s) {   // remaining steps, alternating A/B
            float* dst = (src == B.ua) ? B.ub : B.ua;
            if ((rc = fused_step(b, B, src, dst, st))) return rc;
            src = dst;
        }
    }
    const size_t n4 = T / 4;
    const int blocks = (int)std::min<size_t>((n4 + 255) / 256, (size_t)152 * 16);
    EVX_TIMED("batch_axpy", st, batch_axpy_kernel<<<blocks, 256, 0, st>>>(
        src, B.upd, u_out, traj ? traj + (size_t)(nsteps - 1) * T : nullptr, n4, nonfinite));
    count_launch();
    return check_launch("batch_axpy_kernel");
    });
}

int evx_batch_adjoint(evx_batch* b, const float* states, int nsteps, const float* lam_in, float* lam_out,
                      double* grads, void* ws, void* stream) {
    return evx_batch_adjoint_spectra(b, states, nullptr, nsteps, lam_in, lam_out, grads, ws, stream);
}

int evx_batch_adjoint_spectra(evx_batch* b, const float* states, const float* spectra, int nsteps,
                              const float* lam_in, float* lam_out, double* grads, void* ws, void* stream) {
    if (!b) return fail(EVX_ERR_BAD_ARG, "batch is NULL");
    if (!lam_in || !lam_out || !ws || (!states && nsteps > 0)) return fail(EVX_ERR_BAD_ARG, "NULL buffer");
    if (lam_in == lam_out) return fail(EVX_ERR_BAD_ARG, "lam_in and lam_out must not alias");
    if (((reinterpret_cast<uintptr_t>(lam_in) | reinterpret_cast<uintptr_t>(lam_out) |
          reinterpret_cast<uintptr_t>(states) | reinterpret_cast<uintptr_t>(spectra)) & 15) ||
        (reinterpret_cast<uintptr_t>(ws) & 255))
        return fail(EVX_ERR_BAD_ARG, "buffers must be 16-byte aligned (workspace 256-byte)");
    if (nsteps < 0) return fail(EVX_ERR_BAD_ARG, "nsteps must be >= 0");
    const size_t T = b->total;
    if (nsteps == 0)
        return check_cuda(cudaMemcpyAsync(lam_out, lam_in, T * sizeof(float), cudaMemcpyDeviceToDevice,
                                          as_stream(stream)), "copy");
    const GraphKey key{4, key_p(states), key_p(spectra), (uint64_t)nsteps, key_p(lam_in), key_p(lam_out),
                       key_p(grads), key_p(ws)};
    return b->graphs.run(key, as_stream(stream), [&](cudaStream_t st) -> int {
    int rc;
    if ((rc = bind_plans(b, ws, st))) return rc;
    const Bufs B = bufs(b, ws);
    float* gbuf = B.r;
    float* hbuf = B.r + T;
    float2* spec_h = B.spec + b->total_spec;
    const bool want = grads != nullptr;
    const bool spectral = want && spectra != nullptr;   // gradient sums by Parseval against the stored spectra
    const float* lam = lam_in;
    for (int s = nsteps - 1; s >= 0; --s) {
        float* dst = (s % 2 == 0) ? lam_out : B.lam;
        if ((rc = batch_r2c(b, lam, B.spec, st))) return rc;
        if (spectral) {
            float2* ds = reinterpret_cast<float2*>(const_cast<float*>(spectra) + (size_t)s * b->spec_floats);
            if (b->any_kspace) {
                EVX_TIMED("batch_kspace_adj_spec", st,
                          batch_kspace_adj_spec_kernel<<<dim3(b->kspace_blocks, b->n), 256, 0, st>>>(
                              B.spec, ds, B.xpart, b->d_kinst, b->d_k2));
                count_launch();
                if ((rc = check_launch("batch_kspace_adj_spec_kernel"))) return rc;
            }
            if ((rc = batch_xpass(b, 3, B.spec, nullptr, st, ds, B.xpart))) return rc;
            if ((rc = batch_c2r(b, B.spec, gbuf, st))) return rc;
            const float* us = states + (size_t)s * T;
            if ((rc = batch_pullback_launch(2, us, gbuf, lam, nullptr, nullptr, dst, B.part, b->d_inst, b->d_items,
                                            b->n_items, B.cnt + 1, b->grid_pb[2], st)))
                return rc;
            EVX_TIMED("batch_grad_reduce", st, batch_grad_reduce_spec_kernel<<<b->n, 256, 0, st>>>(
                                                   B.part, B.xpart, b->d_rinst, grads));
            count_launch();
            if ((rc = check_launch("batch_grad_reduce_spec_kernel"))) return rc;
            lam = dst;
            continue;
        }
        if (b->any_kspace) {
            EVX_TIMED("batch_kspace_adj", st,
                      batch_kspace_adj_kernel<<<dim3(b->kspace_blocks, b->n), 256, 0, st>>>(
                          B.spec, want ? spec_h : nullptr, b->d_kinst, b->d_k2));
            count_launch();
            if ((rc = check_launch("batch_kspace_adj_kernel"))) return rc;
        }
        if ((rc = batch_xpass(b, want ? 2 : 1, B.spec, want ? spec_h : nullptr, st))) return rc;
        if ((rc = batch_c2r(b, B.spec, gbuf, st))) return rc;
        if (want && (rc = batch_c2r(b, spec_h, hbuf, st))) return rc;
        const float* us = states + (size_t)s * T;
        if ((rc = batch_pullback_launch(want ? 1 : 0, us, gbuf, lam, hbuf, us + T, dst, B.part, b->d_inst, b->d_items,
                                        b->n_items, B.cnt + 1, b->grid_pb[want ? 1 : 0], st)))
            return rc;
        if (want) {
            EVX_TIMED("batch_grad_reduce", st, batch_grad_reduce_kernel<<<b->n, 256, 0, st>>>(B.part, b->d_rinst, grads));
            count_launch();
            if ((rc = check_launch("batch_grad_reduce_kernel"))) return rc;
        }
        lam = dst;
    }
    return EVX_OK;
    });
}

}  // extern "C"
