// Mean-squared-error loss between a final state and a target field, and its
// gradient: loss = mean((u - t)^2), lam = 2*(u - t)/n.  This seeds the adjoint
// of an inversion (the loss the reference's parameter-estimation workflow
// minimises between simulated and observed fields, evoxels/inversion.py:105-124).
// Per-block partial sums go to caller scratch and one block reduces them in a
// fixed order, so the loss is deterministic.  Also the frame check of the
// solver loop: a NaN flag over a field, computed on the device so that the
// frame's host copy needs no extra pass (evoxels/solvers.py:163-165).
#include <algorithm>

#include "evx_common.cuh"
#include "evx_prof.cuh"

namespace evx {
namespace {

constexpr int MSE_THREADS = 256;
constexpr int MSE_MAX_BLOCKS = 152 * 8;

__global__ void __launch_bounds__(MSE_THREADS)
mse_grad_kernel(const float* __restrict__ u, const float* __restrict__ t, size_t n, float scale,
                float* __restrict__ lam, double* __restrict__ part) {
    __shared__ double red[MSE_THREADS / 32];
    // per-thread float partial sums (a few dozen terms each), double across threads
    float accf = 0.f;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    size_t tail0 = 0;
    // 16-byte accesses where every array allows them, the last n % 4 elements one by one
    if (((reinterpret_cast<uintptr_t>(u) | reinterpret_cast<uintptr_t>(t) | reinterpret_cast<uintptr_t>(lam)) & 15) == 0) {
        const size_t n4 = n / 4;
        for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n4; e += stride) {
            const float4 a = __ldg(reinterpret_cast<const float4*>(u) + e), b = __ldg(reinterpret_cast<const float4*>(t) + e);
            const float4 d = make_float4(a.x - b.x, a.y - b.y, a.z - b.z, a.w - b.w);
            if (lam) reinterpret_cast<float4*>(lam)[e] = make_float4(scale * d.x, scale * d.y, scale * d.z, scale * d.w);
            accf = fmaf(d.x, d.x, accf);
            accf = fmaf(d.y, d.y, accf);
            accf = fmaf(d.z, d.z, accf);
            accf = fmaf(d.w, d.w, accf);
        }
        tail0 = n4 * 4;
    }
    for (size_t e = tail0 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
        const float d = __ldg(u + e) - __ldg(t + e);
        if (lam) lam[e] = scale * d;
        accf = fmaf(d, d, accf);
    }
    double acc = accf;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < MSE_THREADS / 32; ++w) s += red[w];
        part[blockIdx.x] = s;
    }
}

__global__ void mse_reduce_kernel(const double* __restrict__ part, int nblk, double inv_n, double* __restrict__ loss) {
    __shared__ double s[256];
    double a = 0.0;
    for (int b = threadIdx.x; b < nblk; b += 256) a += part[b];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) *loss = s[0] * inv_n;
}

// *flag = 1 if any x[i] is NaN (the caller zeroes it); float4 loads when aligned.
__global__ void nan_flag_kernel(const float* __restrict__ x, size_t n, int* __restrict__ flag) {
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    bool bad = false;
    size_t tail0 = 0;
    if ((reinterpret_cast<uintptr_t>(x) & 15) == 0) {
        const float4* x4 = reinterpret_cast<const float4*>(x);
        const size_t n4 = n / 4;
        for (size_t e = (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n4; e += stride) {
            const float4 v = __ldg(x4 + e);
            bad |= isnan(v.x) || isnan(v.y) || isnan(v.z) || isnan(v.w);
        }
        tail0 = n4 * 4;
    }
    for (size_t e = tail0 + (size_t)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) bad |= isnan(__ldg(x + e));
    if (__any_sync(0xffffffffu, bad) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

int mse_blocks(size_t n) {
    return (int)std::max<size_t>(1, std::min<size_t>((n + MSE_THREADS - 1) / MSE_THREADS, MSE_MAX_BLOCKS));
}

}  // namespace
}  // namespace evx

using namespace evx;

extern "C" {

size_t evx_mse_scratch_bytes(size_t n) { return (size_t)mse_blocks(n) * sizeof(double); }

int evx_mse_grad(const float* u, const float* target, size_t n, float* lam, double* loss, void* scratch,
                 size_t scratch_bytes, void* stream) {
    if (!u || !target || !loss) return fail(EVX_ERR_BAD_ARG, "NULL pointer");
    if (n == 0) return fail(EVX_ERR_BAD_SHAPE, "empty field");
    const int nb = mse_blocks(n);
    if (!scratch || scratch_bytes < (size_t)nb * sizeof(double))
        return fail(EVX_ERR_WORKSPACE, "scratch needs %zu bytes", (size_t)nb * sizeof(double));
    cudaStream_t st = as_stream(stream);
    double* part = static_cast<double*>(scratch);
    const float scale = (float)(2.0 / (double)n);
    EVX_TIMED("mse_grad", st, mse_grad_kernel<<<nb, MSE_THREADS, 0, st>>>(u, target, n, scale, lam, part));
    EVX_TIMED("mse_reduce", st, mse_reduce_kernel<<<1, 256, 0, st>>>(part, nb, 1.0 / (double)n, loss));
    count_launch(2);
    return check_launch("evx_mse_grad");
}

int evx_nan_flag(const float* x, size_t n, int* flag, void* stream) {
    if (!flag || (n && !x)) return fail(EVX_ERR_BAD_ARG, "NULL pointer");
    cudaStream_t st = as_stream(stream);
    int rc = check_cuda(cudaMemsetAsync(flag, 0, sizeof(int), st), "evx_nan_flag reset");
    if (rc || n == 0) return rc;
    const int nb = (int)std::max<size_t>(1, std::min<size_t>((n / 4 + MSE_THREADS - 1) / MSE_THREADS, 152 * 8));
    EVX_TIMED("nan_flag", st, nan_flag_kernel<<<nb, MSE_THREADS, 0, st>>>(x, n, flag));
    count_launch();
    return check_launch("nan_flag_kernel");
}

}  // extern "C"
