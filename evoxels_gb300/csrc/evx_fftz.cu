// Real transforms along z with a y-contiguous half spectrum: the z pass of
// the (y, z) transforms of the x-pass plans.  R2C reads the real rows
// in[x][y][z] and writes spec[x][kz][y] (kz in [0, nz/2], unnormalised, cuFFT's
// values); C2R reads spec[x][kz][y] and writes out[x][y][z] (the imaginary parts
// of the kz = 0 and kz = nz/2 entries ignored, as a C2R transform does).  With
// y contiguous, the y transform is one batched contiguous 1-D C2C (cuFFT) over
// all (x, kz) columns, in place, and the x-pass sees pencils m = kz*ny + ky.
//
// A block of 256 threads owns YG = 2*(256/TZ) rows of one x plane at a time
// (persistent blocks stride over (x, row group) items).  Two real rows a, b are
// one complex row c = a + i b, transformed by the four-step FFT of evx_fft.cuh
// with TZ threads per row pair (EZ values each, exchange in shared memory
// within the warp); A(k) = (C(k) + conj C(nz-k))/2, B(k) = (C(k) - conj
// C(nz-k))/(2i) with the partner values by warp shuffles.  The row group's
// half spectrum is staged in shared memory as T[kz][y] (row pitch YG+1) and
// leaves as coalesced runs of YG values along y.  C2R mirrors it: coalesced
// runs into T, each pair gathers C(k) = A(k) + i B(k) (k <= nz/2) and
// C(nz-k) = conj A(k) + i conj B(k), one inverse FFT gives a + i b.
//
// No waits of their own: __syncthreads and __syncwarp only.
#include <algorithm>
#include <mutex>

#include "evx_ch_plan.cuh"
#include "evx_fft.cuh"

namespace evx {
namespace {

using namespace fft;

__host__ __device__ constexpr int zsplit(int n) { return n == 512 ? 32 : (n >= 16 ? 16 : n); }

template <int NZ>
struct ZT {
    static constexpr int NH = NZ / 2, NH1 = NH + 1;
    static constexpr int EZ = zsplit(NZ), TZ = NZ / EZ, QZ = EZ / TZ;
    static constexpr int PAIRS = 256 / TZ, YG = 2 * PAIRS;   // row pairs / rows per item
    static constexpr int KS = TZ + 1, PS = EZ * KS;           // padded z exchange per pair
    static constexpr int TP = YG + 2;   // staging row pitch (complex): rows a, b of a pair are one 16-byte word
    static constexpr size_t SMEM = ((size_t)PAIRS * PS + (size_t)NH1 * TP) * sizeof(float2);
    static_assert(EZ >= TZ && EZ % TZ == 0, "unsupported split");
};

// z exchange of one row pair: xi(k1, j) = base + k1*KS + j
struct ZCol {
    int base, n2, ks;
    __device__ __forceinline__ int xi(int k1, int j) const { return base + k1 * ks + j; }
};

// MINB: resident blocks the register budget is sized for; TWS: split twiddles
// (nz = 256 only); PF: the next item's rows loaded during the current transform.
template <int NZ, int MINB = 1, bool TWS = false, bool PF = true>
__global__ void __launch_bounds__(256, MINB)
zt_r2c_kernel(const float* __restrict__ in, float2* __restrict__ out, int nx, int ny, bool vec) {
    using G = ZT<NZ>;
    static_assert(!TWS || (G::EZ == 16 && G::TZ == 16), "split twiddles are for 16 x 16 columns");
    constexpr int EZ = G::EZ, TZ = G::TZ, QZ = G::QZ, NH = G::NH, NH1 = G::NH1, YG = G::YG, TP = G::TP;
    extern __shared__ __align__(16) float2 sm[];
    float2* Z = sm;                              // [PAIRS][EZ][KS]
    float2* T = sm + G::PAIRS * G::PS;           // [NH1][TP]
    const int tid = threadIdx.x;
    const int t = tid % TZ, g = tid / TZ;
    const ZCol zc{g * G::PS, t, G::KS};
    float2 tw[TWS ? 1 : EZ];                     // this thread's stage twiddles
    Tw16<false> tws;
    if constexpr (TWS) tws.init(t);
    else fwd_twiddles<EZ, TZ>(tw, t);
    const int groups = (ny + YG - 1) / YG;
    const long items = (long)nx * groups;
    // the item's two rows, loaded one item ahead (in flight during the previous item's transform)
    auto load_rows = [&](long it, float2 (&w)[EZ]) {
        const int x = (int)(it / groups), y0 = (int)(it - (long)x * groups) * YG;
        const float* plane = in + (size_t)x * ny * NZ;
        const int ya = y0 + 2 * g, yb = ya + 1;
        const bool la = ya < ny, lb = yb < ny;
#pragma unroll
        for (int e = 0; e < EZ; ++e) {
            const int z = TZ * e + t;
            w[e] = make_float2(la ? __ldg(plane + (size_t)ya * NZ + z) : 0.f, lb ? __ldg(plane + (size_t)yb * NZ + z) : 0.f);
        }
    };
    float2 vn[PF ? EZ : 1];
    if constexpr (PF) {
        if (blockIdx.x < items) load_rows(blockIdx.x, vn);
    }
    for (long it = blockIdx.x; it < items; it += gridDim.x) {
        const int x = (int)(it / groups), y0 = (int)(it - (long)x * groups) * YG;
        float2 v[EZ];
        if constexpr (PF) {
#pragma unroll
            for (int e = 0; e < EZ; ++e) v[e] = vn[e];
            if (it + gridDim.x < items) load_rows(it + gridDim.x, vn);
        } else {
            load_rows(it, v);
        }
        if constexpr (TWS) fwd_stage1_tw16<true>(v, Z, zc, tws);
        else fwd_stage1_tw<EZ, TZ, true>(v, Z, zc, tw);   // a pair's TZ threads share a warp
        fwd_stage2<EZ, TZ>(v);
        // v[q*TZ + k2] = C(k1 + EZ*k2), k1 = t*QZ + q.  Partner C(NZ - k): for
        // k1 != 0 it is k1' = EZ - k1, k2' = TZ-1-k2 (lane TZ-t for q = 0, TZ-1-t
        // otherwise); for k1 = 0 (t = 0, q = 0) it is k2' = (TZ - k2) % TZ, own.
#pragma unroll
        for (int q = 0; q < QZ; ++q) {
            const int k1 = t * QZ + q;
            const int qs = q == 0 ? 0 : QZ - q;
            const int src = q == 0 ? (TZ - t) % TZ : TZ - 1 - t;
#pragma unroll
            for (int k2 = 0; k2 <= TZ / 2; ++k2) {
                const float2 pv = v[qs * TZ + (TZ - 1 - k2)];
                float2 cp;
                cp.x = __shfl_sync(0xffffffffu, pv.x, src, TZ);
                cp.y = __shfl_sync(0xffffffffu, pv.y, src, TZ);
                if (k1 == 0) cp = v[(TZ - k2) % TZ];
                const float2 c = v[q * TZ + k2];
                const int kz = k1 + EZ * k2;
                if (kz > NH || (k2 == TZ / 2 && k1 != 0)) continue;
                // A = (C + conj Cp)/2, B = (C - conj Cp)/(2i): rows a, b of the pair in one store
                *reinterpret_cast<float4*>(T + kz * TP + 2 * g) =
                    make_float4(0.5f * (c.x + cp.x), 0.5f * (c.y - cp.y), 0.5f * (c.y + cp.y), -0.5f * (c.x - cp.x));
            }
        }
        __syncthreads();   // T complete
        const int rows = min(YG, ny - y0);
        float2* orow = out + (size_t)x * NH1 * ny + y0;
        // two y values per thread and store (vec: even ny, 16-byte aligned output)
        for (int e = tid; e < NH1 * (YG / 2); e += 256) {
            const int kz = e / (YG / 2), yl = 2 * (e - kz * (YG / 2));
            const float4 w = *reinterpret_cast<const float4*>(T + kz * TP + yl);
            float2* o = orow + (size_t)kz * ny + yl;
            if (vec && yl + 1 < rows) {
                *reinterpret_cast<float4*>(o) = w;
            } else {
                if (yl < rows) o[0] = make_float2(w.x, w.y);
                if (yl + 1 < rows) o[1] = make_float2(w.z, w.w);
            }
        }
        __syncthreads();   // T and Z are rewritten by the next item
    }
}

// 16-byte asynchronous global -> shared copy (zero-filled when !full) and its groups.
__device__ __forceinline__ void cp_async16(float2* dst, const float2* src, bool full) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(dst));
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(s), "l"(src), "r"(full ? 16 : 0) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prev() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// DB: the staging area T is double-buffered and, on the vectorised path, the
// next item's spectrum runs are copied into the idle buffer by cp.async while
// the current item is transformed (the R2C's one-item-ahead prefetch, without
// the registers); otherwise the thread's staging loads go through registers.
template <int NZ, bool DB = false>
__global__ void __launch_bounds__(256)
zt_c2r_kernel(const float2* __restrict__ in, float* __restrict__ out, int nx, int ny, bool vec) {
    using G = ZT<NZ>;
    constexpr int EZ = G::EZ, TZ = G::TZ, QZ = G::QZ, NH = G::NH, NH1 = G::NH1, YG = G::YG, TP = G::TP;
    extern __shared__ __align__(16) float2 sm[];
    float2* Z = sm;
    float2* T = sm + G::PAIRS * G::PS;           // [DB ? 2 : 1][NH1][TP]
    const int tid = threadIdx.x;
    const int t = tid % TZ, g = tid / TZ;
    const ZCol zc{g * G::PS, t, G::KS};
    float2 tw[EZ];                               // this thread's stage twiddles
    inv_twiddles<EZ, TZ>(tw, t);
    const int groups = (ny + YG - 1) / YG;
    const long items = (long)nx * groups;
    constexpr int HY = YG / 2, NST = NH1 * HY, PER = (NST + 255) / 256;
    const bool db = DB && vec;
    // queue the copies of item it2's half spectrum (two y values per copy) into Tb
    auto issue = [&](long it2, float2* Tb) {
        const int x2 = (int)(it2 / groups), y2 = (int)(it2 - (long)x2 * groups) * YG;
        const int rows2 = min(YG, ny - y2);
        const float2* irow2 = in + (size_t)x2 * NH1 * ny + y2;
#pragma unroll
        for (int p = 0; p < PER; ++p) {
            const int e = tid + 256 * p;
            if (e < NST) {
                const int kz = e / HY, yl = 2 * (e - kz * HY);
                const bool full = yl < rows2;    // vec: rows2 is even, so yl + 1 < rows2 too
                cp_async16(Tb + kz * TP + yl, full ? irow2 + (size_t)kz * ny + yl : irow2, full);
            }
        }
        cp_async_commit();
    };
    if (db && blockIdx.x < items) issue(blockIdx.x, T);
    int buf = 0;
    for (long it = blockIdx.x; it < items; it += gridDim.x, buf ^= 1) {
        const int x = (int)(it / groups), y0 = (int)(it - (long)x * groups) * YG;
        const int rows = min(YG, ny - y0);
        const float2* irow = in + (size_t)x * NH1 * ny + y0;
        const float2* Tc = T;
        if (db) {
            // the idle buffer was last read before the previous item's closing barrier
            Tc = T + buf * (NH1 * TP);
            if (it + gridDim.x < items) issue(it + gridDim.x, T + (buf ^ 1) * (NH1 * TP));
            else cp_async_commit();              // empty group: the wait below stays uniform
            cp_async_wait_prev();                // this item's copies have landed
        } else {
            // all of the thread's loads in flight at once (two y values each; vec: even ny,
            // 16-byte aligned input), then into T
            float4 w[PER];
#pragma unroll
            for (int p = 0; p < PER; ++p) {
                const int e = tid + 256 * p, kz = e / HY, yl = 2 * (e - kz * HY);
                const float2* src = irow + (size_t)kz * ny + yl;
                float4 v4 = make_float4(0.f, 0.f, 0.f, 0.f);
                if (e < NH1 * HY) {
                    if (vec && yl + 1 < rows) {
                        v4 = __ldg(reinterpret_cast<const float4*>(src));
                    } else {
                        if (yl < rows) { const float2 q = __ldg(src); v4.x = q.x; v4.y = q.y; }
                        if (yl + 1 < rows) { const float2 q = __ldg(src + 1); v4.z = q.x; v4.w = q.y; }
                    }
                }
                w[p] = v4;
            }
#pragma unroll
            for (int p = 0; p < PER; ++p) {
                const int e = tid + 256 * p;
                if (e < NH1 * HY) *reinterpret_cast<float4*>(T + (e / HY) * TP + 2 * (e % HY)) = w[p];
            }
        }
        __syncthreads();
        const int a = 2 * g, b = a + 1;
        float2 v[EZ];
#pragma unroll
        for (int q = 0; q < QZ; ++q)
#pragma unroll
            for (int k2 = 0; k2 < TZ; ++k2) {
                const int k = t * QZ + q + EZ * k2;
                const int kk = k <= NH ? k : NZ - k;
                const float4 AB = *reinterpret_cast<const float4*>(Tc + kk * TP + a);  // (A, B) of the pair
                float2 c;
                if (k == 0 || k == NH) c = make_float2(AB.x, AB.z);                    // real parts only
                else if (k < NH) c = make_float2(AB.x - AB.w, AB.y + AB.z);            // A + iB
                else c = make_float2(AB.x + AB.w, AB.z - AB.y);                        // conj A + i conj B
                v[q * TZ + k2] = c;
            }
        inv_stage2_tw<EZ, TZ>(v, Z, zc, tw);
        inv_stage1<EZ, TZ, true>(v, Z, zc);      // a pair's TZ threads share a warp
        float* plane = out + (size_t)x * ny * NZ;
        const int ya = y0 + a, yb = ya + 1;
        if (ya < ny) {
#pragma unroll
            for (int e = 0; e < EZ; ++e) plane[(size_t)ya * NZ + TZ * e + t] = v[e].x;
        }
        if (yb < ny) {
#pragma unroll
            for (int e = 0; e < EZ; ++e) plane[(size_t)yb * NZ + TZ * e + t] = v[e].y;
        }
        __syncthreads();   // T is rewritten by the next item
    }
}

constexpr int MAX_DEVICES = 64;
int g_tw_rc[MAX_DEVICES];
std::once_flag g_tw_once[MAX_DEVICES];

int zt_init() {
    int dev = 0;
    int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= MAX_DEVICES) return fail(EVX_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::call_once(g_tw_once[dev], [dev] { g_tw_rc[dev] = check_cuda(upload_w512(), "twiddle table upload"); });
    return g_tw_rc[dev];
}

template <class K>
int zt_grid(K kern, size_t smem, long items, int* grid) {
    int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "z transform shared memory attribute");
    if (rc) return rc;
    int dev = 0, sms = 0, per = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if ((rc = check_cuda(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kern, 256, smem), "z transform occupancy")))
        return rc;
    *grid = (int)std::max<long>(1, std::min<long>(items, (long)std::max(1, sms) * std::max(1, per)));
    return EVX_OK;
}

template <class K>
int zt_go(K kern, bool fwd, long items, int nx, int ny, const void* in, void* out, size_t smem, cudaStream_t st) {
    int grid = 0, rc;
    if ((rc = zt_grid(kern, smem, items, &grid))) return rc;
    const bool vec = (ny % 2) == 0 && (reinterpret_cast<uintptr_t>(fwd ? out : in) & 15) == 0;
    if (fwd) {
        EVX_TIMED("fft_z_r2c", st, reinterpret_cast<void (*)(const float*, float2*, int, int, bool)>(kern)<<<grid, 256, smem, st>>>(
                                       static_cast<const float*>(in), static_cast<float2*>(out), nx, ny, vec));
    } else {
        EVX_TIMED("fft_z_c2r", st, reinterpret_cast<void (*)(const float2*, float*, int, int, bool)>(kern)<<<grid, 256, smem, st>>>(
                                       static_cast<const float2*>(in), static_cast<float*>(out), nx, ny, vec));
    }
    count_launch();
    return check_launch(fwd ? "zt_r2c_kernel" : "zt_c2r_kernel");
}

// R2C for nz = 256: at most 128 registers (2 blocks per SM; 143 unbounded,
// which left one block per SM) with the split twiddles that make room for the
// next item's rows: 36 -> 31 us at 256^3.  The C2R is not register-limited.
template <int NZ>
int zt_launch_t(bool fwd, int nx, int ny, const void* in, void* out, cudaStream_t st) {
    using G = ZT<NZ>;
    const long items = (long)nx * ((ny + G::YG - 1) / G::YG);
    if (fwd) {
        constexpr bool S = NZ == 256;
        return zt_go(zt_r2c_kernel<NZ, S ? 2 : 1, S, true>, true, items, nx, ny, in, out, G::SMEM, st);
    }
    // C2R for nz = 256: double-buffered staging (2 x 34 KB more shared memory, still 2 blocks per SM)
    if constexpr (NZ == 256)
        return zt_go(zt_c2r_kernel<NZ, true>, false, items, nx, ny, in, out,
                     G::SMEM + (size_t)G::NH1 * G::TP * sizeof(float2), st);
    else
        return zt_go(zt_c2r_kernel<NZ>, false, items, nx, ny, in, out, G::SMEM, st);
}

int zt_launch(bool fwd, int nx, int ny, int nz, const void* in, void* out, cudaStream_t st) {
    int rc = zt_init();
    if (rc) return rc;
    switch (nz) {
        case 32: return zt_launch_t<32>(fwd, nx, ny, in, out, st);
        case 64: return zt_launch_t<64>(fwd, nx, ny, in, out, st);
        case 128: return zt_launch_t<128>(fwd, nx, ny, in, out, st);
        case 256: return zt_launch_t<256>(fwd, nx, ny, in, out, st);
        default: return fail(EVX_ERR_UNSUPPORTED, "z transform: nz = %d", nz);
    }
}

}  // namespace

bool zt_supported(int nz) { return nz == 32 || nz == 64 || nz == 128 || nz == 256; }

int fft_zt_r2c(int nx, int ny, int nz, const float* in, float2* out, cudaStream_t st) {
    return zt_launch(true, nx, ny, nz, in, out, st);
}

int fft_zt_c2r(int nx, int ny, int nz, const float2* in, float* out, cudaStream_t st) {
    return zt_launch(false, nx, ny, nz, in, out, st);
}

}  // namespace evx

using namespace evx;

extern "C" {

int evx_fft_z_r2c(const float* in, float* out, int nx, int ny, int nz, void* stream) {
    if (!in || !out) return fail(EVX_ERR_BAD_ARG, "NULL pointer");
    if (nx < 1 || ny < 1) return fail(EVX_ERR_BAD_SHAPE, "nx and ny must be >= 1");
    if (reinterpret_cast<uintptr_t>(out) & 7) return fail(EVX_ERR_BAD_ARG, "out must be 8-byte aligned");
    return fft_zt_r2c(nx, ny, nz, in, reinterpret_cast<float2*>(out), as_stream(stream));
}

int evx_fft_z_c2r(const float* in, float* out, int nx, int ny, int nz, void* stream) {
    if (!in || !out) return fail(EVX_ERR_BAD_ARG, "NULL pointer");
    if (nx < 1 || ny < 1) return fail(EVX_ERR_BAD_SHAPE, "nx and ny must be >= 1");
    if (reinterpret_cast<uintptr_t>(in) & 7) return fail(EVX_ERR_BAD_ARG, "in must be 8-byte aligned");
    return fft_zt_c2r(nx, ny, nz, reinterpret_cast<const float2*>(in), out, as_stream(stream));
}

}  // extern "C"
