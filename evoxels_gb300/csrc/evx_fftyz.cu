// Fused 2-D (y, z) real-to-complex and complex-to-real transforms of every x
// plane of a field: one read and one write per transform where cuFFT's
// batched 2-D plans make two passes (a z kernel and a y kernel).  Output and
// input use cuFFT's layout and scaling: spec[x][ky][kz], kz in [0, nz/2],
// unnormalised.
//
// A thread-block cluster of CS CTAs owns one x plane at a time (persistent
// clusters stride over x).  Each CTA keeps KC = (nz/2)/CS columns of the
// plane's half spectrum for all ny rows in shared memory, S[y][kz - rank*KC].
// The kz = 0 and kz = nz/2 columns of a real row are real, so both share the
// column slot kz = 0 as (re, im) = (Z0, Znyq); that makes nz/2 columns, an
// even split.
//
// R2C, per plane:
//   z stage  each CTA transforms ny/CS rows, two real rows a, b packed as one
//            complex row c = a + i b (four-step FFT of evx_fft.cuh, TZ threads
//            per row pair); A(k) = (C(k) + conj C(nz-k))/2, B(k) = (C(k) -
//            conj C(nz-k))/(2i), the partner values by warp shuffles.  Each
//            value goes to the S of the CTA owning its column (distributed
//            shared memory), so the transpose between the stages costs no HBM.
//   cluster barrier
//   y stage  each CTA transforms its KC columns along y in place in S and
//            writes rows of spec; the packed column is split again,
//            Z0(ky) = (P(ky) + conj P(-ky))/2, Znyq(ky) = (P(ky) - conj P(-ky))/(2i).
//   cluster barrier (S is rewritten by the next plane)
// C2R mirrors it: y stage on the CTA's columns (the packed column loaded as
// Z0 + i Znyq, whose inverse transforms are both real), cluster barrier, z
// stage per row pair gathering its half spectrum from all CTAs of the cluster
// and the Hermitian extension, C(k) = A(k) + i B(k), C(nz-k) = conj A(k) +
// i conj B(k), one complex inverse FFT giving a + i b.
//
// No waits of its own: the only synchronisation is __syncthreads and the
// cluster barrier, reached by every thread of every CTA the same number of
// times (the plane loop depends on the cluster index only).  A cluster barrier
// at entry makes sure every CTA of the cluster runs before any distributed
// shared memory access, and the last one of each plane that no CTA leaves
// while another may still access its shared memory.
#include <cooperative_groups.h>

#include <algorithm>
#include <cstdlib>
#include <mutex>

#include "evx_ch_plan.cuh"
#include "evx_fft.cuh"

namespace cg = cooperative_groups;

namespace evx {
namespace {

using namespace fft;

// (N1, N2) four-step split of a transform length
__host__ __device__ constexpr int split_n1(int n) { return n == 512 ? 32 : (n >= 16 ? 16 : n); }

template <int NY, int NZ, int CS>
struct YZ {
    static constexpr int NH = NZ / 2;            // column slots (kz = 0 packs kz = nz/2)
    static constexpr int NH1 = NZ / 2 + 1;       // row length of the spectrum
    static constexpr int KC = NH / CS;           // columns per CTA
    static constexpr int RY = NY / CS;           // rows per CTA in the z stage
    static constexpr int PAIRS = RY / 2;
    // z stage: EZ x TZ, TZ threads per row pair, GZ pairs per round
    static constexpr int EZ = split_n1(NZ), TZ = NZ / EZ, GZ = 256 / TZ;
    static constexpr int ZROUNDS = (PAIRS + GZ - 1) / GZ;
    static constexpr int KS = TZ + 1;            // padded k1 row of the z exchange
    static constexpr int PS = EZ * KS;           // per-pair exchange block
    // y stage: PY columns per round, N2Y threads per column
    static constexpr int PYT = 256 / (NY / split_n1(NY));
    static constexpr int PY = PYT < KC ? PYT : KC;
    static constexpr int N2Y = 256 / PY, N1Y = NY / N2Y;
    static constexpr int YROUNDS = KC / PY;
    static constexpr size_t SMEM = ((size_t)NY * KC + (size_t)GZ * PS) * sizeof(float2);
    static_assert(NH % CS == 0 && RY % 2 == 0 && KC % PY == 0, "unsupported split");
    static_assert(N1Y >= N2Y && N1Y % N2Y == 0 && EZ >= TZ, "unsupported split");
};

// Cluster barrier without release/acquire: for the end of a plane, where the
// only hazard is the next plane's distributed writes overtaking reads that have
// already returned (no wait for this thread's global stores to land).
__device__ __forceinline__ void cluster_sync_relaxed() {
    asm volatile("barrier.cluster.arrive.relaxed.aligned;\n\tbarrier.cluster.wait.aligned;" ::: "memory");
}

// z-stage column: the exchange block of one row pair, xi(k1, j) = base + k1*KS + j
struct ZCol {
    int base, n2, ks;
    __device__ __forceinline__ int xi(int k1, int j) const { return base + k1 * ks + j; }
};

template <int NY, int NZ, int CS>
__global__ void __cluster_dims__(CS, 1, 1) __launch_bounds__(256, 2)
yz_r2c_kernel(const float* __restrict__ in, float2* __restrict__ out, int nx) {
    using G = YZ<NY, NZ, CS>;
    constexpr int EZ = G::EZ, TZ = G::TZ, KC = G::KC, NH = G::NH, NH1 = G::NH1;
    constexpr int QZ = EZ / TZ;
    extern __shared__ __align__(16) float2 sm[];
    float2* S = sm;                          // [NY][KC]
    float2* Z = sm + NY * KC;                // z exchange [GZ][EZ][KS]; packed-column scratch
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int cid = blockIdx.x / CS, ncl = gridDim.x / CS;
    const int tid = threadIdx.x;
    static_assert(KC % EZ == 0, "column owner must follow from k2");
    float2* Sr[CS];                          // every CTA's S, mapped once
#pragma unroll
    for (int r = 0; r < CS; ++r) Sr[r] = cl.map_shared_rank(S, r);
    cl.sync();

    for (int x = cid; x < nx; x += ncl) {
        const float* plane = in + (size_t)x * NY * NZ;
        if (tid == 0 && x + ncl < nx) {      // next plane's rows of this CTA into L2
            const float* nxt = plane + (size_t)ncl * NY * NZ + (size_t)rank * G::RY * NZ;
            asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(nxt), "r"((unsigned)(G::RY * NZ * 4))
                         : "memory");
        }
        // ---- z stage: row pairs of this CTA's rows
        const int t = tid % TZ, g = tid / TZ;
        const ZCol zc{g * G::PS, t, G::KS};
        float2 twz[EZ];                      // z-stage twiddles of this thread (lanes differ in t)
        fwd_twiddles<EZ, TZ>(twz, t);
#pragma unroll 1
        for (int rnd = 0; rnd < G::ZROUNDS; ++rnd) {
            const int pair = rnd * G::GZ + g;
            const bool live = pair < G::PAIRS;
            const int ya = rank * G::RY + 2 * (live ? pair : 0), yb = ya + 1;
            float2 v[EZ];
#pragma unroll
            for (int e = 0; e < EZ; ++e) {
                const int z = TZ * e + t;
                v[e] = live ? make_float2(__ldg(plane + ya * NZ + z), __ldg(plane + yb * NZ + z)) : make_float2(0.f, 0.f);
            }
            fwd_stage1_tw<EZ, TZ, true>(v, Z, zc, twz);   // a row pair's TZ threads share a warp
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
                    if (!live || kz > NH || (k2 == TZ / 2 && k1 != 0)) continue;
                    // A = (C + conj Cp)/2, B = (C - conj Cp)/(2i)
                    const float2 A = make_float2(0.5f * (c.x + cp.x), 0.5f * (c.y - cp.y));
                    const float2 B = make_float2(0.5f * (c.y + cp.y), -0.5f * (c.x - cp.x));
                    if (kz == NH) {          // Nyquist: imaginary half of slot 0 (rank 0)
                        Sr[0][ya * KC].y = A.x;
                        Sr[0][yb * KC].y = B.x;
                    } else if (kz == 0) {
                        Sr[0][ya * KC].x = A.x;
                        Sr[0][yb * KC].x = B.x;
                    } else {
                        // owner (EZ*k2)/KC is a compile-time index (k1 < EZ, KC a multiple of EZ)
                        float2* so = Sr[(EZ * k2) / KC < CS ? (EZ * k2) / KC : CS - 1];
                        so[ya * KC + kz % KC] = A;
                        so[yb * KC + kz % KC] = B;
                    }
                }
            }
            __syncwarp();                    // the group's Z block is rewritten by the next round
        }
        cl.sync();
        // ---- y stage: this CTA's columns, in place in S
        constexpr int PY = G::PY, N1Y = G::N1Y, N2Y = G::N2Y, QY = N1Y / N2Y;
        const int p = tid % PY, n2 = tid / PY;
#pragma unroll 1
        for (int ry = 0; ry < G::YROUNDS; ++ry) {
            const int col = ry * PY + p;
            const int kz = rank * KC + col;
            const Col<N1Y, N2Y> c{col, n2, KC};
            float2 v[N1Y];
#pragma unroll
            for (int n1 = 0; n1 < N1Y; ++n1) v[n1] = S[(N2Y * n1 + n2) * KC + col];
            fwd_stage1<N1Y, N2Y>(v, S, c);
            fwd_stage2<N1Y, N2Y>(v);
            float2* orow = out + (size_t)x * NY * NH1;
            if (rank == 0 && ry == 0) {      // uniform in the CTA: split the packed column
                __syncthreads();
                if (p == 0) {
#pragma unroll
                    for (int q = 0; q < QY; ++q)
#pragma unroll
                        for (int k2 = 0; k2 < N2Y; ++k2) Z[(n2 * QY + q) + N1Y * k2] = v[q * N2Y + k2];
                }
                __syncthreads();
            }
#pragma unroll
            for (int q = 0; q < QY; ++q)
#pragma unroll
                for (int k2 = 0; k2 < N2Y; ++k2) {
                    const int ky = n2 * QY + q + N1Y * k2;
                    const float2 c = v[q * N2Y + k2];
                    if (kz == 0) {
                        const float2 cp = Z[(NY - ky) % NY];
                        orow[(size_t)ky * NH1] = make_float2(0.5f * (c.x + cp.x), 0.5f * (c.y - cp.y));
                        orow[(size_t)ky * NH1 + NH] = make_float2(0.5f * (c.y + cp.y), -0.5f * (c.x - cp.x));
                    } else {
                        orow[(size_t)ky * NH1 + kz] = c;
                    }
                }
        }
        cluster_sync_relaxed();
    }
}

template <int NY, int NZ, int CS>
__global__ void __cluster_dims__(CS, 1, 1) __launch_bounds__(256, 2)
yz_c2r_kernel(const float2* __restrict__ in, float* __restrict__ out, int nx) {
    using G = YZ<NY, NZ, CS>;
    constexpr int EZ = G::EZ, TZ = G::TZ, KC = G::KC, NH = G::NH, NH1 = G::NH1;
    constexpr int QZ = EZ / TZ;
    extern __shared__ __align__(16) float2 sm[];
    float2* S = sm;                          // [NY][KC]
    float2* Z = sm + NY * KC;                // z exchange [GZ][EZ][KS]
    cg::cluster_group cl = cg::this_cluster();
    const int rank = (int)cl.block_rank();
    const int cid = blockIdx.x / CS, ncl = gridDim.x / CS;
    const int tid = threadIdx.x;
    cl.sync();

    for (int x = cid; x < nx; x += ncl) {
        const float2* irow = in + (size_t)x * NY * NH1;
        // ---- y stage (inverse): this CTA's columns into S, natural row order
        constexpr int PY = G::PY, N1Y = G::N1Y, N2Y = G::N2Y, QY = N1Y / N2Y;
        const int p = tid % PY, n2 = tid / PY;
#pragma unroll 1
        for (int ry = 0; ry < G::YROUNDS; ++ry) {
            const int col = ry * PY + p;
            const int kz = rank * KC + col;
            const Col<N1Y, N2Y> c{col, n2, KC};
            float2 v[N1Y];
#pragma unroll
            for (int q = 0; q < QY; ++q)
#pragma unroll
                for (int k2 = 0; k2 < N2Y; ++k2) {
                    const int ky = n2 * QY + q + N1Y * k2;
                    if (kz == 0) {           // Z0 + i Znyq
                        const float2 a = irow[(size_t)ky * NH1], b = irow[(size_t)ky * NH1 + NH];
                        v[q * N2Y + k2] = make_float2(a.x - b.y, a.y + b.x);
                    } else {
                        v[q * N2Y + k2] = irow[(size_t)ky * NH1 + kz];
                    }
                }
            inv_stage2<N1Y, N2Y>(v, S, c);
            inv_stage1<N1Y, N2Y>(v, S, c);
#pragma unroll
            for (int n1 = 0; n1 < N1Y; ++n1) S[(N2Y * n1 + n2) * KC + col] = v[n1];
        }
        cl.sync();
        // ---- z stage (inverse): row pairs of this CTA's rows
        float* plane = out + (size_t)x * NY * NZ;
        const int t = tid % TZ, g = tid / TZ;
        const ZCol zc{g * G::PS, t, G::KS};
        float2 twz[EZ];                      // z-stage twiddles of this thread (lanes differ in t)
        inv_twiddles<EZ, TZ>(twz, t);
        const float2* s0 = cl.map_shared_rank(S, 0);
#pragma unroll 1
        for (int rnd = 0; rnd < G::ZROUNDS; ++rnd) {
            const int pair = rnd * G::GZ + g;
            const bool live = pair < G::PAIRS;
            const int ya = rank * G::RY + 2 * (live ? pair : 0), yb = ya + 1;
            float2 v[EZ];
#pragma unroll
            for (int q = 0; q < QZ; ++q)
#pragma unroll
                for (int k2 = 0; k2 < TZ; ++k2) {
                    const int k = t * QZ + q + EZ * k2;
                    float2 c;
                    if (k == 0 || k == NH) {
                        const float2 pa = s0[ya * KC], pb = s0[yb * KC];
                        c = k == 0 ? make_float2(pa.x, pb.x) : make_float2(pa.y, pb.y);
                    } else if (k < NH) {
                        const float2* so = cl.map_shared_rank(S, k / KC);
                        const float2 A = so[ya * KC + k % KC], B = so[yb * KC + k % KC];
                        c = make_float2(A.x - B.y, A.y + B.x);
                    } else {
                        const int kk = NZ - k;
                        const float2* so = cl.map_shared_rank(S, kk / KC);
                        const float2 A = so[ya * KC + kk % KC], B = so[yb * KC + kk % KC];
                        c = make_float2(A.x + B.y, B.x - A.y);
                    }
                    v[q * TZ + k2] = c;
                }
            inv_stage2_tw<EZ, TZ>(v, Z, zc, twz);
            inv_stage1<EZ, TZ, true>(v, Z, zc);   // a row pair's TZ threads share a warp
            if (live) {
#pragma unroll
                for (int e = 0; e < EZ; ++e) {
                    plane[ya * NZ + TZ * e + t] = v[e].x;
                    plane[yb * NZ + TZ * e + t] = v[e].y;
                }
            }
            __syncwarp();                    // the group's Z block is rewritten by the next round
        }
        cluster_sync_relaxed();
    }
}

// ---- host side -------------------------------------------------------------------
constexpr int MAX_DEVICES = 64;
int g_tw_rc[MAX_DEVICES];
std::once_flag g_tw_once[MAX_DEVICES];

bool yz_env_off() {   // EVX_FFT_YZ=0: keep cuFFT's (y, z) plans everywhere
    static const bool off = [] {
        const char* e = std::getenv("EVX_FFT_YZ");
        return e && e[0] == '0';
    }();
    return off;
}

int yz_init() {
    int dev = 0;
    int rc = check_cuda(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc) return rc;
    if (dev < 0 || dev >= MAX_DEVICES) return fail(EVX_ERR_UNSUPPORTED, "device ordinal %d out of range", dev);
    std::call_once(g_tw_once[dev], [dev] {
        g_tw_rc[dev] = check_cuda(upload_w512(), "twiddle table upload");
    });
    return g_tw_rc[dev];
}

template <class K>
int yz_grid(K kern, size_t smem, int cs, int nx, int* grid) {
    int rc = check_cuda(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem),
                        "(y,z) transform shared memory attribute");
    if (rc) return rc;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(cs * std::max(1, nx));
    cfg.blockDim = dim3(256);
    cfg.dynamicSmemBytes = smem;
    int ncl = 0;
    rc = check_cuda(cudaOccupancyMaxActiveClusters(&ncl, kern, &cfg), "(y,z) transform cluster occupancy");
    if (rc) return rc;
    if (ncl < 1) return fail(EVX_ERR_UNSUPPORTED, "(y,z) transform cluster of %d CTAs does not fit", cs);
    *grid = cs * std::min(ncl, nx);
    return EVX_OK;
}

template <int NY, int NZ, int CS>
int yz_launch_t(bool fwd, const void* in, void* out, int nx, cudaStream_t st) {
    using G = YZ<NY, NZ, CS>;
    static int grid_f = 0, grid_i = 0, nx_f = -1, nx_i = -1;   // per instantiation
    int rc;
    if (fwd) {
        if (nx != nx_f) {
            if ((rc = yz_grid(yz_r2c_kernel<NY, NZ, CS>, G::SMEM, CS, nx, &grid_f))) return rc;
            nx_f = nx;
        }
        EVX_TIMED("fft_yz_r2c", st, yz_r2c_kernel<NY, NZ, CS><<<grid_f, 256, G::SMEM, st>>>(
                                        static_cast<const float*>(in), static_cast<float2*>(out), nx));
    } else {
        if (nx != nx_i) {
            if ((rc = yz_grid(yz_c2r_kernel<NY, NZ, CS>, G::SMEM, CS, nx, &grid_i))) return rc;
            nx_i = nx;
        }
        EVX_TIMED("fft_yz_c2r", st, yz_c2r_kernel<NY, NZ, CS><<<grid_i, 256, G::SMEM, st>>>(
                                        static_cast<const float2*>(in), static_cast<float*>(out), nx));
    }
    count_launch();
    return check_launch(fwd ? "yz_r2c_kernel" : "yz_c2r_kernel");
}

// cluster size: KC = 32 columns per CTA (fewer when nz/2 < 32)
template <int NY, int NZ>
int yz_launch_n(bool fwd, const void* in, void* out, int nx, cudaStream_t st) {
    constexpr int CS = NZ / 2 >= 32 ? NZ / 64 : 1;
    return yz_launch_t<NY, NZ, (CS < 1 ? 1 : CS)>(fwd, in, out, nx, st);
}

template <int NY>
int yz_launch_y(bool fwd, int nz, const void* in, void* out, int nx, cudaStream_t st) {
    switch (nz) {
        case 64: return yz_launch_n<NY, 64>(fwd, in, out, nx, st);
        case 128: return yz_launch_n<NY, 128>(fwd, in, out, nx, st);
        case 256: return yz_launch_n<NY, 256>(fwd, in, out, nx, st);
        default: return fail(EVX_ERR_UNSUPPORTED, "(y,z) transform: nz = %d", nz);
    }
}

int yz_launch(bool fwd, int nx, int ny, int nz, const void* in, void* out, cudaStream_t st) {
    int rc = yz_init();
    if (rc) return rc;
    if (!yz_supported(ny, nz)) return fail(EVX_ERR_UNSUPPORTED, "(y,z) transform of %d x %d", ny, nz);
    switch (ny) {
        case 64: return yz_launch_y<64>(fwd, nz, in, out, nx, st);
        case 128: return yz_launch_y<128>(fwd, nz, in, out, nx, st);
        case 256: return yz_launch_y<256>(fwd, nz, in, out, nx, st);
        default: return fail(EVX_ERR_UNSUPPORTED, "(y,z) transform: ny = %d", ny);
    }
}

}  // namespace

bool yz_supported(int ny, int nz) {
    auto ok = [](int n) { return n == 64 || n == 128 || n == 256; };
    return ok(ny) && ok(nz) && !yz_env_off();
}

int fft_yz_r2c(int nx, int ny, int nz, const float* in, float2* out, cudaStream_t st) {
    return yz_launch(true, nx, ny, nz, in, out, st);
}

int fft_yz_c2r(int nx, int ny, int nz, const float2* in, float* out, cudaStream_t st) {
    return yz_launch(false, nx, ny, nz, in, out, st);
}

}  // namespace evx

using namespace evx;

extern "C" {

int evx_fft_yz_r2c(const float* in, float* out, int nx, int ny, int nz, void* stream) {
    if (!in || !out) return fail(EVX_ERR_BAD_ARG, "NULL pointer");
    if (nx < 1) return fail(EVX_ERR_BAD_SHAPE, "nx must be >= 1");
    if (reinterpret_cast<uintptr_t>(out) & 7) return fail(EVX_ERR_BAD_ARG, "out must be 8-byte aligned");
    return fft_yz_r2c(nx, ny, nz, in, reinterpret_cast<float2*>(out), as_stream(stream));
}

int evx_fft_yz_c2r(const float* in, float* out, int nx, int ny, int nz, void* stream) {
    if (!in || !out) return fail(EVX_ERR_BAD_ARG, "NULL pointer");
    if (nx < 1) return fail(EVX_ERR_BAD_SHAPE, "nx must be >= 1");
    if (reinterpret_cast<uintptr_t>(in) & 7) return fail(EVX_ERR_BAD_ARG, "in must be 8-byte aligned");
    return fft_yz_c2r(nx, ny, nz, reinterpret_cast<const float2*>(in), out, as_stream(stream));
}

}  // extern "C"
