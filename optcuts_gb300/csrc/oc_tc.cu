// BF16 tensor-core products for the learned proposal's MLP.
//
// One CTA of 128 threads computes a 128 x N tile (N <= 128) of
//   C = alpha * op(A) op(B) + beta * C (+ bias)
// Per K-stage of 64: the threads load their rows of A and B (any strides,
// so transposed operands need no copies), round them to BF16 and store them
// in shared memory in the canonical K-major layout without swizzle (core
// matrices of 8 rows x 16 bytes: K-adjacent ones 128 bytes apart, row
// groups 1024 bytes apart); one thread issues four tcgen05.mma (K = 16
// each) into an FP32 accumulator in tensor memory and commits them to an
// mbarrier, which every thread waits on (bounded) before the next stage
// overwrites the operands.  The epilogue reads the accumulator with
// tcgen05.ld (warp w owns rows 32w..32w+31, one row per thread).

#include "oc_tc.h"

#include <cuda_bf16.h>

#include <atomic>
#include <cstdint>

namespace oc {
namespace {

constexpr int kTcM = 128, kTcN = 128, kTcK = 64;
constexpr int kTcThreads = 128;
constexpr uint32_t kTmemCols = 128;             // FP32 accumulator columns (power of two >= 32)
constexpr uint32_t kCoreK = 128, kCoreM = 1024;  // bytes between K- / row-adjacent core matrices
constexpr int kWaitPolls = 1 << 20;

__device__ __forceinline__ uint32_t smem_u32(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// shared-memory matrix descriptor (tcgen05): start address, leading (K)
// and stride (row-group) byte offsets, version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr)
{
    uint64_t d = 0;
    d |= static_cast<uint64_t>((addr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>((kCoreK >> 4) & 0x3FFFu) << 16;
    d |= static_cast<uint64_t>((kCoreM >> 4) & 0x3FFFu) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    return d;
}

// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B,
// both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
           (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int polls = kWaitPolls)
{
    for (int i = 0; i < polls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// rows [r0, r0 + 128) of X(row, k) = X[row * srow + k * sk] for k in
// [k0, k0 + 64), rounded to BF16, into the K-major core-matrix layout
__device__ __forceinline__ void stage_rows(uint8_t* dst, const float* __restrict__ X, long long srow, long long sk,
                                           int rows, int r0, int K, int k0, int r)
{
    const int row = r0 + r;
    const bool live = row < rows;
    const float* base = X + (live ? row * srow : 0);
#pragma unroll 2
    for (int kc = 0; kc < kTcK / 8; ++kc) {
        uint32_t w[4];
#pragma unroll
        for (int h = 0; h < 4; ++h) {
            const int k = k0 + kc * 8 + 2 * h;
            const float x0 = (live && k < K) ? base[k * sk] : 0.0f;
            const float x1 = (live && k + 1 < K) ? base[(k + 1) * sk] : 0.0f;
            const __nv_bfloat162 v = __floats2bfloat162_rn(x0, x1);
            w[h] = *reinterpret_cast<const uint32_t*>(&v);
        }
        *reinterpret_cast<uint4*>(dst + (r >> 3) * kCoreM + kc * kCoreK + (r & 7) * 16) = make_uint4(w[0], w[1], w[2], w[3]);
    }
}

__global__ void __launch_bounds__(kTcThreads) k_gemm_tc(int M, int N, int K, const float* __restrict__ A,
                                                        long long sam, long long sak, const float* __restrict__ B,
                                                        long long sbk, long long sbn, float* __restrict__ C,
                                                        long long ldc, float alpha, float beta,
                                                        const float* __restrict__ bias, int nInst, int waitPolls,
                                                        int* err)
{
    __shared__ __align__(1024) uint8_t sA[kTcM * kTcK * 2];
    __shared__ __align__(1024) uint8_t sB[kTcN * kTcK * 2];
    __shared__ __align__(8) uint64_t mbar;
    __shared__ uint32_t tmemBase;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int m0 = blockIdx.y * kTcM, n0 = blockIdx.x * kTcN;
    const uint32_t bar = smem_u32(&mbar);
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmemBase)),
                     "r"(kTmemCols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = tmemBase;
    const uint32_t idesc = idesc_bf16(kTcM, nInst);
    uint32_t parity = 0;
    bool ok = true;
    for (int k0 = 0; k0 < K && ok; k0 += kTcK) {
        stage_rows(sA, A, sam, sak, M, m0, K, k0, tid);
        stage_rows(sB, B, sbn, sbk, N, n0, K, k0, tid);
        // the generic-proxy stores, visible to the tensor core's async proxy
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        __syncthreads();
        if (tid == 0) {
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
#pragma unroll
            for (int s = 0; s < kTcK / 16; ++s) {
                const uint64_t da = smem_desc(smem_u32(sA) + s * 2 * kCoreK);
                const uint64_t db = smem_desc(smem_u32(sB) + s * 2 * kCoreK);
                const uint32_t accumulate = (k0 > 0 || s > 0) ? 1u : 0u;
                asm volatile(
                    "{\n\t.reg .pred p;\n\t"
                    "setp.ne.b32 p, %4, 0;\n\t"
                    "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
                    "l"(da), "l"(db), "r"(idesc), "r"(accumulate)
                    : "memory");
            }
            asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                         : "memory");
        }
        ok = mbar_wait(bar, parity, waitPolls);
        parity ^= 1u;
        // a block whose wait ran out stops here; every thread sees the same
        // mbarrier, but make the decision uniform anyway
        ok = __syncthreads_and(ok);
    }
    if (!ok) {
        if (tid == 0) atomicExch(err, 1);
        // the MMAs of the last stage may still be in flight: give them one
        // more bounded wait before the tensor memory is released
        mbar_wait(bar, parity ^ 1u);
    }
    else {
        asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
        const int row = m0 + warp * 32 + lane;
        for (int c0 = 0; c0 < nInst; c0 += 16) {
            uint32_t v[16];
            const uint32_t taddr = tmem + (static_cast<uint32_t>(warp * 32) << 16) + static_cast<uint32_t>(c0);
            asm volatile(
                "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
                "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
                : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
                  "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]),
                  "=r"(v[15])
                : "r"(taddr)
                : "memory");
            asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
            if (row < M) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int n = n0 + c0 + j;
                    if (n < N) {
                        float x = alpha * __uint_as_float(v[j]);
                        if (beta != 0.0f) x += beta * C[row * ldc + n];
                        if (bias) x += bias[n];
                        C[row * ldc + n] = x;
                    }
                }
            }
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 0)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(kTmemCols) : "memory");
}

constexpr int kTileM = 64, kTileN = 64, kTileK = 16;

__global__ void __launch_bounds__(256) k_gemm_bf16(int M, int N, int K, const float* __restrict__ A, long long sam,
                                                   long long sak, const float* __restrict__ B, long long sbk,
                                                   long long sbn, float* __restrict__ C, long long ldc, float alpha,
                                                   float beta, const float* __restrict__ bias)
{
    __shared__ __nv_bfloat16 As[kTileK][kTileM + 2];
    __shared__ __nv_bfloat16 Bs[kTileK][kTileN + 2];
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;   // 16 x 16 threads, 4 x 4 outputs each
    const int m0 = blockIdx.y * kTileM, n0 = blockIdx.x * kTileN;
    float acc[4][4] = {};
    for (int k0 = 0; k0 < K; k0 += kTileK) {
        for (int e = threadIdx.x; e < kTileK * kTileM; e += 256) {
            const int kk = e / kTileM, mm = e % kTileM;
            const int m = m0 + mm, k = k0 + kk;
            As[kk][mm] = __float2bfloat16(m < M && k < K ? A[m * sam + k * sak] : 0.0f);
        }
        for (int e = threadIdx.x; e < kTileK * kTileN; e += 256) {
            const int kk = e / kTileN, nn = e % kTileN;
            const int n = n0 + nn, k = k0 + kk;
            Bs[kk][nn] = __float2bfloat16(n < N && k < K ? B[k * sbk + n * sbn] : 0.0f);
        }
        __syncthreads();
#pragma unroll
        for (int kk = 0; kk < kTileK; ++kk) {
            float a[4], b[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) a[i] = __bfloat162float(As[kk][ty * 4 + i]);
#pragma unroll
            for (int j = 0; j < 4; ++j) b[j] = __bfloat162float(Bs[kk][tx * 4 + j]);
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 4; ++j) acc[i][j] = fmaf(a[i], b[j], acc[i][j]);
        }
        __syncthreads();
    }
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int m = m0 + ty * 4 + i, n = n0 + tx * 4 + j;
            if (m < M && n < N) {
                float v = alpha * acc[i][j];
                if (beta != 0.0f) v += beta * C[m * ldc + n];
                if (bias) v += bias[n];
                C[m * ldc + n] = v;
            }
        }
}

} // namespace

namespace {
std::atomic<int> g_waitPolls{-1};   // -1: kWaitPolls
}

void tc_set_wait_polls(int polls) { g_waitPolls.store(polls < 0 ? -1 : polls); }

cudaError_t gemm_tc(cudaStream_t st, int M, int N, int K, const float* A, long long sam, long long sak, const float* B,
                    long long sbk, long long sbn, float* C, long long ldc, float alpha, float beta, const float* bias,
                    int* err)
{
    if (M <= 0 || N <= 0) return cudaSuccess;
    if (K <= 0 || !err) return cudaErrorInvalidValue;
    const int nInst = N >= kTcN ? kTcN : ((N + 15) / 16) * 16;
    dim3 grid((N + kTcN - 1) / kTcN, (M + kTcM - 1) / kTcM);
    const int polls = g_waitPolls.load();
    k_gemm_tc<<<grid, kTcThreads, 0, st>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, alpha, beta, bias, nInst,
                                           polls >= 0 ? polls : kWaitPolls, err);
    return cudaGetLastError();
}

void gemm_cuda_cores(cudaStream_t st, int M, int N, int K, const float* A, long long sam, long long sak,
                     const float* B, long long sbk, long long sbn, float* C, long long ldc, float alpha, float beta,
                     const float* bias)
{
    if (M <= 0 || N <= 0) return;
    dim3 grid((N + kTileN - 1) / kTileN, (M + kTileM - 1) / kTileM);
    k_gemm_bf16<<<grid, 256, 0, st>>>(M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, alpha, beta, bias);
}

} // namespace oc
