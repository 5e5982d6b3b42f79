// BF16 products on the 5th-generation tensor cores (oc_tc.cu): the
// learned proposal's MLP layers.
#pragma once

#include "oc_internal.h"

namespace oc {

// C[m, n] = alpha * sum_k A(m, k) B(k, n) + beta * C[m, n] (+ bias[n]) with
// A(m, k) = A[m * sam + k * sak] and B(k, n) = B[k * sbk + n * sbn] (FP32 in
// global memory, rounded to BF16 on the way into shared memory), products
// by tcgen05.mma (kind::f16, 128 x N tiles, N <= 128 per tile) accumulated
// in FP32 in tensor memory.  A wait that runs out sets *err to 1.
cudaError_t gemm_tc(cudaStream_t st, int M, int N, int K, const float* A, long long sam, long long sak, const float* B,
                    long long sbk, long long sbn, float* C, long long ldc, float alpha, float beta, const float* bias,
                    int* err);

// The bound of the in-loop mbarrier waits of later gemm_tc launches, in
// polls (0: give up at once; -1: the default, 2^20; process-wide).  A wait
// that runs out raises *err, waits for the MMAs in flight with the default
// bound, releases the tensor memory and returns: a bound of 0 is how the
// timeout path is tested without a fault.
void tc_set_wait_polls(int polls);

// The same product on the CUDA cores (BF16 operands, FP32 accumulation):
// the reference the tensor-core kernel is tested against, and the form for
// the one-column products (K or N of 1) of the network.
void gemm_cuda_cores(cudaStream_t st, int M, int N, int K, const float* A, long long sam, long long sak,
                     const float* B, long long sbk, long long sbn, float* C, long long ldc, float alpha, float beta,
                     const float* bias);

} // namespace oc
