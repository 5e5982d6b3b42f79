// Small MLP for the topology step's learned proposal (oc_mlp.cu).
#pragma once

#include "oc_internal.h"

#include <string>

namespace oc {

struct Mlp {
    int in = 0, hidden = 0, step = 0;
    cudaStream_t st = nullptr;
    // parameters (FP32 master, BF16-rounded copy used by the products),
    // Adam moments, gradient
    float *master = nullptr, *wbf = nullptr, *m1 = nullptr, *v1 = nullptr, *grad = nullptr, *sse = nullptr;
    // row buffers
    int capRows = 0;
    float *bufX = nullptr, *bufT = nullptr, *bufH1 = nullptr, *bufH2 = nullptr, *bufY = nullptr;
    float *bufD1 = nullptr, *bufD2 = nullptr, *bufDy = nullptr;

    // products on the tensor cores (else the CUDA-core kernel); a device
    // flag the tensor-core kernel sets when a wait runs out; the last launch
    // error of a product
    bool tensorCores = true;
    int* errFlag = nullptr;
    cudaError_t launchError = cudaSuccess;

    int nParams() const;
    int init(int nIn, int nHidden, unsigned seed, cudaStream_t s, std::string* err);
    void release();
    int ensure_rows(int n);
    void forward(int n);    // rows in bufX -> bufY
    void backward(int n);   // targets in bufT -> grad, sum of squared errors in *sse
    void adam(float lr);
    void gemm(int M, int N, int K, const float* A, long long sam, long long sak, const float* B, long long sbk,
              long long sbn, float* C, long long ldc, float alpha, float beta, const float* bias);
    // after a synchronize: OC_OK, or OC_ERR_TIMEOUT / OC_ERR_CUDA (flags cleared)
    int check();
};

void k_round_bf16_launch(const float* w, float* out, int n, cudaStream_t st);
void k_gather_rows_launch(const float* X, const float* t, const int* idx, int n, int in, float* Xo, float* to,
                          cudaStream_t st);

} // namespace oc

struct oc_mlp {
    oc_ctx* ctx = nullptr;
    oc::Mlp m;
};
