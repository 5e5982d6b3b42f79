// Learned proposal for the topology step: a 3-layer MLP (in -> 128 -> 128 -> 1,
// ReLU) with BF16 weights and activations feeding FP32-accumulated
// products, trained on the device by the project's own forward / backward
// kernels and Adam on FP32 master weights.
//
// Every product has the form C[M x N] (+)= op(A)[M x K] * op(B)[K x N] with
// A, B given with explicit strides (no transposed copies).  Those with K and
// N of at least 16 (both hidden layers, forward and backward) run on the
// tensor cores (oc_tc.cu, tcgen05.mma); the one-column products of the
// output layer on the CUDA cores.

#include "oc_mlp.h"
#include "oc_tc.h"

#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <random>
#include <vector>

namespace oc {
namespace {

__global__ void k_relu(float* __restrict__ x, long long n)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n) x[i] = fmaxf(x[i], 0.0f);
}

// dH *= (H > 0)
__global__ void k_relu_back(float* __restrict__ dH, const float* __restrict__ H, long long n)
{
    const long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (i < n && !(H[i] > 0.0f)) dH[i] = 0.0f;
}

// dy = 2 (y - t) / n, and the batch's squared error into partials
__global__ void k_mse_grad(const float* __restrict__ y, const float* __restrict__ t, int n, float* __restrict__ dy,
                           float* __restrict__ sse)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    float e = 0.0f;
    if (i < n) {
        const float d = y[i] - t[i];
        dy[i] = 2.0f * d / n;
        e = d * d;
    }
    for (int o = 16; o > 0; o >>= 1) e += __shfl_down_sync(0xffffffffu, e, o);
    if ((threadIdx.x & 31) == 0) atomicAdd(sse, e);
}

// column sums: out[n] = sum_m X[m * ld + n]
__global__ void k_colsum(const float* __restrict__ X, int M, int N, long long ld, float* __restrict__ out)
{
    const int n = blockIdx.x * blockDim.x + threadIdx.x;
    if (n >= N) return;
    float s = 0.0f;
    for (int m = 0; m < M; ++m) s += X[m * ld + n];
    out[n] = s;
}

__global__ void k_adam(float* __restrict__ w, float* __restrict__ mo, float* __restrict__ ve,
                       const float* __restrict__ g, int n, float lr, float b1, float b2, float eps, float c1, float c2)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float m = b1 * mo[i] + (1.0f - b1) * gi;
    const float v = b2 * ve[i] + (1.0f - b2) * gi * gi;
    mo[i] = m;
    ve[i] = v;
    w[i] -= lr * (m / c1) / (sqrtf(v / c2) + eps);
}

// weights used by the products: rounded to BF16 (kept as float values)
__global__ void k_round_bf16(const float* __restrict__ w, float* __restrict__ out, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] = __bfloat162float(__float2bfloat16(w[i]));
}

int blocks(long long n, int t = 256) { return static_cast<int>((n + t - 1) / t); }

} // namespace

void Mlp::gemm(int M, int N, int K, const float* A, long long sam, long long sak, const float* B, long long sbk,
               long long sbn, float* C, long long ldc, float alpha, float beta, const float* bias)
{
    if (tensorCores && K >= 16 && N >= 16) {
        const cudaError_t e = gemm_tc(st, M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, alpha, beta, bias, errFlag);
        if (e != cudaSuccess) launchError = e;
    }
    else {
        gemm_cuda_cores(st, M, N, K, A, sam, sak, B, sbk, sbn, C, ldc, alpha, beta, bias);
    }
}


void k_round_bf16_launch(const float* w, float* out, int n, cudaStream_t st)
{
    k_round_bf16<<<blocks(n), 256, 0, st>>>(w, out, n);
}

// parameter block layout: W1 [H x I], b1 [H], W2 [H x H], b2 [H], W3 [H], b3 [1]
int Mlp::nParams() const { return hidden * in + hidden + hidden * hidden + hidden + hidden + 1; }

int Mlp::init(int nIn, int nHidden, unsigned seed, cudaStream_t s, std::string* err)
{
    in = nIn;
    hidden = nHidden;
    st = s;
    const int P = nParams();
    std::vector<float> w(P, 0.0f);
    std::mt19937 rng(seed);
    auto fill = [&](int off, int fanIn, int count) {   // He-uniform
        std::uniform_real_distribution<float> U(-std::sqrt(6.0f / fanIn), std::sqrt(6.0f / fanIn));
        for (int i = 0; i < count; ++i) w[off + i] = U(rng);
    };
    fill(0, in, hidden * in);
    fill(hidden * in + hidden, hidden, hidden * hidden);
    fill(hidden * in + hidden + hidden * hidden + hidden, hidden, hidden);
    cudaError_t e = cudaSuccess;
    for (float** p : {&master, &wbf, &m1, &v1, &grad}) {
        if (e == cudaSuccess) e = cudaMalloc(p, sizeof(float) * P);
        if (e == cudaSuccess) e = cudaMemsetAsync(*p, 0, sizeof(float) * P, st);
    }
    if (e == cudaSuccess) e = cudaMalloc(&sse, sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc(&errFlag, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(errFlag, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(master, w.data(), sizeof(float) * P, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) k_round_bf16<<<blocks(P), 256, 0, st>>>(master, wbf, P);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) {
        if (err) *err = std::string("mlp init: ") + cudaGetErrorString(e);
        return OC_ERR_CUDA;
    }
    step = 0;
    return OC_OK;
}

void Mlp::release()
{
    for (float* p : {master, wbf, m1, v1, grad, sse, bufX, bufT, bufH1, bufH2, bufY, bufD1, bufD2, bufDy}) cudaFree(p);
    master = wbf = m1 = v1 = grad = sse = nullptr;
    bufX = bufT = bufH1 = bufH2 = bufY = bufD1 = bufD2 = bufDy = nullptr;
    cudaFree(errFlag);
    errFlag = nullptr;
    capRows = 0;
}

int Mlp::check()
{
    int flag = 0;
    if (cudaMemcpyAsync(&flag, errFlag, sizeof(int), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return OC_ERR_CUDA;
    const cudaError_t le = launchError;
    launchError = cudaSuccess;
    if (le != cudaSuccess) return OC_ERR_CUDA;
    if (flag) {
        cudaMemsetAsync(errFlag, 0, sizeof(int), st);
        return OC_ERR_TIMEOUT;
    }
    return OC_OK;
}

int Mlp::ensure_rows(int n)
{
    if (n <= capRows) return OC_OK;
    for (float* p : {bufX, bufT, bufH1, bufH2, bufY, bufD1, bufD2, bufDy}) cudaFree(p);
    cudaError_t e = cudaSuccess;
    const size_t r = static_cast<size_t>(n);
    if (e == cudaSuccess) e = cudaMalloc(&bufX, sizeof(float) * r * in);
    if (e == cudaSuccess) e = cudaMalloc(&bufT, sizeof(float) * r);
    if (e == cudaSuccess) e = cudaMalloc(&bufH1, sizeof(float) * r * hidden);
    if (e == cudaSuccess) e = cudaMalloc(&bufH2, sizeof(float) * r * hidden);
    if (e == cudaSuccess) e = cudaMalloc(&bufY, sizeof(float) * r);
    if (e == cudaSuccess) e = cudaMalloc(&bufD1, sizeof(float) * r * hidden);
    if (e == cudaSuccess) e = cudaMalloc(&bufD2, sizeof(float) * r * hidden);
    if (e == cudaSuccess) e = cudaMalloc(&bufDy, sizeof(float) * r);
    if (e != cudaSuccess) return OC_ERR_CUDA;
    capRows = n;
    return OC_OK;
}

// forward over n rows of bufX: bufH1, bufH2 (post-ReLU), bufY
void Mlp::forward(int n)
{
    const float* W1 = wbf;
    const float* b1 = W1 + hidden * in;
    const float* W2 = b1 + hidden;
    const float* b2 = W2 + hidden * hidden;
    const float* W3 = b2 + hidden;
    const float* b3 = W3 + hidden;
    // H1 = X W1^T + b1: A = X (n x in), B(k, j) = W1[j * in + k]
    gemm(n, hidden, in, bufX, in, 1, W1, 1, in, bufH1, hidden, 1.0f, 0.0f, b1);
    k_relu<<<blocks((long long)n * hidden), 256, 0, st>>>(bufH1, (long long)n * hidden);
    gemm(n, hidden, hidden, bufH1, hidden, 1, W2, 1, hidden, bufH2, hidden, 1.0f, 0.0f, b2);
    k_relu<<<blocks((long long)n * hidden), 256, 0, st>>>(bufH2, (long long)n * hidden);
    gemm(n, 1, hidden, bufH2, hidden, 1, W3, 1, hidden, bufY, 1, 1.0f, 0.0f, b3);
}

// gradient of the mean squared error over n rows (bufX, bufT) into grad
void Mlp::backward(int n)
{
    const float* W2 = wbf + hidden * in + hidden;
    const float* W3 = W2 + hidden * hidden + hidden;
    float* gW1 = grad;
    float* gb1 = gW1 + hidden * in;
    float* gW2 = gb1 + hidden;
    float* gb2 = gW2 + hidden * hidden;
    float* gW3 = gb2 + hidden;
    float* gb3 = gW3 + hidden;
    cudaMemsetAsync(sse, 0, sizeof(float), st);
    k_mse_grad<<<blocks(n), 256, 0, st>>>(bufY, bufT, n, bufDy, sse);
    // layer 3: gW3[j] = sum_m dy[m] H2[m, j]; gb3 = sum dy; dH2 = dy W3 (x) relu'
    gemm(1, hidden, n, bufDy, 0, 1, bufH2, hidden, 1, gW3, hidden, 1.0f, 0.0f, nullptr);
    k_colsum<<<1, 32, 0, st>>>(bufDy, n, 1, 1, gb3);
    gemm(n, hidden, 1, bufDy, 1, 1, W3, 0, 1, bufD2, hidden, 1.0f, 0.0f, nullptr);
    k_relu_back<<<blocks((long long)n * hidden), 256, 0, st>>>(bufD2, bufH2, (long long)n * hidden);
    // layer 2: gW2[j, k] = sum_m dH2[m, j] H1[m, k]; dH1 = dH2 W2 (x) relu'
    gemm(hidden, hidden, n, bufD2, 1, hidden, bufH1, hidden, 1, gW2, hidden, 1.0f, 0.0f, nullptr);
    k_colsum<<<blocks(hidden, 128), 128, 0, st>>>(bufD2, n, hidden, hidden, gb2);
    gemm(n, hidden, hidden, bufD2, hidden, 1, W2, hidden, 1, bufD1, hidden, 1.0f, 0.0f, nullptr);
    k_relu_back<<<blocks((long long)n * hidden), 256, 0, st>>>(bufD1, bufH1, (long long)n * hidden);
    // layer 1: gW1[j, k] = sum_m dH1[m, j] X[m, k]
    gemm(hidden, in, n, bufD1, 1, hidden, bufX, in, 1, gW1, in, 1.0f, 0.0f, nullptr);
    k_colsum<<<blocks(hidden, 128), 128, 0, st>>>(bufD1, n, hidden, hidden, gb1);
}

__global__ void k_gather_rows(const float* __restrict__ X, const float* __restrict__ t, const int* __restrict__ idx,
                              int n, int in, float* __restrict__ Xo, float* __restrict__ to)
{
    const int r = blockIdx.x;
    if (r >= n) return;
    const int s = idx[r];
    for (int k = threadIdx.x; k < in; k += blockDim.x) Xo[(size_t)r * in + k] = X[(size_t)s * in + k];
    if (threadIdx.x == 0) to[r] = t[s];
}

void k_gather_rows_launch(const float* X, const float* t, const int* idx, int n, int in, float* Xo, float* to,
                          cudaStream_t st)
{
    if (n > 0) k_gather_rows<<<n, 64, 0, st>>>(X, t, idx, n, in, Xo, to);
}

void Mlp::adam(float lr)
{
    ++step;
    const float b1 = 0.9f, b2 = 0.999f;
    const float c1 = 1.0f - std::pow(b1, static_cast<float>(step)), c2 = 1.0f - std::pow(b2, static_cast<float>(step));
    const int P = nParams();
    k_adam<<<blocks(P), 256, 0, st>>>(master, m1, v1, grad, P, lr, b1, b2, 1e-8f, c1, c2);
    k_round_bf16<<<blocks(P), 256, 0, st>>>(master, wbf, P);
}

int mlp_predict_host(Mlp& m, const float* X, int n, float* y)
{
    const int chunk = 65536;
    for (int r0 = 0; r0 < n; r0 += chunk) {
        const int r = n - r0 < chunk ? n - r0 : chunk;
        if (m.ensure_rows(r)) return OC_ERR_CUDA;
        if (cudaMemcpyAsync(m.bufX, X + (size_t)r0 * m.in, sizeof(float) * (size_t)r * m.in, cudaMemcpyHostToDevice,
                            m.st) != cudaSuccess)
            return OC_ERR_CUDA;
        m.forward(r);
        if (cudaMemcpyAsync(y + r0, m.bufY, sizeof(float) * r, cudaMemcpyDeviceToHost, m.st) != cudaSuccess)
            return OC_ERR_CUDA;
    }
    if (cudaStreamSynchronize(m.st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return OC_ERR_CUDA;
    return m.check();
}

} // namespace oc

// ---------------------------------------------------------------- C ABI
#define OC_EXPORT extern "C" __attribute__((visibility("default")))


OC_EXPORT int oc_mlp_create(oc_ctx* ctx, int nIn, int nHidden, unsigned seed, oc_mlp** out)
{
    if (!ctx || !out || nIn <= 0 || nHidden <= 0 || nIn > 1024 || nHidden > 1024) return OC_ERR_INVALID;
    *out = nullptr;
    oc_mlp* p = new (std::nothrow) oc_mlp;
    if (!p) return OC_ERR_NOMEM;
    p->ctx = ctx;
    std::string err;
    const int rc = p->m.init(nIn, nHidden, seed, oc::ctx_stream(ctx), &err);
    if (rc) {
        p->m.release();
        delete p;
        return rc;
    }
    *out = p;
    return OC_OK;
}

OC_EXPORT int oc_mlp_destroy(oc_mlp* p)
{
    if (!p) return OC_ERR_INVALID;
    p->m.release();
    delete p;
    return OC_OK;
}

OC_EXPORT int oc_mlp_get_params(oc_mlp* p, float* params)
{
    if (!p || !params) return OC_ERR_INVALID;
    if (cudaMemcpyAsync(params, p->m.master, sizeof(float) * p->m.nParams(), cudaMemcpyDeviceToHost, p->m.st) != cudaSuccess ||
        cudaStreamSynchronize(p->m.st) != cudaSuccess)
        return OC_ERR_CUDA;
    return OC_OK;
}

OC_EXPORT int oc_mlp_set_params(oc_mlp* p, const float* params)
{
    if (!p || !params) return OC_ERR_INVALID;
    const int P = p->m.nParams();
    if (cudaMemcpyAsync(p->m.master, params, sizeof(float) * P, cudaMemcpyHostToDevice, p->m.st) != cudaSuccess)
        return OC_ERR_CUDA;
    oc::k_round_bf16_launch(p->m.master, p->m.wbf, P, p->m.st);
    return cudaStreamSynchronize(p->m.st) == cudaSuccess ? OC_OK : OC_ERR_CUDA;
}

OC_EXPORT int oc_mlp_num_params(const oc_mlp* p, int* n)
{
    if (!p || !n) return OC_ERR_INVALID;
    *n = p->m.nParams();
    return OC_OK;
}

// y = f(X) for n rows (X n x in, row-major)
OC_EXPORT int oc_mlp_predict(oc_mlp* p, const float* X, int n, float* y)
{
    if (!p || !X || !y || n < 0) return OC_ERR_INVALID;
    if (n == 0) return OC_OK;
    return oc::mlp_predict_host(p->m, X, n, y);
}

// gradient of the mean squared error of n rows (for checking the backward pass)
OC_EXPORT int oc_mlp_gradient(oc_mlp* p, const float* X, const float* t, int n, float* grad, float* loss)
{
    if (!p || !X || !t || !grad || n <= 0) return OC_ERR_INVALID;
    oc::Mlp& m = p->m;
    if (m.ensure_rows(n)) return OC_ERR_CUDA;
    cudaMemcpyAsync(m.bufX, X, sizeof(float) * (size_t)n * m.in, cudaMemcpyHostToDevice, m.st);
    cudaMemcpyAsync(m.bufT, t, sizeof(float) * n, cudaMemcpyHostToDevice, m.st);
    m.forward(n);
    m.backward(n);
    float sse = 0.0f;
    cudaMemcpyAsync(grad, m.grad, sizeof(float) * m.nParams(), cudaMemcpyDeviceToHost, m.st);
    cudaMemcpyAsync(&sse, m.sse, sizeof(float), cudaMemcpyDeviceToHost, m.st);
    if (cudaStreamSynchronize(m.st) != cudaSuccess || cudaGetLastError() != cudaSuccess) return OC_ERR_CUDA;
    if (const int rc = m.check()) return rc;
    if (loss) *loss = sse / n;
    return OC_OK;
}

// Adam on mini-batches (shuffled each epoch); *finalLoss = mean squared
// error of the last epoch's batches
OC_EXPORT int oc_mlp_train(oc_mlp* p, const float* X, const float* t, int n, int epochs, int batch, float lr,
                           unsigned seed, float* finalLoss)
{
    if (!p || !X || !t || n <= 0 || epochs <= 0 || batch <= 0) return OC_ERR_INVALID;
    oc::Mlp& m = p->m;
    float *dX = nullptr, *dT = nullptr;
    int* dIdx = nullptr;
    if (cudaMalloc(&dX, sizeof(float) * (size_t)n * m.in) != cudaSuccess || cudaMalloc(&dT, sizeof(float) * n) != cudaSuccess ||
        cudaMalloc(&dIdx, sizeof(int) * n) != cudaSuccess || m.ensure_rows(batch)) {
        cudaFree(dX); cudaFree(dT); cudaFree(dIdx);
        return OC_ERR_CUDA;
    }
    cudaMemcpyAsync(dX, X, sizeof(float) * (size_t)n * m.in, cudaMemcpyHostToDevice, m.st);
    cudaMemcpyAsync(dT, t, sizeof(float) * n, cudaMemcpyHostToDevice, m.st);
    std::vector<int> idx(n);
    for (int i = 0; i < n; ++i) idx[i] = i;
    std::mt19937 rng(seed);
    double lastSse = 0.0;
    int lastRows = 0;
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(idx.begin(), idx.end(), rng);
        cudaMemcpyAsync(dIdx, idx.data(), sizeof(int) * n, cudaMemcpyHostToDevice, m.st);
        lastSse = 0.0;
        lastRows = 0;
        for (int b0 = 0; b0 < n; b0 += batch) {
            const int r = n - b0 < batch ? n - b0 : batch;
            oc::k_gather_rows_launch(dX, dT, dIdx + b0, r, m.in, m.bufX, m.bufT, m.st);
            m.forward(r);
            m.backward(r);
            m.adam(lr);
            if (ep == epochs - 1) {
                float sse = 0.0f;
                cudaMemcpyAsync(&sse, m.sse, sizeof(float), cudaMemcpyDeviceToHost, m.st);
                cudaStreamSynchronize(m.st);
                lastSse += sse;
                lastRows += r;
            }
        }
        // the host shuffle of the next epoch reuses dIdx: wait for this one
        if (const int rc = m.check()) {
            cudaFree(dX); cudaFree(dT); cudaFree(dIdx);
            return rc;
        }
    }
    const bool ok = cudaStreamSynchronize(m.st) == cudaSuccess && cudaGetLastError() == cudaSuccess;
    cudaFree(dX); cudaFree(dT); cudaFree(dIdx);
    if (finalLoss) *finalLoss = lastRows ? static_cast<float>(lastSse / lastRows) : 0.0f;
    return ok ? OC_OK : OC_ERR_CUDA;
}

// products of the network on the tensor cores (1, the default) or on the
// CUDA cores (0)
OC_EXPORT int oc_mlp_set_tensor_cores(oc_mlp* p, int on)
{
    if (!p) return OC_ERR_INVALID;
    p->m.tensorCores = on != 0;
    return OC_OK;
}

OC_EXPORT int oc_tc_set_wait_polls(int polls)
{
    if (polls < -1) return OC_ERR_INVALID;
    oc::tc_set_wait_polls(polls);
    return OC_OK;
}

// C (M x N, row-major, host) = A(m, k) B(k, n) with host operands and
// strides in elements, BF16 operands and FP32 accumulation, on the tensor
// cores (tensorCores 1) or the CUDA cores (0)
OC_EXPORT int oc_bf16_gemm(oc_ctx* ctx, int M, int N, int K, const float* A, long long sam, long long sak,
                           const float* B, long long sbk, long long sbn, float* C, int tensorCores)
{
    if (!ctx || !A || !B || !C || M <= 0 || N <= 0 || K <= 0 || sam < 0 || sak < 0 || sbk < 0 || sbn < 0)
        return OC_ERR_INVALID;
    const long long aSpan = (M - 1) * sam + (K - 1) * sak + 1, bSpan = (K - 1) * sbk + (N - 1) * sbn + 1;
    cudaStream_t st = oc::ctx_stream(ctx);
    float *dA = nullptr, *dB = nullptr, *dC = nullptr;
    int* dErr = nullptr;
    cudaError_t e = cudaMalloc(&dA, sizeof(float) * aSpan);
    if (e == cudaSuccess) e = cudaMalloc(&dB, sizeof(float) * bSpan);
    if (e == cudaSuccess) e = cudaMalloc(&dC, sizeof(float) * (size_t)M * N);
    if (e == cudaSuccess) e = cudaMalloc(&dErr, sizeof(int));
    if (e == cudaSuccess) e = cudaMemsetAsync(dErr, 0, sizeof(int), st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dA, A, sizeof(float) * aSpan, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dB, B, sizeof(float) * bSpan, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) {
        if (tensorCores) e = oc::gemm_tc(st, M, N, K, dA, sam, sak, dB, sbk, sbn, dC, N, 1.0f, 0.0f, nullptr, dErr);
        else oc::gemm_cuda_cores(st, M, N, K, dA, sam, sak, dB, sbk, sbn, dC, N, 1.0f, 0.0f, nullptr);
    }
    if (e == cudaSuccess) e = cudaGetLastError();
    int flag = 0;
    if (e == cudaSuccess) e = cudaMemcpyAsync(C, dC, sizeof(float) * (size_t)M * N, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, dErr, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    cudaFree(dA); cudaFree(dB); cudaFree(dC); cudaFree(dErr);
    if (e != cudaSuccess) return OC_ERR_CUDA;
    return flag ? OC_ERR_TIMEOUT : OC_OK;
}
