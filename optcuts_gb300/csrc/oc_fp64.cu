// FP64 per-triangle kernels of the geometry step: energy, gradient,
// inversion-free step bound, step forward, inversion check and the
// deterministic reductions behind them.
//
// This translation unit is compiled with -fmad=false so that every
// expression rounds exactly as the reference's scalar x86-64 code does
// (no fused multiply-add there either); with IEEE division and square root
// the per-triangle energies, gradients and step bounds are bit-identical to
// src/Energy/SymDirichletEnergy.cpp.  Sums over triangles use a fixed-order
// two-pass reduction, so results are deterministic run to run.

#include "oc_elem.cuh"
#include "oc_internal.h"

#include <algorithm>
#include <cstdint>
#include <mutex>

namespace oc {
namespace {

__device__ __forceinline__ double warp_sum(double v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}

// Block-wide sum of NT values per thread; thread 0 writes NT partials.
template <int NT>
__device__ __forceinline__ void block_sum_store(double (&v)[NT], int nTrials, double* out)
{
    __shared__ double sh[NT][32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < NT; ++k) {
        if (k < nTrials) {
            double s = warp_sum(v[k]);
            if (lane == 0) sh[k][warp] = s;
        }
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            if (k < nTrials) {
                double s = lane < nw ? sh[k][lane] : 0.0;
                s = warp_sum(s);
                if (lane == 0) out[k] = s;
            }
        }
    }
}

struct Corners {
    double2 U1, U2, U3;
};

__device__ __forceinline__ double2 at(const double2* uv, const double2* dir, double alpha, int v)
{
    double2 p = uv[v];
    if (dir) {
        const double2 d = dir[v];
        p.x = p.x + alpha * d.x;   // Optimizer::stepForward, Optimizer.cpp:667-668
        p.y = p.y + alpha * d.y;
    }
    return p;
}

template <int NT>
__global__ void __launch_bounds__(256) k_energy(DeviceMesh m, const double2* __restrict__ uv,
                                                const double2* __restrict__ dir, Alphas alphas, int nTrials,
                                                int uniform, double* partials)
{
    double acc[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) acc[k] = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m.nF; t += gridDim.x * blockDim.x) {
        const int i0 = m.F0[t], i1 = m.F1[t], i2 = m.F2[t];
        const double w = uniform ? 1.0 : m.w[t];
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            if (k < nTrials) {
                const double a = alphas.a[k];
                acc[k] += elem_energy(m, t, w, at(uv, dir, a, i0), at(uv, dir, a, i1), at(uv, dir, a, i2));
            }
        }
    }
    block_sum_store<NT>(acc, nTrials, partials + (size_t)blockIdx.x * kMaxTrials);
}

__global__ void k_energy_elem(DeviceMesh m, int uniform, double* out)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.nF) return;
    const double w = uniform ? 1.0 : m.w[t];
    out[t] = elem_energy(m, t, w, m.uv[m.F0[t]], m.uv[m.F1[t]], m.uv[m.F2[t]]);
}

// Fixed-order final reduction of nBlocks x nVals partials (single block).
__global__ void k_reduce_final(const double* partials, int nBlocks, int nVals, double* out)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ double sh[32];
    for (int k = 0; k < nVals; ++k) {
        double s = 0.0;
        for (int b = threadIdx.x; b < nBlocks; b += blockDim.x) s += partials[(size_t)b * kMaxTrials + k];
        s = warp_sum(s);
        if (lane == 0) sh[warp] = s;
        __syncthreads();
        if (warp == 0) {
            double v = lane < (int)(blockDim.x >> 5) ? sh[lane] : 0.0;
            v = warp_sum(v);
            if (lane == 0) out[k] = v;
        }
        __syncthreads();
    }
}

// Corner gradients of every triangle, written to cornerBuf[k * nF + t].
__global__ void __launch_bounds__(256) k_grad_corners(DeviceMesh m, int uniform, double2* __restrict__ cornerBuf)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.nF) return;
    double2 g[3];
    tri_corner_grads(m.uv[m.F0[t]], m.uv[m.F1[t]], m.uv[m.F2[t]], m.A2[t], m.e0[t], m.e1[t], m.e01[t],
                     uniform ? 1.0 : m.w[t], g);
    cornerBuf[t] = g[0];
    cornerBuf[m.nF + t] = g[1];
    cornerBuf[2 * m.nF + t] = g[2];
}

// Per-vertex gather in triangle order (the reference's scatter order), fixed
// rows zeroed (SymDirichletEnergy.cpp:300-303), times energyParams[0]
// (Optimizer.cpp:786); block partials of ||g||^2.
__global__ void __launch_bounds__(256) k_grad_gather(DeviceMesh m, const double2* __restrict__ cornerBuf, double scale,
                                                     double2* __restrict__ g, double* partials)
{
    double acc[1] = {0.0};
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < m.nV; v += gridDim.x * blockDim.x) {
        double sx = 0.0, sy = 0.0;
        for (int p = m.vcPtr[v]; p < m.vcPtr[v + 1]; ++p) {
            const double2 c = cornerBuf[m.vcIdx[p]];
            sx = sx + c.x;
            sy = sy + c.y;
        }
        if (m.fixedMask[v]) { sx = 0.0; sy = 0.0; }
        sx = scale * sx;
        sy = scale * sy;
        g[v] = make_double2(sx, sy);
        acc[0] += sx * sx + sy * sy;
    }
    block_sum_store<1>(acc, 1, partials + (size_t)blockIdx.x * kMaxTrials);
}

// Augmented gradient with a scaffold, over the whole vertex numbering (mesh
// vertices, then air-only vertices): Optimizer::computeGradient scales the
// mesh gradient by energyParams[0] (Optimizer.cpp:786), then
// Scaffold::augmentGradient (Scaffold.cpp:210-230) adds w * g_air on the
// boundary vertices and sets w * g_air on the air-only ones.  Both gathers
// follow triangle order; the air mesh's fixed rows are zeroed before the
// scaling, as SymDirichletEnergy::computeGradient does for any mesh.
__global__ void __launch_bounds__(256) k_grad_gather_scaf(DeviceMesh m, const double2* __restrict__ cornerBuf,
                                                          double scale, DeviceMesh a,
                                                          const double2* __restrict__ airCorner, double airScale,
                                                          double2* __restrict__ g, double* partials)
{
    double acc[1] = {0.0};
    for (int v = blockIdx.x * blockDim.x + threadIdx.x; v < a.nV; v += gridDim.x * blockDim.x) {
        double gx = 0.0, gy = 0.0;
        const bool onMesh = v < m.nV;
        if (onMesh) {
            double sx = 0.0, sy = 0.0;
            for (int p = m.vcPtr[v]; p < m.vcPtr[v + 1]; ++p) {
                const double2 c = cornerBuf[m.vcIdx[p]];
                sx = sx + c.x;
                sy = sy + c.y;
            }
            if (m.fixedMask[v]) { sx = 0.0; sy = 0.0; }
            gx = scale * sx;
            gy = scale * sy;
        }
        const int p0 = a.vcPtr[v], p1 = a.vcPtr[v + 1];
        if (p1 > p0) {
            double sx = 0.0, sy = 0.0;
            for (int p = p0; p < p1; ++p) {
                const double2 c = airCorner[a.vcIdx[p]];
                sx = sx + c.x;
                sy = sy + c.y;
            }
            if (a.fixedMask[v]) { sx = 0.0; sy = 0.0; }
            if (onMesh) {
                gx = gx + airScale * sx;
                gy = gy + airScale * sy;
            }
            else {
                gx = airScale * sx;
                gy = airScale * sy;
            }
        }
        g[v] = make_double2(gx, gy);
        acc[0] += gx * gx + gy * gy;
    }
    block_sum_store<1>(acc, 1, partials + (size_t)blockIdx.x * kMaxTrials);
}

// SymDirichletEnergy::initStepSize (SymDirichletEnergy.cpp:555-609); the
// minimum over triangles is taken with an atomicMin on the bit pattern of
// positive doubles (order-independent, hence deterministic).
__global__ void __launch_bounds__(256) k_init_step(DeviceMesh m, const double2* __restrict__ dir, double stepSize,
                                                   unsigned long long* minBits)
{
    double best = stepSize;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m.nF; t += gridDim.x * blockDim.x) {
        const int i0 = m.F0[t], i1 = m.F1[t], i2 = m.F2[t];
        const double bound = tri_step_bound(m.uv[i0], m.uv[i1], m.uv[i2], dir[i0], dir[i1], dir[i2], stepSize);
        if (bound < best) best = bound;
    }
    // block min via shuffles (exact), then one atomic per block
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) best = fmin(best, __shfl_down_sync(0xffffffffu, best, o));
    if ((threadIdx.x & 31) == 0) {
        // every bound of a valid (non-inverted) triangle is positive; a
        // non-positive or NaN bound is clamped to 0 so the host sees it
        const double v = (best > 0.0) ? best : 0.0;
        atomicMin(minBits, static_cast<unsigned long long>(__double_as_longlong(v)));
    }
}

// Three blocks per SM (168 registers, a few hundred bytes spilled) against
// two at the unconstrained 218 registers: 2.38 -> 2.34 ms for the Hessian
// phase of a 199k-triangle Newton step, the same bits.
__global__ void __launch_bounds__(128, 3) k_hessian(DeviceMesh m, int uniform, double* __restrict__ hb)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.nF) return;
    const double2 U[3] = {m.uv[m.F0[t]], m.uv[m.F1[t]], m.uv[m.F2[t]]};
    double H[6][6];
    tri_hessian(U, m.A2[t], m.e0d[t], m.e1d[t], m.e01d[t], uniform ? 1.0 : m.w[t], H);
    store_hessian_blocks(H, t, m.nF, hb);
}

__global__ void k_set_bits(unsigned long long* dst, double v)
{
    *dst = static_cast<unsigned long long>(__double_as_longlong(v));
}

__global__ void k_step_forward(const double2* __restrict__ uv0, const double2* __restrict__ dir, double alpha,
                               double2* __restrict__ uv, int nV)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= nV) return;
    const double2 p = uv0[v], d = dir[v];
    uv[v] = make_double2(p.x + alpha * d.x, p.y + alpha * d.y);
}

// TriMesh::checkInversion (TriMesh.cpp:1710-1756): count of triangles with
// signed double area < 0, into minBits (as a plain counter).
__global__ void k_check_inversion(DeviceMesh m, unsigned long long* count)
{
    unsigned int bad = 0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < m.nF; t += gridDim.x * blockDim.x) {
        const double2 U1 = m.uv[m.F0[t]], U2 = m.uv[m.F1[t]], U3 = m.uv[m.F2[t]];
        const double e00 = U2.x - U1.x, e01 = U2.y - U1.y, e10 = U3.x - U1.x, e11 = U3.y - U1.y;
        const double dbArea = e00 * e11 - e01 * e10;
        if (dbArea < 0.0) ++bad;
    }
    for (int o = 16; o > 0; o >>= 1) bad += __shfl_down_sync(0xffffffffu, bad, o);
    if ((threadIdx.x & 31) == 0 && bad) atomicAdd(count, static_cast<unsigned long long>(bad));
}

// SymDirichletEnergy::computeDivGradPerVert with its standard-deviation
// filter (SymDirichletEnergy.cpp:108-147): per vertex, the standard
// deviation of its incident corner gradients (mean and deviations summed in
// triangle order; 0 for a vertex with one incident triangle).
__global__ void __launch_bounds__(256) k_divgrad(DeviceMesh m, const double2* __restrict__ cornerBuf,
                                                 double* __restrict__ out)
{
    const int v = blockIdx.x * blockDim.x + threadIdx.x;
    if (v >= m.nV) return;
    const int p0 = m.vcPtr[v], p1 = m.vcPtr[v + 1];
    const int n = p1 - p0;
    double mx = 0.0, my = 0.0;
    for (int p = p0; p < p1; ++p) {
        const double2 c = cornerBuf[m.vcIdx[p]];
        mx = mx + c.x;
        my = my + c.y;
    }
    mx = mx / n;
    my = my / n;
    double sd = 0.0;
    for (int p = p0; p < p1; ++p) {
        const double2 c = cornerBuf[m.vcIdx[p]];
        const double dx = c.x - mx, dy = c.y - my;
        sd = sd + (dx * dx + dy * dy);
    }
    out[v] = (n == 1) ? 0.0 : sqrt(sd / (n - 1.0));
}

} // namespace

int reduce_blocks_for(int n)
{
    int b = (n + 255) / 256;
    if (b > kMaxReduceBlocks) b = kMaxReduceBlocks;
    return b < 1 ? 1 : b;
}

// ------------------------------------------------- allocation-free energy
// Variant of k_energy for caller-owned, reference-layout device arrays (F
// nF x 3, rest nF x 8), with its block partials in a file-scope device array
// instead of an allocation.  Callers that cannot allocate (a host framework
// owning all device memory, externally captured graphs) use it through
// oc_sd_energy_trials_noalloc.
namespace {

constexpr int kNoAllocBlocks = kMaxReduceBlocks;
static __device__ __align__(256) double g_noallocPartials[kNoAllocBlocks * kMaxTrials];

template <int NT>
__global__ void __launch_bounds__(256) k_energy_aos(const int* __restrict__ F, const double2* __restrict__ uv,
                                                    const double2* __restrict__ dir, const double* __restrict__ rest,
                                                    double surfaceArea, int nF, Alphas alphas, int nTrials,
                                                    int uniform, double* partials)
{
    double acc[NT];
#pragma unroll
    for (int k = 0; k < NT; ++k) acc[k] = 0.0;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nF; t += gridDim.x * blockDim.x) {
        const int i0 = F[3 * t], i1 = F[3 * t + 1], i2 = F[3 * t + 2];
        const double* r = rest + 8 * (size_t)t;
        const double w = uniform ? 1.0 : r[0] / surfaceArea;
        const double A2 = r[1], e0 = r[2], e1 = r[3], e01 = r[4];
#pragma unroll
        for (int k = 0; k < NT; ++k) {
            if (k < nTrials) {
                const double a = alphas.a[k];
                const double2 U1 = at(uv, dir, a, i0), U2 = at(uv, dir, a, i1), U3 = at(uv, dir, a, i2);
                const double a0 = U2.x - U1.x, a1 = U2.y - U1.y;
                const double b0 = U3.x - U1.x, b1 = U3.y - U1.y;
                const double area_U = 0.5 * (a0 * b1 - a1 * b0);
                acc[k] += w * (1.0 + A2 / area_U / area_U) *
                          (((b0 * b0 + b1 * b1) * e0 + (a0 * a0 + a1 * a1) * e1) / 4 / A2 -
                           (b0 * a0 + b1 * a1) * e01 / 2 / A2);
            }
        }
    }
    block_sum_store<NT>(acc, nTrials, partials + (size_t)blockIdx.x * kMaxTrials);
}

std::mutex g_noallocMu;
double* g_noallocPtr[256] = {};

} // namespace

void launch_hessian(const DeviceMesh& m, int uniform, double* hb, cudaStream_t st, int projection)
{
    if (projection == OC_HESSIAN_REDUCED) return launch_hessian_reduced(m, uniform, hb, st, 0.0);
    if (projection == OC_HESSIAN_HYBRID) return launch_hessian_reduced(m, uniform, hb, st, kHybridDensity);
    k_hessian<<<(m.nF + 127) / 128, 128, 0, st>>>(m, uniform, hb);
}

void launch_reduce_final(Scratch& s, int nBlocks, int nVals, cudaStream_t st, double* out)
{
    k_reduce_final<<<1, 256, 0, st>>>(s.partials, nBlocks, nVals, out ? out : s.result);
}

void launch_energy(const DeviceMesh& m, const double2* uv, const double2* dir, const double* alphas, int nTrials,
                   int uniform, double scale, Scratch& s, cudaStream_t st, double* out)
{
    (void)scale;
    Alphas a = {{0, 0, 0, 0, 0, 0, 0, 0}};
    for (int k = 0; k < nTrials && k < 8; ++k) a.a[k] = alphas ? alphas[k] : 0.0;
    const int nb = reduce_blocks_for(m.nF);
    if (nTrials <= 1)
        k_energy<1><<<nb, 256, 0, st>>>(m, uv, dir, a, 1, uniform, s.partials);
    else if (nTrials <= 4)
        k_energy<4><<<nb, 256, 0, st>>>(m, uv, dir, a, nTrials, uniform, s.partials);
    else
        k_energy<8><<<nb, 256, 0, st>>>(m, uv, dir, a, nTrials, uniform, s.partials);
    launch_reduce_final(s, nb, nTrials < 1 ? 1 : nTrials, st, out);
}

void launch_energy_elem(const DeviceMesh& m, int uniform, double* out, cudaStream_t st)
{
    k_energy_elem<<<(m.nF + 255) / 256, 256, 0, st>>>(m, uniform, out);
}

void launch_gradient(const DeviceMesh& m, int uniform, double scale, double2* cornerBuf, double2* g, Scratch& s,
                     cudaStream_t st)
{
    k_grad_corners<<<(m.nF + 255) / 256, 256, 0, st>>>(m, uniform, cornerBuf);
    const int nb = reduce_blocks_for(m.nV);
    k_grad_gather<<<nb, 256, 0, st>>>(m, cornerBuf, scale, g, s.partials);
    launch_reduce_final(s, nb, 1, st);
}

void launch_gradient_scaf(const DeviceMesh& m, double scale, double2* cornerBuf, const DeviceMesh& air,
                          double airScale, double2* airCornerBuf, double2* g, Scratch& s, cudaStream_t st)
{
    k_grad_corners<<<(m.nF + 255) / 256, 256, 0, st>>>(m, 0, cornerBuf);
    k_grad_corners<<<(air.nF + 255) / 256, 256, 0, st>>>(air, 1, airCornerBuf);
    const int nb = reduce_blocks_for(air.nV);
    k_grad_gather_scaf<<<nb, 256, 0, st>>>(m, cornerBuf, scale, air, airCornerBuf, airScale, g, s.partials);
    launch_reduce_final(s, nb, 1, st);
}

void launch_init_step(const DeviceMesh& m, const double2* dir, double stepSize, Scratch& s, cudaStream_t st,
                      bool reset)
{
    if (reset) k_set_bits<<<1, 1, 0, st>>>(s.minBits, stepSize);
    k_init_step<<<reduce_blocks_for(m.nF), 256, 0, st>>>(m, dir, stepSize, s.minBits);
}

void launch_divgrad(const DeviceMesh& m, double2* cornerBuf, double* divGrad, cudaStream_t st)
{
    k_grad_corners<<<(m.nF + 255) / 256, 256, 0, st>>>(m, 0, cornerBuf);
    k_divgrad<<<(m.nV + 255) / 256, 256, 0, st>>>(m, cornerBuf, divGrad);
}

void launch_step_forward(const double2* uv0, const double2* dir, double alpha, double2* uv, int nV, cudaStream_t st)
{
    k_step_forward<<<(nV + 255) / 256, 256, 0, st>>>(uv0, dir, alpha, uv, nV);
}

void launch_check_inversion(const DeviceMesh& m, Scratch& s, cudaStream_t st)
{
    cudaMemsetAsync(s.minBits, 0, sizeof(unsigned long long), st);
    k_check_inversion<<<reduce_blocks_for(m.nF), 256, 0, st>>>(m, s.minBits);
}

// Device address of the file-scope partials array for the current device;
// looked up once per device (host code cannot use the symbol directly: its
// host-side name is only a stand-in for the device array).
static int noalloc_scratch(double** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 256) return OC_ERR_CUDA;
    std::lock_guard<std::mutex> lock(g_noallocMu);
    if (!g_noallocPtr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noallocPartials) != cudaSuccess || !p) return OC_ERR_CUDA;
        g_noallocPtr[dev] = static_cast<double*>(p);
    }
    *out = g_noallocPtr[dev];
    return OC_OK;
}

} // namespace oc

extern "C" __attribute__((visibility("default"))) int
oc_sd_energy_trials_noalloc(const int* F, const double* UV, const double* dir, const double* rest, double surfaceArea,
                            int nF, const double* alphas, int nTrials, int uniformWeight, double* energies,
                            void* stream)
{
    using namespace oc;
    if (!F || !UV || !rest || !energies || nF <= 0 || !(surfaceArea > 0.0)) return OC_ERR_INVALID;
    if (nTrials < 1 || nTrials > kMaxTrials) return OC_ERR_INVALID;   // scratch holds 8 trials per block
    if (dir && !alphas) return OC_ERR_INVALID;
    double* partials = nullptr;
    int rc = noalloc_scratch(&partials);
    if (rc) return rc;
    Alphas a = {{0, 0, 0, 0, 0, 0, 0, 0}};
    for (int k = 0; k < nTrials; ++k) a.a[k] = alphas ? alphas[k] : 0.0;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    const int nb = reduce_blocks_for(nF);
    if (nb > kNoAllocBlocks) return OC_ERR_INVALID;   // the static partials hold kNoAllocBlocks blocks
    const double2* uv = reinterpret_cast<const double2*>(UV);
    const double2* d = reinterpret_cast<const double2*>(dir);
    if (nTrials == 1)
        k_energy_aos<1><<<nb, 256, 0, st>>>(F, uv, d, rest, surfaceArea, nF, a, 1, uniformWeight, partials);
    else if (nTrials <= 4)
        k_energy_aos<4><<<nb, 256, 0, st>>>(F, uv, d, rest, surfaceArea, nF, a, nTrials, uniformWeight, partials);
    else
        k_energy_aos<8><<<nb, 256, 0, st>>>(F, uv, d, rest, surfaceArea, nF, a, nTrials, uniformWeight, partials);
    k_reduce_final<<<1, 256, 0, st>>>(partials, nb, nTrials, energies);
    return cudaGetLastError() == cudaSuccess ? OC_OK : OC_ERR_CUDA;
}
