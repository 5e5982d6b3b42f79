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

#include "oc_internal.h"

#include <cooperative_groups.h>

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

// SymDirichletEnergy::getEnergyValPerElem body (SymDirichletEnergy.cpp:32-44).
__device__ __forceinline__ double elem_energy(const DeviceMesh& m, int t, double w, const double2 U1,
                                              const double2 U2, const double2 U3)
{
    const double a0 = U2.x - U1.x, a1 = U2.y - U1.y;   // U2m1
    const double b0 = U3.x - U1.x, b1 = U3.y - U1.y;   // U3m1
    const double area_U = 0.5 * (a0 * b1 - a1 * b0);
    const double A2 = m.A2[t];
    return w * (1.0 + A2 / area_U / area_U) *
           (((b0 * b0 + b1 * b1) * m.e0[t] + (a0 * a0 + a1 * a1) * m.e1[t]) / 4 / A2 -
            (b0 * a0 + b1 * a1) * m.e01[t] / 2 / A2);
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

// SymDirichletEnergy::computeGradient per-corner terms (SymDirichletEnergy.cpp:
// 267-297; also computeLocalGradient, :215-256) of one triangle.
__device__ __forceinline__ void tri_corner_grads(const double2 U1, const double2 U2, const double2 U3, double A2,
                                                 double e0, double e1, double e01, double w, double2 g[3])
{
    const double a0 = U2.x - U1.x, a1 = U2.y - U1.y;   // U2m1
    const double b0 = U3.x - U1.x, b1 = U3.y - U1.y;   // U3m1
    const double area_U = 0.5 * (a0 * b1 - a1 * b0);
    const double leftTerm = 1.0 + A2 / area_U / area_U;
    const double rightTerm = ((b0 * b0 + b1 * b1) * e0 + (a0 * a0 + a1 * a1) * e1) / 4 / A2 -
                             (b0 * a0 + b1 * a1) * e01 / 2 / A2;
    const double areaRatio = A2 / area_U / area_U / area_U;
    {
        const double eo0 = U3.x - U2.x, eo1 = U3.y - U2.y;
        const double dL0 = areaRatio * eo1, dL1 = areaRatio * -eo0;
        const double dR0 = ((e01 - e0) * b0 + (e01 - e1) * a0) / 2.0 / A2;
        const double dR1 = ((e01 - e0) * b1 + (e01 - e1) * a1) / 2.0 / A2;
        g[0] = make_double2(w * (dL0 * rightTerm + dR0 * leftTerm), w * (dL1 * rightTerm + dR1 * leftTerm));
    }
    {
        const double eo0 = U1.x - U3.x, eo1 = U1.y - U3.y;
        const double dL0 = areaRatio * eo1, dL1 = areaRatio * -eo0;
        const double dR0 = (e1 * a0 - e01 * b0) / 2.0 / A2;
        const double dR1 = (e1 * a1 - e01 * b1) / 2.0 / A2;
        g[1] = make_double2(w * (dL0 * rightTerm + dR0 * leftTerm), w * (dL1 * rightTerm + dR1 * leftTerm));
    }
    {
        const double eo0 = U2.x - U1.x, eo1 = U2.y - U1.y;
        const double dL0 = areaRatio * eo1, dL1 = areaRatio * -eo0;
        const double dR0 = (e0 * b0 - e01 * a0) / 2.0 / A2;
        const double dR1 = (e0 * b1 - e01 * a1) / 2.0 / A2;
        g[2] = make_double2(w * (dL0 * rightTerm + dR0 * leftTerm), w * (dL1 * rightTerm + dR1 * leftTerm));
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

// SymDirichletEnergy::initStepSize per triangle (SymDirichletEnergy.cpp:
// 555-609): the bound from det(U + alpha V) > 0, or stepSize when none.
__device__ __forceinline__ double tri_step_bound(const double2 U1, const double2 U2, const double2 U3, const double2 V1,
                                                 const double2 V2, const double2 V3, double stepSize)
{
    const double U2m1x = U2.x - U1.x, U2m1y = U2.y - U1.y;
    const double U3m1x = U3.x - U1.x, U3m1y = U3.y - U1.y;
    const double V2m1x = V2.x - V1.x, V2m1y = V2.y - V1.y;
    const double V3m1x = V3.x - V1.x, V3m1y = V3.y - V1.y;
    const double a = V2m1x * V3m1y - V2m1y * V3m1x;
    const double b = U2m1x * V3m1y - U2m1y * V3m1x + V2m1x * U3m1y - V2m1y * U3m1x;
    const double c = U2m1x * U3m1y - U2m1y * U3m1x;
    const double delta = b * b - 4.0 * a * c;
    double bound = stepSize;
    if (a > 0.0) {
        if ((b < 0.0) && (delta >= 0.0)) bound = 2.0 * c / (-b + sqrt(delta));
    }
    else if (a < 0.0) {
        if (b < 0.0) bound = 2.0 * c / (-b + sqrt(delta));
        else bound = (-b - sqrt(delta)) / 2.0 / a;
    }
    else {
        if (b < 0.0) bound = -c / b;
    }
    return bound;
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

// Cyclic Jacobi eigen-decomposition of a symmetric 6x6: A is destroyed (its
// diagonal holds the eigenvalues), V receives the eigenvectors as columns.
__device__ void jacobi_eig6(double A[6][6], double V[6][6])
{
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
    double fro = 0.0;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) fro += A[i][j] * A[i][j];
    double prevOff = 0.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < 6; ++p)
            for (int q = p + 1; q < 6; ++q) off += A[p][q] * A[p][q];
        // converged, or no longer decreasing (the off-diagonal mass has
        // reached the rounding floor, below which 1e-34 is not reachable)
        if (off <= 1e-34 * fro || (sweep > 0 && off >= prevOff)) break;
        prevOff = off;
        for (int p = 0; p < 6; ++p) {
            for (int q = p + 1; q < 6; ++q) {
                const double apq = A[p][q];
                if (apq == 0.0) continue;
                const double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(theta * theta + 1.0));
                const double c = 1.0 / sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < 6; ++k) {
                    const double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < 6; ++k) {
                    const double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < 6; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
        }
    }
}

// Cyclic Jacobi eigen-decomposition of a symmetric 4x4 (A destroyed: its
// diagonal holds the eigenvalues; V the eigenvectors as columns); stops at
// convergence or when the off-diagonal mass stops decreasing.
template <typename T>
__device__ void jacobi_eig4(T A[4][4], T V[4][4], T tol)
{
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) V[i][j] = (i == j) ? T(1) : T(0);
    T fro = T(0);
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) fro += A[i][j] * A[i][j];
    T prevOff = T(0);
    for (int sweep = 0; sweep < 40; ++sweep) {
        T off = T(0);
        for (int p = 0; p < 4; ++p)
            for (int q = p + 1; q < 4; ++q) off += A[p][q] * A[p][q];
        if (off <= tol * fro || (sweep > 0 && off >= prevOff)) break;
        prevOff = off;
        for (int p = 0; p < 4; ++p)
            for (int q = p + 1; q < 4; ++q) {
                const T apq = A[p][q];
                if (apq == T(0)) continue;
                const T theta = (A[q][q] - A[p][p]) / (T(2) * apq);
                const T t = (theta >= T(0) ? T(1) : T(-1)) / (fabs(theta) + sqrt(theta * theta + T(1)));
                const T c = T(1) / sqrt(t * t + T(1)), sn = t * c;
                for (int k = 0; k < 4; ++k) {
                    const T akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - sn * akq;
                    A[k][q] = sn * akp + c * akq;
                }
                for (int k = 0; k < 4; ++k) {
                    const T apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - sn * aqk;
                    A[q][k] = sn * apk + c * aqk;
                }
                for (int k = 0; k < 4; ++k) {
                    const T vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - sn * vkq;
                    V[k][q] = sn * vkp + c * vkq;
                }
            }
    }
}

// makePD of a triangle's 6x6 Hessian for the local topology solves, in the
// 4-dimensional complement of the two rigid translations (H t = 0 for them,
// so H = Q K Q^T with K = Q^T H Q): Q = B (x) I2, B the orthonormal 3x2 basis
// [-1/sqrt2, -1/sqrt6; 1/sqrt2, -1/sqrt6; 0, 2/sqrt6] of the vectors
// orthogonal to (1, 1, 1).  K PSD up to -1e-13 of its largest diagonal
// leaves H unchanged (makePD's early return); otherwise K = V Lambda V^T,
// negative eigenvalues clamped to zero and H = (Q V) Lambda+ (Q V)^T: the same
// projection as the 6x6 eigen-clamp, at about a fifth of its arithmetic.
// T = float projects in FP32 (scaled by the largest |K_ii|).
template <typename T>
__device__ void project_psd_reduced(double H[6][6])
{
    const double r2 = 0.70710678118654752440, r6 = 0.40824829046386301637;
    const double B[3][2] = {{-r2, -r6}, {r2, -r6}, {0.0, 2.0 * r6}};
    double Tm[4][6];   // Q^T H
    for (int k = 0; k < 2; ++k)
        for (int b = 0; b < 2; ++b)
            for (int c = 0; c < 6; ++c) {
                double acc = 0.0;
                for (int i = 0; i < 3; ++i) acc = acc + B[i][k] * H[2 * i + b][c];
                Tm[2 * k + b][c] = acc;
            }
    double K[4][4];
    for (int r = 0; r < 4; ++r)
        for (int l = 0; l < 2; ++l)
            for (int d = 0; d < 2; ++d) {
                double acc = 0.0;
                for (int j = 0; j < 3; ++j) acc = acc + Tm[r][2 * j + d] * B[j][l];
                K[r][2 * l + d] = acc;
            }
    for (int r = 0; r < 4; ++r)   // symmetric up to rounding: use the mean
        for (int c = r + 1; c < 4; ++c) {
            const double m = 0.5 * (K[r][c] + K[c][r]);
            K[r][c] = m;
            K[c][r] = m;
        }
    double dmax = 0.0;
    for (int i = 0; i < 4; ++i) dmax = fmax(dmax, fabs(K[i][i]));
    {   // LDL^T without pivoting: no pivot below -1e-13 dmax -> PSD
        double A[4][4];
        for (int i = 0; i < 4; ++i)
            for (int j = 0; j < 4; ++j) A[i][j] = K[i][j];
        const double tol = 1e-13 * dmax;
        bool psd = true;
        for (int k = 0; k < 4 && psd; ++k) {
            const double d = A[k][k];
            if (d < -tol) psd = false;
            else if (d > tol)
                for (int i = k + 1; i < 4; ++i) {
                    const double l = A[i][k] / d;
                    for (int j = k + 1; j <= i; ++j) A[i][j] = A[i][j] - l * A[j][k];
                }
        }
        if (psd) return;
    }
    const double scale = dmax > 0.0 ? dmax : 1.0;
    T A[4][4], V[4][4];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) A[i][j] = static_cast<T>(K[i][j] / scale);
    jacobi_eig4<T>(A, V, sizeof(T) == 8 ? T(1e-34) : T(1e-14));
    double lam[4];
    for (int m = 0; m < 4; ++m) lam[m] = A[m][m] < T(0) ? 0.0 : static_cast<double>(A[m][m]) * scale;
    double W[6][4];   // Q V
    for (int i = 0; i < 3; ++i)
        for (int a = 0; a < 2; ++a)
            for (int m = 0; m < 4; ++m)
                W[2 * i + a][m] = B[i][0] * static_cast<double>(V[a][m]) + B[i][1] * static_cast<double>(V[2 + a][m]);
    for (int r = 0; r < 6; ++r)
        for (int c = r; c < 6; ++c) {
            double acc = 0.0;
            for (int m = 0; m < 4; ++m) acc = acc + W[r][m] * lam[m] * W[c][m];
            H[r][c] = acc;
            H[c][r] = acc;
        }
}

// Per-triangle Hessian (SymDirichletEnergy.cpp:440-522) projected to PSD by
// the 6x6 eigen-clamp of IglUtils::makePD (IglUtils.hpp:71-90): unchanged
// when the smallest eigenvalue is >= 0, otherwise V max(Lambda, 0) V^T.
// The full 6x6 decomposition matters: for stiff elements (entries up to
// ~1e26 at a Tutte start) the rounding-level translation components it keeps
// change the Newton direction, and reducing to the 4-dimensional
// translation-free part first does not reproduce the reference.
// Output: the upper triangle as 21 values per triangle (SoA).
// localMode 0: exact (the global Newton); 1: the reduced 4x4 projection
// (local solves, FP64); 2: as 1 with the eigen-decomposition in FP32
__device__ void tri_hessian(const double2 U[3], double triAreaSq, double e0d, double e1d, double e01d, double w,
                            double H[6][6], int localMode = 0)
{
    const double U2m1[2] = {U[1].x - U[0].x, U[1].y - U[0].y};
    const double U3m1[2] = {U[2].x - U[0].x, U[2].y - U[0].y};
    const double area_U = 0.5 * (U2m1[0] * U3m1[1] - U2m1[1] * U3m1[0]);
    const double areaRatio = triAreaSq / area_U / area_U / area_U;
    const double dAR = 3.0 / 2.0 * areaRatio / area_U;
    const double leftTerm = 1.0 + triAreaSq / area_U / area_U;
    const double rightTerm = ((U3m1[0] * U3m1[0] + U3m1[1] * U3m1[1]) * e0d +
                              (U2m1[0] * U2m1[0] + U2m1[1] * U2m1[1]) * e1d) / 2. -
                             (U3m1[0] * U2m1[0] + U3m1[1] * U2m1[1]) * e01d;
    double ort[3][2];
    ort[0][0] = U[2].y - U[1].y; ort[0][1] = -(U[2].x - U[1].x);
    ort[1][0] = U[0].y - U[2].y; ort[1][1] = -(U[0].x - U[2].x);
    ort[2][0] = U[1].y - U[0].y; ort[2][1] = -(U[1].x - U[0].x);
    double dL[3][2], dR[3][2];
    for (int k = 0; k < 3; ++k) { dL[k][0] = areaRatio * ort[k][0]; dL[k][1] = areaRatio * ort[k][1]; }
    for (int c = 0; c < 2; ++c) {
        dR[0][c] = (e01d - e0d) * U3m1[c] + (e01d - e1d) * U2m1[c];
        dR[1][c] = e1d * U2m1[c] - e01d * U3m1[c];
        dR[2][c] = e0d * U3m1[c] - e01d * U2m1[c];
    }
    const double d2R[3][3] = {{e0d + e1d - 2.0 * e01d, e01d - e1d, e01d - e0d},
                              {e01d - e1d, e1d, -e01d},
                              {e01d - e0d, -e01d, e0d}};
    const double skew[3][3] = {{0, 1, -1}, {-1, 0, 1}, {1, -1, 0}};
    for (int i = 0; i < 3; ++i) {
        for (int j = i; j < 3; ++j) {
            for (int a = 0; a < 2; ++a) {
                for (int b = 0; b < 2; ++b) {
                    double d2L = dAR * ort[i][a] * ort[j][b];
                    if (i != j) d2L += areaRatio * skew[i][j] * ((a == 0 && b == 1) ? -1.0 : ((a == 1 && b == 0) ? 1.0 : 0.0));
                    const double v = w * (d2L * rightTerm + dL[i][a] * dR[j][b] +
                                          (a == b ? d2R[i][j] * leftTerm : 0.0) + dR[i][a] * dL[j][b]);
                    H[2 * i + a][2 * j + b] = v;
                    H[2 * j + b][2 * i + a] = v;
                }
            }
        }
    }
    if (localMode == 1) {
        project_psd_reduced<double>(H);
        return;
    }
    if (localMode == 2) {
        project_psd_reduced<float>(H);
        return;
    }
    double A[6][6], V[6][6];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) A[i][j] = H[i][j];
    jacobi_eig6(A, V);
    double lam[6], lmin = A[0][0];
    for (int i = 0; i < 6; ++i) {
        lam[i] = A[i][i];
        if (lam[i] < lmin) lmin = lam[i];
    }
    if (lmin < 0.0) {
        for (int i = 0; i < 6; ++i)
            if (lam[i] < 0.0) lam[i] = 0.0;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) {
                double s = 0.0;
                for (int k = 0; k < 6; ++k) s += V[i][k] * lam[k] * V[j][k];
                H[i][j] = s;
            }
    }
}

__global__ void __launch_bounds__(128) k_hessian(DeviceMesh m, int uniform, double* __restrict__ hb)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.nF) return;
    const int nF = m.nF;
    const double2 U[3] = {m.uv[m.F0[t]], m.uv[m.F1[t]], m.uv[m.F2[t]]};
    double H[6][6];
    tri_hessian(U, m.A2[t], m.e0d[t], m.e1d[t], m.e01d[t], uniform ? 1.0 : m.w[t], H);
    for (int a = 0; a < 3; ++a) {
        hb[(3 * a + 0) * (size_t)nF + t] = H[2 * a][2 * a];
        hb[(3 * a + 1) * (size_t)nF + t] = H[2 * a][2 * a + 1];
        hb[(3 * a + 2) * (size_t)nF + t] = H[2 * a + 1][2 * a + 1];
    }
    for (int a = 0; a < 3; ++a)
        for (int b = a + 1; b < 3; ++b) {
            const int p = a + b - 1;   // (0,1) -> 0, (0,2) -> 1, (1,2) -> 2
            for (int i = 0; i < 2; ++i)
                for (int j = 0; j < 2; ++j) hb[(9 + 4 * p + 2 * i + j) * (size_t)nF + t] = H[2 * a + i][2 * b + j];
        }
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

// ---------------------------------------------------- local topology solves
// The projected-Newton loop the reference runs on a candidate's local mesh
// (Optimizer with useDense, energyParams {1}, relGL2Tol 1e-6,
// solve(maxIter): Optimizer.cpp:203-261, 505-652; dense Hessian
// SymDirichletEnergy.cpp:306-427 + LDLT), one local problem per group of
// TPP threads (CL = 1) or per thread-block cluster of CL blocks of TPP
// threads.  Threads own triangles; a block sums its contiguous range of
// triangles in triangle order on single threads, and a cluster adds its
// blocks' partial sums in rank order (every block reads them all through
// distributed shared memory, so all blocks hold the same totals and run
// the same serial steps).  The arithmetic depends only on (TPP, CL), which
// the host picks from the triangle count, so results are deterministic.
// TPP 8 and 32 pack several problems into a 128-thread block (sub-warp
// groups); TPP 128 gives one problem a block; clusters spread the
// few-hundred-triangle fans around high-valence vertices over several SMs.
namespace cg = cooperative_groups;

constexpr int kLocalParts = 36;   // values combined across a cluster at once

template <int TPP>
struct LocalShared {
    double2 pos[kLocalMaxFree], pos0[kLocalMaxFree];
    double dir[2 * kLocalMaxFree], g[2 * kLocalMaxFree];
    double H[2 * kLocalMaxFree][2 * kLocalMaxFree];
    double bc[2];                      // broadcast slots
    double part[2][kLocalParts];       // cluster partials (double-buffered)
    double triE[TPP];
    double triG[TPP][6];
    double triH[TPP][21];
    int triSlot[TPP][3];
};

template <int TPP, int CL>
struct LocalGroup {
    unsigned mask;
    int sub, rank, buf;
    __device__ __forceinline__ void sync() const
    {
        if constexpr (TPP <= 32) __syncwarp(mask);
        else __syncthreads();
    }
};

// largest block: 128 threads (several problems per block for TPP <= 32)
template <int TPP, int CL>
__host__ __device__ constexpr int local_threads() { return (TPP >= 128 || CL > 1) ? TPP : 128; }

template <int TPP, int CL>
constexpr size_t local_smem(int threads) { return (threads / TPP) * sizeof(LocalShared<TPP>); }

__device__ __forceinline__ int sym21(int i, int j)   // packed upper triangle of a 6x6
{
    if (i > j) { const int t = i; i = j; j = t; }
    return i * 6 - i * (i - 1) / 2 + (j - i);
}

// corner positions and free slots of local triangle t, at pos (+ alpha dir)
template <int TPP>
__device__ __forceinline__ void local_corners(const LocalBatch& b, const LocalProblem& P, const LocalShared<TPP>& S,
                                              int t, const double2* pos, bool withDir, double alpha, double2 U[3],
                                              int slot[3])
{
    for (int k = 0; k < 3; ++k) {
        const int lv = b.ltCorner[3 * (P.triOff + t) + k];
        const int sl = b.lvSlot[P.vertOff + lv];
        slot[k] = sl;
        if (sl >= 0) {
            double2 p = pos[sl];
            if (withDir) {
                p.x = p.x + alpha * S.dir[2 * sl];
                p.y = p.y + alpha * S.dir[2 * sl + 1];
            }
            U[k] = p;
        }
        else {
            U[k] = b.lvPos[P.vertOff + lv];
        }
    }
}

// value computed by the group's first thread, seen by all
template <int TPP, int CL>
__device__ __forceinline__ double local_bcast(LocalShared<TPP>& S, const LocalGroup<TPP, CL>& G, double v)
{
    if (G.sub == 0) S.bc[0] = v;
    G.sync();
    v = S.bc[0];
    G.sync();
    return v;
}

// Combines per-block partials across the cluster: the thread owning `slot`
// (>= 0) gets the rank-ordered sum (op 0), min (1) or max (2) of every
// block's value of that slot.  Called by every thread of the cluster.
template <int TPP, int CL>
__device__ __forceinline__ double cluster_combine(LocalShared<TPP>& S, LocalGroup<TPP, CL>& G, double v, int slot,
                                                  int op)
{
    if constexpr (CL == 1) {
        return v;
    }
    else {
        double* part = S.part[G.buf];
        if (slot >= 0) part[slot] = v;
        cg::cluster_group cl = cg::this_cluster();
        cl.sync();
        double tot = v;
        if (slot >= 0)
            for (int r = 0; r < CL; ++r) {
                const double x = cl.map_shared_rank(part, r)[slot];
                tot = r == 0 ? x : (op == 0 ? tot + x : (op == 1 ? fmin(tot, x) : fmax(tot, x)));
            }
        // the other buffer next time: a block rewrites this one only after
        // the next combine's cluster barrier, when every read of it is done
        G.buf ^= 1;
        return tot;
    }
}

// local energy (weights triArea / localArea) at pos0 + alpha dir or at pos,
// over triangles [lo, hi) of this block, combined across the cluster
template <int TPP, int CL>
__device__ double local_energy(const DeviceMesh& m, const LocalBatch& b, const LocalProblem& P, LocalShared<TPP>& S,
                               LocalGroup<TPP, CL>& G, int lo, int hi, const double2* pos, bool withDir,
                               double alpha)
{
    double acc = 0.0;
    for (int c0 = lo; c0 < hi; c0 += TPP) {
        const int t = c0 + G.sub;
        double e = 0.0;
        if (t < hi) {
            double2 U[3];
            int sl[3];
            local_corners(b, P, S, t, pos, withDir, alpha, U, sl);
            const int g = b.ltGlobal[P.triOff + t];
            e = elem_energy(m, g, m.area[g] / P.localArea, U[0], U[1], U[2]);
        }
        S.triE[G.sub] = e;
        G.sync();
        if (G.sub == 0) {
            const int n = min(TPP, hi - c0);
            for (int k = 0; k < n; ++k) acc = acc + S.triE[k];
        }
        G.sync();
    }
    acc = cluster_combine(S, G, acc, G.sub == 0 ? 0 : -1, 0);
    return local_bcast(S, G, acc);
}

template <int TPP, int CL>
__global__ void __launch_bounds__(local_threads<TPP, CL>(), (TPP >= 128 || CL > 1) ? 1 : 3)
    k_local_newton(DeviceMesh m, double surfaceArea, LocalBatch b)
{
    static_assert(CL == 1 || TPP >= kLocalParts, "a cluster block must own every Hessian entry");
    extern __shared__ __align__(16) unsigned char localSmem[];
    const int groups = static_cast<int>(blockDim.x) / TPP;   // problems per block (TPP <= 32: 1-16)
    const int grp = threadIdx.x / TPP;
    const int pi = CL > 1 ? static_cast<int>(blockIdx.x) / CL : static_cast<int>(blockIdx.x) * groups + grp;
    if (pi >= b.nProb) return;   // uniform per group, block and cluster
    LocalGroup<TPP, CL> G;
    G.sub = threadIdx.x % TPP;
    G.mask = TPP >= 32 ? 0xffffffffu : (((1u << TPP) - 1u) << ((threadIdx.x & 31) & ~(TPP - 1)));
    G.rank = CL > 1 ? static_cast<int>(blockIdx.x) % CL : 0;
    G.buf = 0;
    LocalShared<TPP>& S = reinterpret_cast<LocalShared<TPP>*>(localSmem)[grp];
    const int sub = G.sub;
    const long long clk0 = clock64();
    const LocalProblem P = b.prob[pi];
    const int nDof = 2 * P.nFree;
    // this block's triangles [lo, hi) and initial-energy triangles [ilo, ihi)
    const int per = (P.nTri + CL - 1) / CL, iper = (P.nInit + CL - 1) / CL;
    const int lo = min(P.nTri, G.rank * per), hi = min(P.nTri, lo + per);
    const int ilo = min(P.nInit, G.rank * iper), ihi = min(P.nInit, ilo + iper);
    for (int j = sub; j < P.nVert; j += TPP) {
        const int sl = b.lvSlot[P.vertOff + j];
        if (sl >= 0) S.pos[sl] = b.lvPos[P.vertOff + j];
    }
    G.sync();
    // initial energy: the candidate's global triangles with global weights,
    // rescaled to the local mesh (TriMesh.cpp:2355-2361)
    double initE = 0.0;
    for (int c0 = ilo; c0 < ihi; c0 += TPP) {
        const int k = c0 + sub;
        double e = 0.0;
        if (k < ihi) {
            const int g = b.initTri[P.initOff + k];
            e = elem_energy(m, g, m.w[g], m.uv[m.F0[g]], m.uv[m.F1[g]], m.uv[m.F2[g]]);
        }
        S.triE[sub] = e;
        G.sync();
        if (sub == 0) {
            const int n = min(TPP, ihi - c0);
            for (int q = 0; q < n; ++q) initE = initE + S.triE[q];
        }
        G.sync();
    }
    initE = cluster_combine(S, G, initE, sub == 0 ? 0 : -1, 0);
    initE = local_bcast(S, G, initE * (surfaceArea / P.localArea));
    double lastE = local_energy(m, b, P, S, G, lo, hi, S.pos, false, 0.0);   // precompute
    int status = 0, it = 0, trials = 0;
    bool finite = isfinite(lastE);
    // raw quantities of the starting point (features of the learned
    // proposal), summed in triangle order like everything else
    double raw[kLocalRaw];
    for (int k = 0; k < kLocalRaw; ++k) raw[k] = 0.0;
    {
        // sums: lsum, lsq, g0x, g0y, g1x, g1y, n0, n1, es0, es1; then max eu, max -eu
        double acc[12] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, -1e300};
        for (int c0 = lo; c0 < hi; c0 += TPP) {
            const int t = c0 + sub;
            if (t < hi) {
                double2 U[3];
                int sl[3];
                local_corners(b, P, S, t, S.pos, false, 0.0, U, sl);
                const int g = b.ltGlobal[P.triOff + t];
                const double w = m.area[g] / P.localArea;
                const double e = elem_energy(m, g, w, U[0], U[1], U[2]);
                const double eu = e / (4.0 * w);
                double2 cg3[3];
                tri_corner_grads(U[0], U[1], U[2], m.A2[g], m.e0[g], m.e1[g], m.e01[g], w, cg3);
                double q[4] = {0.0, 0.0, 0.0, 0.0};
                double touch0 = 0.0, touch1 = 0.0;
                for (int k = 0; k < 3; ++k) {
                    if (sl[k] == 0) { q[0] += cg3[k].x; q[1] += cg3[k].y; touch0 = 1.0; }
                    if (sl[k] == 1) { q[2] += cg3[k].x; q[3] += cg3[k].y; touch1 = 1.0; }
                }
                for (int k = 0; k < 4; ++k) S.triG[sub][k] = q[k];
                S.triH[sub][0] = e;
                S.triH[sub][1] = eu;
                S.triH[sub][2] = log(eu);
                S.triH[sub][3] = touch0;
                S.triH[sub][4] = touch1;
            }
            G.sync();
            if (sub == 0) {
                const int n = min(TPP, hi - c0);
                for (int k = 0; k < n; ++k) {
                    const double e = S.triH[k][0], eu = S.triH[k][1], l = S.triH[k][2];
                    acc[0] += l;
                    acc[1] += l * l;
                    for (int c = 0; c < 4; ++c) acc[2 + c] += S.triG[k][c];
                    if (S.triH[k][3] != 0.0) { acc[6] += 1.0; acc[8] += e; }
                    if (S.triH[k][4] != 0.0) { acc[7] += 1.0; acc[9] += e; }
                    acc[10] = fmax(acc[10], eu);
                    acc[11] = fmax(acc[11], -eu);
                }
            }
            G.sync();
        }
        if constexpr (CL > 1) {
            // sub 0 holds the block's 12 partials: spread them over threads
            // 0..11, combine, gather back on sub 0
            if (sub == 0)
                for (int k = 0; k < 12; ++k) S.triE[k] = acc[k];
            G.sync();
            const double mine = sub < 12 ? S.triE[sub] : 0.0;
            const double tot = cluster_combine(S, G, mine, sub < 12 ? sub : -1, sub < 10 ? 0 : 2);
            G.sync();
            if (sub < 12) S.triE[sub] = tot;
            G.sync();
            for (int k = 0; k < 12; ++k) acc[k] = S.triE[k];
            G.sync();
        }
        const double g0x = acc[2], g0y = acc[3], g1x = acc[4], g1y = acc[5];
        raw[0] = lastE;
        raw[5] = acc[10];
        raw[6] = -acc[11];
        raw[7] = acc[0] / P.nTri;
        raw[8] = acc[1] / P.nTri;
        raw[9] = g0x * g0x + g0y * g0y;
        raw[10] = g1x * g1x + g1y * g1y;
        raw[11] = g0x * g1x + g0y * g1y;
        raw[12] = acc[6];
        raw[13] = acc[7];
        raw[14] = acc[8];
        raw[15] = acc[9];
        raw[4] = lastE;   // E1: replaced after the first step
    }
    constexpr int kEntRounds = (36 + TPP - 1) / TPP;
    for (; it < P.maxIter && finite; ++it) {
        // gradient (fixed vertices have no slot: zero rows)
        double gj = 0.0;
        for (int c0 = lo; c0 < hi; c0 += TPP) {
            const int t = c0 + sub;
            if (t < hi) {
                double2 U[3];
                int sl[3];
                local_corners(b, P, S, t, S.pos, false, 0.0, U, sl);
                const int g = b.ltGlobal[P.triOff + t];
                double2 cg3[3];
                tri_corner_grads(U[0], U[1], U[2], m.A2[g], m.e0[g], m.e1[g], m.e01[g], m.area[g] / P.localArea, cg3);
                for (int k = 0; k < 3; ++k) {
                    S.triG[sub][2 * k] = cg3[k].x;
                    S.triG[sub][2 * k + 1] = cg3[k].y;
                    S.triSlot[sub][k] = sl[k];
                }
            }
            G.sync();
            if (sub < nDof) {
                const int n = min(TPP, hi - c0);
                for (int q = 0; q < n; ++q)
                    for (int k = 0; k < 3; ++k)
                        if (S.triSlot[q][k] == (sub >> 1)) gj = gj + S.triG[q][2 * k + (sub & 1)];
            }
            G.sync();
        }
        gj = cluster_combine(S, G, gj, sub < nDof ? sub : -1, 0);
        if (sub < nDof) S.g[sub] = gj;
        G.sync();
        double gsq = 0.0;
        for (int j = 0; j < nDof; ++j) gsq = gsq + S.g[j] * S.g[j];
        if (it == 0) raw[1] = gsq;
        if (gsq < P.targetGRes) {   // Optimizer.cpp:215-221
            status = 1;
            break;
        }
        // dense Hessian of the free DOFs: projected triangle blocks summed in
        // triangle order (IglUtils::addBlockToMatrix, IglUtils.cpp:453-489)
        const int nEnt = nDof * (nDof + 1) / 2;
        double hacc[kEntRounds];
        for (int r = 0; r < kEntRounds; ++r) hacc[r] = 0.0;
        for (int c0 = lo; c0 < hi; c0 += TPP) {
            const int t = c0 + sub;
            if (t < hi) {
                double2 U[3];
                int sl[3];
                local_corners(b, P, S, t, S.pos, false, 0.0, U, sl);
                const int g = b.ltGlobal[P.triOff + t];
                double H6[6][6];
                tri_hessian(U, m.A2[g], m.e0d[g], m.e1d[g], m.e01d[g], m.area[g] / P.localArea, H6,
                            b.fp32Hessian ? 2 : 1);
                for (int i = 0; i < 6; ++i)
                    for (int j = i; j < 6; ++j) S.triH[sub][sym21(i, j)] = H6[i][j];
                for (int k = 0; k < 3; ++k) S.triSlot[sub][k] = sl[k];
            }
            G.sync();
            const int n = min(TPP, hi - c0);
            for (int r = 0; r < kEntRounds; ++r) {
                const int e = sub + TPP * r;
                if (e >= nEnt) continue;
                // entry e -> (i, j), i <= j, row-major upper triangle
                int i = 0, rem = e;
                while (rem >= nDof - i) { rem -= nDof - i; ++i; }
                const int j = i + rem;
                double acc = hacc[r];
                for (int q = 0; q < n; ++q)
                    for (int a = 0; a < 3; ++a) {
                        if (S.triSlot[q][a] != (i >> 1)) continue;
                        for (int c = 0; c < 3; ++c)
                            if (S.triSlot[q][c] == (j >> 1))
                                acc = acc + S.triH[q][sym21(2 * a + (i & 1), 2 * c + (j & 1))];
                    }
                hacc[r] = acc;
            }
            G.sync();
        }
        if constexpr (CL > 1) hacc[0] = cluster_combine(S, G, hacc[0], sub < nEnt ? sub : -1, 0);
        for (int r = 0; r < kEntRounds; ++r) {
            const int e = sub + TPP * r;
            if (e >= nEnt) continue;
            int i = 0, rem = e;
            while (rem >= nDof - i) { rem -= nDof - i; ++i; }
            const int j = i + rem;
            S.H[i][j] = hacc[r];
            S.H[j][i] = hacc[r];
        }
        G.sync();
        // H d = -g by LDL^T with symmetric pivoting on the largest remaining
        // diagonal (Eigen::LDLT); zero pivots give zero components.  Every
        // block of a cluster solves the same system.
        if (sub == 0) {
            double A[2 * kLocalMaxFree][2 * kLocalMaxFree], x[2 * kLocalMaxFree];
            int perm[2 * kLocalMaxFree];
            for (int i = 0; i < nDof; ++i) {
                perm[i] = i;
                x[i] = -S.g[i];
                for (int j = 0; j < nDof; ++j) A[i][j] = S.H[i][j];
            }
            double dmax = 0.0;
            for (int i = 0; i < nDof; ++i) dmax = fmax(dmax, fabs(A[i][i]));
            for (int k = 0; k < nDof; ++k) {
                int piv = k;
                for (int i = k + 1; i < nDof; ++i)
                    if (fabs(A[i][i]) > fabs(A[piv][piv])) piv = i;
                if (piv != k) {
                    for (int j = 0; j < nDof; ++j) { const double t = A[k][j]; A[k][j] = A[piv][j]; A[piv][j] = t; }
                    for (int i = 0; i < nDof; ++i) { const double t = A[i][k]; A[i][k] = A[i][piv]; A[i][piv] = t; }
                    const int tp = perm[k]; perm[k] = perm[piv]; perm[piv] = tp;
                }
                const double d = A[k][k];
                if (!(fabs(d) > 1e-300 + 1e-15 * dmax)) {
                    A[k][k] = 0.0;
                    for (int i = k + 1; i < nDof; ++i) A[i][k] = 0.0;
                    continue;
                }
                for (int i = k + 1; i < nDof; ++i) A[i][k] = A[i][k] / d;
                for (int i = k + 1; i < nDof; ++i)
                    for (int j = k + 1; j <= i; ++j) {
                        A[i][j] = A[i][j] - A[i][k] * d * A[j][k];
                        A[j][i] = A[i][j];
                    }
            }
            double y[2 * kLocalMaxFree];
            for (int i = 0; i < nDof; ++i) y[i] = x[perm[i]];
            for (int i = 0; i < nDof; ++i)
                for (int k = 0; k < i; ++k) y[i] = y[i] - A[i][k] * y[k];
            for (int i = 0; i < nDof; ++i) y[i] = (A[i][i] != 0.0) ? y[i] / A[i][i] : 0.0;
            for (int i = nDof - 1; i >= 0; --i)
                for (int k = i + 1; k < nDof; ++k) y[i] = y[i] - A[k][i] * y[k];
            for (int i = 0; i < nDof; ++i) S.dir[perm[i]] = y[i];
        }
        G.sync();
        // line search (Optimizer.cpp:575-652): injective bound x 0.99, halve
        // until E <= E_last, relative-decrease stop test
        double bound = 1.0;
        for (int t = lo + sub; t < hi; t += TPP) {
            double2 U[3], D[3];
            int sl[3];
            local_corners(b, P, S, t, S.pos, false, 0.0, U, sl);
            for (int k = 0; k < 3; ++k)
                D[k] = sl[k] >= 0 ? make_double2(S.dir[2 * sl[k]], S.dir[2 * sl[k] + 1]) : make_double2(0.0, 0.0);
            bound = fmin(bound, tri_step_bound(U[0], U[1], U[2], D[0], D[1], D[2], 1.0));
        }
        S.triE[sub] = bound;
        G.sync();
        if (sub == 0)
            for (int k = 1; k < TPP; ++k) bound = fmin(bound, S.triE[k]);
        G.sync();
        bound = cluster_combine(S, G, bound, sub == 0 ? 0 : -1, 1);
        bound = local_bcast(S, G, bound);
        double step = bound * 0.99;
        if (sub < P.nFree) S.pos0[sub] = S.pos[sub];
        G.sync();
        bool stopped = false;
        double testE = local_energy(m, b, P, S, G, lo, hi, S.pos0, true, step);
        ++trials;
        while (testE > lastE) {
            step = step / 2.0;
            if (step == 0.0) {
                stopped = true;
                break;
            }
            testE = local_energy(m, b, P, S, G, lo, hi, S.pos0, true, step);
            ++trials;
        }
        if (sub < P.nFree) {
            S.pos[sub].x = S.pos0[sub].x + step * S.dir[2 * sub];
            S.pos[sub].y = S.pos0[sub].y + step * S.dir[2 * sub + 1];
        }
        G.sync();
        const double lastEDec = lastE - testE;
        if ((lastEDec / lastE < 1.0e-6 * step) && (step > 1.0e-3)) stopped = true;
        lastE = testE;
        if (it == 0) {
            raw[2] = step;
            raw[3] = trials;
            raw[4] = testE;
        }
        finite = isfinite(lastE);
        if (stopped) {
            status = 1;
            ++it;
            break;
        }
    }
    if (!finite) status = 2;
    if (sub == 0 && G.rank == 0) {
        LocalResult r;
        r.initE = initE;
        r.lastE = lastE;
        r.eDec = (initE - lastE) * P.localArea / surfaceArea;   // TriMesh.cpp:2381
        for (int k = 0; k < kLocalMaxFree; ++k) r.pos[k] = k < P.nFree ? S.pos[k] : make_double2(0.0, 0.0);
        r.iters = it;
        r.status = status;
        r.trials = trials;
        for (int k = 0; k < kLocalRaw; ++k) r.raw[k] = raw[k];
        r.cycles = clock64() - clk0;
        b.out[pi] = r;
    }
    // no block leaves while another may still read its partials
    if constexpr (CL > 1) cg::this_cluster().sync();
}

} // namespace

int reduce_blocks_for(int n)
{
    int b = (n + 255) / 256;
    if (b > 1216) b = 1216;   // 152 SMs x 8 resident 256-thread blocks
    return b < 1 ? 1 : b;
}

// ------------------------------------------------- allocation-free energy
// Variant of k_energy for caller-owned, reference-layout device arrays (F
// nF x 3, rest nF x 8), with its block partials in a file-scope device array
// instead of an allocation.  Callers that cannot allocate (a host framework
// owning all device memory, externally captured graphs) use it through
// oc_sd_energy_trials_noalloc.
namespace {

constexpr int kNoAllocBlocks = 1216;
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

void launch_hessian(const DeviceMesh& m, int uniform, double* hb, cudaStream_t st)
{
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

namespace {
template <int TPP, int CL>
cudaError_t launch_local_tpp(const DeviceMesh& m, double surfaceArea, const LocalBatch& b, int block, cudaStream_t st)
{
    constexpr int maxThreads = local_threads<TPP, CL>();
    const int threads = (TPP >= 128 || CL > 1) ? maxThreads : std::max(TPP, std::min(maxThreads, block));
    constexpr size_t smemMax = local_smem<TPP, CL>(maxThreads);
    const size_t smem = local_smem<TPP, CL>(threads);
    static const cudaError_t attr = [] {
        cudaError_t e = cudaFuncSetAttribute(k_local_newton<TPP, CL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smemMax));
        if (e == cudaSuccess && CL > 8)
            e = cudaFuncSetAttribute(k_local_newton<TPP, CL>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
        return e;
    }();
    if (attr != cudaSuccess) return attr;
    const int groups = threads / TPP;
    if constexpr (CL == 1) {
        k_local_newton<TPP, CL><<<(b.nProb + groups - 1) / groups, threads, smem, st>>>(m, surfaceArea, b);
        return cudaGetLastError();
    }
    else {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(static_cast<unsigned>(b.nProb) * CL, 1, 1);
        cfg.blockDim = dim3(threads, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = CL;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        return cudaLaunchKernelEx(&cfg, k_local_newton<TPP, CL>, m, surfaceArea, b);
    }
}
} // namespace

// Schedule of a size class from its triangle bound and problem count: the
// 5-8 triangle problems pack four to a warp (a warp's FP64 instruction costs
// the same however many lanes are active), in 128-thread blocks when there
// are enough of them to give every SM two blocks, else in single-warp blocks
// spread over more SMs; larger problems spread over a cluster of blocks so
// that count x cluster blocks give at most about four blocks per SM, each
// block keeping at least 16 triangles.
LocalSchedule local_schedule(int maxTri, int count, int numSMs, int maxCluster)
{
    if (maxTri <= 8) return {8, 1, count / 16 >= 2 * numSMs ? 128 : 32};
    if (maxTri <= 40) return {32, 1, count / 4 >= 2 * numSMs ? 128 : 32};
    int c = 1;
    while (c < maxCluster && 2 * c * count <= 4 * numSMs && maxTri / (2 * c) >= 16) c *= 2;
    if (c == 1) return {128, 1, 128};
    return {64, c, 64};
}

int local_max_cluster()
{
    // 16-block clusters need the non-portable size and room on one GPC
    static const int v = [] {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(16, 1, 1);
        cfg.blockDim = dim3(64, 1, 1);
        cfg.dynamicSmemBytes = local_smem<64, 16>(64);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 16;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaFuncSetAttribute(k_local_newton<64, 16>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_local_newton<64, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(local_smem<64, 16>(64))) != cudaSuccess ||
            cudaOccupancyMaxActiveClusters(&n, k_local_newton<64, 16>, &cfg) != cudaSuccess) {
            cudaGetLastError();
            return 8;
        }
        return n > 0 ? 16 : 8;
    }();
    return v;
}

cudaError_t launch_local_newton(const DeviceMesh& m, double surfaceArea, const LocalBatch& b, LocalSchedule sc,
                                cudaStream_t st)
{
    if (b.nProb <= 0) return cudaSuccess;
    const int bl = sc.block;
    if (sc.tpp == 8 && sc.cluster == 1) return launch_local_tpp<8, 1>(m, surfaceArea, b, bl, st);
    if (sc.tpp == 32 && sc.cluster == 1) return launch_local_tpp<32, 1>(m, surfaceArea, b, bl, st);
    if (sc.tpp == 128 && sc.cluster == 1) return launch_local_tpp<128, 1>(m, surfaceArea, b, bl, st);
    if (sc.tpp == 64 && sc.cluster == 2) return launch_local_tpp<64, 2>(m, surfaceArea, b, bl, st);
    if (sc.tpp == 64 && sc.cluster == 4) return launch_local_tpp<64, 4>(m, surfaceArea, b, bl, st);
    if (sc.tpp == 64 && sc.cluster == 8) return launch_local_tpp<64, 8>(m, surfaceArea, b, bl, st);
    if (sc.tpp == 64 && sc.cluster == 16) return launch_local_tpp<64, 16>(m, surfaceArea, b, bl, st);
    return cudaErrorInvalidValue;
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
    const int nb = reduce_blocks_for(nF);   // <= kNoAllocBlocks
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
