// Per-triangle symmetric Dirichlet kernels shared by the global Newton step
// (oc_fp64.cu, compiled with -fmad=false so its FP64 rounding follows the
// reference's scalar host code operation by operation) and the local
// topology solves (oc_local.cu, compiled with FMA contraction): energy,
// corner gradients, injective step bound, element Hessian with its PSD
// projection.  Each translation unit gets its own copy with its own
// floating-point contraction.
#pragma once

#include "oc_internal.h"

namespace oc {
namespace {

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

// Eigen-decomposition of a symmetric 6x6 to FP64 accuracy with a fraction
// of the FP64 instructions of jacobi_eig6: cyclic Jacobi in FP32 on the
// matrix scaled by its largest entry (a starting basis; FP32 instructions
// are 64x cheaper on GB300), that basis made orthonormal in FP64 (modified
// Gram-Schmidt), A rotated into it, then FP64 cyclic Jacobi sweeps on the
// nearly diagonal result until the off-diagonal mass reaches the rounding
// floor, each rotation updating only the entries it changes.  Only IEEE
// operations (division, square root, and explicit fused multiply-adds where
// a product meets a sum: one rounding, half the FP64 instructions of a
// product and a sum in this file's no-contraction build), so that a host
// restatement with std::fma rounds identically.  On return A's diagonal
// holds the eigenvalues and V the eigenvectors as columns.
__device__ void eig6_mixed(double A[6][6], double V[6][6])
{
    double s = 0.0;
    bool finite = true;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            finite = finite && isfinite(A[i][j]);
            s = fmax(s, fabs(A[i][j]));
        }
    if (!finite || !(s > 0.0)) {
        jacobi_eig6(A, V);
        return;
    }
    float Af[6][6], Vf[6][6];
    const double inv = 1.0 / s;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            Af[i][j] = static_cast<float>(A[i][j] * inv);
            Vf[i][j] = (i == j) ? 1.0f : 0.0f;
        }
    {
        float fro = 0.0f;
        for (int i = 0; i < 6; ++i)
            for (int j = 0; j < 6; ++j) fro += Af[i][j] * Af[i][j];
        float prevOff = 0.0f;
        for (int sweep = 0; sweep < 30; ++sweep) {
            float off = 0.0f;
            for (int p = 0; p < 6; ++p)
                for (int q = p + 1; q < 6; ++q) off += Af[p][q] * Af[p][q];
            if (off <= 1e-14f * fro || (sweep > 0 && off >= prevOff)) break;
            prevOff = off;
            for (int p = 0; p < 6; ++p)
                for (int q = p + 1; q < 6; ++q) {
                    const float apq = Af[p][q];
                    if (apq == 0.0f) continue;
                    const float theta = (Af[q][q] - Af[p][p]) / (2.0f * apq);
                    const float t = (theta >= 0.0f ? 1.0f : -1.0f) / (fabsf(theta) + sqrtf(theta * theta + 1.0f));
                    const float c = 1.0f / sqrtf(t * t + 1.0f), sn = t * c;
                    for (int k = 0; k < 6; ++k) {
                        const float akp = Af[k][p], akq = Af[k][q];
                        Af[k][p] = c * akp - sn * akq;
                        Af[k][q] = sn * akp + c * akq;
                    }
                    for (int k = 0; k < 6; ++k) {
                        const float apk = Af[p][k], aqk = Af[q][k];
                        Af[p][k] = c * apk - sn * aqk;
                        Af[q][k] = sn * apk + c * aqk;
                    }
                    for (int k = 0; k < 6; ++k) {
                        const float vkp = Vf[k][p], vkq = Vf[k][q];
                        Vf[k][p] = c * vkp - sn * vkq;
                        Vf[k][q] = sn * vkp + c * vkq;
                    }
                }
        }
    }
    double Q[6][6];
    for (int c = 0; c < 6; ++c) {
        double v[6];
        for (int r = 0; r < 6; ++r) v[r] = static_cast<double>(Vf[r][c]);
        for (int p = 0; p < c; ++p) {
            double d = 0.0;
            for (int r = 0; r < 6; ++r) d = fma(Q[r][p], v[r], d);
            for (int r = 0; r < 6; ++r) v[r] = fma(-d, Q[r][p], v[r]);
        }
        double n2 = 0.0;
        for (int r = 0; r < 6; ++r) n2 = fma(v[r], v[r], n2);
        const double in = 1.0 / sqrt(n2);
        for (int r = 0; r < 6; ++r) Q[r][c] = v[r] * in;
    }
    double T[6][6];
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) {
            double acc = 0.0;
            for (int k = 0; k < 6; ++k) acc = fma(A[r][k], Q[k][c], acc);
            T[r][c] = acc;
        }
    for (int r = 0; r < 6; ++r)
        for (int c = r; c < 6; ++c) {
            double acc = 0.0;
            for (int k = 0; k < 6; ++k) acc = fma(Q[k][r], T[k][c], acc);
            A[r][c] = acc;
        }
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < r; ++c) A[r][c] = A[c][r];
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) V[i][j] = Q[i][j];
    double fro = 0.0;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) fro = fma(A[i][j], A[i][j], fro);
    double prevOff = 0.0;
    for (int sweep = 0; sweep < 40; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < 6; ++p)
            for (int q = p + 1; q < 6; ++q) off = fma(A[p][q], A[p][q], off);
        if (off <= 1e-34 * fro || (sweep > 0 && off >= prevOff)) break;
        prevOff = off;
        for (int p = 0; p < 6; ++p)
            for (int q = p + 1; q < 6; ++q) {
                const double apq = A[p][q];
                if (apq == 0.0) continue;
                const double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (fabs(theta) + sqrt(fma(theta, theta, 1.0)));
                const double c = 1.0 / sqrt(fma(t, t, 1.0)), sn = t * c;
                A[p][p] = fma(-t, apq, A[p][p]);
                A[q][q] = fma(t, apq, A[q][q]);
                A[p][q] = 0.0;
                A[q][p] = 0.0;
                for (int k = 0; k < 6; ++k) {
                    if (k == p || k == q) continue;
                    const double akp = A[k][p], akq = A[k][q];
                    const double np = fma(c, akp, -(sn * akq)), nq = fma(sn, akp, c * akq);
                    A[k][p] = np;
                    A[p][k] = np;
                    A[k][q] = nq;
                    A[q][k] = nq;
                }
                for (int k = 0; k < 6; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = fma(c, vkp, -(sn * vkq));
                    V[k][q] = fma(sn, vkp, c * vkq);
                }
            }
    }
}

__device__ __forceinline__ double recip_sqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ float recip_sqrt(float x) { return rsqrtf(x); }

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
                // the rotation of the classical formula t = sgn(theta) /
                // (|theta| + sqrt(theta^2 + 1)), theta = delta / apq, written
                // with one division and one square root (the entries are
                // scaled to O(1) by the caller, so delta^2 + apq^2 cannot
                // overflow), and c = 1 / sqrt(1 + t^2) as a reciprocal root
                const T delta = (A[q][q] - A[p][p]) * T(0.5);
                const T t = (delta >= T(0) ? apq : -apq) / (fabs(delta) + sqrt(delta * delta + apq * apq));
                const T c = recip_sqrt(t * t + T(1)), sn = t * c;
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

// Eigen-decomposition of a symmetric 4x4 to FP64 accuracy with few FP64
// instructions (GB300's FP64 pipe charges a warp instruction in full
// whatever its active lanes): cyclic Jacobi in FP32 for a starting basis,
// that basis made orthonormal in FP64 (modified Gram-Schmidt), K rotated
// into it, then FP64 cyclic Jacobi sweeps on the nearly diagonal result
// (quadratic convergence: one or two sweeps), each rotation updating only
// the entries it changes (the 2x2 pivot block in closed form and the two
// affected rows).  On return A's diagonal holds the eigenvalues and V the
// eigenvectors as columns.
__device__ void eig4_mixed(double A[4][4], double V[4][4])
{
    float Af[4][4], Vf[4][4];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) Af[i][j] = static_cast<float>(A[i][j]);
    jacobi_eig4<float>(Af, Vf, 1e-14f);
    double Q[4][4];
    for (int c = 0; c < 4; ++c) {
        double v[4];
        for (int r = 0; r < 4; ++r) v[r] = static_cast<double>(Vf[r][c]);
        for (int p = 0; p < c; ++p) {
            double d = 0.0;
            for (int r = 0; r < 4; ++r) d = d + Q[r][p] * v[r];
            for (int r = 0; r < 4; ++r) v[r] = v[r] - d * Q[r][p];
        }
        double n2 = 0.0;
        for (int r = 0; r < 4; ++r) n2 = n2 + v[r] * v[r];
        const double inv = recip_sqrt(n2);
        for (int r = 0; r < 4; ++r) Q[r][c] = v[r] * inv;
    }
    // B = Q^T A Q (symmetrised), then Jacobi on B with V = Q
    double T[4][4];
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < 4; ++c) {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) acc = acc + A[r][k] * Q[k][c];
            T[r][c] = acc;
        }
    for (int r = 0; r < 4; ++r)
        for (int c = r; c < 4; ++c) {
            double acc = 0.0;
            for (int k = 0; k < 4; ++k) acc = acc + Q[k][r] * T[k][c];
            A[r][c] = acc;
        }
    for (int r = 0; r < 4; ++r)
        for (int c = 0; c < r; ++c) A[r][c] = A[c][r];
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) V[i][j] = Q[i][j];
    double fro = 0.0;
    for (int i = 0; i < 4; ++i)
        for (int j = 0; j < 4; ++j) fro = fro + A[i][j] * A[i][j];
    double prevOff = 0.0;
    for (int sweep = 0; sweep < 40; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < 4; ++p)
            for (int q = p + 1; q < 4; ++q) off = off + A[p][q] * A[p][q];
        // off-diagonal below 1e-15 of the matrix (eigenvalues then exact to
        // the rounding of their own size), or no longer decreasing
        if (off <= 1e-30 * fro || (sweep > 0 && off >= prevOff)) break;
        prevOff = off;
        for (int p = 0; p < 4; ++p)
            for (int q = p + 1; q < 4; ++q) {
                const double apq = A[p][q];
                if (apq == 0.0) continue;
                const double delta = (A[q][q] - A[p][p]) * 0.5;
                const double t = (delta >= 0.0 ? apq : -apq) / (fabs(delta) + sqrt(delta * delta + apq * apq));
                const double c = recip_sqrt(t * t + 1.0), sn = t * c;
                // the pivot block in closed form: a_pp - t a_pq, a_qq + t a_pq, 0
                A[p][p] = A[p][p] - t * apq;
                A[q][q] = A[q][q] + t * apq;
                A[p][q] = 0.0;
                A[q][p] = 0.0;
                for (int k = 0; k < 4; ++k) {
                    if (k == p || k == q) continue;
                    const double akp = A[k][p], akq = A[k][q];
                    const double np = c * akp - sn * akq, nq = sn * akp + c * akq;
                    A[k][p] = np;
                    A[p][k] = np;
                    A[k][q] = nq;
                    A[q][k] = nq;
                }
                for (int k = 0; k < 4; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
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
    if constexpr (sizeof(T) == 8) eig4_mixed(A, V);
    else jacobi_eig4<T>(A, V, T(1e-14));
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
                            double H[6][6], int localMode = 0, double reducedDensity = 0.0)
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
    if (localMode == 1 || (localMode == 3 && leftTerm * rightTerm <= reducedDensity)) {
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
    eig6_mixed(A, V);
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
                for (int k = 0; k < 6; ++k) s = fma(V[i][k] * lam[k], V[j][k], s);
                H[i][j] = s;
            }
    }
}


// The 21 distinct entries of a symmetric 6x6 element block, stored
// structure-of-arrays over the nF triangles: the three diagonal 2x2 blocks
// (xx, xy, yy) in slots 0-8, then the 2x2 blocks of corner pairs (0,1),
// (0,2), (1,2) row-major in slots 9-20.
__device__ inline void store_hessian_blocks(const double H[6][6], int t, int nF, double* __restrict__ hb)
{
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

} // namespace
} // namespace oc
