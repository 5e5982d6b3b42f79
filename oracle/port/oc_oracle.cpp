// CPU restatement ("port") of the reference OptCuts geometry step.
// TEST INFRASTRUCTURE ONLY -- the checker for the CUDA path and the timed
// CPU baseline; the product never links it.  See oc_oracle.h.
//
// Each function follows the reference file:line named beside it.  The
// sparse direct solver stands in for Eigen's SimplicialLDLT
// (src/LinSysSolver/EigenLibSolver.cpp:71-107): an up-looking simplicial
// LDL^T (the published row-by-row algorithm driven by the elimination tree)
// under a geometric nested-dissection ordering of the mesh vertices, in
// place of Eigen's AMD ordering.  Both are exact factorizations; they differ
// only in rounding.

#include "oc_oracle.h"

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <thread>
#include <vector>

namespace {

// ---------------------------------------------------------------- threads
template <typename Body>
void parallel_range(int n, int nThreads, const Body& body)
{
    if (nThreads <= 1 || n < 1024) {
        body(0, n);
        return;
    }
    std::vector<std::thread> pool;
    for (int t = 0; t < nThreads; ++t) {
        int b = static_cast<int>(static_cast<long long>(n) * t / nThreads);
        int e = static_cast<int>(static_cast<long long>(n) * (t + 1) / nThreads);
        pool.emplace_back([=, &body] { body(b, e); });
    }
    for (auto& th : pool) th.join();
}

inline void corner(const double* UV, const int* F, int t, double U[3][2])
{
    for (int k = 0; k < 3; ++k) {
        U[k][0] = UV[2 * F[3 * t + k]];
        U[k][1] = UV[2 * F[3 * t + k] + 1];
    }
}

// Per-element energy, SymDirichletEnergy.cpp:30-44 (same operation order).
inline double elem_energy(const double* r, const double U[3][2], double w)
{
    const double a0 = U[1][0] - U[0][0], a1 = U[1][1] - U[0][1];   // U2m1
    const double b0 = U[2][0] - U[0][0], b1 = U[2][1] - U[0][1];   // U3m1
    const double area_U = 0.5 * (a0 * b1 - a1 * b0);
    const double triAreaSq = r[1], e0 = r[2], e1 = r[3], e01 = r[4];
    return w * (1.0 + triAreaSq / area_U / area_U) *
           (((b0 * b0 + b1 * b1) * e0 + (a0 * a0 + a1 * a1) * e1) / 4 / triAreaSq -
            (b0 * a0 + b1 * a1) * e01 / 2 / triAreaSq);
}

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (n <= 6).
// A is destroyed (its diagonal holds the eigenvalues), V receives the
// eigenvectors as columns.
void jacobi_eig(double A[6][6], double V[6][6], int n)
{
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) V[i][j] = (i == j) ? 1.0 : 0.0;
    double fro = 0.0;
    for (int i = 0; i < n; ++i)
        for (int j = 0; j < n; ++j) fro += A[i][j] * A[i][j];
    double prevOff = 0.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < n; ++p)
            for (int q = p + 1; q < n; ++q) off += A[p][q] * A[p][q];
        // converged, or no longer decreasing (rounding floor)
        if (off <= 1e-34 * fro || (sweep > 0 && off >= prevOff)) break;
        prevOff = off;
        for (int p = 0; p < n; ++p) {
            for (int q = p + 1; q < n; ++q) {
                const double apq = A[p][q];
                if (apq == 0.0) continue;
                const double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
                const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
                for (int k = 0; k < n; ++k) {   // columns p, q
                    const double akp = A[k][p], akq = A[k][q];
                    A[k][p] = c * akp - s * akq;
                    A[k][q] = s * akp + c * akq;
                }
                for (int k = 0; k < n; ++k) {   // rows p, q
                    const double apk = A[p][k], aqk = A[q][k];
                    A[p][k] = c * apk - s * aqk;
                    A[q][k] = s * apk + c * aqk;
                }
                for (int k = 0; k < n; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = c * vkp - s * vkq;
                    V[k][q] = s * vkp + c * vkq;
                }
            }
        }
    }
}

// Symmetric 6x6 eigen-decomposition, the GPU's two-stage order: cyclic
// Jacobi in single precision on A scaled by its largest entry (a starting
// basis), that basis made orthonormal in double precision (modified
// Gram-Schmidt), A rotated into it (B = Q^T A Q, upper triangle mirrored),
// then double-precision cyclic Jacobi sweeps that update only the entries a
// rotation changes (diagonal by a_pp - t a_pq, a_qq + t a_pq), the products
// meeting sums as explicit std::fma.  Compiled without contraction, every
// operation rounds as on the device.  Non-finite or all-zero input falls
// back to jacobi_eig.
void eig6_mixed(double A[6][6], double V[6][6])
{
    double s = 0.0;
    bool finite = true;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            finite = finite && std::isfinite(A[i][j]);
            s = std::fmax(s, std::fabs(A[i][j]));
        }
    if (!finite || !(s > 0.0)) {
        jacobi_eig(A, V, 6);
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
                    const float t = (theta >= 0.0f ? 1.0f : -1.0f) /
                                    (std::fabs(theta) + std::sqrt(theta * theta + 1.0f));
                    const float c = 1.0f / std::sqrt(t * t + 1.0f), sn = t * c;
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
            for (int r = 0; r < 6; ++r) d = std::fma(Q[r][p], v[r], d);
            for (int r = 0; r < 6; ++r) v[r] = std::fma(-d, Q[r][p], v[r]);
        }
        double n2 = 0.0;
        for (int r = 0; r < 6; ++r) n2 = std::fma(v[r], v[r], n2);
        const double in = 1.0 / std::sqrt(n2);
        for (int r = 0; r < 6; ++r) Q[r][c] = v[r] * in;
    }
    double T[6][6];
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < 6; ++c) {
            double acc = 0.0;
            for (int k = 0; k < 6; ++k) acc = std::fma(A[r][k], Q[k][c], acc);
            T[r][c] = acc;
        }
    for (int r = 0; r < 6; ++r)
        for (int c = r; c < 6; ++c) {
            double acc = 0.0;
            for (int k = 0; k < 6; ++k) acc = std::fma(Q[k][r], T[k][c], acc);
            A[r][c] = acc;
        }
    for (int r = 0; r < 6; ++r)
        for (int c = 0; c < r; ++c) A[r][c] = A[c][r];
    std::memcpy(V, Q, sizeof(Q));
    double fro = 0.0;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) fro = std::fma(A[i][j], A[i][j], fro);
    double prevOff = 0.0;
    for (int sweep = 0; sweep < 40; ++sweep) {
        double off = 0.0;
        for (int p = 0; p < 6; ++p)
            for (int q = p + 1; q < 6; ++q) off = std::fma(A[p][q], A[p][q], off);
        if (off <= 1e-34 * fro || (sweep > 0 && off >= prevOff)) break;
        prevOff = off;
        for (int p = 0; p < 6; ++p)
            for (int q = p + 1; q < 6; ++q) {
                const double apq = A[p][q];
                if (apq == 0.0) continue;
                const double theta = (A[q][q] - A[p][p]) / (2.0 * apq);
                const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(std::fma(theta, theta, 1.0)));
                const double c = 1.0 / std::sqrt(std::fma(t, t, 1.0)), sn = t * c;
                A[p][p] = std::fma(-t, apq, A[p][p]);
                A[q][q] = std::fma(t, apq, A[q][q]);
                A[p][q] = 0.0;
                A[q][p] = 0.0;
                for (int k = 0; k < 6; ++k) {
                    if (k == p || k == q) continue;
                    const double akp = A[k][p], akq = A[k][q];
                    const double np = std::fma(c, akp, -(sn * akq)), nq = std::fma(sn, akp, c * akq);
                    A[k][p] = np;
                    A[p][k] = np;
                    A[k][q] = nq;
                    A[q][k] = nq;
                }
                for (int k = 0; k < 6; ++k) {
                    const double vkp = V[k][p], vkq = V[k][q];
                    V[k][p] = std::fma(c, vkp, -(sn * vkq));
                    V[k][q] = std::fma(sn, vkp, c * vkq);
                }
            }
    }
}

// IglUtils::makePD (IglUtils.hpp:71-90): eigen-decompose, clamp negative
// eigenvalues to zero, rebuild; untouched when already PSD.
void make_pd(double H[6][6])
{
    double A[6][6], V[6][6];
    std::memcpy(A, H, sizeof(A));
    eig6_mixed(A, V);
    double lam[6];
    double lmin = 0.0;
    bool any = false;
    for (int i = 0; i < 6; ++i) {
        lam[i] = A[i][i];
        if (!any || lam[i] < lmin) lmin = lam[i];
        any = true;
    }
    if (lmin >= 0.0) return;
    for (int i = 0; i < 6; ++i)
        if (lam[i] < 0.0) lam[i] = 0.0;
    for (int i = 0; i < 6; ++i)
        for (int j = 0; j < 6; ++j) {
            double s = 0.0;
            for (int k = 0; k < 6; ++k) s = std::fma(V[i][k] * lam[k], V[j][k], s);
            H[i][j] = s;
        }
}

// Per-triangle Hessian, SymDirichletEnergy.cpp:440-522.
void elem_hessian(const double* r, const double U[3][2], double w, double H[6][6])
{
    const double U2m1[2] = {U[1][0] - U[0][0], U[1][1] - U[0][1]};
    const double U3m1[2] = {U[2][0] - U[0][0], U[2][1] - U[0][1]};
    const double area_U = 0.5 * (U2m1[0] * U3m1[1] - U2m1[1] * U3m1[0]);
    const double triAreaSq = r[1];
    const double areaRatio = triAreaSq / area_U / area_U / area_U;
    const double dAR = 3.0 / 2.0 * areaRatio / area_U;
    const double e0d = r[5], e1d = r[6], e01d = r[7];
    const double leftTerm = 1.0 + triAreaSq / area_U / area_U;
    const double rightTerm = ((U3m1[0] * U3m1[0] + U3m1[1] * U3m1[1]) * e0d +
                              (U2m1[0] * U2m1[0] + U2m1[1] * U2m1[1]) * e1d) / 2. -
                             (U3m1[0] * U2m1[0] + U3m1[1] * U2m1[1]) * e01d;
    const double eo[3][2] = {{U[2][0] - U[1][0], U[2][1] - U[1][1]},
                             {U[0][0] - U[2][0], U[0][1] - U[2][1]},
                             {U[1][0] - U[0][0], U[1][1] - U[0][1]}};
    double ort[3][2];
    for (int k = 0; k < 3; ++k) { ort[k][0] = eo[k][1]; ort[k][1] = -eo[k][0]; }
    double dL[3][2], dR[3][2];
    for (int k = 0; k < 3; ++k) { dL[k][0] = areaRatio * ort[k][0]; dL[k][1] = areaRatio * ort[k][1]; }
    for (int c = 0; c < 2; ++c) {
        dR[0][c] = (e01d - e0d) * U3m1[c] + (e01d - e1d) * U2m1[c];
        dR[1][c] = e1d * U2m1[c] - e01d * U3m1[c];
        dR[2][c] = e0d * U3m1[c] - e01d * U2m1[c];
    }
    // d2Right_ij (scalar multiples of I) and the dOrtho/dU skew term sign
    const double d2R[3][3] = {{e0d + e1d - 2.0 * e01d, e01d - e1d, e01d - e0d},
                              {e01d - e1d, e1d, -e01d},
                              {e01d - e0d, -e01d, e0d}};
    // skew coefficient s_ij: d2Left_ij += areaRatio * s_ij * [[0,-1],[1,0]]
    const double skew[3][3] = {{0, 1, -1}, {-1, 0, 1}, {1, -1, 0}};
    for (int i = 0; i < 3; ++i) {
        for (int j = i; j < 3; ++j) {
            double B[2][2];
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b) {
                    double d2L = dAR * ort[i][a] * ort[j][b];
                    if (i != j) d2L += areaRatio * skew[i][j] * ((a == 0 && b == 1) ? -1.0 : ((a == 1 && b == 0) ? 1.0 : 0.0));
                    B[a][b] = w * (d2L * rightTerm + dL[i][a] * dR[j][b] +
                                   (a == b ? d2R[i][j] * leftTerm : 0.0) + dR[i][a] * dL[j][b]);
                }
            for (int a = 0; a < 2; ++a)
                for (int b = 0; b < 2; ++b) {
                    H[2 * i + a][2 * j + b] = B[a][b];
                    H[2 * j + b][2 * i + a] = B[a][b];
                }
        }
    }
    make_pd(H);
}

// ---------------------------------------------------------------- solver
struct Solver {
    int nV = 0, n = 0;
    std::vector<int> vptr, vadj;          // vertex adjacency incl. self, sorted
    std::vector<char> isFixed;
    std::vector<int> order, pinv;         // vertex elimination order, inverse
    std::vector<int> triSlot;             // nF*9 -> block slot in vadj (or -1)
    std::vector<double> blk;              // assembled 2x2 blocks per slot (4 each)
    // LDL^T of the permuted DOF matrix
    std::vector<int> parent, Lp, Lnz, Li, flag, pattern;
    std::vector<double> Lx, D, y;
    long long nnzL = 0;
};

void nested_dissection(const Solver& S, const double* Vr, std::vector<int>& verts, std::vector<int>& tag,
                       int& tagCounter, std::vector<int>& out)
{
    // explicit stack of (subset) to avoid deep recursion on large meshes
    struct Item { std::vector<int> v; int stage; std::vector<int> sep; };
    std::vector<Item> st;
    st.push_back({std::move(verts), 0, {}});
    while (!st.empty()) {
        Item& it = st.back();
        if (it.stage == 0) {
            if (it.v.size() <= 64) {
                out.insert(out.end(), it.v.begin(), it.v.end());
                st.pop_back();
                continue;
            }
            double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
            for (int v : it.v)
                for (int c = 0; c < 3; ++c) {
                    lo[c] = std::min(lo[c], Vr[3 * v + c]);
                    hi[c] = std::max(hi[c], Vr[3 * v + c]);
                }
            int ax = 0;
            for (int c = 1; c < 3; ++c)
                if (hi[c] - lo[c] > hi[ax] - lo[ax]) ax = c;
            const size_t mid = it.v.size() / 2;
            std::nth_element(it.v.begin(), it.v.begin() + mid, it.v.end(), [&](int a, int b) {
                const double xa = Vr[3 * a + ax], xb = Vr[3 * b + ax];
                return xa < xb || (xa == xb && a < b);
            });
            const int tg = ++tagCounter;
            for (size_t k = mid; k < it.v.size(); ++k) tag[it.v[k]] = tg;
            std::vector<int> left, right(it.v.begin() + mid, it.v.end());
            std::vector<int> sep;
            for (size_t k = 0; k < mid; ++k) {
                const int v = it.v[k];
                bool touches = false;
                for (int p = S.vptr[v]; p < S.vptr[v + 1]; ++p)
                    if (tag[S.vadj[p]] == tg) { touches = true; break; }
                (touches ? sep : left).push_back(v);
            }
            it.stage = 1;
            it.sep = std::move(sep);
            std::vector<int> l = std::move(left), r = std::move(right);
            it.v.clear();
            // order: left, right, separator  (push right first so left runs first)
            st.push_back({std::move(r), 0, {}});
            st.push_back({std::move(l), 0, {}});
            // sentinel item that emits the separator after both halves
            // (stage 2 marks "emit sep of parent")
            continue;
        }
        // stage 1: both children have been processed -> emit separator
        out.insert(out.end(), it.sep.begin(), it.sep.end());
        st.pop_back();
    }
}

// Permuted DOF k -> (vertex, component).  Upper entries (i <= k) of column k
// are listed by visiting the vertex's adjacency.
template <typename F>
void for_upper(const Solver& S, int k, F fn)
{
    const int vk = S.order[k >> 1], ck = k & 1;
    for (int p = S.vptr[vk]; p < S.vptr[vk + 1]; ++p) {
        const int vc = S.vadj[p];
        const int base = 2 * S.pinv[vc];
        for (int cc = 0; cc < 2; ++cc) {
            const int i = base + cc;
            if (i <= k) fn(i, p, ck, cc);
        }
    }
}

bool symbolic(Solver& S)
{
    const int n = S.n;
    S.parent.assign(n, -1);
    S.flag.assign(n, -1);
    S.Lnz.assign(n, 0);
    for (int k = 0; k < n; ++k) {
        S.flag[k] = k;
        for_upper(S, k, [&](int i, int p, int, int) {
            if (i >= k) return;
            const int vk = S.order[k >> 1], vc = S.vadj[p];
            if ((S.isFixed[vk] || S.isFixed[vc]) && vk != vc) return;   // fixed rows are diagonal only
            for (; S.flag[i] != k; i = S.parent[i]) {
                if (S.parent[i] == -1) S.parent[i] = k;
                S.Lnz[i]++;
                S.flag[i] = k;
            }
        });
    }
    S.Lp.assign(n + 1, 0);
    for (int k = 0; k < n; ++k) S.Lp[k + 1] = S.Lp[k] + S.Lnz[k];
    S.nnzL = S.Lp[n];
    S.Li.assign(S.nnzL, 0);
    S.Lx.assign(S.nnzL, 0.0);
    S.D.assign(n, 0.0);
    S.y.assign(n, 0.0);
    S.pattern.assign(n, 0);
    return true;
}

int numeric(Solver& S)
{
    const int n = S.n;
    std::fill(S.flag.begin(), S.flag.end(), -1);
    std::fill(S.Lnz.begin(), S.Lnz.end(), 0);
    std::vector<int> path(n);
    for (int k = 0; k < n; ++k) {
        int top = n;
        S.flag[k] = k;
        S.y[k] = 0.0;
        for_upper(S, k, [&](int i, int p, int ck, int cc) {
            const int vk = S.order[k >> 1], vc = S.vadj[p];
            if ((S.isFixed[vk] || S.isFixed[vc]) && vk != vc) return;
            S.y[i] += S.blk[4 * p + 2 * ck + cc];
            int len = 0;
            for (; S.flag[i] != k; i = S.parent[i]) {
                path[len++] = i;
                S.flag[i] = k;
            }
            while (len > 0) S.pattern[--top] = path[--len];
        });
        double d = S.y[k];
        S.y[k] = 0.0;
        for (; top < n; ++top) {
            const int i = S.pattern[top];
            const double yi = S.y[i];
            S.y[i] = 0.0;
            const int p2 = S.Lp[i] + S.Lnz[i];
            for (int p = S.Lp[i]; p < p2; ++p) S.y[S.Li[p]] -= S.Lx[p] * yi;
            const double lki = yi / S.D[i];
            d -= lki * yi;
            S.Li[p2] = k;
            S.Lx[p2] = lki;
            S.Lnz[i]++;
        }
        if (d == 0.0 || !std::isfinite(d)) return -1;
        S.D[k] = d;
    }
    return 0;
}

} // namespace

extern "C" {

int ocr_rest_constants(const double* Vr, int nV, const int* F, int nF, double areaThres,
                       double* rest, double* scalars)
{
    (void)nV;
    double surfaceArea = 0.0;
    bool invalid = false;
    for (int t = 0; t < nF; ++t) {
        const double* P1 = Vr + 3 * F[3 * t];
        const double* P2 = Vr + 3 * F[3 * t + 1];
        const double* P3 = Vr + 3 * F[3 * t + 2];
        const double a[3] = {P2[0] - P1[0], P2[1] - P1[1], P2[2] - P1[2]};
        const double b[3] = {P3[0] - P1[0], P3[1] - P1[1], P3[2] - P1[2]};
        const double nrm[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
        double* r = rest + 8 * t;
        r[0] = 0.5 * std::sqrt(nrm[0] * nrm[0] + nrm[1] * nrm[1] + nrm[2] * nrm[2]);
        if (r[0] == 0.0) invalid = true;
        if (r[0] < areaThres) {   // TriMesh.cpp:373-383
            r[0] = areaThres;
            surfaceArea += areaThres;
            r[1] = areaThres * areaThres;
            r[2] = r[3] = 4.0 / std::sqrt(3.0) * areaThres;
            r[4] = r[2] / 2.0;
            r[5] = r[6] = 2.0 / std::sqrt(3.0) / areaThres;
            r[7] = r[5] / 2.0;
        }
        else {
            surfaceArea += r[0];
            r[1] = r[0] * r[0];
            r[2] = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
            r[3] = b[0] * b[0] + b[1] * b[1] + b[2] * b[2];
            r[4] = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
            r[5] = r[2] / 2. / r[1];
            r[6] = r[3] / 2. / r[1];
            r[7] = r[4] / 2. / r[1];
        }
    }
    double avg = 0.0;   // igl::avg_edge_length: every half-edge of every face
    for (int t = 0; t < nF; ++t)
        for (int j = 0; j < 3; ++j) {
            const double* p = Vr + 3 * F[3 * t + j];
            const double* q = Vr + 3 * F[3 * t + (j + 1) % 3];
            avg += std::sqrt((p[0] - q[0]) * (p[0] - q[0]) + (p[1] - q[1]) * (p[1] - q[1]) + (p[2] - q[2]) * (p[2] - q[2]));
        }
    scalars[0] = surfaceArea;
    scalars[1] = avg / (3.0 * nF);
    scalars[2] = std::sqrt(surfaceArea / M_PI);
    return invalid ? -1 : 0;
}

static double surface_area(const double* rest, int nF)
{
    double s = 0.0;
    for (int t = 0; t < nF; ++t) s += rest[8 * t];
    return s;
}

void ocr_energy_elem(const double* rest, const int* F, int nF, const double* UV, int uniformWeight, double* out)
{
    const double normalizer = surface_area(rest, nF);
    for (int t = 0; t < nF; ++t) {
        double U[3][2];
        corner(UV, F, t, U);
        out[t] = elem_energy(rest + 8 * t, U, uniformWeight ? 1.0 : rest[8 * t] / normalizer);
    }
}

double ocr_energy(const double* rest, const int* F, int nF, const double* UV, int uniformWeight)
{
    const double normalizer = surface_area(rest, nF);
    double s = 0.0;
    for (int t = 0; t < nF; ++t) {
        double U[3][2];
        corner(UV, F, t, U);
        s += elem_energy(rest + 8 * t, U, uniformWeight ? 1.0 : rest[8 * t] / normalizer);
    }
    return s;
}

void ocr_gradient(const double* rest, const int* F, int nF, const double* UV, int nV,
                  const int* fixedVert, int nFixed, int uniformWeight, double* g)
{
    const double normalizer = surface_area(rest, nF);
    std::fill(g, g + 2 * nV, 0.0);
    for (int t = 0; t < nF; ++t) {
        const double* r = rest + 8 * t;
        double U[3][2];
        corner(UV, F, t, U);
        const double U2m1[2] = {U[1][0] - U[0][0], U[1][1] - U[0][1]};
        const double U3m1[2] = {U[2][0] - U[0][0], U[2][1] - U[0][1]};
        const double area_U = 0.5 * (U2m1[0] * U3m1[1] - U2m1[1] * U3m1[0]);
        const double triAreaSq = r[1], e0 = r[2], e1 = r[3], e01 = r[4];
        const double leftTerm = 1.0 + triAreaSq / area_U / area_U;
        const double rightTerm = ((U3m1[0] * U3m1[0] + U3m1[1] * U3m1[1]) * e0 +
                                  (U2m1[0] * U2m1[0] + U2m1[1] * U2m1[1]) * e1) / 4 / triAreaSq -
                                 (U3m1[0] * U2m1[0] + U3m1[1] * U2m1[1]) * e01 / 2 / triAreaSq;
        const double areaRatio = triAreaSq / area_U / area_U / area_U;
        const double w = uniformWeight ? 1.0 : r[0] / normalizer;
        const double eo[3][2] = {{U[2][0] - U[1][0], U[2][1] - U[1][1]},
                                 {U[0][0] - U[2][0], U[0][1] - U[2][1]},
                                 {U[1][0] - U[0][0], U[1][1] - U[0][1]}};
        double dR[3][2];
        for (int c = 0; c < 2; ++c) {
            dR[0][c] = ((e01 - e0) * U3m1[c] + (e01 - e1) * U2m1[c]) / 2.0 / triAreaSq;
            dR[1][c] = (e1 * U2m1[c] - e01 * U3m1[c]) / 2.0 / triAreaSq;
            dR[2][c] = (e0 * U3m1[c] - e01 * U2m1[c]) / 2.0 / triAreaSq;
        }
        for (int k = 0; k < 3; ++k) {
            const double dL[2] = {areaRatio * eo[k][1], areaRatio * -eo[k][0]};
            const int v = F[3 * t + k];
            g[2 * v] += w * (dL[0] * rightTerm + dR[k][0] * leftTerm);
            g[2 * v + 1] += w * (dL[1] * rightTerm + dR[k][1] * leftTerm);
        }
    }
    for (int i = 0; i < nFixed; ++i) {
        g[2 * fixedVert[i]] = 0.0;
        g[2 * fixedVert[i] + 1] = 0.0;
    }
}

static void hessian_blocks_mt(const double* rest, const int* F, int nF, const double* UV,
                              int uniformWeight, double* out, int nThreads)
{
    const double normalizer = surface_area(rest, nF);
    parallel_range(nF, nThreads, [&](int b, int e) {
        for (int t = b; t < e; ++t) {
            double U[3][2], H[6][6];
            corner(UV, F, t, U);
            elem_hessian(rest + 8 * t, U, uniformWeight ? 1.0 : rest[8 * t] / normalizer, H);
            std::memcpy(out + 36 * (size_t)t, H, sizeof(H));
        }
    });
}

void ocr_hessian_blocks(const double* rest, const int* F, int nF, const double* UV, int uniformWeight, double* out)
{
    hessian_blocks_mt(rest, F, nF, UV, uniformWeight, out, 1);
}

void ocr_init_step_size(const int* F, int nF, const double* UV, const double* dir, double* stepSize)
{
    double step = *stepSize;
    for (int t = 0; t < nF; ++t) {
        double U[3][2], Vd[3][2];
        corner(UV, F, t, U);
        corner(dir, F, t, Vd);
        const double U2m1[2] = {U[1][0] - U[0][0], U[1][1] - U[0][1]};
        const double U3m1[2] = {U[2][0] - U[0][0], U[2][1] - U[0][1]};
        const double V2m1[2] = {Vd[1][0] - Vd[0][0], Vd[1][1] - Vd[0][1]};
        const double V3m1[2] = {Vd[2][0] - Vd[0][0], Vd[2][1] - Vd[0][1]};
        const double a = V2m1[0] * V3m1[1] - V2m1[1] * V3m1[0];
        const double b = U2m1[0] * V3m1[1] - U2m1[1] * V3m1[0] + V2m1[0] * U3m1[1] - V2m1[1] * U3m1[0];
        const double c = U2m1[0] * U3m1[1] - U2m1[1] * U3m1[0];
        const double delta = b * b - 4.0 * a * c;
        double bound = step;
        if (a > 0.0) {
            if ((b < 0.0) && (delta >= 0.0)) bound = 2.0 * c / (-b + std::sqrt(delta));
        }
        else if (a < 0.0) {
            if (b < 0.0) bound = 2.0 * c / (-b + std::sqrt(delta));
            else bound = (-b - std::sqrt(delta)) / 2.0 / a;
        }
        else {
            if (b < 0.0) bound = -c / b;
        }
        if (bound < step) step = bound;
    }
    *stepSize = step;
}

static ocr_solver* solver_create(int nV, const int* F, int nF, const int* fixedVert, int nFixed, const double* Vr,
                                 const int* givenOrder);

ocr_solver* ocr_solver_create(int nV, const int* F, int nF, const int* fixedVert, int nFixed, const double* Vr)
{
    return solver_create(nV, F, nF, fixedVert, nFixed, Vr, nullptr);
}

ocr_solver* ocr_solver_create_ordered(int nV, const int* F, int nF, const int* fixedVert, int nFixed,
                                      const int* vertexOrder)
{
    return solver_create(nV, F, nF, fixedVert, nFixed, nullptr, vertexOrder);
}

int ocr_solver_negative_pivots(const ocr_solver* s)
{
    const Solver& S = *reinterpret_cast<const Solver*>(s);
    int n = 0;
    for (double d : S.D) n += d < 0.0;
    return n;
}

static ocr_solver* solver_create(int nV, const int* F, int nF, const int* fixedVert, int nFixed, const double* Vr,
                                 const int* givenOrder)
{
    Solver* S = new Solver;
    S->nV = nV;
    S->n = 2 * nV;
    std::vector<std::vector<int>> nb(nV);
    for (int v = 0; v < nV; ++v) nb[v].push_back(v);
    for (int t = 0; t < nF; ++t)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
                if (a != b) nb[F[3 * t + a]].push_back(F[3 * t + b]);
    S->vptr.assign(nV + 1, 0);
    for (int v = 0; v < nV; ++v) {
        std::sort(nb[v].begin(), nb[v].end());
        nb[v].erase(std::unique(nb[v].begin(), nb[v].end()), nb[v].end());
        S->vptr[v + 1] = S->vptr[v] + static_cast<int>(nb[v].size());
    }
    S->vadj.reserve(S->vptr[nV]);
    for (int v = 0; v < nV; ++v) S->vadj.insert(S->vadj.end(), nb[v].begin(), nb[v].end());
    S->isFixed.assign(nV, 0);
    for (int i = 0; i < nFixed; ++i) S->isFixed[fixedVert[i]] = 1;
    S->triSlot.assign(9 * (size_t)nF, -1);
    for (int t = 0; t < nF; ++t)
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const int va = F[3 * t + a], vb = F[3 * t + b];
                const int* lo = S->vadj.data() + S->vptr[va];
                const int* hi = S->vadj.data() + S->vptr[va + 1];
                S->triSlot[9 * (size_t)t + 3 * a + b] = static_cast<int>(std::lower_bound(lo, hi, vb) - S->vadj.data());
            }
    S->blk.assign(4 * S->vadj.size(), 0.0);
    std::vector<int> verts(nV), tag(nV, 0);
    for (int v = 0; v < nV; ++v) verts[v] = v;
    int tagCounter = 0;
    S->order.clear();
    if (givenOrder) S->order.assign(givenOrder, givenOrder + nV);
    else nested_dissection(*S, Vr, verts, tag, tagCounter, S->order);
    S->pinv.assign(nV, 0);
    for (int k = 0; k < nV; ++k) S->pinv[S->order[k]] = k;
    symbolic(*S);
    // keep F for assembly
    S->Lx.shrink_to_fit();
    return reinterpret_cast<ocr_solver*>(S);
}

void ocr_solver_destroy(ocr_solver* s) { delete reinterpret_cast<Solver*>(s); }

long long ocr_solver_nnz_L(const ocr_solver* s) { return reinterpret_cast<const Solver*>(s)->nnzL; }

static int solver_factorize(Solver& S, const double* blocks, double param, int nF)
{
    std::fill(S.blk.begin(), S.blk.end(), 0.0);
    for (int t = 0; t < nF; ++t) {
        const double* H = blocks + 36 * (size_t)t;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const int slot = S.triSlot[9 * (size_t)t + 3 * a + b];
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) S.blk[4 * slot + 2 * i + j] += param * H[6 * (2 * a + i) + 2 * b + j];
            }
    }
    for (int v = 0; v < S.nV; ++v) {   // fixed vertices: param * identity (SymDirichletEnergy.cpp:541-548)
        if (!S.isFixed[v]) continue;
        for (int p = S.vptr[v]; p < S.vptr[v + 1]; ++p) {
            double* B = &S.blk[4 * p];
            if (S.vadj[p] == v) { B[0] = param; B[1] = 0; B[2] = 0; B[3] = param; }
        }
    }
    return numeric(S);
}

int ocr_solver_factorize(ocr_solver* s, const double* blocks, double param)
{
    Solver& S = *reinterpret_cast<Solver*>(s);
    const int nF = static_cast<int>(S.triSlot.size() / 9);
    return solver_factorize(S, blocks, param, nF);
}

void ocr_solver_solve(ocr_solver* s, const double* rhs, double* x)
{
    Solver& S = *reinterpret_cast<Solver*>(s);
    const int n = S.n;
    std::vector<double> z(n);
    for (int k = 0; k < n; ++k) z[k] = rhs[2 * S.order[k >> 1] + (k & 1)];
    for (int j = 0; j < n; ++j) {
        const double zj = z[j];
        for (int p = S.Lp[j]; p < S.Lp[j] + S.Lnz[j]; ++p) z[S.Li[p]] -= S.Lx[p] * zj;
    }
    for (int j = 0; j < n; ++j) z[j] /= S.D[j];
    for (int j = n - 1; j >= 0; --j) {
        double zj = z[j];
        for (int p = S.Lp[j]; p < S.Lp[j] + S.Lnz[j]; ++p) zj -= S.Lx[p] * z[S.Li[p]];
        z[j] = zj;
    }
    for (int k = 0; k < n; ++k) x[2 * S.order[k >> 1] + (k & 1)] = z[k];
}

// solver_factorize for an augmented system: blocks of triangles t < nF
// scaled by param, the rest (air triangles) by airScale; fixed rows get
// param (+ airScale when airFixed marks them) times identity.
static int solver_factorize_scaf(Solver& S, const double* blocks, int nF, int nFa, double param, double airScale,
                                 const std::vector<char>& airFixed)
{
    std::fill(S.blk.begin(), S.blk.end(), 0.0);
    for (int t = 0; t < nF + nFa; ++t) {
        const double* H = blocks + 36 * (size_t)t;
        const double sc = t < nF ? param : airScale;
        for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
                const int slot = S.triSlot[9 * (size_t)t + 3 * a + b];
                for (int i = 0; i < 2; ++i)
                    for (int j = 0; j < 2; ++j) S.blk[4 * slot + 2 * i + j] += sc * H[6 * (2 * a + i) + 2 * b + j];
            }
    }
    for (int v = 0; v < S.nV; ++v) {
        if (!S.isFixed[v]) continue;
        const double d = airFixed[v] ? param + airScale : param;   // Scaffold.cpp:193-199 + Optimizer.cpp:839
        for (int p = S.vptr[v]; p < S.vptr[v + 1]; ++p) {
            double* B = &S.blk[4 * p];
            if (S.vadj[p] == v) { B[0] = d; B[1] = 0; B[2] = 0; B[3] = d; }
        }
    }
    return numeric(S);
}

static int newton_impl(const double* Vr, int nV, const int* F, int nF, const int* fixedVert, int nFixed, double* UV,
                       const ocr_newton_opts* o, const ocr_scaffold* sc, double* traceE, double* traceGsq,
                       double* traceAlpha, double* traceSeconds, int* status)
{
    using clk = std::chrono::steady_clock;
    std::vector<double> rest(8 * (size_t)nF);
    double scal[3];
    ocr_rest_constants(Vr, nV, F, nF, 0.0, rest.data(), scal);
    const double par = o->energyParam;
    // scaffold: air mesh in the augmented numbering (Scaffold.cpp:179-199)
    const int nBnd = sc ? sc->nBnd : 0, nFa = sc ? sc->nAirF : 0;
    const int nW = sc ? nV + sc->nAirV - nBnd : nV;
    std::vector<int> Fw(F, F + 3 * (size_t)nF);
    std::vector<double> restA, Vw(3 * (size_t)nW, 0.0), W(2 * (size_t)nW);
    std::vector<int> airFixedList;
    std::vector<char> airFixed(nW, 0);
    std::copy(Vr, Vr + 3 * (size_t)nV, Vw.begin());
    std::copy(UV, UV + 2 * (size_t)nV, W.begin());
    double airScale = 0.0;
    if (sc) {
        auto whole = [&](int a) { return a < nBnd ? sc->bnd[a] : nV + a - nBnd; };
        std::vector<double> V3(3 * (size_t)sc->nAirV, 0.0);
        for (int i = 0; i < sc->nAirV; ++i) {
            V3[3 * i] = sc->airV[2 * i];
            V3[3 * i + 1] = sc->airV[2 * i + 1];
        }
        restA.resize(8 * (size_t)nFa);
        double sa[3];
        ocr_rest_constants(V3.data(), sc->nAirV, sc->airF, nFa, sc->areaThres, restA.data(), sa);
        for (int k = 0; k < 3 * nFa; ++k) Fw.push_back(whole(sc->airF[k]));
        for (int i = nBnd; i < sc->nAirV; ++i) {
            const int v = whole(i);
            W[2 * v] = sc->airV[2 * i];
            W[2 * v + 1] = sc->airV[2 * i + 1];
            Vw[3 * v] = sc->airV[2 * i];
            Vw[3 * v + 1] = sc->airV[2 * i + 1];
        }
        for (int i = 0; i < nFixed; ++i)
            for (int k = 0; k < nBnd; ++k)
                if (sc->bnd[k] == fixedVert[i]) {
                    airFixed[fixedVert[i]] = 1;
                    airFixedList.push_back(fixedVert[i]);
                }
        airScale = 0.01 * par / nFa;   // w_scaf / |F_air| (Optimizer.cpp:87, 776)
    }
    const int* Fa = Fw.data() + 3 * (size_t)nF;
    auto energy = [&](const double* X, double* eScaf) {
        double e = par * ocr_energy(rest.data(), F, nF, X, 0);
        double es = 0.0;
        if (sc) {
            es = ocr_energy(restA.data(), Fa, nFa, X, 1) * airScale;
            e += es;
        }
        if (eScaf) *eScaf = es;
        return e;
    };
    // Optimizer::precompute (Optimizer.cpp:154-201)
    ocr_solver* solver = ocr_solver_create(nW, Fw.data(), nF + nFa, fixedVert, nFixed, Vw.data());
    const double targetGRes = par * static_cast<double>(nV - nFixed) / nV * o->relGL2Tol;   // Optimizer.cpp:677
    double lastE = energy(W.data(), nullptr);
    traceE[0] = lastE;
    std::vector<double> g(2 * (size_t)nW), ga(2 * (size_t)nW), d(2 * (size_t)nW), W0(2 * (size_t)nW);
    std::vector<double> blocks(36 * (size_t)(nF + nFa));
    int it = 0;
    *status = 0;
    for (; it < o->maxIter; ++it) {
        auto t0 = clk::now();
        // Optimizer::solve (Optimizer.cpp:209-228); augmentGradient (Scaffold.cpp:210-230)
        ocr_gradient(rest.data(), F, nF, W.data(), nV, fixedVert, nFixed, 0, g.data());
        for (int k = 0; k < 2 * nV; ++k) g[k] *= par;
        for (int k = 2 * nV; k < 2 * nW; ++k) g[k] = 0.0;
        if (sc) {
            ocr_gradient(restA.data(), Fa, nFa, W.data(), nW, airFixedList.data(), (int)airFixedList.size(), 1,
                         ga.data());
            std::vector<char> onAir(nW, 0);
            for (int k = 0; k < 3 * nFa; ++k) onAir[Fa[k]] = 1;
            for (int v = 0; v < nW; ++v) {
                if (!onAir[v]) continue;
                if (v < nV) {
                    g[2 * v] += airScale * ga[2 * v];
                    g[2 * v + 1] += airScale * ga[2 * v + 1];
                }
                else {
                    g[2 * v] = airScale * ga[2 * v];
                    g[2 * v + 1] = airScale * ga[2 * v + 1];
                }
            }
        }
        double gsq = 0.0;
        for (double gi : g) gsq += gi * gi;
        traceGsq[it] = gsq;
        if (gsq < targetGRes) {
            *status = 1;
            traceE[it + 1] = lastE;
            traceAlpha[it] = 0.0;
            traceSeconds[it] = std::chrono::duration<double>(clk::now() - t0).count();
            ++it;
            break;
        }
        // Optimizer::solve_oneStep (Optimizer.cpp:505-573)
        hessian_blocks_mt(rest.data(), F, nF, W.data(), 0, blocks.data(), o->nThreads);
        if (sc) hessian_blocks_mt(restA.data(), Fa, nFa, W.data(), 1, blocks.data() + 36 * (size_t)nF, o->nThreads);
        Solver& S = *reinterpret_cast<Solver*>(solver);
        if (solver_factorize_scaf(S, blocks.data(), nF, nFa, par, airScale, airFixed) != 0) {
            ocr_solver_destroy(solver);
            return -1;
        }
        for (auto& gi : g) gi = -gi;
        ocr_solver_solve(solver, g.data(), d.data());
        // Optimizer::lineSearch (Optimizer.cpp:575-652)
        bool stopped = false;
        double step = 1.0;
        ocr_init_step_size(F, nF, W.data(), d.data(), &step);
        if (sc) ocr_init_step_size(Fa, nFa, W.data(), d.data(), &step);
        step *= 0.99;
        double eScaf0 = 0.0, eScaf = 0.0;
        if (sc) lastE = energy(W.data(), &eScaf0);   // Optimizer.cpp:588-592
        std::memcpy(W0.data(), W.data(), sizeof(double) * 2 * nW);
        auto forward = [&](double s) {
            for (int k = 0; k < 2 * nW; ++k) W[k] = W0[k] + s * d[k];
        };
        forward(step);
        double testE = energy(W.data(), &eScaf);
        while (testE > lastE) {
            step /= 2.0;
            if (step == 0.0) { stopped = true; break; }
            forward(step);
            testE = energy(W.data(), &eScaf);
        }
        double lastEDec = lastE - testE;
        if (sc) lastEDec += (-eScaf0 + eScaf);   // Optimizer.cpp:632-634
        if ((lastEDec / lastE < 1.0e-6 * step) && (step > 1.0e-3)) stopped = true;
        lastE = testE;
        traceE[it + 1] = lastE;
        traceAlpha[it] = step;
        traceSeconds[it] = std::chrono::duration<double>(clk::now() - t0).count();
        if (stopped) { *status = 1; ++it; break; }
    }
    std::copy(W.begin(), W.begin() + 2 * (size_t)nV, UV);
    ocr_solver_destroy(solver);
    return it;
}

int ocr_newton(const double* Vr, int nV, const int* F, int nF, const int* fixedVert, int nFixed,
               double* UV, const ocr_newton_opts* o, double* traceE, double* traceGsq,
               double* traceAlpha, double* traceSeconds, int* status)
{
    return newton_impl(Vr, nV, F, nF, fixedVert, nFixed, UV, o, nullptr, traceE, traceGsq, traceAlpha, traceSeconds,
                       status);
}

int ocr_newton_scaffold(const double* Vr, int nV, const int* F, int nF, const int* fixedVert, int nFixed,
                        double* UV, const ocr_newton_opts* o, const ocr_scaffold* scaffold, double* traceE,
                        double* traceGsq, double* traceAlpha, double* traceSeconds, int* status)
{
    return newton_impl(Vr, nV, F, nF, fixedVert, nFixed, UV, o, scaffold, traceE, traceGsq, traceAlpha, traceSeconds,
                       status);
}

} // extern "C"
