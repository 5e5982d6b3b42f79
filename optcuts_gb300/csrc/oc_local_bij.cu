// Bijective local topology solves (TriMesh::computeLocalEdDec_* with the
// scaffold on, TriMesh.cpp:2262-2795; Scaffold's local constructor,
// Scaffold.cpp:150-205) and the host entry point of their loop mesher.

#include "oc_internal.h"
#include "oc_loopmesh.cuh"

#include <vector>

#define OC_EXPORT extern "C" __attribute__((visibility("default")))

OC_EXPORT int oc_air_loop_mesh(const double* pts, int nPts, int maxSteiner, int* nV, double* V, int* nT, int* T,
                               int* status)
{
    if (!pts || !nV || !V || !nT || !T) return OC_ERR_INVALID;
    if (nPts < 3 || nPts > oc::kLoopMaxPts || maxSteiner < 0) return OC_ERR_INVALID;
    std::vector<double2> P(nPts);
    for (int i = 0; i < nPts; ++i) P[i] = make_double2(pts[2 * i], pts[2 * i + 1]);
    // the mesher's state is a few kB: heap, not stack
    std::vector<oc::LoopMesh> M(2);
    std::vector<oc::loopmesh::BadQueue> Q(1);
    const int st = oc::loop_mesh(P.data(), nPts, maxSteiner, M[0], M[1], Q[0]);
    if (status) *status = st;
    if (st & (oc::kLoopBadInput | oc::kLoopNoEar | oc::kLoopFlipCap)) return OC_ERR_INVALID;
    *nV = M[0].nV;
    *nT = M[0].nT;
    for (int i = 0; i < M[0].nV; ++i) {
        V[2 * i] = M[0].P[i].x;
        V[2 * i + 1] = M[0].P[i].y;
    }
    for (int t = 0; t < M[0].nT; ++t)
        for (int k = 0; k < 3; ++k) T[3 * t + k] = M[0].T[t][k];
    return OC_OK;
}

#include "oc_elem.cuh"

namespace oc {
namespace {

// ------------------------------------------------ bijective local solves
// The local projected-Newton loop of a candidate whose local Optimizer runs
// with scaffolding on (Optimizer(localMesh, {SD}, {1}, 0, mute, true,
// UV_bnds, E, bnd, useDense) in TriMesh::computeLocalEdDec_*): every
// iteration first re-meshes the air loop from the current positions
// (`scaffold = Scaffold(result, UV_bnds, E, bnd)` before the first and
// after every further step, Optimizer.cpp:154-158, 249-257), whose
// triangles then carry w_scaf / |F_air| (w_scaf = 0.01 energyParams[0] =
// 0.01) times their uniform-weight symmetric Dirichlet energy with the
// layout at meshing time as rest shape (degenerate-air clamp airThres);
// loop points that are fixed local vertices or air points stay put, the
// Steiner points are free.  Gradient, dense Hessian, injective bound and
// line search run over the local triangles and the air triangles
// (Optimizer.cpp:575-652, 764-843); lastEDec counts the local mesh's
// energy change only (:630-633); the result is the local mesh's energy
// alone (computeEnergyVal(..., excludeScaffold = true)).  One warp per
// problem; lane 0 runs the loop mesher and the LDL^T.
constexpr int kBijFree = kLocalMaxFree + kLoopMaxSteiner;   // free vertices: local slots, then Steiner points
constexpr int kBijDof = 2 * kBijFree;
constexpr int kBijProbs = 2;                                // problems (warps) per block

struct BijShared {
    LoopMesh M;
    double air[kLoopMaxTri][7];     // triAreaSq, e0SqLen, e1SqLen, e0dote1, *_div_dbAreaSq
    int apSlot[kLoopMaxV];          // free slot of an air vertex, -1 fixed
    double2 apFix[kLoopMaxV];       // position of a fixed air vertex
    double2 pos[kBijFree], pos0[kBijFree];
    double dir[kBijDof], g[kBijDof];
    double H[kBijDof][kBijDof];
    double bc;
    double triE[32];
    double triG[32][6];
    double triH[32][21];
    int triSlot[32][3];
    int nAirT, nSteiner, mstatus, maxSteiner;
    double wAir;
};

__device__ __forceinline__ double sd_energy(double2 U1, double2 U2, double2 U3, double A2, double e0, double e1,
                                            double e01, double w)
{
    const double a0 = U2.x - U1.x, a1 = U2.y - U1.y;
    const double b0 = U3.x - U1.x, b1 = U3.y - U1.y;
    const double area_U = 0.5 * (a0 * b1 - a1 * b0);
    return w * (1.0 + A2 / area_U / area_U) *
           (((b0 * b0 + b1 * b1) * e0 + (a0 * a0 + a1 * a1) * e1) / 4 / A2 - (b0 * a0 + b1 * a1) * e01 / 2 / A2);
}

__device__ __forceinline__ int bsym21(int i, int j)
{
    if (i > j) { const int t = i; i = j; j = t; }
    return i * 6 - i * (i - 1) / 2 + (j - i);
}

__device__ __forceinline__ double warp_bcast(BijShared& S, double v)
{
    if ((threadIdx.x & 31) == 0) S.bc = v;
    __syncwarp();
    v = S.bc;
    __syncwarp();
    return v;
}

// corners of local triangle t at pos (or pos0 + alpha dir)
__device__ __forceinline__ void mesh_corners(const LocalBatch& b, const LocalProblem& P, const BijShared& S, int t,
                                             bool withDir, double alpha, double2 U[3], int slot[3])
{
    for (int k = 0; k < 3; ++k) {
        const int lv = b.ltCorner[3 * (P.triOff + t) + k];
        const int sl = b.lvSlot[P.vertOff + lv];
        slot[k] = sl;
        if (sl >= 0)
            U[k] = withDir ? make_double2(S.pos0[sl].x + alpha * S.dir[2 * sl], S.pos0[sl].y + alpha * S.dir[2 * sl + 1])
                           : S.pos[sl];
        else
            U[k] = b.lvPos[P.vertOff + lv];
    }
}

__device__ __forceinline__ void air_corners(const BijShared& S, int t, bool withDir, double alpha, double2 U[3],
                                            int slot[3])
{
    for (int k = 0; k < 3; ++k) {
        const int a = S.M.T[t][k];
        const int sl = S.apSlot[a];
        slot[k] = sl;
        if (sl >= 0)
            U[k] = withDir ? make_double2(S.pos0[sl].x + alpha * S.dir[2 * sl], S.pos0[sl].y + alpha * S.dir[2 * sl + 1])
                           : S.pos[sl];
        else
            U[k] = S.apFix[a];
    }
}

// local mesh energy (weights triArea / localArea), triangle order
__device__ double bij_mesh_energy(const DeviceMesh& m, const LocalBatch& b, const LocalProblem& P, BijShared& S,
                                  bool withDir, double alpha)
{
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    for (int c0 = 0; c0 < P.nTri; c0 += 32) {
        const int t = c0 + lane;
        double e = 0.0;
        if (t < P.nTri) {
            double2 U[3];
            int sl[3];
            mesh_corners(b, P, S, t, withDir, alpha, U, sl);
            const int g = b.ltGlobal[P.triOff + t];
            e = elem_energy(m, g, m.area[g] / P.localArea, U[0], U[1], U[2]);
        }
        S.triE[lane] = e;
        __syncwarp();
        if (lane == 0) {
            const int n = min(32, P.nTri - c0);
            for (int k = 0; k < n; ++k) acc = acc + S.triE[k];
        }
        __syncwarp();
    }
    return warp_bcast(S, acc);
}

// air energy: w_scaf / |F_air| times the uniform-weight sum (Optimizer.cpp:774-777)
__device__ double bij_air_energy(BijShared& S, bool withDir, double alpha)
{
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    for (int c0 = 0; c0 < S.nAirT; c0 += 32) {
        const int t = c0 + lane;
        double e = 0.0;
        if (t < S.nAirT) {
            double2 U[3];
            int sl[3];
            air_corners(S, t, withDir, alpha, U, sl);
            e = sd_energy(U[0], U[1], U[2], S.air[t][0], S.air[t][1], S.air[t][2], S.air[t][3], 1.0);
        }
        S.triE[lane] = e;
        __syncwarp();
        if (lane == 0) {
            const int n = min(32, S.nAirT - c0);
            for (int k = 0; k < n; ++k) acc = acc + S.triE[k];
        }
        __syncwarp();
    }
    return warp_bcast(S, acc * S.wAir);
}

__global__ void __launch_bounds__(32 * kBijProbs) k_local_newton_bij(DeviceMesh m, double surfaceArea, LocalBatch b)
{
    __shared__ BijShared shared[kBijProbs];
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int pi = blockIdx.x * kBijProbs + w;
    if (pi >= b.nProb) return;   // whole warp
    BijShared& S = shared[w];
    const long long clk0 = clock64();
    const LocalProblem P = b.prob[pi];
    if (P.nAir < 0) {
        // abandoned by the reference before its solve (overlapping or
        // self-intersecting air loops): energy decrease -DBL_MAX
        if (lane == 0) {
            LocalResult r = {};
            r.eDec = -1.7976931348623157e308;
            r.status = 3;
            b.out[pi] = r;
        }
        return;
    }
    const int nFreeMesh = P.nFree;
    for (int j = lane; j < P.nVert; j += 32) {
        const int sl = b.lvSlot[P.vertOff + j];
        if (sl >= 0) S.pos[sl] = b.lvPos[P.vertOff + j];
    }
    if (lane == 0) {
        S.mstatus = 0;
        S.maxSteiner = 0;
    }
    __syncwarp();
    // initial energy: the candidate's global triangles with global weights,
    // rescaled to the local mesh
    double initE = 0.0;
    for (int c0 = 0; c0 < P.nInit; c0 += 32) {
        const int k = c0 + lane;
        double e = 0.0;
        if (k < P.nInit) {
            const int g = b.initTri[P.initOff + k];
            e = elem_energy(m, g, m.w[g], m.uv[m.F0[g]], m.uv[m.F1[g]], m.uv[m.F2[g]]);
        }
        S.triE[lane] = e;
        __syncwarp();
        if (lane == 0) {
            const int n = min(32, P.nInit - c0);
            for (int q = 0; q < n; ++q) initE = initE + S.triE[q];
        }
        __syncwarp();
    }
    initE = warp_bcast(S, initE * (surfaceArea / P.localArea));
    double lastE = 0.0;
    int status = 0, it = 0, trials = 0;
    bool failed = false;
    constexpr int kEntRounds = (kBijDof * (kBijDof + 1) / 2 + 31) / 32;
    for (;;) {
        if (it >= P.maxIter) break;
        // ---- the local scaffold from the current positions
        if (lane == 0) {
            double2 pts[kLoopMaxPts];
            for (int i = 0; i < P.nAir; ++i) {
                const int lv = b.apLocal[P.airOff + i];
                double2 p;
                int sl = -1;
                if (lv >= 0) {
                    sl = b.lvSlot[P.vertOff + lv];
                    p = sl >= 0 ? S.pos[sl] : b.lvPos[P.vertOff + lv];
                }
                else {
                    p = b.apPos[P.airOff + i];
                }
                pts[i] = p;
                S.apSlot[i] = sl;
                S.apFix[i] = p;
            }
            LoopMesh B;
            loopmesh::BadQueue Q;
            const int ms = loop_mesh(pts, P.nAir, kLoopMaxSteiner, S.M, B, Q);
            S.mstatus |= ms;
            const bool bad = (ms & (kLoopBadInput | kLoopNoEar | kLoopFlipCap)) != 0;
            S.nAirT = bad ? 0 : S.M.nT;
            S.nSteiner = bad ? 0 : S.M.nV - P.nAir;
            S.maxSteiner = max(S.maxSteiner, S.nSteiner);
            for (int s = 0; s < S.nSteiner; ++s) {
                S.apSlot[P.nAir + s] = nFreeMesh + s;
                S.pos[nFreeMesh + s] = S.M.P[P.nAir + s];
                S.apFix[P.nAir + s] = S.M.P[P.nAir + s];
            }
            S.wAir = S.nAirT > 0 ? 0.01 / S.nAirT : 0.0;
        }
        __syncwarp();
        if (S.nAirT == 0) {
            failed = true;
            break;
        }
        // rest constants of the air triangles: their layout now, z = 0
        // (Scaffold.cpp:187-190; TriMesh::computeFeatures, TriMesh.cpp:355-393)
        for (int t = lane; t < S.nAirT; t += 32) {
            const double2 P1 = S.M.P[S.M.T[t][0]], P2 = S.M.P[S.M.T[t][1]], P3 = S.M.P[S.M.T[t][2]];
            const double ax = P2.x - P1.x, ay = P2.y - P1.y, bx = P3.x - P1.x, by = P3.y - P1.y;
            const double nz = ax * by - ay * bx;
            double area = 0.5 * sqrt(nz * nz);
            double* r = S.air[t];
            if (area < P.airThres) {
                area = P.airThres;
                r[0] = area * area;
                r[1] = r[2] = 4.0 / sqrt(3.0) * area;
                r[3] = r[1] / 2.0;
                r[4] = r[5] = 2.0 / sqrt(3.0) / area;
                r[6] = r[4] / 2.0;
            }
            else {
                r[0] = area * area;
                r[1] = ax * ax + ay * ay;
                r[2] = bx * bx + by * by;
                r[3] = ax * bx + ay * by;
                r[4] = r[1] / 2. / r[0];
                r[5] = r[2] / 2. / r[0];
                r[6] = r[3] / 2. / r[0];
            }
        }
        __syncwarp();
        const int nFree = nFreeMesh + S.nSteiner;
        const int nDof = 2 * nFree;
        // ---- gradient: the local mesh's, plus w_air times the air mesh's
        // on the loop vertices and the Steiner points (Scaffold::augmentGradient)
        double gm = 0.0, ga = 0.0;
        for (int c0 = 0; c0 < P.nTri; c0 += 32) {
            const int t = c0 + lane;
            if (t < P.nTri) {
                double2 U[3];
                int sl[3];
                mesh_corners(b, P, S, t, false, 0.0, U, sl);
                const int g = b.ltGlobal[P.triOff + t];
                double2 cg3[3];
                tri_corner_grads(U[0], U[1], U[2], m.A2[g], m.e0[g], m.e1[g], m.e01[g], m.area[g] / P.localArea, cg3);
                for (int k = 0; k < 3; ++k) {
                    S.triG[lane][2 * k] = cg3[k].x;
                    S.triG[lane][2 * k + 1] = cg3[k].y;
                    S.triSlot[lane][k] = sl[k];
                }
            }
            __syncwarp();
            if (lane < nDof) {
                const int n = min(32, P.nTri - c0);
                for (int q = 0; q < n; ++q)
                    for (int k = 0; k < 3; ++k)
                        if (S.triSlot[q][k] == (lane >> 1)) gm = gm + S.triG[q][2 * k + (lane & 1)];
            }
            __syncwarp();
        }
        for (int c0 = 0; c0 < S.nAirT; c0 += 32) {
            const int t = c0 + lane;
            if (t < S.nAirT) {
                double2 U[3];
                int sl[3];
                air_corners(S, t, false, 0.0, U, sl);
                double2 cg3[3];
                tri_corner_grads(U[0], U[1], U[2], S.air[t][0], S.air[t][1], S.air[t][2], S.air[t][3], 1.0, cg3);
                for (int k = 0; k < 3; ++k) {
                    S.triG[lane][2 * k] = cg3[k].x;
                    S.triG[lane][2 * k + 1] = cg3[k].y;
                    S.triSlot[lane][k] = sl[k];
                }
            }
            __syncwarp();
            if (lane < nDof) {
                const int n = min(32, S.nAirT - c0);
                for (int q = 0; q < n; ++q)
                    for (int k = 0; k < 3; ++k)
                        if (S.triSlot[q][k] == (lane >> 1)) ga = ga + S.triG[q][2 * k + (lane & 1)];
            }
            __syncwarp();
        }
        if (lane < nDof) S.g[lane] = (lane >> 1) < nFreeMesh ? gm + S.wAir * ga : S.wAir * ga;
        __syncwarp();
        double gsq = 0.0;
        for (int j = 0; j < nDof; ++j) gsq = gsq + S.g[j] * S.g[j];
        if (gsq < P.targetGRes) {   // Optimizer.cpp:215-221
            status = 1;
            break;
        }
        // ---- dense Hessian: projected local blocks, plus w_air times the
        // projected air blocks (Scaffold::augmentProxyMatrix, dense form)
        const int nEnt = nDof * (nDof + 1) / 2;
        double hm[kEntRounds], ha[kEntRounds];
        for (int r = 0; r < kEntRounds; ++r) hm[r] = ha[r] = 0.0;
        for (int pass = 0; pass < 2; ++pass) {
            const int nT = pass == 0 ? P.nTri : S.nAirT;
            for (int c0 = 0; c0 < nT; c0 += 32) {
                const int t = c0 + lane;
                if (t < nT) {
                    double2 U[3];
                    int sl[3];
                    double H6[6][6];
                    if (pass == 0) {
                        mesh_corners(b, P, S, t, false, 0.0, U, sl);
                        const int g = b.ltGlobal[P.triOff + t];
                        tri_hessian(U, m.A2[g], m.e0d[g], m.e1d[g], m.e01d[g], m.area[g] / P.localArea, H6,
                                    b.fp32Hessian ? 2 : 1);
                    }
                    else {
                        air_corners(S, t, false, 0.0, U, sl);
                        tri_hessian(U, S.air[t][0], S.air[t][4], S.air[t][5], S.air[t][6], 1.0, H6,
                                    b.fp32Hessian ? 2 : 1);
                    }
                    for (int i = 0; i < 6; ++i)
                        for (int j = i; j < 6; ++j) S.triH[lane][bsym21(i, j)] = H6[i][j];
                    for (int k = 0; k < 3; ++k) S.triSlot[lane][k] = sl[k];
                }
                __syncwarp();
                const int n = min(32, nT - c0);
                for (int r = 0; r < kEntRounds; ++r) {
                    const int e = lane + 32 * r;
                    if (e >= nEnt) continue;
                    int i = 0, rem = e;
                    while (rem >= nDof - i) { rem -= nDof - i; ++i; }
                    const int j = i + rem;
                    double acc = pass == 0 ? hm[r] : ha[r];
                    for (int q = 0; q < n; ++q)
                        for (int a = 0; a < 3; ++a) {
                            if (S.triSlot[q][a] != (i >> 1)) continue;
                            for (int c = 0; c < 3; ++c)
                                if (S.triSlot[q][c] == (j >> 1))
                                    acc = acc + S.triH[q][bsym21(2 * a + (i & 1), 2 * c + (j & 1))];
                        }
                    if (pass == 0) hm[r] = acc;
                    else ha[r] = acc;
                }
                __syncwarp();
            }
        }
        for (int r = 0; r < kEntRounds; ++r) {
            const int e = lane + 32 * r;
            if (e >= nEnt) continue;
            int i = 0, rem = e;
            while (rem >= nDof - i) { rem -= nDof - i; ++i; }
            const int j = i + rem;
            const double v = hm[r] + S.wAir * ha[r];
            S.H[i][j] = v;
            S.H[j][i] = v;
        }
        __syncwarp();
        // ---- H d = -g: LDL^T with symmetric pivoting on the largest
        // remaining diagonal (Eigen::LDLT), in place in S.H
        if (lane == 0) {
            int perm[kBijDof];
            double y[kBijDof];
            for (int i = 0; i < nDof; ++i) {
                perm[i] = i;
                y[i] = -S.g[i];
            }
            double dmax = 0.0;
            for (int i = 0; i < nDof; ++i) dmax = fmax(dmax, fabs(S.H[i][i]));
            for (int k = 0; k < nDof; ++k) {
                int piv = k;
                for (int i = k + 1; i < nDof; ++i)
                    if (fabs(S.H[i][i]) > fabs(S.H[piv][piv])) piv = i;
                if (piv != k) {
                    for (int j = 0; j < nDof; ++j) { const double t = S.H[k][j]; S.H[k][j] = S.H[piv][j]; S.H[piv][j] = t; }
                    for (int i = 0; i < nDof; ++i) { const double t = S.H[i][k]; S.H[i][k] = S.H[i][piv]; S.H[i][piv] = t; }
                    const int tp = perm[k]; perm[k] = perm[piv]; perm[piv] = tp;
                }
                const double d = S.H[k][k];
                if (!(fabs(d) > 1e-300 + 1e-15 * dmax)) {
                    S.H[k][k] = 0.0;
                    for (int i = k + 1; i < nDof; ++i) S.H[i][k] = 0.0;
                    continue;
                }
                for (int i = k + 1; i < nDof; ++i) S.H[i][k] = S.H[i][k] / d;
                for (int i = k + 1; i < nDof; ++i)
                    for (int j = k + 1; j <= i; ++j) {
                        S.H[i][j] = S.H[i][j] - S.H[i][k] * d * S.H[j][k];
                        S.H[j][i] = S.H[i][j];
                    }
            }
            double x[kBijDof];
            for (int i = 0; i < nDof; ++i) x[i] = y[perm[i]];
            for (int i = 0; i < nDof; ++i)
                for (int k = 0; k < i; ++k) x[i] = x[i] - S.H[i][k] * x[k];
            for (int i = 0; i < nDof; ++i) x[i] = (S.H[i][i] != 0.0) ? x[i] / S.H[i][i] : 0.0;
            for (int i = nDof - 1; i >= 0; --i)
                for (int k = i + 1; k < nDof; ++k) x[i] = x[i] - S.H[k][i] * x[k];
            for (int i = 0; i < nDof; ++i) S.dir[perm[i]] = x[i];
        }
        __syncwarp();
        // ---- line search (Optimizer.cpp:575-652) over both meshes
        double bound = 1.0;
        for (int pass = 0; pass < 2; ++pass) {
            const int nT = pass == 0 ? P.nTri : S.nAirT;
            for (int t = lane; t < nT; t += 32) {
                double2 U[3], D[3];
                int sl[3];
                if (pass == 0) mesh_corners(b, P, S, t, false, 0.0, U, sl);
                else air_corners(S, t, false, 0.0, U, sl);
                for (int k = 0; k < 3; ++k)
                    D[k] = sl[k] >= 0 ? make_double2(S.dir[2 * sl[k]], S.dir[2 * sl[k] + 1]) : make_double2(0.0, 0.0);
                bound = fmin(bound, tri_step_bound(U[0], U[1], U[2], D[0], D[1], D[2], 1.0));
            }
        }
        for (int o = 16; o > 0; o >>= 1) bound = fmin(bound, __shfl_xor_sync(0xffffffffu, bound, o));
        double step = bound * 0.99;
        if (lane < nFree) S.pos0[lane] = S.pos[lane];
        __syncwarp();
        // energy with the new scaffold at the current layout
        const double eAir0 = bij_air_energy(S, false, 0.0);
        lastE = bij_mesh_energy(m, b, P, S, false, 0.0) + eAir0;
        bool stopped = false;
        double eAir = bij_air_energy(S, true, step);
        double testE = bij_mesh_energy(m, b, P, S, true, step) + eAir;
        ++trials;
        while (testE > lastE) {
            step = step / 2.0;
            if (step == 0.0) {
                stopped = true;
                break;
            }
            eAir = bij_air_energy(S, true, step);
            testE = bij_mesh_energy(m, b, P, S, true, step) + eAir;
            ++trials;
        }
        if (lane < nFree) {
            S.pos[lane].x = S.pos0[lane].x + step * S.dir[2 * lane];
            S.pos[lane].y = S.pos0[lane].y + step * S.dir[2 * lane + 1];
        }
        __syncwarp();
        const double lastEDec = (lastE - testE) + (eAir - eAir0);
        if ((lastEDec / lastE < 1.0e-6 * step) && (step > 1.0e-3)) stopped = true;
        lastE = testE;
        ++it;
        if (!isfinite(lastE)) {
            status = 2;
            break;
        }
        if (stopped) {
            status = 1;
            break;
        }
    }
    // the local mesh's energy at the final layout (excludeScaffold)
    const double curE = bij_mesh_energy(m, b, P, S, false, 0.0);
    if (lane == 0) {
        LocalResult r;
        r.initE = initE;
        r.lastE = curE;
        r.eDec = failed ? -1.7976931348623157e308 : (initE - curE) * P.localArea / surfaceArea;
        for (int k = 0; k < kLocalMaxFree; ++k) r.pos[k] = k < nFreeMesh ? S.pos[k] : make_double2(0.0, 0.0);
        r.iters = it;
        r.status = failed ? 3 : (isfinite(curE) ? status : 2);
        r.trials = trials;
        for (int k = 0; k < kLocalRaw; ++k) r.raw[k] = 0.0;
        r.cycles = clock64() - clk0;
        r.airStatus = S.mstatus;
        r.airSteiner = S.maxSteiner;
        b.out[pi] = r;
    }
}

} // namespace

cudaError_t launch_local_newton_bij(const DeviceMesh& m, double surfaceArea, const LocalBatch& b, cudaStream_t st)
{
    if (b.nProb <= 0) return cudaSuccess;
    k_local_newton_bij<<<(b.nProb + kBijProbs - 1) / kBijProbs, 32 * kBijProbs, 0, st>>>(m, surfaceArea, b);
    return cudaGetLastError();
}

} // namespace oc
