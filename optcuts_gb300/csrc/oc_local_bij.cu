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
// alone (computeEnergyVal(..., excludeScaffold = true)).
//
// One warp per problem.  GB300's FP64 pipe takes a warp instruction whole
// whatever its active lanes, so the local and air triangles go through
// every per-triangle step together (one lane each: one pass of the element
// Hessians instead of two), and the LDL^T spreads each elimination step
// over the lanes; lane 0 runs the loop mesher and the fixed-order sums.
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
    int perm[kBijDof];
    double H[kBijDof][kBijDof];
    double bc[2];
    double triE[32], triA[32];
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
    if ((threadIdx.x & 31) == 0) S.bc[0] = v;
    __syncwarp();
    v = S.bc[0];
    __syncwarp();
    return v;
}

// triangle t of the combined list: the local triangles, then the air
// triangles; corners at pos (or pos0 + alpha dir), free slots, rest
// constants and weight (air: w_scaf / |F_air| for gradient and Hessian)
struct TriView {
    double2 U[3];
    int slot[3];
    double A2, e0, e1, e01, e0d, e1d, e01d, w;
    bool air;
};

__device__ __forceinline__ double2 at_slot(const BijShared& S, int sl, bool withDir, double alpha)
{
    return withDir ? make_double2(S.pos0[sl].x + alpha * S.dir[2 * sl], S.pos0[sl].y + alpha * S.dir[2 * sl + 1])
                   : S.pos[sl];
}

__device__ __forceinline__ void tri_view(const DeviceMesh& m, const LocalBatch& b, const LocalProblem& P,
                                         const BijShared& S, int t, bool withDir, double alpha, TriView& v)
{
    if (t < P.nTri) {
        for (int k = 0; k < 3; ++k) {
            const int lv = b.ltCorner[3 * (P.triOff + t) + k];
            const int sl = b.lvSlot[P.vertOff + lv];
            v.slot[k] = sl;
            v.U[k] = sl >= 0 ? at_slot(S, sl, withDir, alpha) : b.lvPos[P.vertOff + lv];
        }
        const int g = b.ltGlobal[P.triOff + t];
        v.A2 = m.A2[g];
        v.e0 = m.e0[g];
        v.e1 = m.e1[g];
        v.e01 = m.e01[g];
        v.e0d = m.e0d[g];
        v.e1d = m.e1d[g];
        v.e01d = m.e01d[g];
        v.w = m.area[g] / P.localArea;
        v.air = false;
    }
    else {
        const int a = t - P.nTri;
        for (int k = 0; k < 3; ++k) {
            const int q = S.M.T[a][k];
            const int sl = S.apSlot[q];
            v.slot[k] = sl;
            v.U[k] = sl >= 0 ? at_slot(S, sl, withDir, alpha) : S.apFix[q];
        }
        const double* r = S.air[a];
        v.A2 = r[0];
        v.e0 = r[1];
        v.e1 = r[2];
        v.e01 = r[3];
        v.e0d = r[4];
        v.e1d = r[5];
        v.e01d = r[6];
        v.w = S.wAir;
        v.air = true;
    }
}

// the local mesh's energy (weights triArea / localArea) and the air
// energy (w_scaf / |F_air| times the uniform-weight sum, Optimizer.cpp:
// 774-777), each summed in triangle order, in one pass
__device__ void bij_energies(const DeviceMesh& m, const LocalBatch& b, const LocalProblem& P, BijShared& S,
                             bool withDir, double alpha, double& eMesh, double& eAir)
{
    const int lane = threadIdx.x & 31;
    const int nAll = P.nTri + S.nAirT;
    double am = 0.0, aa = 0.0;
    for (int c0 = 0; c0 < nAll; c0 += 32) {
        const int t = c0 + lane;
        double e = 0.0;
        if (t < nAll) {
            TriView v;
            tri_view(m, b, P, S, t, withDir, alpha, v);
            e = sd_energy(v.U[0], v.U[1], v.U[2], v.A2, v.e0, v.e1, v.e01, v.air ? 1.0 : v.w);
        }
        S.triE[lane] = e;
        __syncwarp();
        if (lane == 0) {
            const int n = min(32, nAll - c0);
            for (int k = 0; k < n; ++k) {
                if (c0 + k < P.nTri) am = am + S.triE[k];
                else aa = aa + S.triE[k];
            }
            S.bc[0] = am;
            S.bc[1] = aa * S.wAir;
        }
        __syncwarp();
    }
    if (nAll == 0 && lane == 0) S.bc[0] = S.bc[1] = 0.0;
    __syncwarp();
    eMesh = S.bc[0];
    eAir = S.bc[1];
    __syncwarp();
}

__device__ double bij_mesh_energy(const DeviceMesh& m, const LocalBatch& b, const LocalProblem& P, BijShared& S)
{
    const int lane = threadIdx.x & 31;
    double acc = 0.0;
    for (int c0 = 0; c0 < P.nTri; c0 += 32) {
        const int t = c0 + lane;
        double e = 0.0;
        if (t < P.nTri) {
            TriView v;
            tri_view(m, b, P, S, t, false, 0.0, v);
            e = sd_energy(v.U[0], v.U[1], v.U[2], v.A2, v.e0, v.e1, v.e01, v.w);
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
        S.nAirT = 0;
        S.wAir = 0.0;
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
    // raw quantities of the starting point for the learned proposal's
    // features, the local mesh's alone and as the unconstrained solve
    // records them: energy, per-triangle unweighted energies (max, min,
    // mean log, mean log^2), gradients at free slots 0 and 1, triangles
    // touching them and their energy; the first step fills the rest
    double raw[kLocalRaw];
    for (int k = 0; k < kLocalRaw; ++k) raw[k] = 0.0;
    {
        double acc[12] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, -1e300};
        for (int c0 = 0; c0 < P.nTri; c0 += 32) {
            const int t = c0 + lane;
            if (t < P.nTri) {
                TriView v;
                tri_view(m, b, P, S, t, false, 0.0, v);
                const double e = sd_energy(v.U[0], v.U[1], v.U[2], v.A2, v.e0, v.e1, v.e01, v.w);
                const double eu = e / (4.0 * v.w);
                double2 cg3[3];
                tri_corner_grads(v.U[0], v.U[1], v.U[2], v.A2, v.e0, v.e1, v.e01, v.w, cg3);
                double q[4] = {0.0, 0.0, 0.0, 0.0};
                double touch0 = 0.0, touch1 = 0.0;
                for (int k = 0; k < 3; ++k) {
                    if (v.slot[k] == 0) { q[0] += cg3[k].x; q[1] += cg3[k].y; touch0 = 1.0; }
                    if (v.slot[k] == 1) { q[2] += cg3[k].x; q[3] += cg3[k].y; touch1 = 1.0; }
                }
                for (int k = 0; k < 4; ++k) S.triG[lane][k] = q[k];
                S.triH[lane][0] = e;
                S.triH[lane][1] = eu;
                S.triH[lane][2] = log(eu);
                S.triH[lane][3] = touch0;
                S.triH[lane][4] = touch1;
            }
            __syncwarp();
            if (lane == 0) {
                const int n = min(32, P.nTri - c0);
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
            __syncwarp();
        }
        const double E0 = bij_mesh_energy(m, b, P, S);
        raw[0] = E0;
        raw[4] = E0;
        raw[5] = acc[10];
        raw[6] = -acc[11];
        raw[7] = acc[0] / P.nTri;
        raw[8] = acc[1] / P.nTri;
        raw[9] = acc[2] * acc[2] + acc[3] * acc[3];
        raw[10] = acc[4] * acc[4] + acc[5] * acc[5];
        raw[11] = acc[2] * acc[4] + acc[3] * acc[5];
        raw[12] = acc[6];
        raw[13] = acc[7];
        raw[14] = acc[8];
        raw[15] = acc[9];
    }
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
        const int nAll = P.nTri + S.nAirT;
        // ---- gradient: the local mesh's plus w_air times the air mesh's
        // (Scaffold::augmentGradient), one pass over both meshes
        double gj = 0.0;
        for (int c0 = 0; c0 < nAll; c0 += 32) {
            const int t = c0 + lane;
            if (t < nAll) {
                TriView v;
                tri_view(m, b, P, S, t, false, 0.0, v);
                double2 cg3[3];
                tri_corner_grads(v.U[0], v.U[1], v.U[2], v.A2, v.e0, v.e1, v.e01, v.w, cg3);
                for (int k = 0; k < 3; ++k) {
                    S.triG[lane][2 * k] = cg3[k].x;
                    S.triG[lane][2 * k + 1] = cg3[k].y;
                    S.triSlot[lane][k] = v.slot[k];
                }
            }
            __syncwarp();
            if (lane < nDof) {
                const int n = min(32, nAll - c0);
                for (int q = 0; q < n; ++q)
                    for (int k = 0; k < 3; ++k)
                        if (S.triSlot[q][k] == (lane >> 1)) gj = gj + S.triG[q][2 * k + (lane & 1)];
            }
            __syncwarp();
        }
        if (lane < nDof) S.g[lane] = gj;
        __syncwarp();
        double gsq = 0.0;
        for (int j = 0; j < nDof; ++j) gsq = gsq + S.g[j] * S.g[j];
        if (it == 0) raw[1] = gsq;
        if (gsq < P.targetGRes) {   // Optimizer.cpp:215-221
            status = 1;
            break;
        }
        // ---- dense Hessian: projected local and air blocks (the air ones
        // weighted w_air, Scaffold::augmentProxyMatrix's dense form), one pass
        const int nEnt = nDof * (nDof + 1) / 2;
        double hacc[kEntRounds];
        for (int r = 0; r < kEntRounds; ++r) hacc[r] = 0.0;
        for (int c0 = 0; c0 < nAll; c0 += 32) {
            const int t = c0 + lane;
            if (t < nAll) {
                TriView v;
                tri_view(m, b, P, S, t, false, 0.0, v);
                double H6[6][6];
                tri_hessian(v.U, v.A2, v.e0d, v.e1d, v.e01d, v.w, H6, b.fp32Hessian ? 2 : 1);
                for (int i = 0; i < 6; ++i)
                    for (int j = i; j < 6; ++j) S.triH[lane][bsym21(i, j)] = H6[i][j];
                for (int k = 0; k < 3; ++k) S.triSlot[lane][k] = v.slot[k];
            }
            __syncwarp();
            const int n = min(32, nAll - c0);
            for (int r = 0; r < kEntRounds; ++r) {
                const int e = lane + 32 * r;
                if (e >= nEnt) break;
                int i = 0, rem = e;
                while (rem >= nDof - i) { rem -= nDof - i; ++i; }
                const int j = i + rem;
                double acc = hacc[r];
                for (int q = 0; q < n; ++q)
                    for (int a = 0; a < 3; ++a) {
                        if (S.triSlot[q][a] != (i >> 1)) continue;
                        for (int c = 0; c < 3; ++c)
                            if (S.triSlot[q][c] == (j >> 1))
                                acc = acc + S.triH[q][bsym21(2 * a + (i & 1), 2 * c + (j & 1))];
                    }
                hacc[r] = acc;
            }
            __syncwarp();
        }
        for (int r = 0; r < kEntRounds; ++r) {
            const int e = lane + 32 * r;
            if (e >= nEnt) break;
            int i = 0, rem = e;
            while (rem >= nDof - i) { rem -= nDof - i; ++i; }
            const int j = i + rem;
            S.H[i][j] = hacc[r];
            S.H[j][i] = hacc[r];
        }
        if (lane < nDof) S.perm[lane] = lane;
        __syncwarp();
        // ---- H d = -g: LDL^T with symmetric pivoting on the largest
        // remaining diagonal (Eigen::LDLT), each step over the lanes (the
        // arithmetic of every entry as a single thread would do it)
        double dmax = 0.0;
        for (int i = 0; i < nDof; ++i) dmax = fmax(dmax, fabs(S.H[i][i]));
        for (int k = 0; k < nDof; ++k) {
            int piv = k;
            for (int i = k + 1; i < nDof; ++i)
                if (fabs(S.H[i][i]) > fabs(S.H[piv][piv])) piv = i;
            if (piv != k) {
                for (int j = lane; j < nDof; j += 32) {
                    const double t = S.H[k][j];
                    S.H[k][j] = S.H[piv][j];
                    S.H[piv][j] = t;
                }
                __syncwarp();
                for (int i = lane; i < nDof; i += 32) {
                    const double t = S.H[i][k];
                    S.H[i][k] = S.H[i][piv];
                    S.H[i][piv] = t;
                }
                if (lane == 0) {
                    const int tp = S.perm[k];
                    S.perm[k] = S.perm[piv];
                    S.perm[piv] = tp;
                }
                __syncwarp();
            }
            const double d = S.H[k][k];
            if (!(fabs(d) > 1e-300 + 1e-15 * dmax)) {
                __syncwarp();
                if (lane == 0) S.H[k][k] = 0.0;
                for (int i = k + 1 + lane; i < nDof; i += 32) S.H[i][k] = 0.0;
                __syncwarp();
                continue;
            }
            for (int i = k + 1 + lane; i < nDof; i += 32) S.H[i][k] = S.H[i][k] / d;
            __syncwarp();
            // the trailing update, pairs (i, j), k < j <= i, over the lanes
            const int mRem = nDof - k - 1;
            const int nPairs = mRem * (mRem + 1) / 2;
            for (int p = lane; p < nPairs; p += 32) {
                int ii = 0, rem = p;
                while (rem > ii) { rem -= ii + 1; ++ii; }
                const int i = k + 1 + ii, j = k + 1 + rem;
                const double v = S.H[i][j] - S.H[i][k] * d * S.H[j][k];
                S.H[i][j] = v;
                S.H[j][i] = v;
            }
            __syncwarp();
        }
        if (lane == 0) {
            double x[kBijDof];
            for (int i = 0; i < nDof; ++i) x[i] = -S.g[S.perm[i]];
            for (int i = 0; i < nDof; ++i)
                for (int k = 0; k < i; ++k) x[i] = x[i] - S.H[i][k] * x[k];
            for (int i = 0; i < nDof; ++i) x[i] = (S.H[i][i] != 0.0) ? x[i] / S.H[i][i] : 0.0;
            for (int i = nDof - 1; i >= 0; --i)
                for (int k = i + 1; k < nDof; ++k) x[i] = x[i] - S.H[k][i] * x[k];
            for (int i = 0; i < nDof; ++i) S.dir[S.perm[i]] = x[i];
        }
        __syncwarp();
        // ---- line search (Optimizer.cpp:575-652) over both meshes
        double bound = 1.0;
        for (int t = lane; t < nAll; t += 32) {
            TriView v;
            tri_view(m, b, P, S, t, false, 0.0, v);
            double2 D[3];
            for (int k = 0; k < 3; ++k)
                D[k] = v.slot[k] >= 0 ? make_double2(S.dir[2 * v.slot[k]], S.dir[2 * v.slot[k] + 1])
                                      : make_double2(0.0, 0.0);
            bound = fmin(bound, tri_step_bound(v.U[0], v.U[1], v.U[2], D[0], D[1], D[2], 1.0));
        }
        for (int o = 16; o > 0; o >>= 1) bound = fmin(bound, __shfl_xor_sync(0xffffffffu, bound, o));
        double step = bound * 0.99;
        if (lane < nFree) S.pos0[lane] = S.pos[lane];
        __syncwarp();
        // energy with the new scaffold at the current layout
        double eMesh0, eAir0, eMesh, eAir;
        bij_energies(m, b, P, S, false, 0.0, eMesh0, eAir0);
        lastE = eMesh0 + eAir0;
        bool stopped = false;
        bij_energies(m, b, P, S, true, step, eMesh, eAir);
        double testE = eMesh + eAir;
        ++trials;
        while (testE > lastE) {
            step = step / 2.0;
            if (step == 0.0) {
                stopped = true;
                break;
            }
            bij_energies(m, b, P, S, true, step, eMesh, eAir);
            testE = eMesh + eAir;
            ++trials;
        }
        if (lane < nFree) {
            S.pos[lane].x = S.pos0[lane].x + step * S.dir[2 * lane];
            S.pos[lane].y = S.pos0[lane].y + step * S.dir[2 * lane + 1];
        }
        __syncwarp();
        const double lastEDec = (lastE - testE) + (eAir - eAir0);
        if ((lastEDec / lastE < 1.0e-6 * step) && (step > 1.0e-3)) stopped = true;
        if (it == 0) {
            raw[2] = step;
            raw[3] = trials;
            raw[4] = eMesh;   // the local mesh's energy after the first step
        }
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
    const double curE = bij_mesh_energy(m, b, P, S);
    if (lane == 0) {
        LocalResult r;
        r.initE = initE;
        r.lastE = curE;
        r.eDec = failed ? -1.7976931348623157e308 : (initE - curE) * P.localArea / surfaceArea;
        for (int k = 0; k < kLocalMaxFree; ++k) r.pos[k] = k < nFreeMesh ? S.pos[k] : make_double2(0.0, 0.0);
        r.iters = it;
        r.status = failed ? 3 : (isfinite(curE) ? status : 2);
        r.trials = trials;
        for (int k = 0; k < kLocalRaw; ++k) r.raw[k] = raw[k];
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
