// Batched local projected-Newton solves of the topology step's candidates
// (TriMesh::computeLocalEdDec_*, TriMesh.cpp:2263-2862, with the Optimizer's
// dense path).  Compiled with FMA contraction (unlike the global step's
// oc_fp64.cu): the local solves are checked against the oracle to a
// tolerance, not bit for bit.

#include "oc_elem.cuh"
#include "oc_internal.h"

#include <cooperative_groups.h>

#include <algorithm>
#include <cstdint>

namespace oc {
namespace {

// ---------------------------------------------------- local topology solves
// The projected-Newton loop the reference runs on a candidate's local mesh
// (Optimizer with useDense, energyParams {1}, relGL2Tol 1e-6,
// solve(maxIter): Optimizer.cpp:203-261, 505-652; dense Hessian
// SymDirichletEnergy.cpp:306-427 + LDLT), one local problem per group of
// TPP threads (CL = 1) or per thread-block cluster of blocks of TPP threads
// (CL = 2: clustered, the cluster's size read at run time).  Threads own triangles; a block sums its contiguous range of
// triangles in triangle order on single threads, and a cluster adds its
// blocks' partial sums in rank order (every block reads them all through
// distributed shared memory, so all blocks hold the same totals and run
// the same serial steps).  The arithmetic depends only on the schedule,
// which the host picks from the triangle count, so results are deterministic.
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
    int sub, rank, ncl, buf;   // ncl: blocks in this problem's cluster (1 unclustered)
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
            for (int r = 0; r < G.ncl; ++r) {
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
    int ncl = 1, rank = 0;
    if constexpr (CL > 1) {
        cg::cluster_group cl = cg::this_cluster();
        ncl = static_cast<int>(cl.num_blocks());
        rank = static_cast<int>(cl.block_rank());
    }
    const int pi = CL > 1 ? static_cast<int>(blockIdx.x) / ncl : static_cast<int>(blockIdx.x) * groups + grp;
    // packed groups (TPP < 32) stay alive past the last problem, solving a
    // copy of it without writing a result, so that their warp can reconverge
    // once per Newton iteration; the other forms leave (uniform per block
    // and cluster)
    const bool valid = pi < b.nProb;
    if (TPP >= 32 && !valid) return;
    LocalGroup<TPP, CL> G;
    G.sub = threadIdx.x % TPP;
    G.mask = TPP >= 32 ? 0xffffffffu : (((1u << TPP) - 1u) << ((threadIdx.x & 31) & ~(TPP - 1)));
    G.rank = rank;
    G.ncl = ncl;
    G.buf = 0;
    LocalShared<TPP>& S = reinterpret_cast<LocalShared<TPP>*>(localSmem)[grp];
    const int sub = G.sub;
    const long long clk0 = clock64();
    const LocalProblem P = b.prob[valid ? pi : b.nProb - 1];
    const int nDof = 2 * P.nFree;
    // this block's triangles [lo, hi) and initial-energy triangles [ilo, ihi)
    const int per = (P.nTri + ncl - 1) / ncl, iper = (P.nInit + ncl - 1) / ncl;
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
    bool running = true;
    for (;;) {
        running = running && it < P.maxIter && finite;
        if constexpr (TPP < 32) {
            if (!__any_sync(0xffffffffu, running)) break;
        }
        else {
            if (!running) break;
        }
        if (running) do {
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
            running = false;
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
            running = false;
            break;
        }
        ++it;
        } while (false);
        // packed groups: reconverge the warp once per iteration, so that the
        // next iteration's element Hessians run for all of its problems at
        // once instead of one group after another
        if constexpr (TPP < 32) __syncwarp();
    }
    if (!finite) status = 2;
    if (valid && sub == 0 && G.rank == 0) {
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

namespace {
template <int TPP, int CL>
cudaError_t launch_local_tpp(const DeviceMesh& m, double surfaceArea, const LocalBatch& b, int block, int cluster,
                             cudaStream_t st)
{
    constexpr int maxThreads = local_threads<TPP, CL>();
    const int threads = (TPP >= 128 || CL > 1) ? maxThreads : std::max(TPP, std::min(maxThreads, block));
    constexpr size_t smemMax = local_smem<TPP, CL>(maxThreads);
    const size_t smem = local_smem<TPP, CL>(threads);
    static const cudaError_t attr = [] {
        cudaError_t e = cudaFuncSetAttribute(k_local_newton<TPP, CL>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             static_cast<int>(smemMax));
        if (e == cudaSuccess && CL > 1)
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
        cfg.gridDim = dim3(static_cast<unsigned>(b.nProb) * cluster, 1, 1);
        cfg.blockDim = dim3(threads, 1, 1);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = st;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = cluster;
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
// spread over more SMs; larger problems spread over a cluster of blocks, one
// warp's worth (32) of triangles per block, as long as count x cluster
// blocks stay within about four blocks per SM.
LocalSchedule local_schedule(int maxTri, int count, int numSMs, int maxCluster)
{
    if (maxTri <= 8) return {8, 1, count / 16 >= 2 * numSMs ? 128 : 32};
    if (maxTri <= 40) return {32, 1, count / 4 >= 2 * numSMs ? 128 : 32};
    int c = std::min(maxCluster, (maxTri + 31) / 32);
    while (c > 1 && c * count > 4 * numSMs) --c;
    if (c <= 1) return {128, 1, 128};
    return {64, c, 64};
}

int local_max_cluster()
{
    // 16-block clusters need the non-portable size and room on one GPC
    static const int v = [] {
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(16, 1, 1);
        cfg.blockDim = dim3(64, 1, 1);
        cfg.dynamicSmemBytes = local_smem<64, 2>(64);
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeClusterDimension;
        at[0].val.clusterDim.x = 16;
        at[0].val.clusterDim.y = 1;
        at[0].val.clusterDim.z = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        int n = 0;
        if (cudaFuncSetAttribute(k_local_newton<64, 2>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1) !=
                cudaSuccess ||
            cudaFuncSetAttribute(k_local_newton<64, 2>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 static_cast<int>(local_smem<64, 2>(64))) != cudaSuccess ||
            cudaOccupancyMaxActiveClusters(&n, k_local_newton<64, 2>, &cfg) != cudaSuccess) {
            cudaGetLastError();
            return 8;
        }
        return n > 0 ? 16 : 8;
    }();
    return v;
}

namespace {

// Element Hessians of the global Newton step with the translation-free 4x4
// PSD projection (FMA contraction on; the 6x6 form is k_hessian in oc_fp64.cu)
__global__ void __launch_bounds__(128) k_hessian_reduced(DeviceMesh m, int uniform, double density,
                                                         double* __restrict__ hb)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= m.nF) return;
    const double2 U[3] = {m.uv[m.F0[t]], m.uv[m.F1[t]], m.uv[m.F2[t]]};
    double H[6][6];
    tri_hessian(U, m.A2[t], m.e0d[t], m.e1d[t], m.e01d[t], uniform ? 1.0 : m.w[t], H, density > 0.0 ? 3 : 1,
                density);
    store_hessian_blocks(H, t, m.nF, hb);
}

} // namespace

void launch_hessian_reduced(const DeviceMesh& m, int uniform, double* hb, cudaStream_t st, double density)
{
    if (m.nF > 0) k_hessian_reduced<<<(m.nF + 127) / 128, 128, 0, st>>>(m, uniform, density, hb);
}

cudaError_t launch_local_newton(const DeviceMesh& m, double surfaceArea, const LocalBatch& b, LocalSchedule sc,
                                cudaStream_t st)
{
    if (b.nProb <= 0) return cudaSuccess;
    const int bl = sc.block;
    if (sc.cluster == 1) {
        if (sc.tpp == 8) return launch_local_tpp<8, 1>(m, surfaceArea, b, bl, 1, st);
        if (sc.tpp == 32) return launch_local_tpp<32, 1>(m, surfaceArea, b, bl, 1, st);
        if (sc.tpp == 128) return launch_local_tpp<128, 1>(m, surfaceArea, b, bl, 1, st);
    }
    else if (sc.tpp == 64 && sc.cluster >= 2 && sc.cluster <= 16) {
        // clustered form: the cluster size is read at run time
        return launch_local_tpp<64, 2>(m, surfaceArea, b, bl, sc.cluster, st);
    }
    return cudaErrorInvalidValue;
}

} // namespace oc
