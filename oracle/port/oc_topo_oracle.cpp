// CPU restatement of the reference's topology queries (bijectivity off).
// TEST INFRASTRUCTURE ONLY: the checker for the device topology queries and
// the timed CPU baseline of a topology step; the product never links it.
//
// Follows src/TriMesh.cpp: querySplit (548-724), queryMerge (800-930),
// computeLocalLDec (2105-2260), computeLocalEdDec_inSplit (2262-2391),
// computeLocalEdDec_merge (2393-2505), computeLocalEdDec_bSplit
// (2507-2794), queryLocalEdDec_bSplit (2796-2862), isBoundaryVert
// (2032-2083), cutPath's interior branch (1449-1475), splitEdgeOnBoundary's
// vertex duplication (2864-2957), and SymDirichletEnergy::
// computeDivGradPerVert (108-147).  The local solve is the Optimizer's dense
// projected Newton (Optimizer.cpp:203-652 with useDense, energyParams {1},
// relGL2Tol 1e-6, 100 iterations) with an LDL^T of symmetric pivoting on
// the largest remaining diagonal (the scheme of Eigen's LDLT).  Candidates
// run in parallel on nThreads (the reference's tbb::parallel_for).

#include "oc_oracle.h"

#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>
#include <map>
#include <set>
#include <thread>
#include <utility>
#include <vector>

namespace {

struct Mesh {
    int nV = 0, nF = 0;
    std::vector<int> F;
    std::vector<double> Vr, V;
    std::map<std::pair<int, int>, int> edge2Tri;
    std::vector<std::set<int>> vNeighbor;

    void features()
    {
        edge2Tri.clear();
        vNeighbor.assign(nV, {});
        for (int t = 0; t < nF; ++t)
            for (int k = 0; k < 3; ++k) {
                const int a = F[3 * t + k], b = F[3 * t + (k + 1) % 3];
                edge2Tri[{a, b}] = t;
                vNeighbor[a].insert(b);
                vNeighbor[b].insert(a);
            }
    }
    int tri(int a, int b) const
    {
        auto it = edge2Tri.find({a, b});
        return it == edge2Tri.end() ? -1 : it->second;
    }
    bool isBoundaryVert(int v) const
    {
        for (int nb : vNeighbor[v])
            if (tri(v, nb) < 0 || tri(nb, v) < 0) return true;
        return false;
    }
    bool isBoundaryVert(int vI, int vNb, std::vector<int>& tris, bool toBound) const
    {
        tris.clear();
        int f = toBound ? tri(vNb, vI) : tri(vI, vNb);
        if (f < 0) return true;
        int vNew = vNb;
        while (true) {
            tris.push_back(f);
            for (int i = 0; i < 3; ++i) {
                const int x = F[3 * f + i];
                if (x != vI && x != vNew) { vNew = x; break; }
            }
            if (vNew == vNb) return false;
            f = toBound ? tri(vNew, vI) : tri(vI, vNew);
            if (f < 0) return true;
        }
    }
};

// SymDirichletEnergy::getEnergyValByElemID with the mesh's own weights
double elem_E(const double* rest, double w, const double U1[2], const double U2[2], const double U3[2])
{
    const double a0 = U2[0] - U1[0], a1 = U2[1] - U1[1], b0 = U3[0] - U1[0], b1 = U3[1] - U1[1];
    const double area_U = 0.5 * (a0 * b1 - a1 * b0);
    return w * (1.0 + rest[1] / area_U / area_U) *
           (((b0 * b0 + b1 * b1) * rest[2] + (a0 * a0 + a1 * a1) * rest[3]) / 4 / rest[1] -
            (b0 * a0 + b1 * a1) * rest[4] / 2 / rest[1]);
}

// The local Optimizer run: dense projected Newton on a small mesh.
// Returns eDec = (initE - E) * localArea / surfaceArea; V is updated.
struct Local {
    std::vector<double> Vr, V;   // local rest (3D) and UV
    std::vector<int> F;          // local triangles
    std::vector<int> fixed;      // local fixed vertices
};

double local_solve(Local& L, double initE_global, double surfaceArea, int maxIter)
{
    const int nV = static_cast<int>(L.V.size() / 2), nF = static_cast<int>(L.F.size() / 3);
    std::vector<double> rest(8 * (size_t)nF);
    double sc[3];
    ocr_rest_constants(L.Vr.data(), nV, L.F.data(), nF, 0.0, rest.data(), sc);
    const double localArea = sc[0];
    const double initE = initE_global * (surfaceArea / localArea);
    std::vector<char> isFixed(nV, 0);
    for (int v : L.fixed) isFixed[v] = 1;
    std::vector<int> dof(2 * nV, -1);
    int n = 0;
    for (int v = 0; v < nV; ++v)
        if (!isFixed[v]) { dof[2 * v] = n++; dof[2 * v + 1] = n++; }
    const double targetGRes = 1.0 * static_cast<double>(nV - (int)L.fixed.size()) / static_cast<double>(nV) * 1.0e-6;
    double lastE = ocr_energy(rest.data(), L.F.data(), nF, L.V.data(), 0);
    std::vector<double> g(2 * nV), blocks(36 * (size_t)nF), d(2 * nV), V0;
    for (int it = 0; it < maxIter; ++it) {
        ocr_gradient(rest.data(), L.F.data(), nF, L.V.data(), nV, L.fixed.data(), (int)L.fixed.size(), 0, g.data());
        double gsq = 0.0;
        for (double x : g) gsq += x * x;
        if (gsq < targetGRes) break;
        ocr_hessian_blocks(rest.data(), L.F.data(), nF, L.V.data(), 0, blocks.data());
        std::vector<double> H((size_t)n * n, 0.0), b(n);
        for (int t = 0; t < nF; ++t)
            for (int a = 0; a < 3; ++a)
                for (int c = 0; c < 3; ++c)
                    for (int i = 0; i < 2; ++i)
                        for (int j = 0; j < 2; ++j) {
                            const int r = dof[2 * L.F[3 * t + a] + i], s = dof[2 * L.F[3 * t + c] + j];
                            if (r >= 0 && s >= 0) H[(size_t)r * n + s] += blocks[36 * (size_t)t + 6 * (2 * a + i) + 2 * c + j];
                        }
        for (int v = 0; v < 2 * nV; ++v)
            if (dof[v] >= 0) b[dof[v]] = -g[v];
        // LDL^T with symmetric pivoting (largest remaining diagonal)
        std::vector<int> perm(n);
        for (int i = 0; i < n; ++i) perm[i] = i;
        double dmax = 0.0;
        for (int i = 0; i < n; ++i) dmax = std::max(dmax, std::fabs(H[(size_t)i * n + i]));
        auto A = [&](int i, int j) -> double& { return H[(size_t)i * n + j]; };
        for (int k = 0; k < n; ++k) {
            int piv = k;
            for (int i = k + 1; i < n; ++i)
                if (std::fabs(A(i, i)) > std::fabs(A(piv, piv))) piv = i;
            if (piv != k) {
                for (int j = 0; j < n; ++j) std::swap(A(k, j), A(piv, j));
                for (int i = 0; i < n; ++i) std::swap(A(i, k), A(i, piv));
                std::swap(perm[k], perm[piv]);
            }
            const double dk = A(k, k);
            if (!(std::fabs(dk) > 1e-300 + 1e-15 * dmax)) {
                A(k, k) = 0.0;
                for (int i = k + 1; i < n; ++i) A(i, k) = 0.0;
                continue;
            }
            for (int i = k + 1; i < n; ++i) A(i, k) /= dk;
            for (int i = k + 1; i < n; ++i)
                for (int j = k + 1; j <= i; ++j) {
                    A(i, j) -= A(i, k) * dk * A(j, k);
                    A(j, i) = A(i, j);
                }
        }
        std::vector<double> y(n);
        for (int i = 0; i < n; ++i) y[i] = b[perm[i]];
        for (int i = 0; i < n; ++i)
            for (int k = 0; k < i; ++k) y[i] -= A(i, k) * y[k];
        for (int i = 0; i < n; ++i) y[i] = A(i, i) != 0.0 ? y[i] / A(i, i) : 0.0;
        for (int i = n - 1; i >= 0; --i)
            for (int k = i + 1; k < n; ++k) y[i] -= A(k, i) * y[k];
        std::fill(d.begin(), d.end(), 0.0);
        for (int v = 0; v < 2 * nV; ++v)
            if (dof[v] >= 0) {
                for (int i = 0; i < n; ++i)
                    if (perm[i] == dof[v]) d[v] = y[i];
            }
        // line search
        double step = 1.0;
        ocr_init_step_size(L.F.data(), nF, L.V.data(), d.data(), &step);
        step *= 0.99;
        V0 = L.V;
        bool stopped = false;
        auto forward = [&](double s) {
            for (int k = 0; k < 2 * nV; ++k) L.V[k] = V0[k] + s * d[k];
        };
        forward(step);
        double testE = ocr_energy(rest.data(), L.F.data(), nF, L.V.data(), 0);
        while (testE > lastE) {
            step /= 2.0;
            if (step == 0.0) { stopped = true; break; }
            forward(step);
            testE = ocr_energy(rest.data(), L.F.data(), nF, L.V.data(), 0);
        }
        const double lastEDec = lastE - testE;
        if ((lastEDec / lastE < 1.0e-6 * step) && (step > 1.0e-3)) stopped = true;
        lastE = testE;
        if (stopped) break;
    }
    return (initE - lastE) * localArea / surfaceArea;
}

// local mesh over `tris` (first appearance), optionally with vertex b mapped onto a
struct LocalBuild {
    std::map<int, int> g2l;
    Local L;
    void build(const Mesh& M, const std::vector<int>& tris, const std::set<int>& freeVert, int a = -1, int b = -1,
               const double* mergedPos = nullptr)
    {
        for (int t : tris)
            for (int k = 0; k < 3; ++k) {
                int g = M.F[3 * t + k];
                const bool merged = (g == a || g == b) && a >= 0;
                auto it = g2l.find(g);
                if (it == g2l.end() && merged) it = g2l.find(g == a ? b : a);
                int l;
                if (it == g2l.end()) {
                    l = static_cast<int>(L.V.size() / 2);
                    if (!freeVert.count(g)) L.fixed.push_back(l);
                    L.Vr.insert(L.Vr.end(), {M.Vr[3 * g], M.Vr[3 * g + 1], M.Vr[3 * g + 2]});
                    if (merged) L.V.insert(L.V.end(), {mergedPos[0], mergedPos[1]});
                    else L.V.insert(L.V.end(), {M.V[2 * g], M.V[2 * g + 1]});
                    g2l[g] = l;
                    if (merged) g2l[g == a ? b : a] = l;
                }
                else {
                    l = it->second;
                }
                L.F.push_back(l);
            }
    }
    int add_copy(int l)
    {
        const int n = static_cast<int>(L.V.size() / 2);
        L.Vr.insert(L.Vr.end(), {L.Vr[3 * l], L.Vr[3 * l + 1], L.Vr[3 * l + 2]});
        L.V.insert(L.V.end(), {L.V[2 * l], L.V[2 * l + 1]});
        return n;
    }
};

double init_energy(const Mesh& M, const double* rest, double surfaceArea, const std::vector<int>& tris)
{
    double e = 0.0;
    for (int t : tris) {
        const int* f = &M.F[3 * t];
        e += elem_E(rest + 8 * (size_t)t, rest[8 * (size_t)t] / surfaceArea, &M.V[2 * f[0]], &M.V[2 * f[1]], &M.V[2 * f[2]]);
    }
    return e;
}

double rdist(const Mesh& M, int a, int b)
{
    const double dx = M.Vr[3 * a] - M.Vr[3 * b], dy = M.Vr[3 * a + 1] - M.Vr[3 * b + 1], dz = M.Vr[3 * a + 2] - M.Vr[3 * b + 2];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

void replace(std::vector<int>& F, const std::vector<int>& tris, const std::vector<int>& localTris, int from, int to)
{
    // tris: global ids in local order; localTris: the global ids whose local copy changes
    for (size_t k = 0; k < tris.size(); ++k)
        if (std::find(localTris.begin(), localTris.end(), tris[k]) != localTris.end())
            for (int c = 0; c < 3; ++c)
                if (F[3 * k + c] == from) { F[3 * k + c] = to; break; }
}

} // namespace

extern "C" int ocr_topology_query(int nV, const int* F, int nF, const double* Vrest, const double* UV, const int* cohE,
                                  int nCohE, int opType, double lambda_t, double filterExp, int nThreads,
                                  int maxCand, double* EwDec, double* ec, int* path, double* pos, int* posRows,
                                  int* nCand, double* seconds)
{
    const auto t0 = std::chrono::steady_clock::now();
    Mesh M;
    M.nV = nV;
    M.nF = nF;
    M.F.assign(F, F + 3 * (size_t)nF);
    M.Vr.assign(Vrest, Vrest + 3 * (size_t)nV);
    M.V.assign(UV, UV + 2 * (size_t)nV);
    M.features();
    std::vector<double> rest(8 * (size_t)nF);
    double sc[3];
    ocr_rest_constants(Vrest, nV, F, nF, 0.0, rest.data(), sc);
    const double surfaceArea = sc[0], avgEdgeLen = sc[1], R = sc[2];
    struct Cand { double EwDec = -DBL_MAX, ec0 = DBL_MAX, ec1 = DBL_MAX; std::vector<int> path; std::vector<double> pos; };
    std::vector<Cand> out;
    std::vector<int> verts;
    if (opType == 0 || opType == 1) {
        // computeDivGradPerVert (standard-deviation filter)
        std::vector<double> mean(2 * nV, 0.0), sd(nV, 0.0), lg(6 * (size_t)nF);
        std::vector<int> cnt(nV, 0);
        for (int t = 0; t < nF; ++t) {
            // per-corner gradients: the scatter of ocr_gradient, one triangle at a time
            std::vector<double> g1(2 * nV, 0.0);
            const int f[3] = {F[3 * t], F[3 * t + 1], F[3 * t + 2]};
            double gt[6];
            {
                std::vector<double> tv = {UV[2 * f[0]], UV[2 * f[0] + 1], UV[2 * f[1]], UV[2 * f[1] + 1], UV[2 * f[2]],
                                          UV[2 * f[2] + 1]};
                const int lf[3] = {0, 1, 2};
                double r8[8];
                std::memcpy(r8, &rest[8 * (size_t)t], sizeof(r8));
                double g6[6];
                // gradient of the single triangle with the global weight
                std::vector<double> rr(r8, r8 + 8);
                rr[0] = rest[8 * (size_t)t];
                ocr_gradient(rr.data(), lf, 1, tv.data(), 3, nullptr, 0, 1, g6);
                const double w = rest[8 * (size_t)t] / surfaceArea;
                for (int k = 0; k < 6; ++k) gt[k] = w * g6[k];
            }
            for (int k = 0; k < 3; ++k) {
                lg[6 * (size_t)t + 2 * k] = gt[2 * k];
                lg[6 * (size_t)t + 2 * k + 1] = gt[2 * k + 1];
                mean[2 * f[k]] += gt[2 * k];
                mean[2 * f[k] + 1] += gt[2 * k + 1];
                cnt[f[k]]++;
            }
        }
        for (int v = 0; v < nV; ++v) {
            mean[2 * v] /= cnt[v];
            mean[2 * v + 1] /= cnt[v];
        }
        for (int t = 0; t < nF; ++t)
            for (int k = 0; k < 3; ++k) {
                const int v = F[3 * t + k];
                const double dx = lg[6 * (size_t)t + 2 * k] - mean[2 * v], dy = lg[6 * (size_t)t + 2 * k + 1] - mean[2 * v + 1];
                sd[v] += dx * dx + dy * dy;
            }
        std::map<double, int> sorted;
        for (int v = 0; v < nV; ++v) {
            if (M.vNeighbor[v].size() <= 2) continue;
            const double dg = cnt[v] == 1 ? 0.0 : std::sqrt(sd[v] / (cnt[v] - 1.0));
            if (opType == 0) {
                if (M.isBoundaryVert(v)) sorted[-dg / 1.0] = v;
            }
            else if (!M.isBoundaryVert(v)) {
                bool toB = false;
                for (int nb : M.vNeighbor[v]) toB = toB || M.isBoundaryVert(nb);
                if (!toB) sorted[-dg / 1.0] = v;
            }
        }
        int amt = static_cast<int>(std::pow(static_cast<double>(sorted.size()), opType == 0 ? 0.8 : filterExp));
        if (amt < 2) amt = 2;
        for (const auto& kv : sorted) {
            verts.push_back(kv.second);
            if ((int)verts.size() >= amt) break;
        }
        out.resize(verts.size());
        auto work = [&](int ci) {
            const int vI = verts[ci];
            Cand& C = out[ci];
            std::vector<int> umbrella;
            const int nbMin = *M.vNeighbor[vI].begin();
            if (M.isBoundaryVert(vI, nbMin, umbrella, false)) {
                C.path = {0, 0};
                for (int nbVI : M.vNeighbor[vI]) {
                    if (M.tri(vI, nbVI) < 0 || M.tri(nbVI, vI) < 0) continue;
                    const bool cut = M.isBoundaryVert(nbVI);
                    std::vector<int> tris, t1, t2;
                    M.isBoundaryVert(vI, nbVI, tris, false);
                    M.isBoundaryVert(vI, nbVI, t1, true);
                    tris.insert(tris.end(), t1.begin(), t1.end());
                    if (cut)
                        for (int cw = 0; cw < 2; ++cw) {
                            M.isBoundaryVert(nbVI, vI, t2, cw != 0);
                            for (int t : t2)
                                if (std::find(tris.begin(), tris.end(), t) == tris.end()) tris.push_back(t);
                        }
                    std::set<int> freeV{vI};
                    if (cut) freeV.insert(nbVI);
                    LocalBuild B;
                    B.build(M, tris, freeV);
                    const double initE = init_energy(M, rest.data(), surfaceArea, tris);
                    const int lb = B.g2l[vI], li = B.g2l[nbVI];
                    const int cb = B.add_copy(lb);
                    replace(B.L.F, tris, t1, lb, cb);
                    int ci2 = -1;
                    if (cut) {
                        std::vector<int> sideI;
                        M.isBoundaryVert(nbVI, vI, sideI, true);
                        ci2 = B.add_copy(li);
                        replace(B.L.F, tris, sideI, li, ci2);
                    }
                    const double SDDec = local_solve(B.L, initE, surfaceArea, 100);
                    const double seInc = rdist(M, vI, nbVI) / R * (1.0 + 1.0) / 2.0;
                    const double cur = (1.0 - lambda_t) * SDDec - lambda_t * seInc;
                    if (cur > C.EwDec) {
                        C.EwDec = cur;
                        C.ec0 = -SDDec;
                        C.ec1 = seInc;
                        C.path = {vI, nbVI};
                        C.pos = {B.L.V[2 * lb], B.L.V[2 * lb + 1], B.L.V[2 * cb], B.L.V[2 * cb + 1]};
                        if (cut)
                            C.pos.insert(C.pos.end(), {B.L.V[2 * ci2], B.L.V[2 * ci2 + 1], B.L.V[2 * li], B.L.V[2 * li + 1]});
                    }
                }
            }
            else {
                C.path = {0, 0, 0};
                const int n = static_cast<int>(umbrella.size());
                const double initE = init_energy(M, rest.data(), surfaceArea, umbrella);
                auto after = [&](int t) {
                    for (int i = 0; i < 3; ++i)
                        if (M.F[3 * t + i] == vI) return M.F[3 * t + (i + 1) % 3];
                    return -1;
                };
                for (int s = 0; s + 1 < n; ++s) {
                    const int p0 = after(umbrella[s]);
                    for (int e = s + 1; e < n; ++e) {
                        const int p2 = after(umbrella[e]);
                        std::vector<int> left;
                        int vNew = p0;
                        while (true) {
                            const int f = M.tri(vI, vNew);
                            left.push_back(f);
                            for (int i = 0; i < 3; ++i) {
                                const int x = M.F[3 * f + i];
                                if (x != vI && x != vNew) { vNew = x; break; }
                            }
                            if (vNew == p2 || vNew == p0) break;
                        }
                        LocalBuild B;
                        B.build(M, umbrella, {vI});
                        const int lv = B.g2l[vI];
                        const int cv = B.add_copy(lv);
                        replace(B.L.F, umbrella, left, lv, cv);
                        const double SDDec = local_solve(B.L, initE, surfaceArea, 100);
                        const double seInc = (rdist(M, p0, vI) * (1.0 + 1.0) + rdist(M, vI, p2) * (1.0 + 1.0)) / R / 2.0;
                        const double Ew = (1.0 - lambda_t) * SDDec - lambda_t * seInc;
                        if (Ew > C.EwDec) {
                            C.EwDec = Ew;
                            C.ec0 = -SDDec;
                            C.ec1 = seInc;
                            C.path = {p0, vI, p2};
                            C.pos = {B.L.V[2 * cv], B.L.V[2 * cv + 1], B.L.V[2 * lv], B.L.V[2 * lv + 1]};
                        }
                    }
                }
                if (C.EwDec != -DBL_MAX) C.EwDec *= 0.5;
            }
        };
        const int nc = static_cast<int>(verts.size());
        const int nt = std::max(1, std::min(nThreads, nc));
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; ++t)
            pool.emplace_back([&, t] {
                for (int ci = t; ci < nc; ci += nt) work(ci);
            });
        for (auto& th : pool) th.join();
    }
    else {
        const double eps_IC = 1.0e-6 * avgEdgeLen;
        for (int ci = 0; ci < nCohE; ++ci) {
            const int* ce = cohE + 4 * (size_t)ci;
            int fork;
            if (ce[0] == ce[2]) fork = 0;
            else if (ce[1] == ce[3]) fork = 1;
            else continue;
            const int va = ce[1 - fork], vb = ce[3 - fork];
            std::vector<int> tris;
            int firstAmt = 0;
            for (int m2 = 0; m2 < 2; ++m2) {
                const int v = m2 ? vb : va;
                for (int nb : M.vNeighbor[v]) {
                    const int f = M.tri(v, nb);
                    if (f >= 0) tris.push_back(f);
                }
                if (!m2) firstAmt = static_cast<int>(tris.size());
            }
            double mp[2] = {(M.V[2 * va] + M.V[2 * vb]) / 2.0, (M.V[2 * va + 1] + M.V[2 * vb + 1]) / 2.0};
            std::vector<double> W = M.V;
            auto inverted = [&](const double* p) {
                W[2 * va] = W[2 * vb] = p[0];
                W[2 * va + 1] = W[2 * vb + 1] = p[1];
                bool bad = false;
                for (int t : tris) {
                    const int* f = &M.F[3 * t];
                    const double e00 = W[2 * f[1]] - W[2 * f[0]], e01 = W[2 * f[1] + 1] - W[2 * f[0] + 1];
                    const double e10 = W[2 * f[2]] - W[2 * f[0]], e11 = W[2 * f[2] + 1] - W[2 * f[0] + 1];
                    if (e00 * e11 - e01 * e10 < 0.0) bad = true;
                }
                return bad;
            };
            if (inverted(mp)) {
                std::vector<double> cm, cv;
                for (size_t k = 0; k < tris.size(); ++k) {
                    const int t = tris[k], vm = (int)k < firstAmt ? va : vb;
                    for (int i = 0; i < 3; ++i)
                        if (M.F[3 * t + i] == vm) {
                            const int i1 = M.F[3 * t + (i + 1) % 3], i2 = M.F[3 * t + (i + 2) % 3];
                            const double cx = W[2 * i2 + 1] - W[2 * i1 + 1], cy = W[2 * i1] - W[2 * i2];
                            const double nr = std::sqrt(cx * cx + cy * cy);
                            cm.push_back(cx / nr);
                            cm.push_back(cy / nr);
                            cv.push_back((W[2 * i1] * W[2 * i2 + 1] - W[2 * i1 + 1] * W[2 * i2]) / nr);
                            break;
                        }
                }
                for (int iter = 0; iter < 70; ++iter) {
                    double maxRes = -DBL_MAX;
                    for (size_t k = 0; k < cv.size(); ++k) {
                        const double res = cm[2 * k] * mp[0] + cm[2 * k + 1] * mp[1] - cv[k];
                        if (res > -eps_IC) {
                            mp[0] -= (res + eps_IC) * cm[2 * k];
                            mp[1] -= (res + eps_IC) * cm[2 * k + 1];
                        }
                        maxRes = std::max(maxRes, res);
                    }
                    if (maxRes < 0.0) break;
                }
                if (inverted(mp)) continue;
            }
            const int p0 = fork ? ce[0] : ce[3], p1 = fork ? ce[1] : ce[2], p2 = fork ? ce[2] : ce[1];
            double seDec = rdist(M, p0, p1) / R * (1.0 + 1.0) / 2.0;
            for (int nb : M.vNeighbor[p0])
                if (nb != p1 && M.isBoundaryVert(nb) && M.vNeighbor[p2].count(nb)) {
                    seDec += rdist(M, p0, nb) / R * (1.0 + 1.0) / 2.0;
                    break;
                }
            LocalBuild B;
            B.build(M, tris, {p0, p2}, p0, p2, mp);
            const double initE = init_energy(M, rest.data(), surfaceArea, tris);
            const double SDInc = -local_solve(B.L, initE, surfaceArea, 100);
            Cand C;
            C.EwDec = lambda_t * seDec - (1.0 - lambda_t) * SDInc;
            C.ec0 = SDInc;
            C.ec1 = -seDec;
            C.path = {p0, p1, p2};
            const int lm = B.g2l[p0];
            C.pos = {B.L.V[2 * lm], B.L.V[2 * lm + 1]};
            out.push_back(C);
        }
    }
    const int n = std::min(static_cast<int>(out.size()), maxCand);
    for (int c = 0; c < n; ++c) {
        EwDec[c] = out[c].EwDec;
        ec[2 * c] = out[c].ec0;
        ec[2 * c + 1] = out[c].ec1;
        for (int k = 0; k < 3; ++k) path[3 * c + k] = k < (int)out[c].path.size() ? out[c].path[k] : -1;
        posRows[c] = static_cast<int>(out[c].pos.size() / 2);
        for (size_t k = 0; k < out[c].pos.size(); ++k) pos[8 * (size_t)c + k] = out[c].pos[k];
    }
    *nCand = static_cast<int>(out.size());
    if (seconds) *seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    return 0;
}
