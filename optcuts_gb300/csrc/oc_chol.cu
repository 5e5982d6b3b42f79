// Multifrontal sparse Cholesky on the device -- the exact Newton solve.
//
// The reference factorises the Newton matrix with Eigen's SimplicialLDLT
// (src/LinSysSolver/EigenLibSolver.cpp:71-107) on one host thread; at
// 200k triangles that is ~94% of its iteration time.  Block-Jacobi PCG does
// not converge on these systems (a Tutte start has condition numbers near
// 1e14), so the default solver here is an exact factorisation too:
//
//  * symbolic (host, once per topology): nested dissection of the vertex
//    graph by BFS level sets; each dissection node is one dense front whose
//    rows are its own vertices followed by the ancestor vertices its subtree
//    touches; per-topology maps for assembling the block-CSR values into the
//    fronts, for the children's extend-add and for the tiled kernels' work;
//  * numeric (device, every iteration): fronts are processed bottom-up one
//    tree level at a time; within a level every front is factorised by the
//    same batched tile kernels (32 x 32 FP64 tiles: LDL^T of the diagonal
//    tile, triangular solve of the panel, trailing update), so one launch
//    serves all fronts of a level; in large factorizations the independent
//    subtrees below the tree's top chain run this on streams of their own
//    (events join them, all inside one captured graph);
//  * solve: forward and backward substitution front by front, level by
//    level, with the children's update vectors extend-added in a fixed
//    order (deterministic, no atomics).
//
// All arithmetic is FP64.  The factorisation is LDL^T without pivoting, the
// reference's own (SimplicialLDLT): a PSD-projected matrix with near-null
// modes can produce tiny negative pivots in rounding, which LDL^T carries;
// a zero or non-finite pivot is replaced by 1e-300 and counted.

#include "oc_chol.h"

#include <chrono>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <deque>
#include <functional>
#include <numeric>
#include <thread>

namespace oc {

// ------------------------------------------------------------------ symbolic
namespace {

// Nested dissection of `verts` by BFS level sets from a pseudo-peripheral
// vertex, into `nodes` in postorder (children first, the separator last;
// node ids local to this call's list).  Subtrees of more than kNdParallel
// vertices are dissected on their own host threads and spliced in the same
// order, so the result equals the sequential dissection.  tag / level are
// shared arrays over all vertices (the subtrees' vertex sets are disjoint);
// tags only need to be distinct, so the counter is atomic.
constexpr size_t kNdParallel = 4096;

void nd_build(const int* rowPtr, const int* col, std::vector<int>& verts, std::vector<int>& tag,
              std::atomic<int>& tagCounter, std::vector<int>& level, std::vector<NdNode>& nodes, int leafSize,
              int depth, const double* xy)
{
    const int myTag = ++tagCounter;
    for (int v : verts) tag[v] = myTag;
    auto make_leaf = [&]() { nodes.push_back(NdNode{verts, {}}); };
    if ((int)verts.size() <= leafSize) return make_leaf();
    std::vector<int> left, right, sep;
    // BFS level sets: two passes, the second from the last vertex the first
    // reached; the separator is the level holding the median vertex.
    // false when the set is too shallow to split
    auto bfs_split = [&](std::vector<int>& L, std::vector<int>& R, std::vector<int>& S) {
        std::vector<int> q;
        q.reserve(verts.size());
        auto bfs = [&](int s0) {
            q.clear();
            for (int v : verts) level[v] = -1;
            level[s0] = 0;
            q.push_back(s0);
            for (size_t h = 0; h < q.size(); ++h) {
                const int v = q[h];
                for (int p = rowPtr[v]; p < rowPtr[v + 1]; ++p) {
                    const int u = col[p];
                    if (tag[u] == myTag && level[u] < 0) {
                        level[u] = level[v] + 1;
                        q.push_back(u);
                    }
                }
            }
        };
        bfs(verts[0]);
        bfs(q.back());
        const int reached = static_cast<int>(q.size());
        const int maxLevel = level[q.back()];
        if (maxLevel < 2) return false;
        std::vector<int> cnt(maxLevel + 1, 0);
        for (int i = 0; i < reached; ++i) cnt[level[q[i]]]++;
        const int total = static_cast<int>(verts.size());
        int sepLevel = 1, cum = 0;
        for (int l = 0; l <= maxLevel; ++l) {
            cum += cnt[l];
            if (2 * cum >= total) { sepLevel = l; break; }
        }
        sepLevel = std::max(1, std::min(sepLevel, maxLevel - 1));
        for (int v : verts) {
            const int l = level[v];
            if (l < 0 || l > sepLevel) R.push_back(v);
            else if (l < sepLevel) L.push_back(v);
            else S.push_back(v);
        }
        return true;
    };
    // geometric bisection at the median along the longer extent: the lower
    // half's vertices with a neighbour in the upper half are the separator
    auto geo_split = [&](std::vector<int>& L, std::vector<int>& R, std::vector<int>& S) {
        double lo[2] = {xy[2 * (size_t)verts[0]], xy[2 * (size_t)verts[0] + 1]}, hi[2] = {lo[0], lo[1]};
        for (int v : verts)
            for (int a = 0; a < 2; ++a) {
                lo[a] = std::min(lo[a], xy[2 * (size_t)v + a]);
                hi[a] = std::max(hi[a], xy[2 * (size_t)v + a]);
            }
        const int ax = (hi[0] - lo[0]) >= (hi[1] - lo[1]) ? 0 : 1;
        std::vector<int> byCoord(verts);
        const size_t half = byCoord.size() / 2;
        std::nth_element(byCoord.begin(), byCoord.begin() + half, byCoord.end(), [&](int a, int b) {
            const double xa = xy[2 * (size_t)a + ax], xb = xy[2 * (size_t)b + ax];
            return xa < xb || (xa == xb && a < b);
        });
        for (size_t i = 0; i < byCoord.size(); ++i) level[byCoord[i]] = i < half ? 0 : 1;
        for (int v : verts) {
            if (level[v] == 1) {
                R.push_back(v);
                continue;
            }
            bool cut = false;
            for (int p = rowPtr[v]; p < rowPtr[v + 1] && !cut; ++p) {
                const int u = col[p];
                cut = tag[u] == myTag && level[u] == 1;
            }
            (cut ? S : L).push_back(v);
        }
        if (S.empty() && !L.empty()) {   // halves not connected here: one vertex as the separator
            S.push_back(L.back());
            L.pop_back();
        }
    };
    // with coordinates, the smaller of the two separators among the
    // balanced splits (neither side above 70% of the rest); BFS alone without
    std::vector<int> gl, gr, gs;
    if (xy) geo_split(gl, gr, gs);
    const bool bfsOk = bfs_split(left, right, sep);
    if (xy) {
        auto balanced = [](const std::vector<int>& L, const std::vector<int>& R) {
            const size_t n = L.size() + R.size();
            return 10 * std::max(L.size(), R.size()) <= 7 * n;
        };
        const bool gb = balanced(gl, gr), bb = bfsOk && balanced(left, right);
        const bool useGeo = !bfsOk || (gb && !bb) || (gb == bb && gs.size() < sep.size());
        if (useGeo) {
            left.swap(gl);
            right.swap(gr);
            sep.swap(gs);
        }
    }
    else if (!bfsOk)
        return make_leaf();
    if (sep.empty() || (left.empty() && right.empty())) return make_leaf();
    // the two halves: each into its own node list, the larger of them on a
    // second thread when both are big (a thread of its own: the recursion
    // measured slower on the host pool's workers)
    std::vector<NdNode> ln, rn;
    const bool par = depth < 6 && left.size() > kNdParallel && right.size() > kNdParallel;
    if (par) {
        std::thread th([&] { nd_build(rowPtr, col, right, tag, tagCounter, level, rn, leafSize, depth + 1, xy); });
        nd_build(rowPtr, col, left, tag, tagCounter, level, ln, leafSize, depth + 1, xy);
        th.join();
    }
    else {
        if (!left.empty()) nd_build(rowPtr, col, left, tag, tagCounter, level, ln, leafSize, depth + 1, xy);
        if (!right.empty()) nd_build(rowPtr, col, right, tag, tagCounter, level, rn, leafSize, depth + 1, xy);
    }
    // splice: left subtree, right subtree (ids shifted), then the separator
    const int base = static_cast<int>(nodes.size());
    std::vector<int> kids;
    for (auto& n : ln) {
        for (int& c : n.children) c += base;
        nodes.push_back(std::move(n));
    }
    if (!ln.empty()) kids.push_back(static_cast<int>(nodes.size()) - 1);
    const int base2 = static_cast<int>(nodes.size());
    for (auto& n : rn) {
        for (int& c : n.children) c += base2;
        nodes.push_back(std::move(n));
    }
    if (!rn.empty()) kids.push_back(static_cast<int>(nodes.size()) - 1);
    nodes.push_back(NdNode{std::move(sep), std::move(kids)});
}

int tiles_of(int k, int m) { return (k + kTile - 1) / kTile + (m - k + kTile - 1) / kTile; }

// rows of L21 per forward-GEMV task on a level whose largest pivot count is
// maxK: 256 for the narrow kernel of small fronts, else 32 (k_fwd_rect)
int kRectRowsFor(int maxK) { return maxK <= kNarrowK ? kNarrowRows : kRectRows; }

// Tile t of a front's columns (pivot tiles first, then the rows below):
// first row/column and extent.
__host__ __device__ __forceinline__ void tile_bounds(int k, int m, int t, int& start, int& len)
{
    const int nP = (k + kTile - 1) / kTile;
    start = t < nP ? t * kTile : k + (t - nP) * kTile;
    const int end = t < nP ? k : m;
    len = end - start < kTile ? end - start : kTile;
}

// rows of a tile row per panel-solve block (one warp per row)
constexpr int kPanelRows = 8;
// trailing updates in 32 x 32 blocks (2 x 2 per thread): finer than 64 x 64
// blocks, so the launches' last waves leave less of the GPU idle.  Measured
// per factorisation: 199k 14.68 ms with 64 x 64 blocks wherever a launch had
// at least eight per SM, 13.99 ms with 32 x 32 everywhere; 2M triangles 212
// against 203 ms; the same bits either way (each entry takes the same FMA
// chain over the panel's columns)
constexpr int kUpdSmall = 32;

// The smallest factorization (flops) whose independent subtrees get streams
// of their own.  The split saves time on every graph replay but doubles the
// graph's launches, so capturing and instantiating it after a pattern change
// costs more (~1 ms more at 199k triangles).  Measured per Newton step (eight
// streams against one): 5k triangles, 3.8e7 flops, factorization 0.90 -> 0.83
// ms, but a whole 5k outer loop with its 38 pattern changes 0.83 -> 0.89 s;
// 41k torus, 1.2e9 flops, re-analysed every step, factorization 3.96 -> 3.80
// ms and the step 16.0 -> 16.3 ms; 199k, 8.9e9 flops, pattern kept, 14.0 ->
// 12.5 ms.
constexpr double kStreamMinFlops = 4e9;

} // namespace

void chol_analyze(CholPlan& P, int nV, const int* rowPtr, const int* col, int leafSize,
                  const std::vector<int>* rootVerts, const double* xy)
{
    const auto t0 = std::chrono::steady_clock::now();
    {
        const int cl = P.solveCluster, fs = P.factStreams;
        const CholPlan::Keep keep = P.keep;
        P = CholPlan{};
        P.solveCluster = cl;
        P.factStreams = fs;
        P.keep = keep;
    }
    // the bisection needs an order on the coordinates: BFS alone unless all are finite
    if (xy)
        for (long long i = 0; i < 2LL * nV; ++i)
            if (!std::isfinite(xy[i])) {
                xy = nullptr;
                break;
            }
    std::vector<NdNode> nodes;
    std::vector<int> tag(nV, 0), level(nV, -1);
    std::atomic<int> tagCounter{0};
    // components: run the dissection on every connected set of vertices
    // (the forced root vertices excluded: tag 0 keeps the BFS out of them)
    std::vector<int> roots;
    {
        std::vector<char> seen(nV, 0);
        if (rootVerts)
            for (int v : *rootVerts) seen[v] = 1;
        for (int s = 0; s < nV; ++s) {
            if (seen[s]) continue;
            std::vector<int> comp{s};
            seen[s] = 1;
            for (size_t h = 0; h < comp.size(); ++h) {
                const int v = comp[h];
                for (int p = rowPtr[v]; p < rowPtr[v + 1]; ++p)
                    if (!seen[col[p]]) { seen[col[p]] = 1; comp.push_back(col[p]); }
            }
            std::vector<NdNode> sub;
            nd_build(rowPtr, col, comp, tag, tagCounter, level, sub, leafSize, 0, xy);
            const int base = static_cast<int>(nodes.size());
            for (auto& n : sub) {
                for (int& c : n.children) c += base;
                nodes.push_back(std::move(n));
            }
            roots.push_back(static_cast<int>(nodes.size()) - 1);
        }
    }
    if (rootVerts && !rootVerts->empty()) nodes.push_back(NdNode{*rootVerts, roots});
    const int rootNode = (rootVerts && !rootVerts->empty()) ? static_cast<int>(nodes.size()) - 1 : -1;
    const double ndMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    chol_analyze_nodes(P, nV, rowPtr, col, nodes, rootNode);
    P.nd.swap(nodes);
    P.ndMs = ndMs;
    P.fullFlops = P.flops;
    P.incremental = 0;
}

void chol_analyze_nodes(CholPlan& P, int nV, const int* rowPtr, const int* col, const std::vector<NdNode>& nodes,
                        int rootNode)
{
    const auto t0 = std::chrono::steady_clock::now();
    {
        const double ndMs = P.ndMs, fullFlops = P.fullFlops;
        const int inc = P.incremental, cl = P.solveCluster, fs = P.factStreams;
        const CholPlan::Keep keep = P.keep;
        P = CholPlan{};
        P.ndMs = ndMs;
        P.fullFlops = fullFlops;
        P.incremental = inc;
        P.solveCluster = cl;
        P.factStreams = fs;
        P.keep = keep;
    }
    P.nV = nV;
    P.nDof = 2 * nV;
    P.ndRoot = rootNode;
    // nodes are created children-first: creation order is a postorder
    const int nF = static_cast<int>(nodes.size());
    P.nFronts = nF;
    std::vector<int> parent(nF, -1);
    for (int f = 0; f < nF; ++f)
        for (int c : nodes[f].children) parent[c] = f;
    std::vector<int> pos(nV, -1);
    P.vertOrder.reserve(nV);
    std::vector<int> vstart(nF);
    for (int f = 0; f < nF; ++f) {
        vstart[f] = static_cast<int>(P.vertOrder.size());
        for (int v : nodes[f].S) {
            pos[v] = static_cast<int>(P.vertOrder.size());
            P.vertOrder.push_back(v);
        }
    }
    P.permDof.resize(P.nDof);
    for (int k = 0; k < nV; ++k) {
        P.permDof[2 * k] = 2 * P.vertOrder[k];
        P.permDof[2 * k + 1] = 2 * P.vertOrder[k] + 1;
    }
    // front levels (leaves 0) and the fronts of each level
    std::vector<int> flev(nF, 0);
    int nLev = 0;
    for (int f = 0; f < nF; ++f) {
        for (int c : nodes[f].children) flev[f] = std::max(flev[f], flev[c] + 1);
        nLev = std::max(nLev, flev[f] + 1);
    }
    std::vector<int> levOff(nLev + 1, 0), levList(nF);
    for (int f = 0; f < nF; ++f) levOff[flev[f] + 1]++;
    for (int l = 0; l < nLev; ++l) levOff[l + 1] += levOff[l];
    {
        std::vector<int> fill(levOff.begin(), levOff.end() - 1);
        for (int f = 0; f < nF; ++f) levList[fill[flev[f]]++] = f;
    }
    // boundary sets (ancestor vertices each subtree touches), bottom-up: the
    // fronts of one level are independent
    std::vector<std::vector<int>> B(nF);
    for (int l = 0; l < nLev; ++l)
        host_parallel_for(levOff[l + 1] - levOff[l], 64, [&](size_t i0, size_t i1) {
            std::vector<int> cand;
            for (size_t i = i0; i < i1; ++i) {
                const int f = levList[levOff[l] + i];
                const int last = vstart[f] + static_cast<int>(nodes[f].S.size()) - 1;
                cand.clear();
                for (int v : nodes[f].S)
                    for (int p = rowPtr[v]; p < rowPtr[v + 1]; ++p)
                        if (pos[col[p]] > last) cand.push_back(pos[col[p]]);
                for (int c : nodes[f].children)
                    for (int u : B[c])
                        if (u > last) cand.push_back(u);
                std::sort(cand.begin(), cand.end());
                cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
                B[f].assign(cand.begin(), cand.end());   // elimination positions, ascending
            }
        });
    // fronts: sizes and offsets in one pass, then the row lists in parallel
    P.fk.resize(nF); P.fm.resize(nF); P.fparent = parent; P.flevel = flev; P.fdofStart.resize(nF);
    P.foff.resize(nF); P.fupd.resize(nF); P.frowOff.resize(nF); P.relOff.resize(nF);
    P.childOff.assign(nF + 1, 0);
    long long pool = 0, upd = 0;
    size_t rows = 0, rels = 0;
    for (int f = 0; f < nF; ++f) {
        const int ns = static_cast<int>(nodes[f].S.size());
        const int k = 2 * ns, m = 2 * (ns + static_cast<int>(B[f].size()));
        P.fk[f] = k;
        P.fm[f] = m;
        P.fdofStart[f] = 2 * vstart[f];
        P.foff[f] = pool;
        pool += (long long)m * m;
        P.fupd[f] = upd;
        upd += m - k;
        P.frowOff[f] = static_cast<int>(rows);
        rows += m;
        P.relOff[f] = static_cast<int>(rels);
        if (parent[f] >= 0) rels += m - k;
        P.maxM = std::max(P.maxM, m);
        P.childOff[f + 1] = P.childOff[f] + static_cast<int>(nodes[f].children.size());
        const double kk = k, mm = m, r = mm - kk;
        P.flops += kk * kk * kk / 3.0 + kk * kk * r + kk * r * r;
    }
    P.poolSize = pool;
    P.updSize = upd;
    P.rowIdx.resize(rows);
    host_parallel_for(nF, 256, [&](size_t f0, size_t f1) {
        for (size_t f = f0; f < f1; ++f) {
            int* out = P.rowIdx.data() + P.frowOff[f];
            const int ns = static_cast<int>(nodes[f].S.size());
            for (int i = 0; i < ns; ++i) {
                *out++ = 2 * (vstart[f] + i);
                *out++ = 2 * (vstart[f] + i) + 1;
            }
            for (int u : B[f]) {
                *out++ = 2 * u;
                *out++ = 2 * u + 1;
            }
        }
    });
    P.childList.resize(P.childOff[nF]);
    for (int f = 0; f < nF; ++f)
        std::copy(nodes[f].children.begin(), nodes[f].children.end(), P.childList.begin() + P.childOff[f]);
    // child update row -> parent row (both row lists ascending)
    std::atomic<int> bad{0};
    P.relIdx.resize(rels);
    host_parallel_for(nF, 256, [&](size_t f0, size_t f1) {
        for (size_t f = f0; f < f1; ++f) {
            const int pf = parent[f];
            if (pf < 0) continue;
            const int* prow = P.rowIdx.data() + P.frowOff[pf];
            const int pm = P.fm[pf];
            const int* it = prow;
            int* out = P.relIdx.data() + P.relOff[f];
            for (int i = P.fk[f]; i < P.fm[f]; ++i) {
                const int dof = P.rowIdx[P.frowOff[f] + i];
                it = std::lower_bound(it, prow + pm, dof);
                if (it == prow + pm || *it != dof) {   // structure invariant violated
                    bad = 1;
                    *out++ = 0;
                    it = prow;
                    continue;
                }
                *out++ = static_cast<int>(it - prow);
            }
        }
    });
    // levels
    for (int f = 0; f < nF; ++f) P.nLevels = std::max(P.nLevels, P.flevel[f] + 1);
    P.levelFrontOff.assign(P.nLevels + 1, 0);
    for (int f = 0; f < nF; ++f) P.levelFrontOff[P.flevel[f] + 1]++;
    for (int l = 0; l < P.nLevels; ++l) P.levelFrontOff[l + 1] += P.levelFrontOff[l];
    P.levelFronts.resize(nF);
    {
        std::vector<int> fill(P.levelFrontOff.begin(), P.levelFrontOff.end() - 1);
        for (int f = 0; f < nF; ++f) P.levelFronts[fill[P.flevel[f]]++] = f;
    }
    // factorization groups, for launches on up to factStreams streams.  A
    // subtree is cut below its top chain, at the first node with two to four
    // big children (big: at least 5% of the factor flops; a chain node's small
    // children stay with the chain): the big subtrees run concurrently, the
    // first on the subtree's stream, the others on streams of their own, and
    // the chain, with every small subtree hanging off it, joins them.  Cuts
    // are made largest subtree first while streams are left; uncut subtrees
    // are leaf groups.  Groups are numbered in postorder, so every group
    // comes after those it waits for.  Factorizations below kStreamMinFlops
    // stay on one stream (see there).
    std::vector<int> grp(nF, 0);
    {
        std::vector<double> fl(nF, 0.0);   // subtree flops (children come first)
        for (int f = 0; f < nF; ++f) {
            const double kk = P.fk[f], r = (double)P.fm[f] - P.fk[f];
            fl[f] += kk * kk * kk / 3.0 + kk * kk * r + kk * r * r;
            for (int c : nodes[f].children) fl[f] += fl[c];
        }
        std::vector<int> roots;
        double total = 0.0;
        for (int f = 0; f < nF; ++f)
            if (parent[f] < 0) {
                roots.push_back(f);
                total += fl[f];
            }
        const auto big = [&](int c) { return fl[c] >= 0.05 * total; };
        // subtree r (-1: the forest of all roots) -> its big children below
        // the chain of nodes with one big child
        auto split_of = [&](int r) {
            std::vector<int> bigK;
            for (;;) {
                bigK.clear();
                for (int c : r < 0 ? roots : nodes[r].children)
                    if (big(c)) bigK.push_back(c);
                if (bigK.size() != 1) return bigK;
                r = bigK[0];
            }
        };
        const int top = roots.size() == 1 ? roots[0] : -1;
        std::vector<char> cut(nF + 1, 0);   // indexed by subtree root + 1
        {
            std::vector<int> leaves{top};
            int streams = 1;
            for (;;) {
                int best = -2;
                double bestFl = -1.0;
                for (int r : leaves) {
                    const size_t k = split_of(r).size();
                    const double rf = r < 0 ? total : fl[r];
                    if (k >= 2 && k <= 4 && streams + (int)k - 1 <= P.factStreams && total >= kStreamMinFlops &&
                        rf > bestFl) {
                        best = r;
                        bestFl = rf;
                    }
                }
                if (best == -2) break;
                cut[best + 1] = 1;
                const std::vector<int> kids = split_of(best);
                streams += static_cast<int>(kids.size()) - 1;
                leaves.erase(std::find(leaves.begin(), leaves.end(), best));
                leaves.insert(leaves.end(), kids.begin(), kids.end());
            }
        }
        // r's subtree into group g, except the subtrees of `stop`
        auto mark = [&](int r, const std::vector<int>& stop, int g) {
            std::vector<int> stack{r};
            while (!stack.empty()) {
                const int f = stack.back();
                stack.pop_back();
                grp[f] = g;
                for (int c : nodes[f].children)
                    if (std::find(stop.begin(), stop.end(), c) == stop.end()) stack.push_back(c);
            }
        };
        int streamsUsed = 1;
        // returns the group that finishes subtree r
        std::function<int(int, int)> build = [&](int r, int stream) -> int {
            std::vector<int> kids, kidGroups;
            if (cut[r + 1]) {
                kids = split_of(r);
                for (size_t i = 0; i < kids.size(); ++i)
                    kidGroups.push_back(build(kids[i], i == 0 ? stream : streamsUsed++));
            }
            const int g = static_cast<int>(P.grpStream.size());
            P.grpStream.push_back(stream);
            for (int d : kidGroups)   // waits between streams only
                if (P.grpStream[d] != stream) P.grpWait.push_back(d);
            P.grpWaitOff.push_back(static_cast<int>(P.grpWait.size()));
            if (r < 0) {   // the forest: every tree that is not one of the big subtrees
                for (int c : roots)
                    if (std::find(kids.begin(), kids.end(), c) == kids.end()) mark(c, kids, g);
            }
            else mark(r, kids, g);   // a leaf group, or the chain with its small subtrees
            return g;
        };
        P.grpWaitOff.assign(1, 0);
        build(top, 0);
        P.nFactStreams = streamsUsed;
        if ((int)P.grpStream.size() > CholPlan::kMaxFactGroups) {   // cannot happen: <= 2 x streams - 1
            std::fill(grp.begin(), grp.end(), 0);
            P.grpStream.assign(1, 0);
            P.grpWaitOff.assign(2, 0);
            P.grpWait.clear();
            P.nFactStreams = 1;
        }
    }
    P.frontGroup = grp;
    const int nGrp = static_cast<int>(P.grpStream.size());
    std::vector<std::vector<int>> glf(static_cast<size_t>(nGrp) * P.nLevels);
    for (int l = 0; l < P.nLevels; ++l)
        for (int i = P.levelFrontOff[l]; i < P.levelFrontOff[l + 1]; ++i) {
            const int f = P.levelFronts[i];
            glf[static_cast<size_t>(grp[f]) * P.nLevels + l].push_back(f);
        }
    // launch schedule: per group and level, extend-add per child slot, the
    // first panel's diagonal tiles, then per panel the panel solve and the
    // trailing update (whose first block also factors the next panel's
    // diagonal tile).  Each (group, level) is built on its own host task,
    // then the lists are joined group by group in level order.
    struct LevelSched {
        std::vector<TileTask> tasks;
        std::vector<CholPlan::Launch> launches;
    };
    std::vector<LevelSched> sched(static_cast<size_t>(nGrp) * P.nLevels);
    host_run_tasks(sched.size(), [&](size_t item) {
        const int l = static_cast<int>(item % P.nLevels);
        std::vector<TileTask>& T = sched[item].tasks;
        std::vector<CholPlan::Launch>& Ls = sched[item].launches;
        const int* lf = glf[item].data();
        const int nl = static_cast<int>(glf[item].size());
        int maxKids = 0, maxPanels = 0;
        for (int i = 0; i < nl; ++i) {
            const int f = lf[i];
            maxKids = std::max(maxKids, P.childOff[f + 1] - P.childOff[f]);
            maxPanels = std::max(maxPanels, (P.fk[f] + kTile - 1) / kTile);
        }
        for (int c = 0; c < maxKids; ++c) {
            const int off = static_cast<int>(T.size());
            for (int i = 0; i < nl; ++i) {
                const int f = lf[i];
                if (P.childOff[f + 1] - P.childOff[f] <= c) continue;
                const int ch = P.childList[P.childOff[f] + c];
                const int u = P.fm[ch] - P.fk[ch];
                for (int j0 = 0; j0 < u; j0 += 16) T.push_back(TileTask{ch, f, j0, std::min(j0 + 16, u)});
            }
            const int cnt = static_cast<int>(T.size()) - off;
            if (cnt) Ls.push_back({0, l, 0, off, cnt, c});
        }
        {   // the first panel's diagonal tiles (the later ones are factored
            // at the end of the previous panel's trailing update)
            const int off = static_cast<int>(T.size());
            for (int i = 0; i < nl; ++i)
                if (P.fk[lf[i]] > 0) T.push_back(TileTask{lf[i], 0, 0, 0});
            if ((int)T.size() > off) Ls.push_back({4, l, 0, off, (int)T.size() - off, 0});
        }
        for (int p = 0; p < maxPanels; ++p) {
            // panel: one CTA per tile row below the factored diagonal tile
            int off = static_cast<int>(T.size());
            for (int i = 0; i < nl; ++i) {
                const int f = lf[i];
                if ((P.fk[f] + kTile - 1) / kTile <= p) continue;
                const int nt = tiles_of(P.fk[f], P.fm[f]);
                for (int ti = p + 1; ti < nt; ++ti) {
                    int r0, h;
                    tile_bounds(P.fk[f], P.fm[f], ti, r0, h);
                    for (int g = 0; g * kPanelRows < h; ++g) T.push_back(TileTask{f, ti, g, p});
                }
            }
            if ((int)T.size() > off) Ls.push_back({1, l, p, off, (int)T.size() - off, 0});
            // trailing region [s, m) x [s, m), s = end of panel p, in the
            // lower triangle of kUpdSmall x kUpdSmall blocks
            off = static_cast<int>(T.size());
            for (int i = 0; i < nl; ++i) {
                const int f = lf[i];
                if ((P.fk[f] + kTile - 1) / kTile <= p) continue;
                const int s0 = std::min((p + 1) * kTile, P.fk[f]);
                const int nb = (P.fm[f] - s0 + kUpdSmall - 1) / kUpdSmall;
                for (int bj = 0; bj < nb; ++bj)
                    for (int bi = bj; bi < nb; ++bi) T.push_back(TileTask{f, bi, bj, p});
            }
            if ((int)T.size() > off) Ls.push_back({5, l, p, off, (int)T.size() - off, 0});
        }
    });
    {
        std::vector<size_t> base(sched.size() + 1, 0);
        for (size_t i = 0; i < sched.size(); ++i) base[i + 1] = base[i] + sched[i].tasks.size();
        P.tasks.resize(base[sched.size()]);
        host_run_tasks(sched.size(), [&](size_t i) {
            std::copy(sched[i].tasks.begin(), sched[i].tasks.end(), P.tasks.begin() + base[i]);
        });
        P.grpLaunchOff.assign(1, 0);
        for (size_t i = 0; i < sched.size(); ++i) {
            for (CholPlan::Launch L : sched[i].launches) {
                L.taskOff += static_cast<int>(base[i]);
                P.launches.push_back(L);
            }
            if ((i + 1) % P.nLevels == 0) P.grpLaunchOff.push_back(static_cast<int>(P.launches.size()));
        }
    }
    // substitution chunks of the rectangular part of each front, per level
    P.rectRowOff.assign(P.nLevels + 1, 0);
    P.rectColOff.assign(P.nLevels + 1, 0);
    P.levelMaxK.assign(P.nLevels, 0);
    P.levelMaxM.assign(P.nLevels, 0);
    for (int l = 0; l < P.nLevels; ++l) {
        for (int i = P.levelFrontOff[l]; i < P.levelFrontOff[l + 1]; ++i) {
            const int f = P.levelFronts[i];
            P.levelMaxK[l] = std::max(P.levelMaxK[l], P.fk[f]);
            P.levelMaxM[l] = std::max(P.levelMaxM[l], P.fm[f]);
        }
        for (int i = P.levelFrontOff[l]; i < P.levelFrontOff[l + 1]; ++i) {
            const int f = P.levelFronts[i];
            const int chunk = kRectRowsFor(P.levelMaxK[l]);
            for (int r0 = P.fk[f]; r0 < P.fm[f]; r0 += chunk) P.rectRowTasks.push_back(make_int2(f, r0));
            if (P.fm[f] > P.fk[f])
                for (int c0 = 0; c0 < P.fk[f]; c0 += kRectCols) P.rectColTasks.push_back(make_int2(f, c0));
        }
        P.rectRowOff[l + 1] = static_cast<int>(P.rectRowTasks.size());
        P.rectColOff[l + 1] = static_cast<int>(P.rectColTasks.size());
    }
    // assembly map: block slot (r, c) with pos[r] >= pos[c] goes to the front owning c
    std::vector<int> owner(nV);
    for (int f = 0; f < nF; ++f)
        for (int v : nodes[f].S) owner[v] = f;
    const int nnzb = rowPtr[nV];
    P.asmDest.assign(nnzb, -1);
    P.asmLd.assign(nnzb, 0);
    P.asmDiag.assign(nnzb, 0);
    host_parallel_for(nV, 2048, [&](size_t r0, size_t r1) {
        for (int r = static_cast<int>(r0); r < static_cast<int>(r1); ++r)
            for (int s = rowPtr[r]; s < rowPtr[r + 1]; ++s) {
                const int c = col[s];
                if (pos[r] < pos[c]) continue;
                const int f = owner[c];
                const int m = P.fm[f];
                const int jc = 2 * (pos[c] - vstart[f]);
                const int* prow = P.rowIdx.data() + P.frowOff[f];
                const int* it = std::lower_bound(prow, prow + m, 2 * pos[r]);
                if (it == prow + m || *it != 2 * pos[r] || jc + 1 >= P.fk[f]) {
                    bad = 1;
                    continue;
                }
                const int ir = static_cast<int>(it - prow);
                P.asmDest[s] = P.foff[f] + ir + (long long)jc * m;
                P.asmLd[s] = m;
                P.asmDiag[s] = (r == c) ? 1 : 0;
            }
    });
    if (bad) P.valid = false;
    P.symMs = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
}

// ------------------------------------------------------------------ kernels
namespace {

__global__ void k_asm_fronts(const Blk2* __restrict__ val, const long long* __restrict__ dest,
                             const int* __restrict__ ld, const unsigned char* __restrict__ diag, int nnzb,
                             double* __restrict__ pool)
{
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nnzb) return;
    const long long d = dest[s];
    if (d < 0) return;
    const Blk2 v = val[s];
    const long long m = ld[s];
    pool[d] = v.a00;
    pool[d + 1] = v.a10;
    pool[d + 1 + m] = v.a11;
    if (!diag[s]) pool[d + m] = v.a01;
}

// extend-add of a child's update matrix into its parent (columns j0..j1)
__global__ void __launch_bounds__(256) k_extend(const TileTask* __restrict__ tasks, const int* __restrict__ fk,
                                                const int* __restrict__ fm, const long long* __restrict__ foff,
                                                const int* __restrict__ relOff, const int* __restrict__ relIdx,
                                                double* __restrict__ pool)
{
    const TileTask t = tasks[blockIdx.x];
    const int ch = t.front, par = t.i;
    const int kc = fk[ch], mc = fm[ch], mp = fm[par];
    const int u = mc - kc, j1 = t.p;
    const double* __restrict__ C = pool + foff[ch];   // the child's and the parent's
    double* __restrict__ Pm = pool + foff[par];       // fronts do not overlap
    const int* rel = relIdx + relOff[ch];
    // the block's columns j0 <= j < j1, rows j <= i < u, numbered column by
    // column; each thread takes every 256th entry, four per round with all
    // loads first (each parent entry is added to once: same sums in any order)
    int j = t.j, off = threadIdx.x;
    while (j < j1 && off >= u - j) off -= u - j, ++j;
    while (j < j1) {
        long long src[4], dst[4];
        int n = 0;
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (j < j1) {
                src[q] = (long long)(kc + j) * mc + kc + j + off;
                dst[q] = (long long)rel[j] * mp + rel[j + off];
                n = q + 1;
                off += blockDim.x;
                while (j < j1 && off >= u - j) off -= u - j, ++j;
            }
        double v[4], w[4];
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (q < n) {
                v[q] = C[src[q]];
                w[q] = Pm[dst[q]];
            }
#pragma unroll
        for (int q = 0; q < 4; ++q)
            if (q < n) Pm[dst[q]] = w[q] + v[q];
    }
}

// LDL^T of the w x w diagonal tile at (s0, s0) of a front, in place (unit-
// lower L below the diagonal, D on it -- the factorisation SimplicialLDLT
// computes; negative pivots pass, a zero or non-finite one is replaced by
// 1e-300 and counted in *flag).  Run by the first kDiagThreads threads of
// the block (four warps, one per SM sub-partition, so the elimination uses
// every FP64 unit of the SM; named barrier 1), in kDiagScratch doubles of
// shared memory: the 32 x 33 tile, the scaled column, the current pivot and
// its reciprocal, and a table of the packed lower triangle's entries in
// column-major order.  Elimination step c scales column c by the pivot's
// reciprocal, which thread 0 computed during step c - 1 right after updating
// that diagonal entry first, while warps 1-3 update the step's other entries
// (r, c2), c < c2 <= r < w.  The operation order of a column-by-column
// right-looking elimination.
constexpr int kDiagThreads = 128;
constexpr int kDiagScratch = kTile * (kTile + 1) + kTile + 2 + (kTile * (kTile + 1) / 2 + 3) / 4;

__device__ __forceinline__ int tri_col_start(int j, int w) { return j * w - (j * (j - 1)) / 2; }

__device__ __forceinline__ void diag_barrier() { asm volatile("bar.sync 1, %0;" ::"n"(kDiagThreads) : "memory"); }

// pivot d (a zero or non-finite value replaced by 1e-300) and 1 / d, the
// correctly rounded reciprocal (the same bits as the division 1.0 / d, by
// the reciprocal's shorter sequence: it is on the tile's dependent chain)
__device__ __forceinline__ void diag_pivot(double dRaw, double* piv, int& nBad)
{
    const bool bad = !(dRaw != 0.0) || !isfinite(dRaw);
    const double d = bad ? 1e-300 : dRaw;
    nBad += bad;
    piv[0] = d;
    piv[1] = __drcp_rn(d);
}

__device__ void ldl_diag_tile(double* __restrict__ F, int m, int s0, int w, double* scratch, int* flag)
{
    double (*T)[kTile + 1] = reinterpret_cast<double(*)[kTile + 1]>(scratch);
    double* Lc = scratch + kTile * (kTile + 1);
    double* piv = Lc + kTile;
    unsigned short* tab = reinterpret_cast<unsigned short*>(piv + 2);   // entry -> (r << 5) | c2
    const int q = threadIdx.x;   // < kDiagThreads
    for (int e = q; e < kTile * w; e += kDiagThreads) {
        const int r = e & (kTile - 1), c = e / kTile;
        if (r < w) T[r][c] = r >= c ? F[(s0 + r) + (long long)(s0 + c) * m] : 0.0;
    }
    const int total = tri_col_start(w, w);
    const float b = 2.0f * w + 1.0f;
    for (int e = q; e < total; e += kDiagThreads) {
        // column c2 of packed entry e: the largest j with start(j) <= e
        int c2 = static_cast<int>(0.5f * (b - sqrtf(b * b - 8.0f * e)));
        c2 = max(0, min(c2, w - 1));
        while (c2 + 1 < w && tri_col_start(c2 + 1, w) <= e) ++c2;
        while (tri_col_start(c2, w) > e) --c2;
        tab[e] = static_cast<unsigned short>(((c2 + (e - tri_col_start(c2, w))) << 5) | c2);
    }
    diag_barrier();
    int nBad = 0;   // thread 0's count
    if (q == 0) diag_pivot(T[0][0], piv, nBad);
    diag_barrier();
    for (int c = 0; c < w; ++c) {
        const double d = piv[0], id = piv[1];
        double lc = 0.0;
        if (q > c && q < w) {
            lc = T[q][c] * id;   // L(q, c)
            Lc[q] = lc;
        }
        diag_barrier();
        const int e0 = tri_col_start(c + 1, w);   // entry (c + 1, c + 1): the next pivot
        if (q == 0) {
            if (c + 1 < w) {
                T[c + 1][c + 1] -= Lc[c + 1] * T[c + 1][c];
                diag_pivot(T[c + 1][c + 1], piv, nBad);
            }
        }
        else if (q >= 32) {
            for (int e = e0 + 1 + (q - 32); e < total; e += kDiagThreads - 32) {
                const int rc = tab[e], r = rc >> 5, c2 = rc & 31;
                T[r][c2] -= Lc[r] * T[c2][c];
            }
        }
        diag_barrier();
        if (q > c && q < w) T[q][c] = lc;
        else if (q == c) T[c][c] = d;
        // the next step reads column c + 1 and the pivot only; column c's
        // writes are ordered before the final copy by later barriers
    }
    diag_barrier();
    for (int e = q; e < kTile * w; e += kDiagThreads) {
        const int r = e & (kTile - 1), c = e / kTile;
        if (r < w && r >= c) F[(s0 + r) + (long long)(s0 + c) * m] = T[r][c];
    }
    if (q == 0 && nBad) atomicAdd(flag, nBad);
}

// The diagonal tile of every front's first panel (one block of four warps
// per front of the level; the later panels' tiles are factored by
// k_ldl_update).
__global__ void __launch_bounds__(kDiagThreads) k_ldl_diag(const TileTask* __restrict__ tasks,
                                                           const int* __restrict__ fk, const int* __restrict__ fm,
                                                           const long long* __restrict__ foff,
                                                           double* __restrict__ pool, int* flag)
{
    __shared__ double scratch[kDiagScratch];
    const TileTask t = tasks[blockIdx.x];
    const int k = fk[t.front], m = fm[t.front];
    int s0, w;
    tile_bounds(k, m, t.p, s0, w);
    ldl_diag_tile(pool + foff[t.front], m, s0, w, scratch, flag);
}

// Panel solve below the (already factored) diagonal tile of panel p:
// L(i, p) = A(i, p) L(p, p)^-T D^-1 for kPanelRows rows of tile row i (task
// j: which group of rows), a row per warp and a column per lane, in the
// operation order of a column-by-column substitution.  A tile row is split
// over several blocks so that the few tile rows of the top fronts spread
// over more SMs.
__global__ void __launch_bounds__(32 * kPanelRows) k_ldl_panel(const TileTask* __restrict__ tasks,
                                                               const int* __restrict__ fk,
                                                               const int* __restrict__ fm,
                                                               const long long* __restrict__ foff,
                                                               double* __restrict__ pool)
{
    static_assert(kTile == 32, "one warp lane per tile column");
    __shared__ double L[kTile][kTile + 1];
    __shared__ double X[kPanelRows][kTile + 1];
    const TileTask t = tasks[blockIdx.x];
    const int k = fk[t.front], m = fm[t.front];
    int s0, w, r0, h;
    tile_bounds(k, m, t.p, s0, w);
    tile_bounds(k, m, t.i, r0, h);
    r0 += kPanelRows * t.j;
    h = min(kPanelRows, h - kPanelRows * t.j);
    double* F = pool + foff[t.front];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    // the factored tile (identity beyond w) and the rows (zero beyond h x w)
    for (int e = threadIdx.x; e < kTile * kTile; e += blockDim.x) {
        const int r = e & (kTile - 1), c = e / kTile;
        double a = r == c ? 1.0 : 0.0;
        if (r < w && c < w && r >= c) a = F[(s0 + r) + (long long)(s0 + c) * m];
        L[r][c] = a;
    }
    for (int e = threadIdx.x; e < kPanelRows * kTile; e += blockDim.x) {
        const int r = e % kPanelRows, c = e / kPanelRows;
        X[r][c] = (r < h && c < w) ? F[(r0 + r) + (long long)(s0 + c) * m] : 0.0;
    }
    __syncthreads();
    double x = X[warp][lane];
    for (int c = 0; c + 1 < w; ++c) {
        const double xc = __shfl_sync(0xffffffffu, x, c);
        if (lane > c) x -= xc * L[lane][c];
    }
    X[warp][lane] = x / L[lane][lane];
    __syncthreads();
    for (int e = threadIdx.x; e < kPanelRows * w; e += blockDim.x) {
        const int r = e % kPanelRows, c = e / kPanelRows;
        if (r < h) F[(r0 + r) + (long long)(s0 + c) * m] = X[r][c];
    }
}

// Trailing update C -= L(:, p) * D_p * L(:, p)^T of the region below and right
// of panel p, in B x B blocks (task: block row bi, block column bj <= bi,
// lower triangle only).  256 threads, P x P accumulators each (B = 16 P);
// the panel columns of both block rows are staged column-major in shared
// memory so a thread's rows (or columns) are 16-byte reads.  Launched with
// B = 32 (kUpdSmall): four times the blocks of B = 64, a quarter of the work
// each, and less of the GPU idle in a launch's last wave.
template <int B, int P>
__global__ void __launch_bounds__(256) k_ldl_update(const TileTask* __restrict__ tasks, const int* __restrict__ fk,
                                                    const int* __restrict__ fm, const long long* __restrict__ foff,
                                                    double* __restrict__ pool, int* flag)
{
    static_assert(B == 16 * P && P % 2 == 0, "16 x 16 threads of P x P");
    // Ai, Aj, and in the tail the diagonal tile's scratch
    constexpr int kSm = 2 * kTile * B > kDiagScratch ? 2 * kTile * B : kDiagScratch;
    __shared__ __align__(16) double sm[kSm];
    double (*Ai)[B] = reinterpret_cast<double(*)[B]>(sm);
    double (*Aj)[B] = reinterpret_cast<double(*)[B]>(sm + kTile * B);
    const TileTask t = tasks[blockIdx.x];
    const int k = fk[t.front], m = fm[t.front];
    int s0, w;
    tile_bounds(k, m, t.p, s0, w);
    const int s = s0 + w;                       // first row/column after the panel
    const int r0 = s + B * t.i, c0 = s + B * t.j;
    const int h = min(B, m - r0), hc = min(B, m - c0);
    double* F = pool + foff[t.front];
    for (int e = threadIdx.x; e < kTile * B; e += blockDim.x) {
        const int r = e % B, c = e / B;
        double ai = 0.0, aj = 0.0;
        if (c < w) {
            const double* col = F + (long long)(s0 + c) * m;
            if (r < h) ai = col[r0 + r] * col[s0 + c];   // L(r, c) * D_c
            if (r < hc) aj = col[c0 + r];
        }
        Ai[c][r] = ai;
        Aj[c][r] = aj;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;   // 16 x 16 threads, P x P each
    double acc[P][P];
#pragma unroll
    for (int i = 0; i < P; ++i)
#pragma unroll
        for (int j = 0; j < P; ++j) acc[i][j] = 0.0;
    // threads whose patch lies outside the block's rows/columns, or wholly
    // above the diagonal of a diagonal block, have nothing to update
    const bool idle = (P * ty >= h) || (P * tx >= hc) || (t.i == t.j && P * ty + P - 1 < P * tx);
    for (int c = 0; c < (idle ? 0 : w); ++c) {
        double a[P], b[P];
#pragma unroll
        for (int i = 0; i < P; i += 2) {
            const double2 av = *reinterpret_cast<const double2*>(&Ai[c][P * ty + i]);
            const double2 bv = *reinterpret_cast<const double2*>(&Aj[c][P * tx + i]);
            a[i] = av.x; a[i + 1] = av.y;
            b[i] = bv.x; b[i + 1] = bv.y;
        }
#pragma unroll
        for (int i = 0; i < P; ++i)
#pragma unroll
            for (int j = 0; j < P; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
    }
    const bool diag = (t.i == t.j);
#pragma unroll
    for (int i = 0; i < P; ++i) {
        const int r = P * ty + i;
        if (r >= h) continue;
#pragma unroll
        for (int j = 0; j < P; ++j) {
            const int cc = P * tx + j;
            if (cc < hc && (!diag || r >= cc)) F[(r0 + r) + (long long)(c0 + cc) * m] -= acc[i][j];
        }
    }
    // the next panel's diagonal tile is the corner of this front's first
    // trailing block: once the block is updated, four warps factor it (in
    // the staging buffers), so the next panel launch reads it factored
    if (t.i == 0 && t.j == 0 && s < k) {
        __syncthreads();
        if (threadIdx.x < kDiagThreads) ldl_diag_tile(F, m, s, min(kTile, k - s), sm, flag);
    }
}

__global__ void k_permute_in(const double* __restrict__ rhs, const int* __restrict__ perm, double sign, int n,
                             double* __restrict__ out)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) out[j] = sign * rhs[perm[j]];
}

__global__ void k_permute_out(const double* __restrict__ xp, const int* __restrict__ perm, int n, double* __restrict__ x)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < n) x[perm[j]] = xp[j];
}

// Bounded waits on shared-memory mbarriers inside one CTA.  A wait that runs
// out (or sees that another thread gave up) sets the CTA's abort flag and
// returns false; every loop then ends, the host reads the kernel's flag.
constexpr int kSolveWaitPolls = 1 << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(unsigned long long* b, int count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(b)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive(unsigned long long* b)
{
    asm volatile("{\n\t.reg .b64 st;\n\tmbarrier.arrive.shared::cta.b64 st, [%0];\n\t}" ::"r"(smem_addr(b)) : "memory");
}

__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* b, uint32_t parity, volatile int* abort)
{
    const uint32_t a = smem_addr(b);
    for (int i = 0; i < kSolveWaitPolls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (*abort) return false;
    }
    *abort = 1;
    return false;
}

// Updaters of the pivot-part kernels: every warp but warp 0 and the warps
// that share its SM sub-partition (warp % 4 == 0).  GB300's FP64 pipe takes
// a warp instruction whole, so an updater's FMAs on warp 0's sub-partition
// queue ahead of the chain's dependent steps (measured: ~9.5 us per 32-row
// block on the top levels with them there).
__host__ __device__ constexpr int upd_warps(int nt) { return nt / 32 - (nt / 32 + 3) / 4; }
__device__ __forceinline__ int upd_rank(int warp) { return warp - 1 - warp / 4; }

// Block sizes of the pivot-part kernels: warp 0 solves, the other NT - 32
// threads update; a level's launch takes the size its largest front needs.
constexpr int kFwdThreads = 384;   // 12 warps: up to 170 registers a thread
constexpr int kSolveThreadsFor(int maxK) { return maxK <= 64 ? 64 : (maxK <= 384 ? 256 : kFwdThreads); }

// Forward substitution, pivot part of one front (one CTA per front of the
// level): gather this front's right-hand side plus the children's update
// vectors (fixed child order), then solve the unit-lower L11 y = b in
// 32-column blocks and store y (not yet divided by D) and the gathered
// right-hand side of the non-pivot rows, which k_fwd_rect then updates.
// Warp specialised, with one block of lookahead: warp 0 solves block j
// (warp-shuffle chain on the staged diagonal block) after applying block
// j-1's columns to block j's own rows; the other warps apply each solved
// block's columns to the rows from block j+2 on.  A block's rows thus take
// the blocks' columns in increasing order and, per block, one FMA chain in
// column order -- the arithmetic of a plain right-looking sweep -- while the
// bulk updates run behind the dependent chain instead of between its steps.
// Hand-offs: per block an mbarrier "solved" (warp 0's 32 lanes) and
// "updated" (the updaters), two of each alternating; waits are bounded.
template <int NT>
__global__ void __launch_bounds__(NT) k_fwd(const int* __restrict__ fronts, const int* __restrict__ fk,
                                                     const int* __restrict__ fm, const long long* __restrict__ foff,
                                                     const long long* __restrict__ fupd, const int* __restrict__ fdof,
                                                     const int* __restrict__ childOff, const int* __restrict__ childList,
                                                     const int* __restrict__ relOff, const int* __restrict__ relIdx,
                                                     const double* __restrict__ pool, double* __restrict__ upd,
                                                     double* __restrict__ y, int* __restrict__ flag)
{
    extern __shared__ double sh[];
    __shared__ double tile[32 * 33];   // the diagonal block, row-major (padded)
    __shared__ unsigned long long solved[2], updated[2];
    __shared__ int abortFlag;
    const int f = fronts[blockIdx.x];
    const int k = fk[f], m = fm[f], d0 = fdof[f];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = threadIdx.x; r < m; r += blockDim.x) sh[r] = r < k ? y[d0 + r] : 0.0;
    if (threadIdx.x == 0) {
        mbar_init(&solved[0], 32);
        mbar_init(&solved[1], 32);
        mbar_init(&updated[0], 32 * upd_warps(NT));
        mbar_init(&updated[1], 32 * upd_warps(NT));
        abortFlag = 0;
    }
    __syncthreads();
    for (int c = childOff[f]; c < childOff[f + 1]; ++c) {
        const int ch = childList[c];
        const int u = fm[ch] - fk[ch];
        const int* rel = relIdx + relOff[ch];
        const double* uc = upd + fupd[ch];
        for (int i = threadIdx.x; i < u; i += blockDim.x) sh[rel[i]] += uc[i];
        __syncthreads();
    }
    const double* L = pool + foff[f];
    const int nb = (k + 31) / 32;
    if (warp == 0) {
        double an = 0.0;   // this block's rows' sums over the previous block's columns
        for (int j = 0; j < nb; ++j) {
            const int c0 = 32 * j, w = min(32, k - c0);
            const int r = c0 + lane;
            // the diagonal block's entries of this lane's row, and the next
            // block's row entries of this block's columns, loads first
            const int n0 = c0 + 32, wn = j + 1 < nb ? min(32, k - n0) : 0;
            double dl[32], ln[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) dl[c] = (lane < w && c < w) ? L[r + (long long)(c0 + c) * m] : 0.0;
#pragma unroll
            for (int c = 0; c < 32; ++c) ln[c] = lane < wn ? L[(n0 + lane) + (long long)(c0 + c) * m] : 0.0;
            // the updaters are done with block j-2 on this block's rows
            if (j >= 2 && !mbar_wait_bounded(&updated[j & 1], ((j - 2) >> 1) & 1, &abortFlag)) break;
            // block j-1's columns on this block's rows, summed along the
            // previous block's chain (one column per step, in column order)
            if (j >= 1 && lane < w) sh[r] -= an;
#pragma unroll
            for (int c = 0; c < 32; ++c)
                if (lane < w) tile[lane * 33 + c] = dl[c];
            __syncwarp();
            double v = lane < w ? sh[r] : 0.0, anNext = 0.0;
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                if (c < w) {   // warp-uniform
                    const double yc = __shfl_sync(0xffffffffu, v, c);
                    if (lane > c && lane < w) v -= tile[lane * 33 + c] * yc;
                    anNext = fma(ln[c], yc, anNext);
                }
            }
            an = anNext;
            if (lane < w) sh[r] = v;
            __syncwarp();
            mbar_arrive(&solved[j & 1]);
        }
    }
    else if (warp & 3) {
        constexpr int NU = 32 * upd_warps(NT);
        const int t = 32 * upd_rank(warp) + lane;
        for (int b = 0; b < nb; ++b) {
            if (!mbar_wait_bounded(&solved[b & 1], (b >> 1) & 1, &abortFlag)) break;
            const int c0 = 32 * b, w = min(32, k - c0);
            // one row per thread and pass, the block's columns loaded at once;
            // each row summed in column order.  Row r always belongs to
            // updater r % NU: a thread finishes block b on its rows before
            // it takes block b + 1, so every row takes the blocks in order
            // whatever the other threads' progress
            const int r0 = c0 + 64;
            for (int r = r0 + ((t - r0) % NU + NU) % NU; r < k; r += NU) {
                double lv[32];
#pragma unroll
                for (int c = 0; c < 32; ++c) lv[c] = c < w ? L[r + (long long)(c0 + c) * m] : 0.0;
                double acc = 0.0;
#pragma unroll
                for (int c = 0; c < 32; ++c)
                    if (c < w) acc = fma(lv[c], sh[c0 + c], acc);
                sh[r] -= acc;
            }
            mbar_arrive(&updated[b & 1]);
        }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < m; r += blockDim.x) {
        if (r < k) y[d0 + r] = sh[r];
        else upd[fupd[f] + (r - k)] = sh[r];
    }
    if (threadIdx.x == 0 && abortFlag) atomicExch(flag, 1);
}

// Forward substitution, non-pivot rows: upd_r -= sum_c L21[r][c] y_c for a
// chunk of kRectRows (32) rows of one front (all fronts of a level per
// launch).  The columns are split over kFwdRectGroups warps, a warp's lanes
// over the chunk's rows (coalesced column segments); each lane keeps
// kRectIlp independent FMA chains (columns c = c0 + j, c0 + j + kRectIlp, ...
// of its warp's range) so that many loads are in flight, the chains are
// added pairwise, and the warps' partial sums are added in warp order: a
// fixed summation order whatever the timing.
constexpr int kFwdRectGroups = 16;
constexpr int kRectIlp = 8;

// Levels of small fronts (every front's pivot count <= kNarrowK): one thread
// per row and all its columns in two chains, kNarrowRows rows per CTA --
// short rows, many fronts, so occupancy matters more than chain length.
__global__ void __launch_bounds__(kNarrowRows) k_fwd_rect_narrow(const int2* __restrict__ tasks,
                                                                const int* __restrict__ fk,
                                                                const int* __restrict__ fm,
                                                                const long long* __restrict__ foff,
                                                                const long long* __restrict__ fupd,
                                                                const int* __restrict__ fdof,
                                                                const double* __restrict__ pool,
                                                                double* __restrict__ upd, const double* __restrict__ y)
{
    __shared__ double ys[kNarrowK];
    const int2 t = tasks[blockIdx.x];
    const int f = t.x, k = fk[f], m = fm[f], d0 = fdof[f];
    for (int c = threadIdx.x; c < k; c += blockDim.x) ys[c] = y[d0 + c];
    __syncthreads();
    const int r = t.y + threadIdx.x;
    if (r >= m) return;
    const double* L = pool + foff[f] + r;
    double s0 = 0.0, s1 = 0.0;
    int c = 0;
    for (; c + 1 < k; c += 2) {
        s0 = fma(L[(long long)c * m], ys[c], s0);
        s1 = fma(L[(long long)(c + 1) * m], ys[c + 1], s1);
    }
    if (c < k) s0 = fma(L[(long long)c * m], ys[c], s0);
    upd[fupd[f] + (r - k)] -= s0 + s1;
}
__global__ void __launch_bounds__(32 * kFwdRectGroups) k_fwd_rect(const int2* __restrict__ tasks,
                                                                 const int* __restrict__ fk, const int* __restrict__ fm,
                                                                 const long long* __restrict__ foff,
                                                                 const long long* __restrict__ fupd,
                                                                 const int* __restrict__ fdof,
                                                                 const double* __restrict__ pool,
                                                                 double* __restrict__ upd, const double* __restrict__ y)
{
    extern __shared__ double ys[];
    __shared__ double part[kFwdRectGroups][32];
    const int2 t = tasks[blockIdx.x];
    const int f = t.x, k = fk[f], m = fm[f], d0 = fdof[f];
    const int lane = threadIdx.x & 31, g = threadIdx.x >> 5;
    for (int c = threadIdx.x; c < k; c += blockDim.x) ys[c] = y[d0 + c];
    __syncthreads();
    const int r = t.y + lane;
    const int span = (k + kFwdRectGroups - 1) / kFwdRectGroups;
    const int cBeg = g * span, cEnd = min(k, cBeg + span);
    double acc[kRectIlp];
#pragma unroll
    for (int j = 0; j < kRectIlp; ++j) acc[j] = 0.0;
    if (r < m) {
        const double* L = pool + foff[f] + r;
        for (int c = cBeg; c < cEnd; c += kRectIlp) {
            double lv[kRectIlp];
#pragma unroll
            for (int j = 0; j < kRectIlp; ++j) lv[j] = c + j < cEnd ? L[(long long)(c + j) * m] : 0.0;
#pragma unroll
            for (int j = 0; j < kRectIlp; ++j)
                if (c + j < cEnd) acc[j] = fma(lv[j], ys[c + j], acc[j]);
        }
    }
#pragma unroll
    for (int w = kRectIlp / 2; w > 0; w /= 2)
#pragma unroll
        for (int j = 0; j < w; ++j) acc[j] += acc[j + w];
    part[g][lane] = acc[0];
    __syncthreads();
    if (g == 0 && r < m) {
        double s = 0.0;
        for (int q = 0; q < kFwdRectGroups; ++q) s += part[q][lane];
        upd[fupd[f] + (r - k)] -= s;
    }
}

// Backward substitution, non-pivot part: t_c = sum_{r >= k} L21[r][c] x_r for
// a chunk of kRectCols pivot columns of one front (a warp per column, its
// lanes over the rows; kRectIlp independent chains per lane, added pairwise,
// then the lanes' sums in a fixed shuffle tree).
template <int ILP>
__global__ void __launch_bounds__(256) k_bwd_rect(const int2* __restrict__ tasks, const int* __restrict__ fk,
                                                  const int* __restrict__ fm, const long long* __restrict__ foff,
                                                  const int* __restrict__ fdof, const int* __restrict__ frowOff,
                                                  const int* __restrict__ rowIdx, const double* __restrict__ pool,
                                                  const double* __restrict__ x, double* __restrict__ tdot)
{
    const int2 t = tasks[blockIdx.x];
    const int f = t.x, k = fk[f], m = fm[f], d0 = fdof[f];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int c = t.y + warp;
    if (c >= k || warp >= kRectCols) return;
    const int* rows = rowIdx + frowOff[f];
    const double* lc = pool + foff[f] + (long long)c * m;
    double acc[ILP];
#pragma unroll
    for (int j = 0; j < ILP; ++j) acc[j] = 0.0;
    for (int r0 = k + lane; r0 < m; r0 += 32 * ILP) {
        double lv[ILP], xv[ILP];
#pragma unroll
        for (int j = 0; j < ILP; ++j) {
            const int r = r0 + 32 * j;
            lv[j] = r < m ? lc[r] : 0.0;
            xv[j] = r < m ? x[rows[r]] : 0.0;
        }
#pragma unroll
        for (int j = 0; j < ILP; ++j) acc[j] = fma(lv[j], xv[j], acc[j]);
    }
#pragma unroll
    for (int w = ILP / 2; w > 0; w /= 2)
#pragma unroll
        for (int j = 0; j < w; ++j) acc[j] += acc[j + w];
    double s = acc[0];
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(0xffffffffu, s, o);
    if (lane == 0) tdot[d0 + c] = s;
}

// Backward substitution, pivot part of one front: x_S = L11^-T (D^-1 y_S - t)
// with t = L21^T x_B from k_bwd_rect (zero for fronts without ancestors), in
// 32-column blocks from the last, right-looking: once block s is solved, its
// rows' contributions L(s, c) x_s are subtracted from every earlier column c.
// Warp specialised like k_fwd: warp 0 subtracts block s + 1's rows from
// block s's own columns (32 x 32) and back-solves block s on the staged
// diagonal block; the other warps subtract each solved block's rows from the
// columns before the block below it, one block behind.  Per column the
// blocks' contributions are subtracted in decreasing block order, each as
// one FMA chain in row order (a fixed order whatever the timing).
template <int NT>
__global__ void __launch_bounds__(NT) k_bwd(const int* __restrict__ fronts, const int* __restrict__ fk,
                                                     const int* __restrict__ fm, const long long* __restrict__ foff,
                                                     const int* __restrict__ fdof, const double* __restrict__ pool,
                                                     const double* __restrict__ y, const double* __restrict__ tdot,
                                                     double* __restrict__ x, int* __restrict__ flag)
{
    extern __shared__ double sh[];
    __shared__ double tile[32 * 33];   // the diagonal block, row-major (padded)
    __shared__ unsigned long long solved[2], updated[2];
    __shared__ int abortFlag;
    const int f = fronts[blockIdx.x];
    const int k = fk[f], m = fm[f], d0 = fdof[f];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double* L = pool + foff[f];
    const bool rect = m > k;
    for (int r = threadIdx.x; r < k; r += blockDim.x)
        sh[r] = y[d0 + r] / L[r + (long long)r * m] - (rect ? tdot[d0 + r] : 0.0);
    if (threadIdx.x == 0) {
        mbar_init(&solved[0], 32);
        mbar_init(&solved[1], 32);
        mbar_init(&updated[0], 32 * upd_warps(NT));
        mbar_init(&updated[1], 32 * upd_warps(NT));
        abortFlag = 0;
    }
    __syncthreads();
    const int nb = (k + 31) / 32;
    // phase parity of block s's hand-off on barrier s & 1 (blocks go from
    // nb - 1 down; a barrier serves every second one)
    auto parity = [nb](int s) { return (uint32_t)(((nb - 1 - s) >> 1) & 1); };
    if (warp == 0) {
        for (int b = nb - 1; b >= 0; --b) {
            const int c0 = 32 * b, w = min(32, k - c0);
            const int c = c0 + lane;
            // the diagonal block's column of this lane and block b + 1's rows
            // of it, loads first (the lookahead sums those rows in row order,
            // so it cannot ride along the block below's chain, which yields
            // its values from the last row down)
            const int r0 = c0 + 32, w1 = b + 1 <= nb - 1 ? min(32, k - r0) : 0;
            double dl[32], lv[32];
#pragma unroll
            for (int r = 0; r < 32; ++r) dl[r] = (lane < w && r < w) ? L[(c0 + r) + (long long)c * m] : 0.0;
#pragma unroll
            for (int r = 0; r < 32; ++r) lv[r] = (lane < w && r < w1) ? L[(r0 + r) + (long long)c * m] : 0.0;
            // the other warps are done with blocks b + 2 and above on these columns
            if (b + 2 <= nb - 1 && !mbar_wait_bounded(&updated[b & 1], parity(b + 2), &abortFlag)) break;
            if (b + 1 <= nb - 1 && lane < w) {   // block b + 1's rows on this block's columns
                double acc = 0.0;
#pragma unroll
                for (int r = 0; r < 32; ++r)
                    if (r < w1) acc = fma(lv[r], sh[r0 + r], acc);
                sh[c] -= acc;
            }
            // tile[r][lane] = L(c0 + r, c0 + lane)
#pragma unroll
            for (int r = 0; r < 32; ++r)
                if (lane < w) tile[r * 33 + lane] = dl[r];
            __syncwarp();
            double v = lane < w ? sh[c] : 0.0;
            for (int r = w - 1; r >= 0; --r) {
                const double xr = __shfl_sync(0xffffffffu, v, r);
                if (lane < r) v -= tile[r * 33 + lane] * xr;
            }
            if (lane < w) sh[c] = v;
            __syncwarp();
            mbar_arrive(&solved[b & 1]);
        }
    }
    else if (warp & 3) {
        constexpr int NU = 32 * upd_warps(NT);
        const int t = 32 * upd_rank(warp) + lane;
        for (int s = nb - 1; s >= 1; --s) {
            if (!mbar_wait_bounded(&solved[s & 1], parity(s), &abortFlag)) break;
            const int r0 = 32 * s, w = min(32, k - r0);
            // block s's rows on the columns before block s - 1
            for (int c = t; c < 32 * (s - 1); c += NU) {
                double lv[32];
#pragma unroll
                for (int r = 0; r < 32; ++r) lv[r] = r < w ? L[(r0 + r) + (long long)c * m] : 0.0;
                double acc = 0.0;
#pragma unroll
                for (int r = 0; r < 32; ++r)
                    if (r < w) acc = fma(lv[r], sh[r0 + r], acc);
                sh[c] -= acc;
            }
            mbar_arrive(&updated[s & 1]);
        }
    }
    __syncthreads();
    for (int r = threadIdx.x; r < k; r += blockDim.x) x[d0 + r] = sh[r];
    if (threadIdx.x == 0 && abortFlag) atomicExch(flag, 1);
}

// ---- cluster substitutions for the top tree levels ----
//
// A level of few large fronts leaves one SM per front walking ~50 dependent
// 32-column blocks, its updates limited by what one SM pulls from memory.
// Here a front gets a thread-block cluster of C CTAs (C <= 8) and its 32-row
// blocks are dealt out round-robin: block j belongs to rank j % C.  Every CTA
// holds the front's whole right-hand side in shared memory.  The owner of a
// block applies the previous block's columns to it (lookahead) and runs the
// same shuffle chain as k_fwd / k_bwd, then pushes the 32 solved values
// into every other CTA's shared memory with asynchronous stores that count
// their bytes off that CTA's per-block mbarrier (st.async ... complete_tx:
// the sender waits for nothing; each receiving CTA posted the bytes it
// expects per block at the start); each CTA's updaters wait (acquire,
// cluster scope) for the block and apply it to the rows (forward) or columns
// (backward) of the blocks it owns.  No cluster-wide barrier per block: the
// chain passes from rank to rank through point-to-point mbarriers, the
// updates spread over C SMs.  Per row / column the contributions are taken in
// the same order and with the same FMA chains as in k_fwd / k_bwd, so the
// results are bit-identical to theirs.  Every wait is bounded; one that runs
// out raises the abort flag of every CTA of the cluster, so all loops end,
// and the kernel's flag reports it as in k_fwd.
constexpr int kClMaxBlocks = 128;   // pivot blocks per front (k <= 4096)
constexpr int kClThreads = 256;

__device__ __forceinline__ uint32_t cl_rank()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ uint32_t cl_size()
{
    uint32_t r;
    asm volatile("mov.u32 %0, %%cluster_nctarank;" : "=r"(r));
    return r;
}

__device__ __forceinline__ void cl_sync()
{
    asm volatile("barrier.cluster.arrive.release.aligned;\n\tbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

// this CTA's shared address a, as seen in cluster rank r's window
__device__ __forceinline__ uint32_t cl_map(uint32_t a, uint32_t r)
{
    uint32_t out;
    asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(out) : "r"(a), "r"(r));
    return out;
}

__device__ __forceinline__ void cl_store_int(uint32_t a, int v)
{
    asm volatile("st.shared::cluster.s32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}

// an asynchronous store of v into another CTA's shared memory that counts
// its 8 bytes off that CTA's mbarrier (remBar, the same CTA's window): the
// sender does not wait for the store, the receiver's barrier completes when
// the bytes it expects have landed
__device__ __forceinline__ void cl_store_async(uint32_t remAddr, double v, uint32_t remBar)
{
    asm volatile("st.async.shared::cluster.mbarrier::complete_tx::bytes.b64 [%0], %1, [%2];" ::"r"(remAddr),
                 "l"(__double_as_longlong(v)), "r"(remBar)
                 : "memory");
}

// this CTA's barrier b expects `bytes` of asynchronous stores (and takes
// its one arrival)
__device__ __forceinline__ void mbar_expect_bytes(unsigned long long* b, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(b)), "r"(bytes) : "memory");
}

// before leaving: every block pushed into this CTA has landed (waits that
// find nothing coming end after a short bound; only after an abort)
__device__ __forceinline__ void cl_drain(unsigned long long* recv, int nb, uint32_t C, uint32_t q)
{
    for (int j = 0; j < nb; ++j) {
        if ((uint32_t)j % C == q) continue;
        const uint32_t a = smem_addr(&recv[j]);
        for (int i = 0; i < (1 << 16); ++i) {
            uint32_t done;
            asm volatile(
                "{\n\t.reg .pred p;\n\t"
                "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
                "selp.u32 %0, 1, 0, p;\n\t}\n"
                : "=r"(done)
                : "r"(a), "r"(0u)
                : "memory");
            if (done) break;
        }
    }
}

// bounded wait with cluster-scope acquire (sees the remote CTAs' stores)
__device__ __forceinline__ bool cl_wait_bounded(unsigned long long* b, uint32_t parity, volatile int* abort)
{
    const uint32_t a = smem_addr(b);
    for (int i = 0; i < kSolveWaitPolls; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        if (*abort) return false;
    }
    *abort = 1;
    return false;
}

// a wait ran out: raise the abort flag of every CTA of the cluster
__device__ __forceinline__ void cl_abort(int* abortFlag, uint32_t C)
{
    const uint32_t a = smem_addr(abortFlag);
    for (uint32_t r = 0; r < C; ++r) cl_store_int(cl_map(a, r), 1);
}

// Forward substitution, pivot part, one cluster per front (see above).
__global__ void __launch_bounds__(kClThreads) k_fwd_cl(const int* __restrict__ fronts, const int* __restrict__ fk,
                                                       const int* __restrict__ fm, const long long* __restrict__ foff,
                                                       const long long* __restrict__ fupd, const int* __restrict__ fdof,
                                                       const int* __restrict__ childOff, const int* __restrict__ childList,
                                                       const int* __restrict__ relOff, const int* __restrict__ relIdx,
                                                       const double* __restrict__ pool, double* __restrict__ upd,
                                                       double* __restrict__ y, int* __restrict__ flag)
{
    extern __shared__ double sh[];
    __shared__ double tile[32 * 33];
    __shared__ unsigned long long recv[kClMaxBlocks], updated[kClMaxBlocks];
    __shared__ double accIn[32];   // this CTA's next block: the previous block's columns on its rows
    __shared__ int abortFlag;
    constexpr int NU = 32 * upd_warps(kClThreads);   // updater threads
    const uint32_t C = cl_size(), q = cl_rank();
    const int f = fronts[blockIdx.x / C];
    const int k = fk[f], m = fm[f], d0 = fdof[f];
    const int nb = (k + 31) / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int r = threadIdx.x; r < m; r += blockDim.x) sh[r] = r < k ? y[d0 + r] : 0.0;
    if (threadIdx.x == 0) {
        // a block's values: this CTA's warp 0 (32 local arrivals) or
        // another rank's asynchronous stores (one arrival here, the bytes)
        for (int j = 0; j < nb; ++j) {
            mbar_init(&recv[j], (uint32_t)j % C == q ? 32 : 1);
            mbar_init(&updated[j], NU);
        }
        abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        // block j's values, and with them, when block j + 1 is this CTA's,
        // its rows' sums over block j's columns
        for (int j = 0; j < nb; ++j)
            if ((uint32_t)j % C != q) {
                uint32_t bytes = 8u * (uint32_t)min(32, k - 32 * j);
                if (j + 1 < nb && (uint32_t)(j + 1) % C == q) bytes += 8u * (uint32_t)min(32, k - 32 * (j + 1));
                mbar_expect_bytes(&recv[j], bytes);
            }
    }
    __syncthreads();
    for (int c = childOff[f]; c < childOff[f + 1]; ++c) {
        const int ch = childList[c];
        const int u = fm[ch] - fk[ch];
        const int* rel = relIdx + relOff[ch];
        const double* uc = upd + fupd[ch];
        for (int i = threadIdx.x; i < u; i += blockDim.x) sh[rel[i]] += uc[i];
        __syncthreads();
    }
    cl_sync();   // every CTA's barriers initialised before the first remote arrive
    const double* L = pool + foff[f];
    if (warp == 0) {
        for (int j = (int)q; j < nb; j += (int)C) {
            const int c0 = 32 * j, w = min(32, k - c0);
            const int r = c0 + lane;
            // the next block's rows (another rank's): their sums over this
            // block's columns are accumulated along the chain, one column per
            // step in column order -- the lookahead k_fwd runs after the chain
            const int n0 = c0 + 32, wn = j + 1 < nb ? min(32, k - n0) : 0;
            double dl[32], ln[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) dl[c] = (lane < w && c < w) ? L[r + (long long)(c0 + c) * m] : 0.0;
#pragma unroll
            for (int c = 0; c < 32; ++c) ln[c] = lane < wn ? L[(n0 + lane) + (long long)(c0 + c) * m] : 0.0;
            // block j-1's values and its columns' sums on these rows (from
            // its owner), and this CTA's updaters done with block j-2 here
            bool ok = j < 1 || cl_wait_bounded(&recv[j - 1], 0, &abortFlag);
            ok = ok && (j < 2 || cl_wait_bounded(&updated[j - 2], 0, &abortFlag));
            if (!__all_sync(0xffffffffu, ok)) break;
            if (j >= 1 && lane < w) sh[r] -= accIn[lane];
#pragma unroll
            for (int c = 0; c < 32; ++c)
                if (lane < w) tile[lane * 33 + c] = dl[c];
            __syncwarp();
            double v = lane < w ? sh[r] : 0.0, an = 0.0;
#pragma unroll
            for (int c = 0; c < 32; ++c) {
                if (c < w) {   // warp-uniform
                    const double yc = __shfl_sync(0xffffffffu, v, c);
                    if (lane > c && lane < w) v -= tile[lane * 33 + c] * yc;
                    an = fma(ln[c], yc, an);
                }
            }
            if (lane < w) sh[r] = v;
            __syncwarp();
            // publish: the w values into every other CTA, counted off its
            // barrier for block j, and the next block's sums to its owner
            // (on the same barrier there); then this CTA's own barrier
            const uint32_t av = smem_addr(&sh[c0 + (lane < w ? lane : 0)]), ab = smem_addr(&recv[j]);
            if (lane < w)
                for (uint32_t t = 1; t < C; ++t) {
                    const uint32_t dst = (q + t) % C;
                    cl_store_async(cl_map(av, dst), v, cl_map(ab, dst));
                }
            if (lane < wn) {
                const uint32_t nxt = (q + 1) % C;
                cl_store_async(cl_map(smem_addr(&accIn[lane]), nxt), an, cl_map(ab, nxt));
            }
            mbar_arrive(&recv[j]);
        }
        if (abortFlag) cl_abort(&abortFlag, C);
    }
    else if (warp & 3) {
        const int t = 32 * upd_rank(warp) + lane;
        // this CTA's rows numbered 32 u + (r % 32) over its blocks q + u C;
        // row number rho always belongs to updater rho % NU (a row takes the
        // blocks in order, as in k_fwd)
        const int nOwnAll = (int)q < nb ? (nb - 1 - (int)q) / (int)C + 1 : 0;
        for (int b = 0; b < nb; ++b) {
            const int c0 = 32 * b, w = min(32, k - c0);
            // this CTA's blocks from b + 2 on: the first is the smallest
            // i >= b + 2 with i % C == q
            const int i0 = b + 2 + (int)((q + C - (uint32_t)((b + 2) % C)) % C);
            const int rho0 = 32 * ((i0 - (int)q) / (int)C);
            const int rhoF = rho0 + ((t - rho0) % NU + NU) % NU;
            // the first row's entries of block b's columns, loaded before the
            // block's values arrive (the factor is final)
            const int rF = rhoF < 32 * nOwnAll ? 32 * ((int)q + (rhoF >> 5) * (int)C) + (rhoF & 31) : k;
            double lv[32];
#pragma unroll
            for (int c = 0; c < 32; ++c) lv[c] = (rF < k && c < w) ? L[rF + (long long)(c0 + c) * m] : 0.0;
            if (!cl_wait_bounded(&recv[b], 0, &abortFlag)) break;
            for (int rho = rhoF; rho < 32 * nOwnAll; rho += NU) {
                const int r = 32 * ((int)q + (rho >> 5) * (int)C) + (rho & 31);
                if (r >= k) continue;
                if (rho != rhoF) {
#pragma unroll
                    for (int c = 0; c < 32; ++c) lv[c] = c < w ? L[r + (long long)(c0 + c) * m] : 0.0;
                }
                double acc = 0.0;
#pragma unroll
                for (int c = 0; c < 32; ++c)
                    if (c < w) acc = fma(lv[c], sh[c0 + c], acc);
                sh[r] -= acc;
            }
            mbar_arrive(&updated[b]);
        }
        if (abortFlag) cl_abort(&abortFlag, C);
    }
    __syncthreads();
    for (int j = (int)q; j < nb; j += (int)C)
        for (int r = 32 * j + threadIdx.x; r < min(k, 32 * j + 32); r += blockDim.x) y[d0 + r] = sh[r];
    if (q == 0)
        for (int r = k + threadIdx.x; r < m; r += blockDim.x) upd[fupd[f] + (r - k)] = sh[r];
    if (threadIdx.x == 0) {
        cl_drain(recv, nb, C, q);
        if (abortFlag) atomicExch(flag, 1);
    }
    cl_sync();   // no CTA leaves while another may still write into it
}

// Backward substitution, pivot part, one cluster per front: column block b
// belongs to rank b % C; blocks go from the last down (see k_bwd).
__global__ void __launch_bounds__(kClThreads) k_bwd_cl(const int* __restrict__ fronts, const int* __restrict__ fk,
                                                       const int* __restrict__ fm, const long long* __restrict__ foff,
                                                       const int* __restrict__ fdof, const double* __restrict__ pool,
                                                       const double* __restrict__ y, const double* __restrict__ tdot,
                                                       double* __restrict__ x, int* __restrict__ flag)
{
    extern __shared__ double sh[];
    __shared__ double tile[32 * 33];
    __shared__ unsigned long long recv[kClMaxBlocks], updated[kClMaxBlocks];
    __shared__ int abortFlag;
    constexpr int NU = 32 * upd_warps(kClThreads);
    const uint32_t C = cl_size(), q = cl_rank();
    const int f = fronts[blockIdx.x / C];
    const int k = fk[f], m = fm[f], d0 = fdof[f];
    const int nb = (k + 31) / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const double* L = pool + foff[f];
    const bool rect = m > k;
    for (int r = threadIdx.x; r < k; r += blockDim.x)
        sh[r] = y[d0 + r] / L[r + (long long)r * m] - (rect ? tdot[d0 + r] : 0.0);
    if (threadIdx.x == 0) {
        // a block's values: this CTA's warp 0 (32 local arrivals) or
        // another rank's asynchronous stores (one arrival here, the bytes)
        for (int j = 0; j < nb; ++j) {
            mbar_init(&recv[j], (uint32_t)j % C == q ? 32 : 1);
            mbar_init(&updated[j], NU);
        }
        abortFlag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        for (int j = 0; j < nb; ++j)
            if ((uint32_t)j % C != q) mbar_expect_bytes(&recv[j], 8u * (uint32_t)min(32, k - 32 * j));
    }
    __syncthreads();
    cl_sync();
    if (warp == 0) {
        // this CTA's blocks, from the last down
        const int top = (nb - 1) - (int)((uint32_t)(nb - 1 + C - q) % C);
        for (int b = top; b >= 0; b -= (int)C) {
            const int c0 = 32 * b, w = min(32, k - c0);
            const int c = c0 + lane;
            const int r0 = c0 + 32, w1 = b + 1 <= nb - 1 ? min(32, k - r0) : 0;
            double dl[32], lv[32];
#pragma unroll
            for (int r = 0; r < 32; ++r) dl[r] = (lane < w && r < w) ? L[(c0 + r) + (long long)c * m] : 0.0;
#pragma unroll
            for (int r = 0; r < 32; ++r) lv[r] = (lane < w && r < w1) ? L[(r0 + r) + (long long)c * m] : 0.0;
            bool ok = b + 1 > nb - 1 || cl_wait_bounded(&recv[b + 1], 0, &abortFlag);
            ok = ok && (b + 2 > nb - 1 || cl_wait_bounded(&updated[b + 2], 0, &abortFlag));
            if (!__all_sync(0xffffffffu, ok)) break;
            if (b + 1 <= nb - 1 && lane < w) {
                double acc = 0.0;
#pragma unroll
                for (int r = 0; r < 32; ++r)
                    if (r < w1) acc = fma(lv[r], sh[r0 + r], acc);
                sh[c] -= acc;
            }
#pragma unroll
            for (int r = 0; r < 32; ++r)
                if (lane < w) tile[r * 33 + lane] = dl[r];
            __syncwarp();
            double v = lane < w ? sh[c] : 0.0;
            for (int r = w - 1; r >= 0; --r) {
                const double xr = __shfl_sync(0xffffffffu, v, r);
                if (lane < r) v -= tile[r * 33 + lane] * xr;
            }
            if (lane < w) sh[c] = v;
            __syncwarp();
            const uint32_t av = smem_addr(&sh[c0 + (lane < w ? lane : 0)]), ab = smem_addr(&recv[b]);
            if (lane < w)
                for (uint32_t t = 1; t < C; ++t) {
                    const uint32_t dst = (q + t) % C;
                    cl_store_async(cl_map(av, dst), v, cl_map(ab, dst));
                }
            mbar_arrive(&recv[b]);
        }
        if (abortFlag) cl_abort(&abortFlag, C);
    }
    else if (warp & 3) {
        const int t = 32 * upd_rank(warp) + lane;
        for (int s = nb - 1; s >= 1; --s) {
            const int r0 = 32 * s, w = min(32, k - r0);
            // this CTA's column blocks up to s - 2: the last is the largest
            // i <= s - 2 with i % C == q
            const int hi = s - 2;
            const int i1 = hi >= 0 ? hi - (int)((uint32_t)(hi + C - q) % C) : -1;
            const int nOwn = i1 >= 0 ? i1 / (int)C + 1 : 0;
            // this CTA's columns numbered 32 u + (c % 32) over its blocks
            // q + u C; column number gam always belongs to updater gam % NU.
            // The first column's entries of block s's rows are loaded before
            // the block's values arrive (the factor is final)
            const int cF = t < 32 * nOwn ? 32 * ((int)q + (t >> 5) * (int)C) + (t & 31) : -1;
            double lv[32];
#pragma unroll
            for (int r = 0; r < 32; ++r) lv[r] = (cF >= 0 && r < w) ? L[(r0 + r) + (long long)cF * m] : 0.0;
            if (!cl_wait_bounded(&recv[s], 0, &abortFlag)) break;
            for (int gam = t; gam < 32 * nOwn; gam += NU) {
                const int c = 32 * ((int)q + (gam >> 5) * (int)C) + (gam & 31);
                if (gam != t) {
#pragma unroll
                    for (int r = 0; r < 32; ++r) lv[r] = r < w ? L[(r0 + r) + (long long)c * m] : 0.0;
                }
                double acc = 0.0;
#pragma unroll
                for (int r = 0; r < 32; ++r)
                    if (r < w) acc = fma(lv[r], sh[r0 + r], acc);
                sh[c] -= acc;
            }
            mbar_arrive(&updated[s]);
        }
        if (abortFlag) cl_abort(&abortFlag, C);
    }
    __syncthreads();
    for (int j = (int)q; j < nb; j += (int)C)
        for (int r = 32 * j + threadIdx.x; r < min(k, 32 * j + 32); r += blockDim.x) x[d0 + r] = sh[r];
    if (threadIdx.x == 0) {
        cl_drain(recv, nb, C, q);   // block 0's values, which no updater waits for
        if (abortFlag) atomicExch(flag, 1);
    }
    cl_sync();
}


} // namespace

int chol_upload(CholPlan& P, std::string* err)
{
    if (!P.valid) {
        if (err) *err = "chol: inconsistent symbolic structure";
        return OC_ERR_INVALID;
    }
    cudaError_t e = cudaSuccess;
    auto chk = [&](cudaError_t x) { if (e == cudaSuccess) e = x; };
    // a buffer of at least `need` elements, grown by a quarter when too small
    auto grow = [&](auto*& ptr, size_t& cap, size_t need) {
        if (e != cudaSuccess || (ptr && cap >= need)) return;
        cudaFree(ptr);
        ptr = nullptr;
        cap = 0;
        const size_t want = need + need / 4 + 64;
        chk(cudaMalloc(reinterpret_cast<void**>(&ptr), sizeof(*ptr) * want));
        if (e == cudaSuccess) cap = want;
    };
    CholPlan::Keep& K = P.keep;
    grow(K.pool, K.poolCap, (size_t)std::max<long long>(P.poolSize, 1));
    grow(K.upd, K.updCap, (size_t)std::max<long long>(P.updSize, 1));
    grow(K.vec, K.vecCap, 3 * (size_t)std::max(P.nDof, 1));
    if (!K.flags) chk(cudaMalloc(reinterpret_cast<void**>(&K.flags), 2 * sizeof(int)));
    // the index arrays, each at a 256-byte-aligned offset of one buffer
    struct Part { void** dst; const void* src; size_t bytes; };
    const Part parts[] = {
        {reinterpret_cast<void**>(&P.dPermDof), P.permDof.data(), sizeof(int) * P.permDof.size()},
        {reinterpret_cast<void**>(&P.dFk), P.fk.data(), sizeof(int) * P.fk.size()},
        {reinterpret_cast<void**>(&P.dFm), P.fm.data(), sizeof(int) * P.fm.size()},
        {reinterpret_cast<void**>(&P.dFdofStart), P.fdofStart.data(), sizeof(int) * P.fdofStart.size()},
        {reinterpret_cast<void**>(&P.dFrowOff), P.frowOff.data(), sizeof(int) * P.frowOff.size()},
        {reinterpret_cast<void**>(&P.dFoff), P.foff.data(), sizeof(long long) * P.foff.size()},
        {reinterpret_cast<void**>(&P.dFupd), P.fupd.data(), sizeof(long long) * P.fupd.size()},
        {reinterpret_cast<void**>(&P.dRowIdx), P.rowIdx.data(), sizeof(int) * P.rowIdx.size()},
        {reinterpret_cast<void**>(&P.dChildOff), P.childOff.data(), sizeof(int) * P.childOff.size()},
        {reinterpret_cast<void**>(&P.dChildList), P.childList.data(), sizeof(int) * P.childList.size()},
        {reinterpret_cast<void**>(&P.dRelOff), P.relOff.data(), sizeof(int) * P.relOff.size()},
        {reinterpret_cast<void**>(&P.dRelIdx), P.relIdx.data(), sizeof(int) * P.relIdx.size()},
        {reinterpret_cast<void**>(&P.dLevelFronts), P.levelFronts.data(), sizeof(int) * P.levelFronts.size()},
        {reinterpret_cast<void**>(&P.dTasks), P.tasks.data(), sizeof(TileTask) * P.tasks.size()},
        {reinterpret_cast<void**>(&P.dAsmDest), P.asmDest.data(), sizeof(long long) * P.asmDest.size()},
        {reinterpret_cast<void**>(&P.dAsmLd), P.asmLd.data(), sizeof(int) * P.asmLd.size()},
        {reinterpret_cast<void**>(&P.dAsmDiag), P.asmDiag.data(), sizeof(unsigned char) * P.asmDiag.size()},
        {reinterpret_cast<void**>(&P.dRectRowTasks), P.rectRowTasks.data(), sizeof(int2) * P.rectRowTasks.size()},
        {reinterpret_cast<void**>(&P.dRectColTasks), P.rectColTasks.data(), sizeof(int2) * P.rectColTasks.size()},
    };
    auto al = [](size_t x) { return (x + 255) & ~size_t(255); };
    size_t total = 0;
    for (const Part& q : parts) total += al(std::max<size_t>(q.bytes, 1));
    grow(K.idx, K.idxCap, total);
    if (e == cudaSuccess) {
        size_t off = 0;
        for (const Part& q : parts) {
            *q.dst = K.idx + off;
            if (q.bytes) chk(cudaMemcpyAsync(K.idx + off, q.src, q.bytes, cudaMemcpyHostToDevice, 0));
            off += al(std::max<size_t>(q.bytes, 1));
        }
        P.pool = K.pool;
        P.upd = K.upd;
        P.yperm = K.vec;
        P.xperm = K.vec + std::max(P.nDof, 1);
        P.tmpDot = K.vec + 2 * (size_t)std::max(P.nDof, 1);
        P.dFlag = K.flags;
        P.dSolveFlag = K.flags + 1;
        if (P.nFactStreams > 1 && !K.fork) {   // the factorization's streams and events
            chk(cudaEventCreateWithFlags(&K.fork, cudaEventDisableTiming));
            for (int a = 0; a < CholPlan::kMaxFactStreams - 1 && e == cudaSuccess; ++a) {
                chk(cudaStreamCreateWithFlags(&K.aux[a], cudaStreamNonBlocking));
                chk(cudaEventCreateWithFlags(&K.join[a], cudaEventDisableTiming));
            }
            for (int g = 0; g < CholPlan::kMaxFactGroups && e == cudaSuccess; ++g)
                chk(cudaEventCreateWithFlags(&K.grpEnd[g], cudaEventDisableTiming));
        }
        chk(cudaMemsetAsync(P.dSolveFlag, 0, sizeof(int), 0));
        chk(cudaStreamSynchronize(0));
    }
    if (e != cudaSuccess) {
        if (err) *err = std::string("chol upload: ") + cudaGetErrorString(e);
        chol_free(P);
        return OC_ERR_CUDA;
    }
    P.onDevice = true;
    return OC_OK;
}

void chol_free(CholPlan& P)
{
    if (P.factGraph) cudaGraphExecDestroy(P.factGraph);
    if (P.solveGraph) cudaGraphExecDestroy(P.solveGraph);
    P.factGraph = P.solveGraph = nullptr;
    P.factKey = nullptr;
    P.solveKey[0] = P.solveKey[1] = nullptr;
    P.dRectRowTasks = P.dRectColTasks = nullptr;
    P.tmpDot = nullptr;
    P.pool = P.upd = P.yperm = P.xperm = nullptr;
    P.dPermDof = P.dFk = P.dFm = P.dFdofStart = P.dFrowOff = nullptr;
    P.dFoff = P.dFupd = nullptr;
    P.dRowIdx = P.dChildOff = P.dChildList = P.dRelOff = P.dRelIdx = P.dLevelFronts = nullptr;
    P.dTasks = nullptr;
    P.dAsmDest = nullptr;
    P.dAsmLd = nullptr;
    P.dAsmDiag = nullptr;
    P.dFlag = nullptr;
    P.dSolveFlag = nullptr;
    P.onDevice = false;
}

void chol_destroy(CholPlan& P)
{
    chol_free(P);
    cudaFree(P.keep.idx);
    cudaFree(P.keep.pool);
    cudaFree(P.keep.upd);
    cudaFree(P.keep.vec);
    cudaFree(P.keep.flags);
    for (int a = 0; a < CholPlan::kMaxFactStreams - 1; ++a) {
        if (P.keep.aux[a]) cudaStreamDestroy(P.keep.aux[a]);
        if (P.keep.join[a]) cudaEventDestroy(P.keep.join[a]);
    }
    for (int g = 0; g < CholPlan::kMaxFactGroups; ++g)
        if (P.keep.grpEnd[g]) cudaEventDestroy(P.keep.grpEnd[g]);
    if (P.keep.fork) cudaEventDestroy(P.keep.fork);
    P.keep = CholPlan::Keep{};
}

static void enqueue_factorize(CholPlan& P, const DeviceBsr& b, cudaStream_t st)
{
    cudaMemsetAsync(P.pool, 0, sizeof(double) * (size_t)P.poolSize, st);
    cudaMemsetAsync(P.dFlag, 0, sizeof(int), st);
    k_asm_fronts<<<(b.nnzb + 255) / 256, 256, 0, st>>>(b.val, P.dAsmDest, P.dAsmLd, P.dAsmDiag, b.nnzb, P.pool);
    // the groups' streams fork off after the assembly; each group waits for
    // the ends of the groups it joins, runs its launches and records its own
    // end; every stream joins st at the end
    const int nS = P.keep.fork ? P.nFactStreams : 1;
    const int nG = static_cast<int>(P.grpStream.size());
    if (nS > 1) {
        cudaEventRecord(P.keep.fork, st);
        for (int a = 1; a < nS; ++a) cudaStreamWaitEvent(P.keep.aux[a - 1], P.keep.fork, 0);
    }
    for (int g = 0; g < nG; ++g) {
        const cudaStream_t ls = (nS > 1 && P.grpStream[g] > 0) ? P.keep.aux[P.grpStream[g] - 1] : st;
        if (nS > 1)
            for (int i = P.grpWaitOff[g]; i < P.grpWaitOff[g + 1]; ++i)
                cudaStreamWaitEvent(ls, P.keep.grpEnd[P.grpWait[i]], 0);
        for (int li = P.grpLaunchOff[g]; li < P.grpLaunchOff[g + 1]; ++li) {
            const CholPlan::Launch& L = P.launches[li];
            const TileTask* t = P.dTasks + L.taskOff;
            switch (L.kind) {
            case 0: k_extend<<<L.taskCount, 256, 0, ls>>>(t, P.dFk, P.dFm, P.dFoff, P.dRelOff, P.dRelIdx, P.pool); break;
            case 1: k_ldl_panel<<<L.taskCount, 32 * kPanelRows, 0, ls>>>(t, P.dFk, P.dFm, P.dFoff, P.pool); break;
            case 4: k_ldl_diag<<<L.taskCount, kDiagThreads, 0, ls>>>(t, P.dFk, P.dFm, P.dFoff, P.pool, P.dFlag); break;
            default:   // 5
                k_ldl_update<kUpdSmall, 2><<<L.taskCount, 256, 0, ls>>>(t, P.dFk, P.dFm, P.dFoff, P.pool, P.dFlag);
                break;
            }
        }
        if (nS > 1) cudaEventRecord(P.keep.grpEnd[g], ls);
    }
    for (int a = 1; a < nS; ++a) {
        cudaEventRecord(P.keep.join[a - 1], P.keep.aux[a - 1]);
        cudaStreamWaitEvent(st, P.keep.join[a - 1], 0);
    }
}

// The launch sequence is fixed per topology, so it is captured once into a
// CUDA graph (keyed by the block-CSR value array it reads) and replayed.
int chol_factorize(CholPlan& P, const DeviceBsr& b, cudaStream_t st, std::string* err, int* nBad)
{
    if (!P.onDevice) return OC_ERR_INVALID;
    if (P.useGraphs && (!P.factGraph || P.factKey != b.val)) {
        if (P.factGraph) cudaGraphExecDestroy(P.factGraph);
        P.factGraph = nullptr;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            enqueue_factorize(P, b, st);
            if (cudaStreamEndCapture(st, &g) == cudaSuccess && g) {
                if (cudaGraphInstantiate(&P.factGraph, g, 0) != cudaSuccess) P.factGraph = nullptr;
                cudaGraphDestroy(g);
            }
        }
        cudaGetLastError();   // a failed capture falls back to direct launches
        P.factKey = b.val;
    }
    if (P.factGraph) cudaGraphLaunch(P.factGraph, st);
    else enqueue_factorize(P, b, st);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        if (err) *err = std::string("chol factorize: ") + cudaGetErrorString(e);
        return OC_ERR_CUDA;
    }
    if (nBad) {
        e = cudaMemcpyAsync(nBad, P.dFlag, sizeof(int), cudaMemcpyDeviceToHost, st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(st);
        if (e != cudaSuccess) {
            if (err) *err = std::string("chol factorize: ") + cudaGetErrorString(e);
            return OC_ERR_CUDA;
        }
    }
    return OC_OK;
}

// Cluster size for a level's pivot-part substitutions: levels of few fronts
// with at least two 32-column blocks per rank get a cluster per front, sized
// so that the level fills up to ~152 CTAs; 1 (one CTA per front) otherwise.
static int solve_cluster_for(const CholPlan& P, int l)
{
    const int cnt = P.levelFrontOff[l + 1] - P.levelFrontOff[l];
    const int nb = (P.levelMaxK[l] + 31) / 32;
    if (P.solveCluster < 2 || nb > kClMaxBlocks) return 1;
    for (int C = std::min(P.solveCluster, 8); C >= 2; C /= 2)
        if (cnt * C <= 152 && nb >= 2 * C) return C;
    return 1;
}

template <typename... A>
static void launch_cluster(void (*kern)(A...), int grid, int C, size_t shm, cudaStream_t st, A... args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(kClThreads);
    cfg.dynamicSmemBytes = shm;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeClusterDimension;
    at[0].val.clusterDim.x = C;
    at[0].val.clusterDim.y = 1;
    at[0].val.clusterDim.z = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    cudaLaunchKernelEx(&cfg, kern, args...);
}

static void enqueue_solve(CholPlan& P, const double2* rhs, double2* x, double sign, cudaStream_t st, size_t shm,
                          size_t shmK)
{
    const int n = P.nDof;
    k_permute_in<<<(n + 255) / 256, 256, 0, st>>>(reinterpret_cast<const double*>(rhs), P.dPermDof, sign, n, P.yperm);
    for (int l = 0; l < P.nLevels; ++l) {
        const int off = P.levelFrontOff[l], cnt = P.levelFrontOff[l + 1] - off;
        const size_t lshm = sizeof(double) * (size_t)std::max(P.levelMaxM[l], 1);
        const int C = solve_cluster_for(P, l);
        if (C > 1)
            launch_cluster(k_fwd_cl, cnt * C, C, lshm, st, (const int*)(P.dLevelFronts + off), (const int*)P.dFk,
                           (const int*)P.dFm, (const long long*)P.dFoff, (const long long*)P.dFupd,
                           (const int*)P.dFdofStart, (const int*)P.dChildOff, (const int*)P.dChildList,
                           (const int*)P.dRelOff, (const int*)P.dRelIdx, (const double*)P.pool, P.upd, P.yperm,
                           P.dSolveFlag);
        else
        switch (kSolveThreadsFor(P.levelMaxK[l])) {
#define OC_FWD(NT)                                                                                                      \
    k_fwd<NT><<<cnt, NT, lshm, st>>>(P.dLevelFronts + off, P.dFk, P.dFm, P.dFoff, P.dFupd, P.dFdofStart, P.dChildOff,     \
                                     P.dChildList, P.dRelOff, P.dRelIdx, P.pool, P.upd, P.yperm, P.dSolveFlag)
        case 64: OC_FWD(64); break;
        case 256: OC_FWD(256); break;
        default: OC_FWD(kFwdThreads); break;
#undef OC_FWD
        }
        const int ro = P.rectRowOff[l], rc = P.rectRowOff[l + 1] - ro;
        if (rc && P.levelMaxK[l] <= kNarrowK)
            k_fwd_rect_narrow<<<rc, kNarrowRows, 0, st>>>(P.dRectRowTasks + ro, P.dFk, P.dFm, P.dFoff, P.dFupd,
                                                          P.dFdofStart, P.pool, P.upd, P.yperm);
        else if (rc)
            k_fwd_rect<<<rc, 32 * kFwdRectGroups, shmK, st>>>(P.dRectRowTasks + ro, P.dFk, P.dFm, P.dFoff, P.dFupd,
                                                              P.dFdofStart, P.pool, P.upd, P.yperm);
    }
    for (int l = P.nLevels - 1; l >= 0; --l) {
        const int off = P.levelFrontOff[l], cnt = P.levelFrontOff[l + 1] - off;
        const int co = P.rectColOff[l], cc = P.rectColOff[l + 1] - co;
        if (cc && P.levelMaxK[l] <= kNarrowK)
            k_bwd_rect<1><<<cc, 32 * kRectCols, 0, st>>>(P.dRectColTasks + co, P.dFk, P.dFm, P.dFoff, P.dFdofStart,
                                                         P.dFrowOff, P.dRowIdx, P.pool, P.xperm, P.tmpDot);
        else if (cc)
            k_bwd_rect<kRectIlp><<<cc, 32 * kRectCols, 0, st>>>(P.dRectColTasks + co, P.dFk, P.dFm, P.dFoff,
                                                                P.dFdofStart, P.dFrowOff, P.dRowIdx, P.pool, P.xperm,
                                                                P.tmpDot);
        const size_t lshm = sizeof(double) * (size_t)std::max(P.levelMaxM[l], 1);
        const int C = solve_cluster_for(P, l);
        if (C > 1)
            launch_cluster(k_bwd_cl, cnt * C, C, lshm, st, (const int*)(P.dLevelFronts + off), (const int*)P.dFk,
                           (const int*)P.dFm, (const long long*)P.dFoff, (const int*)P.dFdofStart,
                           (const double*)P.pool, (const double*)P.yperm, (const double*)P.tmpDot, P.xperm,
                           P.dSolveFlag);
        else
        switch (kSolveThreadsFor(P.levelMaxK[l])) {
#define OC_BWD(NT)                                                                                                      \
    k_bwd<NT><<<cnt, NT, lshm, st>>>(P.dLevelFronts + off, P.dFk, P.dFm, P.dFoff, P.dFdofStart, P.pool, P.yperm,          \
                                     P.tmpDot, P.xperm, P.dSolveFlag)
        case 64: OC_BWD(64); break;
        case 256: OC_BWD(256); break;
        default: OC_BWD(kFwdThreads); break;
#undef OC_BWD
        }
    }
    k_permute_out<<<(n + 255) / 256, 256, 0, st>>>(P.xperm, P.dPermDof, n, reinterpret_cast<double*>(x));
}

int chol_solve_cluster_levels(const CholPlan& P, int* largest)
{
    int n = 0, big = 1;
    for (int l = 0; l < P.nLevels; ++l) {
        const int C = solve_cluster_for(P, l);
        if (C > 1) ++n;
        big = std::max(big, C);
    }
    if (largest) *largest = big;
    return n;
}

void chol_set_factor_streams(CholPlan& P, int streams)
{
    P.factStreams = std::max(1, std::min(streams, (int)CholPlan::kMaxFactStreams));
}

bool chol_groups_ordered(const CholPlan& P)
{
    const int nG = static_cast<int>(P.grpStream.size());
    if (nG < 1 || nG > CholPlan::kMaxFactGroups || (int)P.grpWaitOff.size() != nG + 1 ||
        (int)P.grpLaunchOff.size() != nG + 1 || P.grpLaunchOff[nG] != (int)P.launches.size() ||
        (int)P.frontGroup.size() != P.nFronts)
        return false;
    // hb[a][b]: group a's launches finish before group b's start
    std::vector<std::vector<char>> hb(nG, std::vector<char>(nG, 0));
    for (int g = 0; g < nG; ++g) {
        if (P.grpStream[g] < 0 || P.grpStream[g] >= P.nFactStreams) return false;
        if (P.grpLaunchOff[g] > P.grpLaunchOff[g + 1]) return false;
        for (int h = 0; h < g; ++h)
            if (P.grpStream[h] == P.grpStream[g]) hb[h][g] = 1;
        for (int i = P.grpWaitOff[g]; i < P.grpWaitOff[g + 1]; ++i) {
            if (P.grpWait[i] < 0 || P.grpWait[i] >= g) return false;   // waits only on earlier groups
            hb[P.grpWait[i]][g] = 1;
        }
    }
    for (int k = 0; k < nG; ++k)
        for (int a = 0; a < nG; ++a)
            if (hb[a][k])
                for (int b = 0; b < nG; ++b)
                    if (hb[k][b]) hb[a][b] = 1;
    for (int f = 0; f < P.nFronts; ++f) {
        const int gf = P.frontGroup[f];
        if (gf < 0 || gf >= nG) return false;
        for (int i = P.childOff[f]; i < P.childOff[f + 1]; ++i) {
            const int c = P.childList[i], gc = P.frontGroup[c];
            if (gc == gf ? P.flevel[c] >= P.flevel[f] : !hb[gc][gf]) return false;
        }
    }
    return true;
}

void chol_set_solve_cluster(CholPlan& P, int maxCluster)
{
    P.solveCluster = std::max(1, std::min(maxCluster, 8));
    if (P.solveGraph) cudaGraphExecDestroy(P.solveGraph);
    P.solveGraph = nullptr;
    P.solveKey[0] = P.solveKey[1] = nullptr;
}

int chol_solve_status(CholPlan& P, cudaStream_t st, int* timedOut)
{
    if (!P.onDevice || !timedOut) return OC_ERR_INVALID;
    cudaError_t e = cudaMemcpyAsync(timedOut, P.dSolveFlag, sizeof(int), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    return e == cudaSuccess ? OC_OK : OC_ERR_CUDA;
}

// Forward/backward substitution; captured into a CUDA graph per
// (rhs, x, sign) and replayed.
int chol_solve(CholPlan& P, const double2* rhs, double2* x, double sign, cudaStream_t st, std::string* err)
{
    if (!P.onDevice) return OC_ERR_INVALID;
    int maxK = 0;
    for (int f = 0; f < P.nFronts; ++f) maxK = std::max(maxK, P.fk[f]);
    const size_t shm = sizeof(double) * (size_t)P.maxM, shmK = sizeof(double) * (size_t)std::max(maxK, 1);
    if (shm > 48 * 1024) {
        cudaFuncSetAttribute(k_fwd<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        cudaFuncSetAttribute(k_fwd<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        cudaFuncSetAttribute(k_fwd<kFwdThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        cudaFuncSetAttribute(k_bwd<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        cudaFuncSetAttribute(k_bwd<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        cudaFuncSetAttribute(k_bwd<kFwdThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        cudaFuncSetAttribute(k_fwd_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
        cudaFuncSetAttribute(k_bwd_cl, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shm);
    }
    if (shmK > 48 * 1024) cudaFuncSetAttribute(k_fwd_rect, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shmK);
    if (P.useGraphs && (!P.solveGraph || P.solveKey[0] != rhs || P.solveKey[1] != x || P.solveSign != sign)) {
        if (P.solveGraph) cudaGraphExecDestroy(P.solveGraph);
        P.solveGraph = nullptr;
        cudaGraph_t g = nullptr;
        if (cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal) == cudaSuccess) {
            enqueue_solve(P, rhs, x, sign, st, shm, shmK);
            if (cudaStreamEndCapture(st, &g) == cudaSuccess && g) {
                if (cudaGraphInstantiate(&P.solveGraph, g, 0) != cudaSuccess) P.solveGraph = nullptr;
                cudaGraphDestroy(g);
            }
        }
        cudaGetLastError();
        P.solveKey[0] = rhs;
        P.solveKey[1] = x;
        P.solveSign = sign;
    }
    if (P.solveGraph) cudaGraphLaunch(P.solveGraph, st);
    else enqueue_solve(P, rhs, x, sign, st, shm, shmK);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        if (err) *err = std::string("chol solve: ") + cudaGetErrorString(e);
        return OC_ERR_CUDA;
    }
    return OC_OK;
}

} // namespace oc
