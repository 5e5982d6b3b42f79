// Topology queries (TriMesh::querySplit / queryMerge, src/TriMesh.cpp:548-951)
// with the candidates' local solves batched on the device.
//
// The host enumerates the candidates exactly as the reference does (split
// filter on the per-vertex gradient deviation, boundary and interior split
// paths, zipper-bottom cohesive pairs with the merged-position projection),
// builds every local mesh (TriMesh::computeLocalEdDec_inSplit / _bSplit /
// _merge, TriMesh.cpp:2262-2794, with the local cut or split applied) as a
// packed problem, and the device solves them all in batched launches
// (k_local_newton per size class; with bijectivity on, k_local_newton_bij,
// whose problems also carry the candidates' local air loops).

#include "oc_topo.h"
#include "oc_mlp.h"
#include "oc_loopmesh.cuh"

#include <algorithm>
#include <array>
#include <map>
#include <mutex>
#include <deque>
#include <unordered_map>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <utility>
#include <memory>
#include <thread>

namespace oc {
namespace {

// vertex adjacency and directed half-edges of a triangle mesh (TriMesh's
// vNeighbor and edge2Tri)
struct Topo {
    int nV = 0, nF = 0;
    const int* F = nullptr;
    std::vector<int> hoPtr, hoTo, hoTri;   // outgoing half-edges per vertex
    std::vector<int> nbPtr, nb;            // sorted neighbours per vertex
    std::vector<char> bnd;

    // Counting sorts in chunks on the host pool: chunk c of the items counts
    // per key, the per-key offsets of the chunks follow in chunk order, and
    // each chunk scatters its items in item order, so every list comes out
    // in the order of the sequential counting sort.
    void build(int nV_, const int* F_, int nF_)
    {
        nV = nV_;
        nF = nF_;
        F = F_;
        const int nt = static_cast<int>(std::max<size_t>(1, std::min<size_t>(HostPool::threads(), nF / 8192)));
        std::vector<int> off((size_t)nt * nV);   // per chunk and key: count, then offset within the key
        auto chunk = [](int n, int c, int nt) { return std::make_pair((int)((long long)n * c / nt),
                                                                     (int)((long long)n * (c + 1) / nt)); };
        // key ranges of the per-key passes (offsets, sorts, merges)
        const int nk = static_cast<int>(std::max<size_t>(1, std::min<size_t>(HostPool::threads(), nV / 4096)));
        auto prefix_keys = [&](std::vector<int>& ptr) {
            ptr.assign(nV + 1, 0);
            host_run_tasks(nk, [&](size_t q) {
                const auto r = chunk(nV, (int)q, nk);
                for (int v = r.first; v < r.second; ++v) {
                    int s = 0;
                    for (int c = 0; c < nt; ++c) {
                        const int x = off[(size_t)c * nV + v];
                        off[(size_t)c * nV + v] = s;
                        s += x;
                    }
                    ptr[v + 1] = s;
                }
            });
            for (int v = 0; v < nV; ++v) ptr[v + 1] += ptr[v];
        };
        // out-half-edges per vertex, in triangle order
        host_run_tasks(nt, [&](size_t c) {
            int* o = off.data() + c * nV;
            std::fill(o, o + nV, 0);
            const auto r = chunk(nF, (int)c, nt);
            for (long long i = 3LL * r.first; i < 3LL * r.second; ++i) o[F[i]]++;
        });
        prefix_keys(hoPtr);
        hoTo.resize(3 * (size_t)nF);
        hoTri.resize(3 * (size_t)nF);
        host_run_tasks(nt, [&](size_t c) {
            int* o = off.data() + c * nV;
            const auto r = chunk(nF, (int)c, nt);
            for (int t = r.first; t < r.second; ++t)
                for (int k = 0; k < 3; ++k) {
                    const int a = F[3 * t + k], b = F[3 * t + (k + 1) % 3];
                    const int p = hoPtr[a] + o[a]++;
                    hoTo[p] = b;
                    hoTri[p] = t;
                }
        });
        // out-half-edges of each vertex sorted by target (edge_tri bisects)
        host_run_tasks(nk, [&](size_t q) {
            const auto r = chunk(nV, (int)q, nk);
            for (int a = r.first; a < r.second; ++a) {
                const int p0 = hoPtr[a], p1 = hoPtr[a + 1];
                for (int p = p0 + 1; p < p1; ++p) {   // insertion sort: a handful per vertex
                    const int to = hoTo[p], tri = hoTri[p];
                    int q2 = p;
                    for (; q2 > p0 && hoTo[q2 - 1] > to; --q2) {
                        hoTo[q2] = hoTo[q2 - 1];
                        hoTri[q2] = hoTri[q2 - 1];
                    }
                    hoTo[q2] = to;
                    hoTri[q2] = tri;
                }
            }
        });
        // in-half-edges of each vertex, sources ascending (chunks of sources)
        std::vector<int> hiPtr, hiFrom(3 * (size_t)nF);
        host_run_tasks(nt, [&](size_t c) {
            int* o = off.data() + c * nV;
            std::fill(o, o + nV, 0);
            const auto r = chunk(nV, (int)c, nt);
            for (int p = hoPtr[r.first]; p < hoPtr[r.second]; ++p) o[hoTo[p]]++;
        });
        prefix_keys(hiPtr);
        host_run_tasks(nt, [&](size_t c) {
            int* o = off.data() + c * nV;
            const auto r = chunk(nV, (int)c, nt);
            for (int a = r.first; a < r.second; ++a)
                for (int p = hoPtr[a]; p < hoPtr[a + 1]; ++p) hiFrom[hiPtr[hoTo[p]] + o[hoTo[p]]++] = a;
        });
        // neighbours = out-targets merged with in-sources; a neighbour in
        // only one of the two lists is across a boundary edge
        // (TriMesh::isBoundaryVert, TriMesh.cpp:2069-2083): sizes first,
        // then the lists
        auto merge = [&](int v, int* out, char* border) {
            int i = hoPtr[v], j = hiPtr[v], n = 0;
            const int ie = hoPtr[v + 1], je = hiPtr[v + 1];
            while (i < ie || j < je) {
                int x;
                if (j >= je || (i < ie && hoTo[i] < hiFrom[j])) {
                    x = hoTo[i++];
                    *border = 1;
                }
                else if (i >= ie || hiFrom[j] < hoTo[i]) {
                    x = hiFrom[j++];
                    *border = 1;
                }
                else {
                    x = hoTo[i];
                    ++i;
                    ++j;
                }
                if (out) out[n] = x;
                ++n;
            }
            return n;
        };
        nbPtr.assign(nV + 1, 0);
        bnd.assign(nV, 0);
        host_run_tasks(nk, [&](size_t q) {
            const auto r = chunk(nV, (int)q, nk);
            for (int v = r.first; v < r.second; ++v) nbPtr[v + 1] = merge(v, nullptr, &bnd[v]);
        });
        for (int v = 0; v < nV; ++v) nbPtr[v + 1] += nbPtr[v];
        nb.resize(nbPtr[nV]);
        host_run_tasks(nk, [&](size_t q) {
            const auto r = chunk(nV, (int)q, nk);
            char dummy = 0;
            for (int v = r.first; v < r.second; ++v) merge(v, nb.data() + nbPtr[v], &dummy);
        });
    }

    int edge_tri(int a, int b) const
    {
        int lo = hoPtr[a], hi = hoPtr[a + 1];
        while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (hoTo[mid] < b) lo = mid + 1;
            else hi = mid;
        }
        return lo < hoPtr[a + 1] && hoTo[lo] == b ? hoTri[lo] : -1;
    }

    int degree(int v) const { return nbPtr[v + 1] - nbPtr[v]; }

    bool adjacent(int a, int b) const { return std::binary_search(nb.begin() + nbPtr[a], nb.begin() + nbPtr[a + 1], b); }

    int third(int t, int a, int b) const
    {
        for (int k = 0; k < 3; ++k)
            if (F[3 * t + k] != a && F[3 * t + k] != b) return F[3 * t + k];
        return -1;
    }

    // TriMesh::isBoundaryVert(vI, vI_neighbor, tri_toSep, boundaryEdge,
    // toBound) (TriMesh.cpp:2032-2067): the fan of vI from the edge to
    // vI_neighbor, rotating until a boundary edge (true) or back (false)
    bool walk(int vI, int vNb, bool toBound, std::vector<int>& tris) const
    {
        tris.clear();
        int f = toBound ? edge_tri(vNb, vI) : edge_tri(vI, vNb);
        if (f < 0) return true;
        int vNew = vNb;
        for (int guard = 0; guard <= nF; ++guard) {
            tris.push_back(f);
            vNew = third(f, vI, vNew);
            if (vNew == vNb) return false;
            f = toBound ? edge_tri(vNew, vI) : edge_tri(vI, vNew);
            if (f < 0) return true;
        }
        return false;
    }
};

} // namespace

struct TopoAdjacency {
    Topo T;
};

TopoWorkspace::~TopoWorkspace()
{
    for (auto s : aux)
        if (s) {
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
        }
    for (auto x : ev)
        if (x) cudaEventDestroy(x);
    for (auto* p : buf) cudaFree(p);
}

std::shared_ptr<TopoAdjacency> topo_adjacency(int nV, const int* F, int nF)
{
    auto a = std::make_shared<TopoAdjacency>();
    a->T.build(nV, F, nF);
    return a;
}

namespace {

double rest_dist(const double* Vr, int a, int b)
{
    const double dx = Vr[3 * a] - Vr[3 * b], dy = Vr[3 * a + 1] - Vr[3 * b + 1], dz = Vr[3 * a + 2] - Vr[3 * b + 2];
    return std::sqrt(dx * dx + dy * dy + dz * dz);
}

// packed local problems and what each one belongs to
struct Batch {
    std::vector<LocalProblem> prob;
    std::vector<int> ltGlobal, ltCorner, lvSlot, initTri;
    std::vector<double2> lvPos;
    std::vector<int> apLocal;       // bijective: air-loop points (local vertex or -1)
    std::vector<double2> apPos;     // and their positions when fixed
    struct Tag {
        int cand;          // candidate index
        int a = -1, b = -1, c = -1;   // path entries
        double se = 0.0;   // seam term of this problem (seInc or seDec)
        int nRows = 0;     // newVertPos rows
    };
    std::vector<Tag> tag;
};

// local vertex table over a triangle list (first appearance in row order);
// `alias` maps a global vertex to another whose local vertex it shares
struct LocalMesh {
    std::vector<int> gv;        // local -> global
    std::vector<int> corner;    // 3 per triangle
    std::vector<int>* map = nullptr;   // global -> local of the last build (-1 elsewhere), nV entries
    int find(int g) const
    {
        if (map) return (*map)[g];
        for (size_t i = 0; i < gv.size(); ++i)
            if (gv[i] == g) return static_cast<int>(i);
        return -1;
    }
    void build(const Topo& T, const std::vector<int>& tris, int aliasA = -1, int aliasB = -1)
    {
        if (map) {
            if (map->size() != static_cast<size_t>(T.nV)) map->assign(T.nV, -1);
            for (int g : gv) (*map)[g] = -1;
        }
        gv.clear();
        corner.clear();
        for (int t : tris)
            for (int k = 0; k < 3; ++k) {
                int g = T.F[3 * t + k];
                if (g == aliasB) g = aliasA;
                int l = find(g);
                if (l < 0) {
                    l = static_cast<int>(gv.size());
                    gv.push_back(g);
                    if (map) (*map)[g] = l;
                }
                corner.push_back(l);
            }
    }
};

void emit(Batch& B, const Topo& T, const double* rest, const double* UV, const std::vector<int>& tris,
          const LocalMesh& L, const std::vector<double2>& extraPos, const std::vector<int>& slotOfLocal, int nFree,
          int nFixed, const Batch::Tag& tag)
{
    (void)T;
    LocalProblem P{};
    P.triOff = static_cast<int>(B.ltGlobal.size());
    P.nTri = static_cast<int>(tris.size());
    P.vertOff = static_cast<int>(B.lvPos.size());
    const int nLocal = static_cast<int>(L.gv.size()) + static_cast<int>(extraPos.size());
    P.nVert = nLocal;
    P.initOff = static_cast<int>(B.initTri.size());
    P.nInit = static_cast<int>(tris.size());
    P.nFree = nFree;
    P.maxIter = 100;   // computeLocalEdDec_* default (TriMesh.hpp:166-180)
    double area = 0.0;
    for (int t : tris) area += rest[8 * (size_t)t];   // local computeFeatures order
    P.localArea = area;
    P.targetGRes = 1.0 * static_cast<double>(nLocal - nFixed) / static_cast<double>(nLocal) * 1.0e-6;
    for (size_t i = 0; i < tris.size(); ++i) {
        B.ltGlobal.push_back(tris[i]);
        B.initTri.push_back(tris[i]);
        for (int k = 0; k < 3; ++k) B.ltCorner.push_back(L.corner[3 * i + k]);
    }
    for (size_t l = 0; l < L.gv.size(); ++l) {
        B.lvPos.push_back(make_double2(UV[2 * (size_t)L.gv[l]], UV[2 * (size_t)L.gv[l] + 1]));
        B.lvSlot.push_back(slotOfLocal[l]);
    }
    for (size_t e = 0; e < extraPos.size(); ++e) {
        B.lvPos.push_back(extraPos[e]);
        B.lvSlot.push_back(slotOfLocal[L.gv.size() + e]);
    }
    B.prob.push_back(P);
    B.tag.push_back(tag);
}

// ---------------------------------------------------------------------
// Bijective form: the local air loops (Scaffold::get1RingAirLoop /
// getCornerAirLoop, Scaffold.cpp:339-520) and the separation of the split
// copies (TriMesh::computeLocalEdDec_inSplit / _bSplit, TriMesh.cpp:2326-2372,
// 2597-2660) that the local Scaffold's air loop needs.

double2 d2(double x, double y) { return make_double2(x, y); }

// SymDirichletEnergy::initStepSize per triangle (SymDirichletEnergy.cpp:
// 555-609): the bound from det(U + alpha V) > 0, or stepSize when none
double step_bound_host(double2 U1, double2 U2, double2 U3, double2 V1, double2 V2, double2 V3, double stepSize)
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
        if ((b < 0.0) && (delta >= 0.0)) bound = 2.0 * c / (-b + std::sqrt(delta));
    }
    else if (a < 0.0) {
        if (b < 0.0) bound = 2.0 * c / (-b + std::sqrt(delta));
        else bound = (-b - std::sqrt(delta)) / 2.0 / a;
    }
    else {
        if (b < 0.0) bound = -c / b;
    }
    return bound < stepSize ? bound : stepSize;
}

// the whole-mesh air mesh with its adjacency
struct AirSrc {
    int nAirV = 0, nBnd = 0;
    const double* V = nullptr;
    const int* bnd = nullptr;
    std::vector<int> F;
    Topo T;
    std::vector<int> meshToAir;
    void build(const TopoQueryIn& in)
    {
        nAirV = in.nAirV;
        nBnd = in.nAirBnd;
        V = in.airV;
        bnd = in.airBnd;
        F.assign(in.airF, in.airF + 3 * (size_t)in.nAirF);
        T.build(nAirV, F.data(), in.nAirF);
        meshToAir.assign(in.nV, -1);
        for (int i = 0; i < nBnd; ++i)
            if (bnd[i] >= 0 && bnd[i] < in.nV) meshToAir[bnd[i]] = i;
    }
    double2 pos(int a) const { return d2(V[2 * (size_t)a], V[2 * (size_t)a + 1]); }
    int mesh_of(int a) const { return a >= 0 && a < nBnd ? bnd[a] : -1; }
};

// Scaffold::get1RingAirLoop (Scaffold.cpp:339-388) for mesh vertex v: air
// vertex ids, [1] = v, [2] and [0] the two ends of its air fan (the mesh
// boundary neighbours), [3..] the fan's outer vertices from [2]'s side round
// to [0]'s; false when v has no air fan
bool ring_loop(const AirSrc& A, int v, std::vector<int>& rows)
{
    rows.clear();
    const int a = v >= 0 && v < static_cast<int>(A.meshToAir.size()) ? A.meshToAir[v] : -1;
    if (a < 0 || A.T.degree(a) == 0) return false;
    const int nb0 = A.T.nb[A.T.nbPtr[a]];
    std::vector<int> u0, u;
    A.T.walk(a, nb0, false, u0);
    A.T.walk(a, nb0, true, u);
    std::reverse(u.begin(), u.end());
    u.insert(u.end(), u0.begin(), u0.end());
    if (u.empty()) return false;
    rows.assign(u.size() + 2, -1);
    rows[1] = a;
    for (size_t ti = 0; ti < u.size(); ++ti) {
        const int t = u[ti];
        int k = 0;
        while (k < 3 && A.F[3 * (size_t)t + k] != a) ++k;
        if (k == 3) return false;
        rows[ti + 2] = A.F[3 * (size_t)t + (k + 1) % 3];
        if (ti + 1 == u.size()) rows[0] = A.F[3 * (size_t)t + (k + 2) % 3];
    }
    return A.mesh_of(rows[0]) >= 0 && A.mesh_of(rows[2]) >= 0;
}

// IglUtils::Test2DSegmentSegment with eps = 0 (IglUtils.cpp:647-705; after
// Ericson, Real-Time Collision Detection)
double signed_area2(double2 a, double2 b, double2 c) { return (a.x - c.x) * (b.y - c.y) - (a.y - c.y) * (b.x - c.x); }
bool segments_intersect(double2 a, double2 b, double2 c, double2 d)
{
    const double a1 = signed_area2(a, b, d), a2 = signed_area2(a, b, c);
    if (a1 * a2 <= 0.0) {
        const double a3 = signed_area2(c, d, a), a4 = a3 + a2 - a1;
        if (a3 * a4 <= 0.0) {
            if (std::abs(a1) <= 0.0 && std::abs(a2) <= 0.0) {
                const double abx = b.x - a.x, aby = b.y - a.y;
                const double sq = abx * abx + aby * aby;
                double cc = ((c.x - a.x) * abx + (c.y - a.y) * aby) / sq;
                double cd = ((d.x - a.x) * abx + (d.y - a.y) * aby) / sq;
                if (cc > cd) std::swap(cc, cd);
                return !((cc > 1.0) || (cd < 0.0));
            }
            return true;
        }
    }
    return false;
}

// IglUtils::computeRotAngle (IglUtils.cpp:637-641)
double rot_angle(double2 from, double2 to)
{
    const double nf = std::sqrt(from.x * from.x + from.y * from.y), nt = std::sqrt(to.x * to.x + to.y * to.y);
    const double angle = std::acos(std::max(-1.0, std::min(1.0, (from.x * to.x + from.y * to.y) / nf / nt)));
    return (from.x * to.y - from.y * to.x < 0.0) ? -angle : angle;
}

// Scaffold::getCornerAirLoop (Scaffold.cpp:390-519) for the merge of corner
// (p0, p1, p2): the air loop around the three corners' air fans with p1 and
// p2 removed, started one before p0 (air ids in loop, positions in pts,
// pts[1] = mergedPos); false when the reference abandons the query (the
// loop self-intersects or turns clockwise) or the loop is not found
bool corner_loop(const AirSrc& A, const int corner_mesh[3], double2 mergedPos, std::vector<int>& loop,
                 std::vector<double2>& pts)
{
    int corner[3];
    for (int i = 0; i < 3; ++i) {
        corner[i] = A.meshToAir[corner_mesh[i]];
        if (corner[i] < 0 || A.T.degree(corner[i]) == 0) return false;
    }
    std::vector<int> inc, tmp;
    for (int i = 0; i < 3; ++i) {
        const int nb0 = A.T.nb[A.T.nbPtr[corner[i]]];
        A.T.walk(corner[i], nb0, false, tmp);
        inc.insert(inc.end(), tmp.begin(), tmp.end());
        A.T.walk(corner[i], nb0, true, tmp);
        inc.insert(inc.end(), tmp.begin(), tmp.end());
    }
    std::sort(inc.begin(), inc.end());   // std::set order
    inc.erase(std::unique(inc.begin(), inc.end()), inc.end());
    if (inc.empty()) return false;
    // igl::boundary_loop of the incident triangles: loops traced along the
    // triangles' orientation from the smallest unvisited border vertex, the
    // longest kept
    const int nI = static_cast<int>(inc.size());
    std::vector<int> verts;
    for (int t : inc)
        for (int k = 0; k < 3; ++k) verts.push_back(A.F[3 * (size_t)t + k]);
    std::sort(verts.begin(), verts.end());
    verts.erase(std::unique(verts.begin(), verts.end()), verts.end());
    auto lid = [&](int a) { return static_cast<int>(std::lower_bound(verts.begin(), verts.end(), a) - verts.begin()); };
    const int nVl = static_cast<int>(verts.size());
    std::vector<int> Fl(3 * (size_t)nI);
    for (int f = 0; f < nI; ++f)
        for (int k = 0; k < 3; ++k) Fl[3 * f + k] = lid(A.F[3 * (size_t)inc[f] + k]);
    std::vector<std::vector<int>> VF(nVl);
    for (int f = 0; f < nI; ++f)
        for (int k = 0; k < 3; ++k) VF[Fl[3 * f + k]].push_back(f);
    auto has_edge = [&](int u, int v) {   // a triangle with u -> v
        for (int f : VF[u])
            for (int k = 0; k < 3; ++k)
                if (Fl[3 * f + k] == u && Fl[3 * f + (k + 1) % 3] == v) return true;
        return false;
    };
    std::vector<char> border(nVl, 0);
    for (int f = 0; f < nI; ++f)
        for (int k = 0; k < 3; ++k) {
            const int u = Fl[3 * f + k], v = Fl[3 * f + (k + 1) % 3];
            if (!has_edge(v, u)) border[u] = border[v] = 1;
        }
    std::vector<char> unvisited(border);
    std::vector<int> best;
    for (int s0 = 0; s0 < nVl; ++s0) {
        if (!unvisited[s0]) continue;
        std::vector<int> l{s0};
        unvisited[s0] = 0;
        for (int guard = 0; guard <= nVl; ++guard) {
            const int v = l.back();
            int next = -1;
            for (int f : VF[v]) {
                int k = 0;
                while (Fl[3 * f + k] != v) ++k;
                const int vn = Fl[3 * f + (k + 1) % 3];
                if (unvisited[vn] && !has_edge(vn, v)) {
                    next = vn;
                    break;
                }
            }
            if (next < 0) break;
            l.push_back(next);
            unvisited[next] = 0;
        }
        if (l.size() > best.size()) best.swap(l);
    }
    std::vector<int> L;
    for (int x : best) L.push_back(verts[x]);
    const int n = static_cast<int>(L.size());
    if (n < 5) return false;
    int startI = -1;
    for (int i = 0; i < n && startI < 0; ++i)
        if (L[i] == corner[0]) {
            if (L[(i - 1 + n) % n] == corner[1] && L[(i - 2 + n) % n] == corner[2]) startI = i;
            else return false;
        }
    if (startI < 0) return false;
    // remove corner[2] and corner[1]; start one before corner[0]
    std::vector<int> rest;
    for (int i = 0; i < n; ++i)
        if (i != (startI - 1 + n) % n && i != (startI - 2 + n) % n) rest.push_back(L[i]);
    const int m = n - 2;
    int c0 = 0;
    while (rest[c0] != corner[0]) ++c0;
    loop.clear();
    for (int i = 0; i < m; ++i) loop.push_back(rest[(c0 - 1 + m + i) % m]);
    for (int i = 0; i < 3; ++i)
        if (A.mesh_of(loop[i]) < 0) return false;
    pts.resize(m);
    for (int i = 0; i < m; ++i) pts[i] = A.pos(loop[i]);
    pts[1] = mergedPos;
    // loop edges (i, i + 1), (m - 1, 0): no two non-adjacent ones may meet
    auto e0 = [&](int e) { return pts[e]; };
    auto e1 = [&](int e) { return pts[(e + 1) % m]; };
    for (int eJ = 2; eJ + 1 < m; ++eJ)
        if (segments_intersect(e0(0), e1(0), e0(eJ), e1(eJ))) return false;
    for (int eI = 1; eI + 2 < m; ++eI)
        for (int eJ = eI + 2; eJ < m; ++eJ)
            if (segments_intersect(e0(eI), e1(eI), e0(eJ), e1(eJ))) return false;
    double rot = 0.0;
    auto dir = [&](int e) { return d2(e1(e).x - e0(e).x, e1(e).y - e0(e).y); };
    for (int e = 0; e + 1 < m; ++e) rot += rot_angle(dir(e), dir(e + 1));
    rot += rot_angle(dir(m - 1), dir(0));
    return rot > 0.0;
}

// TriMesh::compute2DInwardNormal (TriMesh.cpp:2085-2103) of local vertex v
// of the local mesh LT at positions P
double2 inward_normal(const Topo& LT, const std::vector<double2>& P, int v)
{
    if (LT.degree(v) == 0) return d2(0.0, 0.0);
    const int nb = LT.nb[LT.nbPtr[v]];
    // the fan's two ends: rotating from nb one way, then the other
    int ends[2] = {-1, -1};
    for (int side = 0; side < 2; ++side) {
        const bool toBound = side == 1;
        int f = toBound ? LT.edge_tri(nb, v) : LT.edge_tri(v, nb);
        int vNew = nb;
        for (int guard = 0; f >= 0 && guard <= LT.nF; ++guard) {
            vNew = LT.third(f, v, vNew);
            if (vNew == nb) return d2(0.0, 0.0);   // interior vertex
            f = toBound ? LT.edge_tri(vNew, v) : LT.edge_tri(v, vNew);
        }
        ends[side] = vNew;
    }
    auto unit = [](double2 x) {
        const double z = x.x * x.x + x.y * x.y;
        if (z > 0.0) {
            const double r = std::sqrt(z);
            return d2(x.x / r, x.y / r);
        }
        return x;
    };
    const double2 b0 = unit(d2(P[ends[0]].x - P[v].x, P[ends[0]].y - P[v].y));
    const double2 b1 = unit(d2(P[ends[1]].x - P[v].x, P[ends[1]].y - P[v].y));
    double2 nrm = unit(d2(b0.x + b1.x, b0.y + b1.y));
    if (b1.x * nrm.y - b1.y * nrm.x < 0.0) nrm = d2(-nrm.x, -nrm.y);
    return nrm;
}

// moves the two copies va, vb apart along their inward normals, a tenth of
// their injective step at a time, until their squared distance reaches
// epsSep or stops growing (TriMesh.cpp:2344-2366)
void separate_copies(const Topo& LT, std::vector<double2>& P, const std::vector<int>& corner, int va, int vb,
                     double epsSep)
{
    double2 sv[2] = {P[va], P[vb]};
    const double2 nrm[2] = {inward_normal(LT, P, va), inward_normal(LT, P, vb)};
    auto sqdist = [](double2 a, double2 b) { return (a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y); };
    double cur = sqdist(sv[0], sv[1]);
    const int nT = static_cast<int>(corner.size() / 3);
    for (int guard = 0; cur < epsSep && guard < 4096; ++guard) {
        for (int i = 0; i < 2; ++i) {
            const int v = i == 0 ? va : vb;
            double step = 1.0;
            for (int t = 0; t < nT; ++t) {
                const int c[3] = {corner[3 * t], corner[3 * t + 1], corner[3 * t + 2]};
                if (c[0] != v && c[1] != v && c[2] != v) continue;
                double2 D[3];
                for (int k = 0; k < 3; ++k) D[k] = c[k] == v ? nrm[i] : d2(0.0, 0.0);
                step = step_bound_host(P[c[0]], P[c[1]], P[c[2]], D[0], D[1], D[2], step);
            }
            sv[i].x += 0.1 * step * nrm[i].x;
            sv[i].y += 0.1 * step * nrm[i].y;
        }
        P[va] = sv[0];
        P[vb] = sv[1];
        const double last = cur;
        cur = sqdist(sv[0], sv[1]);
        if (std::abs(cur - last) / last < 1.0e-3) break;
    }
}

// areaThres_AM of a local Scaffold: sqrt(3)/4 (avgEdgeLen / 2 / 10)^2 with
// the local mesh's igl::avg_edge_length (every triangle's three edges)
// (Scaffold.cpp:34, 150, 189)
double local_air_thres(const double* Vrest, const int* F, const std::vector<int>& tris)
{
    double sum = 0.0;
    long long cnt = 0;
    for (int t : tris)
        for (int j = 0; j < 3; ++j) {
            const int a = F[3 * (size_t)t + j], b = F[3 * (size_t)t + (j + 1) % 3];
            const double dx = Vrest[3 * (size_t)a] - Vrest[3 * (size_t)b];
            const double dy = Vrest[3 * (size_t)a + 1] - Vrest[3 * (size_t)b + 1];
            const double dz = Vrest[3 * (size_t)a + 2] - Vrest[3 * (size_t)b + 2];
            sum += std::sqrt(dx * dx + dy * dy + dz * dz);
            ++cnt;
        }
    const double eps = sum / static_cast<double>(cnt) * 0.5 * 0.1;
    return std::sqrt(3.0) / 4.0 * eps * eps;
}

// attaches an air loop to the last emitted problem (nAir -1: the reference
// abandons this problem, its energy decrease is -DBL_MAX)
void emit_air(Batch& B, const std::vector<int>& local, const std::vector<double2>& pos, double thres, bool reject)
{
    LocalProblem& P = B.prob.back();
    P.airOff = static_cast<int>(B.apLocal.size());
    P.airThres = thres;
    if (reject || local.size() > static_cast<size_t>(kLoopMaxPts) || local.size() < 3) {
        P.nAir = -1;
        return;
    }
    P.nAir = static_cast<int>(local.size());
    B.apLocal.insert(B.apLocal.end(), local.begin(), local.end());
    B.apPos.insert(B.apPos.end(), pos.begin(), pos.end());
}

// the split filter: vertices sorted by -divGrad in a std::map (equal keys
// keep the last vertex), first max(2, pow(count, exponent)) of them
// (TriMesh.cpp:561-629)
std::vector<int> filter_candidates(const std::vector<std::pair<double, int>>& keyed, double exponent, int& poolSize)
{
    // stable sort by key: contiguous chunks stable-sorted on host threads,
    // then merged pairwise (std::merge takes equal keys from the earlier
    // chunk first), which is the stable sort of the whole list
    auto byKey = [](const std::pair<double, int>& x, const std::pair<double, int>& y) { return x.first < y.first; };
    const size_t n = keyed.size();
    std::vector<std::pair<double, int>> s(keyed), tmp(n);
    const size_t nt = std::max<size_t>(1, std::min<size_t>(HostPool::threads(), n / 4096));
    std::vector<size_t> cut(nt + 1);
    for (size_t t = 0; t <= nt; ++t) cut[t] = n * t / nt;
    host_run_tasks(nt, [&](size_t t) { std::stable_sort(s.begin() + cut[t], s.begin() + cut[t + 1], byKey); });
    while (cut.size() > 2) {
        std::vector<size_t> next;
        for (size_t k = 0; k + 1 < cut.size(); k += 2) next.push_back(cut[k]);
        next.push_back(n);
        host_run_tasks((cut.size()) / 2, [&](size_t i) {
            const size_t k = 2 * i;
            if (k + 2 < cut.size())
                std::merge(s.begin() + cut[k], s.begin() + cut[k + 1], s.begin() + cut[k + 1], s.begin() + cut[k + 2],
                           tmp.begin() + cut[k], byKey);
            else
                std::copy(s.begin() + cut[k], s.begin() + cut[k + 1], tmp.begin() + cut[k]);
        });
        s.swap(tmp);
        cut.swap(next);
    }
    std::vector<std::pair<double, int>> uniq;
    for (const auto& kv : s) {
        if (!uniq.empty() && uniq.back().first == kv.first) uniq.back().second = kv.second;
        else uniq.push_back(kv);
    }
    poolSize = static_cast<int>(uniq.size());
    std::vector<int> out;
    if (uniq.empty()) return out;
    int amt = static_cast<int>(std::pow(static_cast<double>(uniq.size()), exponent));
    if (amt < 2) amt = 2;
    for (const auto& kv : uniq) {
        out.push_back(kv.second);
        if ((int)out.size() >= amt) break;
    }
    return out;
}

bool inverted_any(const Topo& T, const std::vector<double>& V, const std::vector<int>& tris)
{
    for (int t : tris) {   // TriMesh::checkInversion(triI), TriMesh.cpp:1710-1733
        const int* f = T.F + 3 * t;
        const double e00 = V[2 * f[1]] - V[2 * f[0]], e01 = V[2 * f[1] + 1] - V[2 * f[0] + 1];
        const double e10 = V[2 * f[2]] - V[2 * f[0]], e11 = V[2 * f[2] + 1] - V[2 * f[0] + 1];
        if (e00 * e11 - e01 * e10 < 0.0) return true;
    }
    return false;
}

} // namespace

namespace {

// ---- schedule autotuner ------------------------------------------------
// On first use of a (device, size class, problem-count bucket, largest
// triangle-count bucket) the candidate schedules of the class are timed on
// the batch itself (CUDA events on the class's stream, one run each after
// the first) and the fastest is kept for later batches of that key.  Opt-in
// (kTopoAutotune): the fixed rule is the default, so that a run's schedule
// -- and with it the rounding of the clustered sums -- does not depend on
// timing.
std::mutex g_schedMu;
std::map<std::array<int, 4>, ScheduleRecord> g_schedTable;

int log2_bucket(int x)
{
    int b = 0;
    while ((1 << (b + 1)) <= x) ++b;
    return b;
}

std::vector<LocalSchedule> schedule_candidates(int cls, int maxTri, int maxCluster)
{
    std::vector<LocalSchedule> c;
    if (cls == 3) c = {{8, 1, 32}, {8, 1, 128}, {32, 1, 32}, {32, 1, 128}};
    else if (cls == 2) c = {{32, 1, 32}, {32, 1, 128}, {128, 1, 128}, {8, 1, 128}};
    else {
        c = {{128, 1, 128}, {32, 1, 128}};
        const int need = (maxTri + 31) / 32;
        for (int cl = 2; cl <= maxCluster && cl <= 16; cl *= 2)
            if (cl <= 2 * need) c.push_back({64, cl, 64});
    }
    return c;
}

} // namespace

std::vector<ScheduleRecord> topo_schedule_table()
{
    std::lock_guard<std::mutex> lock(g_schedMu);
    std::vector<ScheduleRecord> out;
    for (const auto& kv : g_schedTable) out.push_back(kv.second);
    return out;
}

namespace {

// Solves the problems `which` of B into res[k], grouped by size class
// (threads per problem and cluster size from local_schedule), the classes
// launched on their own streams so that the few large fans overlap the many
// small problems; maxIterOverride > 0 caps the Newton iterations.  batchId
// names B: a second call for the same batch (the learned proposal's exact
// pass after its probe) reuses the problem arrays already on the device.
int solve_batch(const TopoQueryIn& in, const Batch& B, unsigned long long batchId, const std::vector<int>& which,
                int maxIterOverride, int fp32, std::vector<LocalResult>& res, std::string* err, bool autotune = false)
{
    if (which.empty()) return OC_OK;
    TopoWorkspace tmp;
    TopoWorkspace& W = in.ws ? *in.ws : tmp;
    // size classes, largest first so that the long poles start first, each
    // with the schedule its size and count call for
    // (the bijective problems, those with an air loop, form a fifth class
    // of their own kernel)
    constexpr int kClasses = 4;
    auto classOfP = [&](const LocalProblem& P) {
        return P.nAir != 0 ? kClasses : P.nTri > 160 ? 0 : P.nTri > 40 ? 1 : P.nTri > 8 ? 2 : 3;
    };
    int count[kClasses + 1] = {}, maxTri[kClasses + 1] = {};
    for (int k : which) {
        const int c = classOfP(B.prob[k]);
        count[c]++;
        maxTri[c] = std::max(maxTri[c], B.prob[k].nTri);
    }
    int dev = 0, numSMs = 152;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&numSMs, cudaDevAttrMultiProcessorCount, dev);
    const int maxCluster = in.bigCluster > 0 ? in.bigCluster : local_max_cluster();
    LocalSchedule sched[kClasses];
    for (int c = 0; c < kClasses; ++c) sched[c] = local_schedule(maxTri[c], count[c], numSMs, maxCluster);
    int start[kClasses + 2] = {};
    for (int c = 0; c <= kClasses; ++c) start[c + 1] = start[c] + count[c];
    std::vector<int> order(which.size());   // position in the class-sorted batch -> index into which
    {
        int fill[kClasses + 1];
        for (int c = 0; c <= kClasses; ++c) fill[c] = start[c];
        for (size_t i = 0; i < which.size(); ++i) order[fill[classOfP(B.prob[which[i]])]++] = static_cast<int>(i);
    }
    std::vector<LocalProblem> prob(which.size());
    for (size_t p = 0; p < which.size(); ++p) {
        prob[p] = B.prob[which[order[p]]];
        if (maxIterOverride > 0) prob[p].maxIter = maxIterOverride;
    }
    LocalBatch db;
    db.fp32Hessian = fp32;
    const size_t sizes[9] = {sizeof(LocalProblem) * prob.size(), sizeof(int) * B.ltGlobal.size(),
                             sizeof(int) * B.ltCorner.size(), sizeof(double2) * B.lvPos.size(),
                             sizeof(int) * B.lvSlot.size(), sizeof(int) * B.initTri.size(),
                             sizeof(LocalResult) * prob.size(), sizeof(int) * B.apLocal.size(),
                             sizeof(double2) * B.apPos.size()};
    const void* src[9] = {prob.data(), B.ltGlobal.data(), B.ltCorner.data(), B.lvPos.data(), B.lvSlot.data(),
                          B.initTri.data(), nullptr, B.apLocal.data(), B.apPos.data()};
    std::vector<LocalResult> out(prob.size());
    cudaError_t e = cudaSuccess;
    const bool reuse = batchId != 0 && W.uploaded == batchId;
    for (int k = 0; k < 9 && e == cudaSuccess; ++k)
        if (W.cap[k] < sizes[k] || !W.buf[k]) {
            if ((k >= 1 && k <= 5) || k >= 7) W.uploaded = 0;
            cudaFree(W.buf[k]);
            W.buf[k] = nullptr;
            W.cap[k] = 0;
            const size_t want = std::max<size_t>(sizes[k] + sizes[k] / 4, 256);
            e = cudaMalloc(&W.buf[k], want);
            if (e == cudaSuccess) W.cap[k] = want;
        }
    const bool upload = !(reuse && W.uploaded == batchId);
    for (int k = 0; k < 9 && e == cudaSuccess; ++k)
        if (k != 6 && sizes[k] > 0 && (k == 0 || upload))
            e = cudaMemcpyAsync(W.buf[k], src[k], sizes[k], cudaMemcpyHostToDevice, in.st);
    if (e == cudaSuccess) W.uploaded = batchId;
    for (int c = 0; c <= kClasses && e == cudaSuccess; ++c)
        if (!W.ev[c]) e = cudaEventCreateWithFlags(&W.ev[c], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventRecord(W.ev[kClasses], in.st);   // uploads done
    if (e == cudaSuccess) {
        db.ltGlobal = static_cast<const int*>(W.buf[1]);
        db.ltCorner = static_cast<const int*>(W.buf[2]);
        db.lvPos = static_cast<const double2*>(W.buf[3]);
        db.lvSlot = static_cast<const int*>(W.buf[4]);
        db.initTri = static_cast<const int*>(W.buf[5]);
        db.apLocal = static_cast<const int*>(W.buf[7]);
        db.apPos = static_cast<const double2*>(W.buf[8]);
        if (count[kClasses]) {
            // the bijective problems: one launch of their own kernel on the
            // fifth stream
            if (!W.aux[kClasses]) e = cudaStreamCreateWithFlags(&W.aux[kClasses], cudaStreamNonBlocking);
            if (e == cudaSuccess && !W.ev[kClasses + 1])
                e = cudaEventCreateWithFlags(&W.ev[kClasses + 1], cudaEventDisableTiming);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(W.aux[kClasses], W.ev[kClasses], 0);
            LocalBatch cb = db;
            cb.prob = static_cast<const LocalProblem*>(W.buf[0]) + start[kClasses];
            cb.out = static_cast<LocalResult*>(W.buf[6]) + start[kClasses];
            cb.nProb = count[kClasses];
            if (e == cudaSuccess) e = launch_local_newton_bij(*in.dm, in.surfaceArea, cb, W.aux[kClasses]);
            if (e == cudaSuccess) e = cudaEventRecord(W.ev[kClasses + 1], W.aux[kClasses]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(in.st, W.ev[kClasses + 1], 0);
        }
        for (int c = 0; c < kClasses && e == cudaSuccess; ++c) {
            if (!count[c]) continue;
            if (!W.aux[c]) {
                // the largest problems (the long pole, on clusters when few)
                // on the highest-priority stream, so that the block scheduler
                // places them before the many small problems' blocks
                int least = 0, greatest = 0;
                cudaDeviceGetStreamPriorityRange(&least, &greatest);
                e = cudaStreamCreateWithPriority(&W.aux[c], cudaStreamNonBlocking, c == 0 ? greatest : least);
            }
            if (e == cudaSuccess) e = cudaStreamWaitEvent(W.aux[c], W.ev[kClasses], 0);
            // clustered large problems (few, latency-bound: the long pole)
            // run alone; the other classes start after them instead of
            // taking their SMs' FP64 pipes
            if (e == cudaSuccess && c > 0 && count[0] && sched[0].cluster > 1)
                e = cudaStreamWaitEvent(W.aux[c], W.ev[0], 0);
            LocalBatch cb = db;
            cb.prob = static_cast<const LocalProblem*>(W.buf[0]) + start[c];
            cb.out = static_cast<LocalResult*>(W.buf[6]) + start[c];
            cb.nProb = count[c];
            if (e == cudaSuccess && autotune) {
                // (a one-iteration probe pass is its own workload)
                const std::array<int, 4> key = {dev, c + (maxIterOverride == 1 ? kClasses : 0), log2_bucket(count[c]),
                                                log2_bucket(maxTri[c])};
                bool known = false;
                {
                    std::lock_guard<std::mutex> lock(g_schedMu);
                    auto it = g_schedTable.find(key);
                    if (it != g_schedTable.end()) {
                        sched[c] = it->second.best;
                        known = true;
                    }
                }
                if (!known) {
                    ScheduleRecord rec{dev, key[1], key[2], key[3], sched[c], sched[c], 0.f, 0.f, 0};
                    cudaEvent_t a = nullptr, z = nullptr;
                    e = cudaEventCreate(&a);
                    if (e == cudaSuccess) e = cudaEventCreate(&z);
                    const auto cands = schedule_candidates(c, maxTri[c], maxCluster);
                    float bestMs = -1.f;
                    for (int pass = 0; pass < 2 && e == cudaSuccess; ++pass)   // pass 0 warms every candidate up
                        for (const LocalSchedule& cs : cands) {
                            if (e != cudaSuccess) break;
                            e = cudaEventRecord(a, W.aux[c]);
                            if (e == cudaSuccess) e = launch_local_newton(*in.dm, in.surfaceArea, cb, cs, W.aux[c]);
                            if (e == cudaSuccess) e = cudaEventRecord(z, W.aux[c]);
                            if (e == cudaSuccess) e = cudaEventSynchronize(z);
                            float ms = 0.f;
                            if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, a, z);
                            if (e != cudaSuccess || pass == 0) continue;
                            if (cs.tpp == rec.rule.tpp && cs.cluster == rec.rule.cluster && cs.block == rec.rule.block)
                                rec.ruleMs = ms;
                            if (bestMs < 0.f || ms < bestMs) {
                                bestMs = ms;
                                rec.best = cs;
                            }
                        }
                    if (a) cudaEventDestroy(a);
                    if (z) cudaEventDestroy(z);
                    if (e == cudaSuccess) {
                        rec.bestMs = bestMs;
                        rec.candidates = static_cast<int>(cands.size());
                        sched[c] = rec.best;
                        std::lock_guard<std::mutex> lock(g_schedMu);
                        g_schedTable[key] = rec;
                    }
                }
            }
            if (e == cudaSuccess) e = launch_local_newton(*in.dm, in.surfaceArea, cb, sched[c], W.aux[c]);
            if (e == cudaSuccess) e = cudaEventRecord(W.ev[c], W.aux[c]);
            if (e == cudaSuccess) e = cudaStreamWaitEvent(in.st, W.ev[c], 0);
        }
        if (e == cudaSuccess) e = cudaMemcpyAsync(out.data(), W.buf[6], sizes[6], cudaMemcpyDeviceToHost, in.st);
        if (e == cudaSuccess) e = cudaStreamSynchronize(in.st);
    }
    if (e != cudaSuccess) {
        cudaStreamSynchronize(in.st);
        for (auto s : W.aux)
            if (s) cudaStreamSynchronize(s);
        W.uploaded = 0;
        if (err) *err = std::string("topology query: ") + cudaGetErrorString(e);
        return OC_ERR_CUDA;
    }
    for (size_t p = 0; p < which.size(); ++p) res[which[order[p]]] = out[p];
    return OC_OK;
}

// Excess of the candidate's local energy over its isometric minimum, in the
// global energy's units: (initE - 4) localArea / surfaceArea.
double excess_global(const LocalProblem& P, const LocalResult& r, double surfaceArea)
{
    return (r.initE - 4.0) * P.localArea / surfaceArea;
}

// The 32 features of one local problem, from its header and the raw
// quantities of its start and first Newton step.
void topo_features(const LocalProblem& P, const LocalResult& r, int opType, const TopoQueryIn& in, float* f)
{
    for (int k = 0; k < kTopoNumFeatures; ++k) f[k] = 0.0f;
    const double E0 = std::max(r.raw[0], 4.0 + 1e-12), E1 = std::max(r.raw[4], 4.0 + 1e-12);
    const double gsq0 = r.raw[1], A = P.localArea;
    auto lg = [](double x) { return std::log10(x + 1e-30) / 10.0; };
    f[0] = opType == kOpBoundarySplit;
    f[1] = opType == kOpInteriorSplit;
    f[2] = opType == kOpMerge;
    f[3] = static_cast<float>(std::log1p(static_cast<double>(P.nTri)) / 3.0);
    f[4] = static_cast<float>(P.nFree / 4.0);
    f[5] = static_cast<float>(std::log(E0 / 4.0));
    f[6] = static_cast<float>(std::log(E1 / 4.0));
    f[7] = static_cast<float>(std::max(-1.0, std::min(1.0, (E0 - E1) / std::max(E0 - 4.0, 1e-12))));
    f[8] = static_cast<float>(r.raw[2]);
    f[9] = static_cast<float>(std::min(r.raw[3], 20.0) / 20.0);
    f[10] = static_cast<float>(lg(gsq0 * A / (E0 * E0)));
    f[11] = static_cast<float>(std::log(std::max(r.raw[5], 1e-30)));
    f[12] = static_cast<float>(std::log(std::max(r.raw[6], 1e-30)));
    f[13] = static_cast<float>(r.raw[7]);
    f[14] = static_cast<float>(std::sqrt(std::max(r.raw[8] - r.raw[7] * r.raw[7], 0.0)));
    f[15] = static_cast<float>(r.raw[12] / P.nTri);
    f[16] = static_cast<float>(r.raw[13] / P.nTri);
    f[17] = static_cast<float>(r.raw[14] / E0);
    f[18] = static_cast<float>(r.raw[15] / E0);
    f[19] = static_cast<float>(lg(r.raw[9] * A / (E0 * E0)));
    f[20] = static_cast<float>(lg(r.raw[10] * A / (E0 * E0)));
    f[21] = static_cast<float>(r.raw[11] / std::sqrt(r.raw[9] * r.raw[10] + 1e-300));
    f[22] = static_cast<float>(std::log(A / P.nTri * in.nF / in.surfaceArea));
    // start and first-step quantities only, so a one-step probe and a full
    // solve give the same row: converged at the start, stop test met at step 1
    f[23] = gsq0 < P.targetGRes ? 1.0f : 0.0f;
    f[24] = (r.raw[2] > 1.0e-3 && (E0 - E1) / E0 < 1.0e-6 * r.raw[2]) ? 1.0f : 0.0f;
    f[25] = static_cast<float>(std::log(std::max(r.initE, 4.0 + 1e-12) / 4.0));
    f[26] = static_cast<float>(std::max(-1.0, std::min(1.0, (r.initE - E1) / std::max(r.initE - 4.0, 1e-12))));
    for (int k = 0; k < kTopoNumFeatures; ++k)
        if (!std::isfinite(f[k])) f[k] = 0.0f;
}

// TriMesh::cohEIndex as computeFeatures builds it (TriMesh.cpp:448-455):
// (c0, c1) -> row, (c3, c2) -> -row - 1, rows without a -1 entry only
std::vector<std::pair<std::pair<int, int>, int>> coh_index(const std::vector<int>& cohE)
{
    std::vector<std::pair<std::pair<int, int>, int>> idx;
    for (size_t i = 0; i < cohE.size() / 4; ++i) {
        const int* c = &cohE[4 * i];
        if (std::min(std::min(c[0], c[1]), std::min(c[2], c[3])) < 0) continue;
        idx.push_back({{c[0], c[1]}, static_cast<int>(i)});
        idx.push_back({{c[3], c[2]}, -static_cast<int>(i) - 1});
    }
    return idx;
}

int* coh_find(std::vector<std::pair<std::pair<int, int>, int>>& idx, int a, int b)
{
    for (auto it = idx.rbegin(); it != idx.rend(); ++it)   // a std::map keeps the last assignment
        if (it->first.first == a && it->first.second == b) return &it->second;
    return nullptr;
}

void coh_set(std::vector<std::pair<std::pair<int, int>, int>>& idx, int a, int b, int v)
{
    if (int* p = coh_find(idx, a, b)) *p = v;
    else idx.push_back({{a, b}, v});
}

void coh_erase(std::vector<std::pair<std::pair<int, int>, int>>& idx, int a, int b)
{
    idx.erase(std::remove_if(idx.begin(), idx.end(),
                             [&](const std::pair<std::pair<int, int>, int>& e) {
                                 return e.first.first == a && e.first.second == b;
                             }),
              idx.end());
}

// TriMesh::isBoundaryVert(vI, vNb, tris, boundaryEdge, toBound) with its
// boundaryEdge output
bool walk_edge(const Topo& T, int vI, int vNb, bool toBound, std::vector<int>& tris, int bEdge[2])
{
    tris.clear();
    int f = toBound ? T.edge_tri(vNb, vI) : T.edge_tri(vI, vNb);
    if (f < 0) {
        bEdge[0] = toBound ? vI : vNb;
        bEdge[1] = toBound ? vNb : vI;
        return true;
    }
    int vNew = vNb;
    for (int guard = 0; guard <= T.nF; ++guard) {
        tris.push_back(f);
        vNew = T.third(f, vI, vNew);
        if (vNew == vNb) return false;
        f = toBound ? T.edge_tri(vNew, vI) : T.edge_tri(vI, vNew);
        if (f < 0) {
            bEdge[0] = toBound ? vI : vNew;
            bEdge[1] = toBound ? vNew : vI;
            return true;
        }
    }
    return false;
}

void replace_in(std::vector<int>& F, const std::vector<int>& tris, int from, int to)
{
    for (int t : tris)
        for (int k = 0; k < 3; ++k)
            if (F[3 * (size_t)t + k] == from) {
                F[3 * (size_t)t + k] = to;
                break;
            }
}

} // namespace

int topo_apply(int opType, const int* path, int pathLen, const double* pos, int posRows, std::vector<int>& F,
               std::vector<double>& Vrest, std::vector<double>& UV, std::vector<int>& cohE, std::string* err,
               int* tails, int* edit)
{
    auto bad = [&](const char* m) {
        if (err) *err = m;
        return OC_ERR_INVALID;
    };
    const int nV = static_cast<int>(Vrest.size() / 3), nF = static_cast<int>(F.size() / 3);
    if (!path || !pos) return bad("topology op: bad arguments");
    for (int i = 0; i < pathLen; ++i)
        if (path[i] < 0 || path[i] >= nV) return bad("topology op: path vertex out of range");
    Topo T;
    T.build(nV, F.data(), nF);
    auto push_vertex = [&](int copyOf, const double* uv) {
        Vrest.insert(Vrest.end(), {Vrest[3 * (size_t)copyOf], Vrest[3 * (size_t)copyOf + 1], Vrest[3 * (size_t)copyOf + 2]});
        UV.insert(UV.end(), {uv[0], uv[1]});
        return static_cast<int>(UV.size() / 2) - 1;
    };
    if (opType == kOpBoundarySplit) {
        // TriMesh::splitEdgeOnBoundary(edge, newVertPos) (TriMesh.cpp:2864-3036)
        if (pathLen != 2) return bad("boundary split: path must be an edge");
        if (T.edge_tri(path[0], path[1]) < 0 || T.edge_tri(path[1], path[0]) < 0)
            return bad("boundary split: not an interior edge");
        int vb = path[0], vi = path[1];
        bool both = false;
        if (T.bnd[path[0]]) {
            if (T.bnd[path[1]]) both = true;
        }
        else {
            if (!T.bnd[path[1]]) return bad("boundary split: the edge does not touch the boundary");
            vb = path[1];
            vi = path[0];
        }
        if (posRows != (both ? 4 : 2)) return bad("boundary split: wrong number of new positions");
        std::vector<int> sepB, sepI;
        int bEb[2] = {-1, -1}, bEi[2] = {-1, -1};
        walk_edge(T, vb, vi, true, sepB, bEb);
        if (both) walk_edge(T, vi, vb, true, sepI, bEi);
        auto idx = coh_index(cohE);
        const int nb = push_vertex(vb, pos + 2);
        if (edit) {
            edit[0] = 0;
            edit[1] = vb;
            edit[2] = both ? vi : -1;
        }
        UV[2 * (size_t)vb] = pos[0];
        UV[2 * (size_t)vb + 1] = pos[1];
        replace_in(F, sepB, vb, nb);
        const int nCE = static_cast<int>(cohE.size() / 4);
        cohE.insert(cohE.end(), {vi, nb, vi, vb});
        coh_set(idx, vi, nb, nCE);
        coh_set(idx, vb, vi, -nCE - 1);
        if (int* f = coh_find(idx, bEb[0], bEb[1])) {
            const int r = *f;
            if (r >= 0) cohE[4 * (size_t)r] = nb;
            else cohE[4 * (size_t)(-r - 1) + 3] = nb;
            coh_erase(idx, bEb[0], bEb[1]);
            coh_set(idx, nb, bEb[1], r);
        }
        if (both) {
            const int ni = push_vertex(vi, pos + 4);
            UV[2 * (size_t)vi] = pos[6];
            UV[2 * (size_t)vi + 1] = pos[7];
            replace_in(F, sepI, vi, ni);
            cohE[4 * (size_t)nCE + 2] = ni;
            coh_erase(idx, vb, vi);
            coh_set(idx, vb, ni, -nCE - 1);
            if (int* f = coh_find(idx, bEi[0], bEi[1])) {
                const int r = *f;
                if (r >= 0) cohE[4 * (size_t)r] = ni;
                else cohE[4 * (size_t)(-r - 1) + 3] = ni;
            }
        }
        if (tails) {   // the interior end is the new tail, none for a cut-through
            tails[0] = both ? -1 : vi;
            tails[1] = tails[2] = -1;
        }
        return OC_OK;
    }
    if (opType == kOpInteriorSplit) {
        // TriMesh::cutPath(path, true, 1, newVertPos), interior branch (TriMesh.cpp:1449-1500)
        if (pathLen != 3 || posRows != 2) return bad("interior split: path of 3 vertices and 2 positions expected");
        const int vI = path[1];
        std::vector<int> left;
        int vNew = path[0];
        for (int guard = 0;; ++guard) {
            const int f = T.edge_tri(vI, vNew);
            if (f < 0 || guard > nF) return bad("interior split: not a valid path");
            left.push_back(f);
            vNew = T.third(f, vI, vNew);
            if (vNew == path[2]) break;
            if (vNew == path[0]) return bad("interior split: not a valid path");
        }
        const int nn = push_vertex(vI, pos);
        if (edit) {
            edit[0] = 0;
            edit[1] = vI;
            edit[2] = -1;
        }
        UV[2 * (size_t)vI] = pos[2];
        UV[2 * (size_t)vI + 1] = pos[3];
        replace_in(F, left, vI, nn);
        cohE.insert(cohE.end(), {nn, path[0], vI, path[0]});
        cohE.insert(cohE.end(), {path[2], nn, path[2], vI});
        if (tails) {
            tails[0] = -1;
            tails[1] = path[0];
            tails[2] = path[2];
        }
        return OC_OK;
    }
    if (opType == kOpMerge) {
        // TriMesh::mergeBoundaryEdges((p0, p1), (p1, p2), newVertPos.row(0)) (TriMesh.cpp:3038-3180)
        if (pathLen != 3 || posRows < 1) return bad("merge: path of 3 vertices expected");
        const int a = path[0], b = path[2];
        if (T.edge_tri(path[1], path[0]) >= 0 || T.edge_tri(path[2], path[1]) >= 0)
            return bad("merge: the edges are not boundary edges");
        auto idx = coh_index(cohE);
        int* ci = coh_find(idx, path[0], path[1]);
        if (!ci) return bad("merge: the edge is not a cohesive edge");
        const int cRow = *ci;
        if (edit) {
            edit[0] = 1;
            edit[1] = a;
            edit[2] = b;
        }
        UV[2 * (size_t)a] = pos[0];
        UV[2 * (size_t)a + 1] = pos[1];
        const int back = nV - 1;
        if (b < back) {
            for (int k = 0; k < 3; ++k) Vrest[3 * (size_t)b + k] = Vrest[3 * (size_t)back + k];
            UV[2 * (size_t)b] = UV[2 * (size_t)back];
            UV[2 * (size_t)b + 1] = UV[2 * (size_t)back + 1];
        }
        Vrest.resize(3 * (size_t)back);
        UV.resize(2 * (size_t)back);
        for (int t = 0; t < nF; ++t)
            for (int k = 0; k < 3; ++k)
                if (F[3 * (size_t)t + k] == b) {
                    F[3 * (size_t)t + k] = a;
                    break;
                }
        if (b < back)
            for (size_t i = 0; i < F.size(); ++i)
                if (F[i] == back) F[i] = b;
        const int nC = static_cast<int>(cohE.size() / 4), cBack = nC - 1;
        const int row = cRow >= 0 ? cRow : -cRow - 1;
        if (row < cBack)
            for (int k = 0; k < 4; ++k) cohE[4 * (size_t)row + k] = cohE[4 * (size_t)cBack + k];
        cohE.resize(4 * (size_t)cBack);
        for (int& c : cohE)
            if (c == b) c = a;
        if (b < back)
            for (int& c : cohE)
                if (c == back) c = b;
        // the merged vertex is the new tail (where it was the last vertex it
        // now sits in b's slot; the reference keeps its old, removed index)
        if (tails) tails[0] = (a == back && b < back) ? b : a;
        // close up a diamond that became whole
        for (size_t i = 0; i < cohE.size() / 4; ++i) {
            int* c = &cohE[4 * i];
            if (c[0] == c[2] && c[1] == c[3]) {
                const size_t last = cohE.size() / 4 - 1;
                if (i < last)
                    for (int k = 0; k < 4; ++k) c[k] = cohE[4 * last + k];
                cohE.resize(4 * last);
                if (tails) tails[0] = -1;
                break;
            }
        }
        return OC_OK;
    }
    return bad("topology op: unknown operation");
}

// The cut graph of a surface of genus >= 1 (igl::cut_to_disk as vendored in
// src/Utils/cut_to_disk.cpp), as the reference's initialisation uses it:
// 1. edges numbered in (min, max) vertex order; faces peeled from each not
//    yet deleted face outwards, a face deleted through an interior edge with
//    exactly one deleted neighbour (a breadth-first queue of such edges);
// 2. degree-1 vertices of the remaining edge graph pruned repeatedly (a
//    queue seeded with the vertices in index order);
// 3. the remaining edges walked into cycles (a walk meeting its own vertex:
//    the loop from that vertex, closed) or, after a dead end and a walk the
//    other way from the reversed list, chains.  The vertex-position map of
//    the first walk is kept across the reversal, as in the source.
// cuts: vertex lists (a closed loop repeats its first vertex).
void topo_cut_to_disk(const int* F, int nF, std::vector<std::vector<int>>& cuts)
{
    cuts.clear();
    if (nF <= 0) return;
    // edges in (min, max) order; faces of each edge in face-corner order
    std::vector<std::pair<long long, int>> he(3 * (size_t)nF);   // (key, corner)
    for (int i = 0; i < nF; ++i)
        for (int j = 0; j < 3; ++j) {
            const long long a = F[3 * (size_t)i + j], b = F[3 * (size_t)i + (j + 1) % 3];
            he[3 * (size_t)i + j] = {(std::min(a, b) << 32) | std::max(a, b), 3 * i + j};
        }
    std::sort(he.begin(), he.end());
    std::vector<int> evA, evB, ef0, ef1, fe(3 * (size_t)nF);
    std::vector<char> bndE;
    for (size_t k = 0; k < he.size();) {
        size_t l = k;
        while (l < he.size() && he[l].first == he[k].first) ++l;
        const int e = static_cast<int>(evA.size());
        evA.push_back(static_cast<int>(he[k].first >> 32));
        evB.push_back(static_cast<int>(he[k].first & 0xffffffffLL));
        ef0.push_back(he[k].second / 3);
        ef1.push_back(l - k > 1 ? he[k + 1].second / 3 : -1);
        bndE.push_back(l - k == 1);
        for (size_t t = k; t < l; ++t) fe[he[t].second] = e;
        k = l;
    }
    const int nE = static_cast<int>(evA.size());
    std::vector<char> delF(nF, 0), delE(nE, 0);
    auto nDel = [&](int e) { return delF[ef0[e]] + delF[ef1[e]]; };
    std::deque<int> q;
    for (int face = 0; face < nF; ++face) {
        if (delF[face]) continue;
        delF[face] = 1;
        for (int j = 0; j < 3; ++j) {
            const int e = fe[3 * (size_t)face + j];
            if (!bndE[e] && nDel(e) == 1) q.push_back(e);
        }
        while (!q.empty()) {
            const int e = q.front();
            q.pop_front();
            int todel = nF;
            if (!delF[ef0[e]]) todel = ef0[e];
            if (!delF[ef1[e]]) todel = ef1[e];
            if (todel == nF) continue;
            delE[e] = 1;
            delF[todel] = 1;
            for (int j = 0; j < 3; ++j) {
                const int e2 = fe[3 * (size_t)todel + j];
                if (!bndE[e2] && nDel(e2) == 1) q.push_back(e2);
            }
        }
    }
    // prune the spines
    std::vector<int> left;
    for (int e = 0; e < nE; ++e)
        if (!delE[e]) left.push_back(e);
    int nV = 0;
    for (long long i = 0; i < 3LL * nF; ++i) nV = std::max(nV, F[i] + 1);
    std::vector<std::vector<int>> vertEdges(nV);
    for (int e : left) {
        vertEdges[evA[e]].push_back(e);
        vertEdges[evB[e]].push_back(e);
    }
    std::vector<int> nbs(nV);
    for (int v = 0; v < nV; ++v) nbs[v] = static_cast<int>(vertEdges[v].size());
    std::fill(delE.begin(), delE.end(), 0);
    for (int v = 0; v < nV; ++v)
        if (vertEdges[v].size() == 1) q.push_back(v);
    while (!q.empty()) {
        const int v = q.front();
        q.pop_front();
        for (int e : vertEdges[v]) {
            if (delE[e]) continue;
            delE[e] = 1;
            for (int w : {evA[e], evB[e]})
                if (--nbs[w] == 1) q.push_back(w);
        }
    }
    std::vector<int> loop;
    for (int e : left)
        if (!delE[e]) loop.push_back(e);
    if (loop.empty()) return;
    std::vector<std::vector<int>> loopVE(nV);
    for (int e : loop) {
        loopVE[evA[e]].push_back(e);
        loopVE[evB[e]].push_back(e);
    }
    std::vector<char> used(nE, 0);
    std::vector<int> verts, edges;
    std::unordered_map<int, int> pos;
    auto walk = [&](int cur, int cure) {   // true when a cycle closes
        while (cur != -1) {
            int nxt = -1, nxe = -1;
            for (int c : loopVE[cur])
                if (!used[c] && c != cure) {
                    nxt = cur == evA[c] ? evB[c] : evA[c];
                    nxe = c;
                    break;
                }
            if (nxt != -1) {
                auto it = pos.find(nxt);
                if (it != pos.end()) {
                    const int i0 = it->second;
                    std::vector<int> cut(verts.begin() + i0, verts.end());
                    cut.push_back(nxt);
                    cuts.push_back(std::move(cut));
                    for (size_t i = i0; i < edges.size(); ++i) used[edges[i]] = 1;
                    used[nxe] = 1;
                    return true;
                }
                pos[nxt] = static_cast<int>(verts.size());
                verts.push_back(nxt);
                edges.push_back(nxe);
            }
            cur = nxt;
            cure = nxe;
        }
        return false;
    };
    for (int e : loop) {
        while (!used[e]) {
            verts = {evA[e], evB[e]};
            edges = {e};
            pos.clear();
            pos[verts[0]] = 0;
            pos[verts[1]] = 1;
            if (walk(evB[e], e)) continue;
            std::reverse(verts.begin(), verts.end());
            std::reverse(edges.begin(), edges.end());
            if (walk(verts.back(), edges.back())) continue;
            cuts.push_back(verts);
            for (int x : edges) used[x] = 1;
        }
    }
}

// TriMesh::cutPath(path, makeCoh = true) (TriMesh.cpp:1393-1517) as the
// initial cutting of a genus >= 1 mesh calls it (main.cpp:1397-1484): from a
// boundary end, every interior edge of the path split on the boundary in
// turn (cut through where both ends are on the boundary); for an interior
// path, the interior cut of its first three vertices, then its remaining
// edges split on the boundary.  Each operation is topo_apply on the faces
// around the path vertices only (global vertex ids): those faces hold every
// half-edge the operation reads (interior edge, boundary vertex, the walk
// around a vertex), so a long path costs the faces it touches, not a
// rebuild of the whole mesh per edge.  made: edges split on the boundary.
int topo_cut_path(const int* path, int pathLen, std::vector<int>& F, std::vector<double>& Vrest,
                  std::vector<double>& UV, std::vector<int>& cohE, int& made, std::string* err)
{
    made = 0;
    const int nF = static_cast<int>(F.size() / 3);
    std::vector<std::vector<int>> inc(Vrest.size() / 3);   // faces around each vertex
    for (int t = 0; t < nF; ++t)
        for (int k = 0; k < 3; ++k) inc[F[3 * (size_t)t + k]].push_back(t);
    std::vector<int> nxt, prv;
    auto around = [&](int v) {
        nxt.clear();
        prv.clear();
        for (int t : inc[v]) {
            const int* r = &F[3 * (size_t)t];
            const int k = r[0] == v ? 0 : (r[1] == v ? 1 : 2);
            nxt.push_back(r[(k + 1) % 3]);
            prv.push_back(r[(k + 2) % 3]);
        }
    };
    auto boundary = [&](int v) {   // TriMesh::isBoundaryVert: the fan does not close
        around(v);
        std::sort(nxt.begin(), nxt.end());
        std::sort(prv.begin(), prv.end());
        return nxt != prv;
    };
    auto interior_edge = [&](int a, int b) {
        around(a);
        return std::find(nxt.begin(), nxt.end(), b) != nxt.end() && std::find(prv.begin(), prv.end(), b) != prv.end();
    };
    auto apply_local = [&](int op, const int* p, int pl, const double* pos, int rows) -> int {
        std::vector<int> faces;
        for (int i = 0; i < pl; ++i) faces.insert(faces.end(), inc[p[i]].begin(), inc[p[i]].end());
        std::sort(faces.begin(), faces.end());
        faces.erase(std::unique(faces.begin(), faces.end()), faces.end());
        std::vector<int> Fs(3 * faces.size());
        for (size_t i = 0; i < faces.size(); ++i)
            for (int k = 0; k < 3; ++k) Fs[3 * i + k] = F[3 * (size_t)faces[i] + k];
        const int rc = topo_apply(op, p, pl, pos, rows, Fs, Vrest, UV, cohE, err);
        if (rc) return rc;
        inc.resize(Vrest.size() / 3);
        for (size_t i = 0; i < faces.size(); ++i) {
            const int t = faces[i];
            for (int k = 0; k < 3; ++k) {
                const int o = F[3 * (size_t)t + k], n = Fs[3 * i + k];
                if (o == n) continue;
                auto& lo = inc[o];
                lo.erase(std::find(lo.begin(), lo.end(), t));
                inc[n].push_back(t);
                F[3 * (size_t)t + k] = n;
            }
        }
        return OC_OK;
    };
    auto split_edges = [&](const int* vs, int n) -> int {
        for (int i = 0; i + 1 < n; ++i) {
            const int ab[2] = {vs[i], vs[i + 1]};
            if (!interior_edge(ab[0], ab[1])) continue;
            const int rows = (boundary(ab[0]) && boundary(ab[1])) ? 4 : 2;
            double pos[8];
            for (int r = 0; r < rows; ++r) {
                pos[2 * r] = UV[2 * (size_t)ab[0]];
                pos[2 * r + 1] = UV[2 * (size_t)ab[0] + 1];
            }
            const int rc = apply_local(kOpBoundarySplit, ab, 2, pos, rows);
            if (rc) return rc;
            ++made;
        }
        return OC_OK;
    };
    const int nV = static_cast<int>(Vrest.size() / 3);
    if (pathLen < 2 || !path) {
        if (err) *err = "cut path: fewer than two vertices";
        return OC_ERR_INVALID;
    }
    for (int i = 0; i < pathLen; ++i)
        if (path[i] < 0 || path[i] >= nV) {
            if (err) *err = "cut path: vertex out of range";
            return OC_ERR_INVALID;
        }
    std::vector<int> pth(path, path + pathLen);
    if (boundary(pth.front()) || boundary(pth.back())) {
        if (!boundary(pth.front())) std::reverse(pth.begin(), pth.end());   // start the cut from the boundary
        return split_edges(pth.data(), pathLen);
    }
    if (pathLen < 3) {
        if (err) *err = "cut path: an interior cut path needs three vertices";
        return OC_ERR_INVALID;
    }
    const double pos[4] = {UV[2 * (size_t)pth[1]], UV[2 * (size_t)pth[1] + 1], UV[2 * (size_t)pth[1]],
                           UV[2 * (size_t)pth[1] + 1]};
    const int rc = apply_local(kOpInteriorSplit, pth.data(), 3, pos, 2);
    if (rc) return rc;
    return split_edges(pth.data() + 2, pathLen - 2);
}

int topo_split_candidates(int nV, const int* F, int nF, const double* divGrad, bool interior, double filterExp,
                          std::vector<int>& cands, int& pool)
{
    Topo T;
    T.build(nV, F, nF);
    std::vector<std::pair<double, int>> keyed;
    for (int v = 0; v < nV; ++v) {
        if (T.degree(v) <= 2) continue;
        if (!interior) {
            if (T.bnd[v]) keyed.push_back({-divGrad[v] / 1.0, v});
        }
        else if (!T.bnd[v]) {
            bool toBound = false;
            for (int p = T.nbPtr[v]; p < T.nbPtr[v + 1] && !toBound; ++p) toBound = T.bnd[T.nb[p]];
            if (!toBound) keyed.push_back({-divGrad[v] / 1.0, v});
        }
    }
    cands = filter_candidates(keyed, interior ? filterExp : 0.8, pool);
    return OC_OK;
}

namespace {

// per-thread scratch and problem batch of the parallel problem assembly
struct BuildCtx {
    std::vector<int> tris, tris1, tris2, vmap;
    std::vector<char> triMark, sideMarkB, sideMarkI;
    LocalMesh L;
    Batch B;
};

// appends src's problems to dst, rebasing their offsets
void append_batch(Batch& dst, const Batch& src)
{
    const int triBase = static_cast<int>(dst.ltGlobal.size()), vertBase = static_cast<int>(dst.lvPos.size()),
              initBase = static_cast<int>(dst.initTri.size());
    const int airBase = static_cast<int>(dst.apLocal.size());
    for (LocalProblem P : src.prob) {
        P.triOff += triBase;
        P.vertOff += vertBase;
        P.initOff += initBase;
        P.airOff += airBase;
        dst.prob.push_back(P);
    }
    dst.apLocal.insert(dst.apLocal.end(), src.apLocal.begin(), src.apLocal.end());
    dst.apPos.insert(dst.apPos.end(), src.apPos.begin(), src.apPos.end());
    dst.ltGlobal.insert(dst.ltGlobal.end(), src.ltGlobal.begin(), src.ltGlobal.end());
    dst.ltCorner.insert(dst.ltCorner.end(), src.ltCorner.begin(), src.ltCorner.end());
    dst.lvPos.insert(dst.lvPos.end(), src.lvPos.begin(), src.lvPos.end());
    dst.lvSlot.insert(dst.lvSlot.end(), src.lvSlot.begin(), src.lvSlot.end());
    dst.initTri.insert(dst.initTri.end(), src.initTri.begin(), src.initTri.end());
    dst.tag.insert(dst.tag.end(), src.tag.begin(), src.tag.end());
}

// the threads' contexts, kept across queries of one mesh size (their
// marker arrays are left all clear and their vertex maps are reset by the
// next local-mesh build, so they are reused without clearing)
struct BuildCache {
    std::vector<std::unique_ptr<BuildCtx>> ctx;
    int nV = -1, nF = -1;
};

// Runs body(ctx, item) for items [0, n) on up to 16 host threads, each a
// contiguous range, and appends the threads' batches to B in item order
// (the same problems in the same order as one thread would build).
template <typename Body>
void build_parallel(const TopoQueryIn& in, size_t n, Batch& B, const Body& body)
{
    BuildCache local;
    BuildCache* cache = &local;
    if (in.ws) {
        if (!in.ws->host) in.ws->host = std::make_shared<BuildCache>();
        cache = static_cast<BuildCache*>(in.ws->host.get());
    }
    if (cache->nV != in.nV || cache->nF != in.nF) {
        cache->ctx.clear();
        cache->nV = in.nV;
        cache->nF = in.nF;
    }
    const int nt = static_cast<int>(std::max<size_t>(1, std::min<size_t>(HostPool::threads(), n / 16 + 1)));
    if (static_cast<int>(cache->ctx.size()) < nt) cache->ctx.resize(nt);
    auto work = [&](int t) {
        std::unique_ptr<BuildCtx>& X = cache->ctx[t];
        if (!X) {
            X = std::make_unique<BuildCtx>();
            X->vmap.assign(in.nV, -1);
            X->triMark.assign(in.nF, 0);
            X->sideMarkB.assign(in.nF, 0);
            X->sideMarkI.assign(in.nF, 0);
            X->L.map = &X->vmap;
        }
        X->B = Batch{};
        const size_t a = n * t / nt, b = n * (t + 1) / nt;
        for (size_t i = a; i < b; ++i) body(*X, i);
    };
    host_run_tasks(nt, [&](size_t t) { work(static_cast<int>(t)); });
    for (int t = 0; t < nt; ++t) append_batch(B, cache->ctx[t]->B);
}

} // namespace

namespace {

// Candidates and local problems of one operation (the enumeration of
// querySplit / queryMerge) appended to B; candidatePool as the reference
// reports it.
int build_op(const TopoQueryIn& in, const Topo& T, int opType, double filterExp, std::vector<TopoCandidate>& out,
             int& candidatePool, Batch& B, std::string* err, const AirSrc* air)
{
    const double R = in.virtualRadius;
    std::vector<int> tris, tris1, tris2;
    std::vector<int> vmap(in.nV, -1);
    std::vector<char> triMark(in.nF, 0), sideMarkB(in.nF, 0), sideMarkI(in.nF, 0);
    LocalMesh L;
    L.map = &vmap;

    if (opType == kOpBoundarySplit || opType == kOpInteriorSplit) {
        if (!in.divGrad && !in.candVerts) {
            if (err) *err = "topology query: no split filter";
            return OC_ERR_INVALID;
        }
        std::vector<std::pair<double, int>> keyed;
        for (int v = 0; v < in.nV && !in.candVerts; ++v) {
            if (T.degree(v) <= 2) continue;   // cannot be split further
            if (opType == kOpBoundarySplit) {
                if (T.bnd[v]) keyed.push_back({-in.divGrad[v] / 1.0, v});   // vertWeight = 1
            }
            else if (!T.bnd[v]) {
                bool toBound = false;
                for (int p = T.nbPtr[v]; p < T.nbPtr[v + 1] && !toBound; ++p) toBound = T.bnd[T.nb[p]];
                if (!toBound) keyed.push_back({-in.divGrad[v] / 1.0, v});
            }
        }
        std::vector<int> cands;
        if (in.candVerts) {
            // propagation: the fracture tails themselves, evaluated as boundary
            // splits (querySplit sets splitInterior = false, TriMesh.cpp:650-665;
            // computeLocalLDec's boundary branch needs a boundary vertex)
            for (int i = 0; i < in.nCandVerts; ++i)
                if (in.candVerts[i] >= 0 && in.candVerts[i] < in.nV && T.bnd[in.candVerts[i]])
                    cands.push_back(in.candVerts[i]);
            candidatePool = static_cast<int>(cands.size());
        }
        else {
            cands = filter_candidates(keyed, opType == kOpBoundarySplit ? 0.8 : filterExp, candidatePool);
        }
        out.resize(cands.size());
        for (size_t ci = 0; ci < cands.size(); ++ci) {
            TopoCandidate& C = out[ci];
            C.EwDec = -DBL_MAX;
            C.ec0 = C.ec1 = DBL_MAX;
            C.path = opType == kOpBoundarySplit ? std::vector<int>{0, 0} : std::vector<int>{0, 0, 0};
        }
        if (opType == kOpBoundarySplit) {
            // computeLocalLDec boundary branch (TriMesh.cpp:2168-2199): every
            // interior edge at each candidate, queryLocalEdDec_bSplit
            // (:2796-2862); one work item per edge
            std::vector<std::pair<int, int>> items;   // (candidate, neighbour)
            for (size_t ci = 0; ci < cands.size(); ++ci) {
                if ((int)(ci % in.shardCount) != in.shardRank) continue;   // another shard's candidate
                const int vI = cands[ci];
                for (int p = T.nbPtr[vI]; p < T.nbPtr[vI + 1]; ++p) {
                    const int nbVI = T.nb[p];
                    if (T.edge_tri(vI, nbVI) < 0 || T.edge_tri(nbVI, vI) < 0) continue;
                    items.push_back({static_cast<int>(ci), nbVI});
                }
            }
            build_parallel(in, items.size(), B, [&](BuildCtx& X, size_t it) {
                auto& tris = X.tris;
                auto& tris1 = X.tris1;
                auto& tris2 = X.tris2;
                auto& triMark = X.triMark;
                auto& sideMarkB = X.sideMarkB;
                auto& sideMarkI = X.sideMarkI;
                auto& L = X.L;
                Batch& B = X.B;
                const size_t ci = static_cast<size_t>(items[it].first);
                const int vI = cands[ci], nbVI = items[it].second;
                const int vb = vI, vi = nbVI;
                const bool cutThrough = T.bnd[vi] != 0;
                T.walk(vb, vi, false, tris);
                T.walk(vb, vi, true, tris1);
                tris.insert(tris.end(), tris1.begin(), tris1.end());
                if (cutThrough) {
                    for (int t : tris) triMark[t] = 1;
                    for (int cw = 0; cw < 2; ++cw) {
                        T.walk(vi, vb, cw != 0, tris2);
                        for (int t : tris2)
                            if (!triMark[t]) {
                                triMark[t] = 1;
                                tris.push_back(t);
                            }
                    }
                    for (int t : tris) triMark[t] = 0;
                }
                // local split (TriMesh::splitEdgeOnBoundary on the local
                // mesh, TriMesh.cpp:2864-3036): the copy of vb takes the
                // fan on the (vi -> vb) side; with cutThrough the copy of
                // vi takes vi's fan from vb towards the boundary
                L.build(T, tris);
                const int lb = L.find(vb), li = L.find(vi);
                const int nLoc = static_cast<int>(L.gv.size());
                std::vector<int> sideB, sideI;
                T.walk(vb, vi, true, sideB);
                if (cutThrough) T.walk(vi, vb, true, sideI);
                else sideI.clear();
                for (int t : sideB) sideMarkB[t] = 1;
                for (int t : sideI) sideMarkI[t] = 1;
                for (size_t k = 0; k < tris.size(); ++k) {
                    const int t = tris[k];
                    const bool inB = sideMarkB[t] != 0;
                    const bool inI = cutThrough && sideMarkI[t] != 0;
                    for (int c = 0; c < 3; ++c) {
                        int& lc = L.corner[3 * k + c];
                        if (inB && lc == lb) lc = nLoc;
                        else if (inI && lc == li) lc = nLoc + 1;
                    }
                }
                for (int t : sideB) sideMarkB[t] = 0;
                for (int t : sideI) sideMarkI[t] = 0;
                std::vector<double2> extra;
                const double2 pb = make_double2(in.UV[2 * (size_t)vb], in.UV[2 * (size_t)vb + 1]);
                const double2 pi = make_double2(in.UV[2 * (size_t)vi], in.UV[2 * (size_t)vi + 1]);
                extra.push_back(pb);
                if (cutThrough) extra.push_back(pi);
                // slots in newVertPos row order: vb, copy of vb, copy of vi, vi
                std::vector<int> slot(nLoc + extra.size(), -1);
                slot[lb] = 0;
                slot[nLoc] = 1;
                int nFree = 2, nFixed = nLoc - 1;
                if (cutThrough) {
                    slot[nLoc + 1] = 2;
                    slot[li] = 3;
                    nFree = 4;
                    nFixed = nLoc - 2;
                }
                Batch::Tag tg;
                tg.cand = static_cast<int>(ci);
                tg.a = vb;
                tg.b = vi;
                tg.se = rest_dist(in.Vrest, vI, nbVI) / R * (1.0 + 1.0) / 2.0;   // seInc
                tg.nRows = cutThrough ? 4 : 2;
                emit(B, T, in.rest, in.UV, tris, L, extra, slot, nFree, nFixed, tg);
                if (air) {
                    // separate the copies, then the air loop: vb's air fan
                    // opened at the split (TriMesh.cpp:2597-2756)
                    const LocalProblem& P = B.prob.back();
                    std::vector<double2> lp(B.lvPos.begin() + P.vertOff, B.lvPos.begin() + P.vertOff + P.nVert);
                    Topo LT;
                    LT.build(P.nVert, L.corner.data(), static_cast<int>(tris.size()));
                    const double dx = in.UV[2 * (size_t)vi] - in.UV[2 * (size_t)vb];
                    const double dy = in.UV[2 * (size_t)vi + 1] - in.UV[2 * (size_t)vb + 1];
                    const double epsSep = (dx * dx + dy * dy) * 1.0e-4;
                    separate_copies(LT, lp, L.corner, lb, nLoc, epsSep);
                    if (cutThrough) separate_copies(LT, lp, L.corner, li, nLoc + 1, epsSep);
                    for (int l = 0; l < P.nVert; ++l) B.lvPos[P.vertOff + l] = lp[l];
                    std::vector<int> rb, ri, al;
                    std::vector<double2> ap;
                    bool reject = !ring_loop(*air, vb, rb);
                    auto meshPt = [&](int airId) {
                        const int l = L.find(air->mesh_of(airId));
                        if (l < 0) reject = true;
                        al.push_back(l);
                        ap.push_back(l >= 0 ? lp[l] : d2(0.0, 0.0));
                    };
                    auto localPt = [&](int l) {
                        al.push_back(l);
                        ap.push_back(lp[l]);
                    };
                    auto airRing = [&](const std::vector<int>& rows) {
                        for (size_t r = 3; r < rows.size(); ++r) {
                            al.push_back(-1);
                            ap.push_back(air->pos(rows[r]));
                        }
                    };
                    if (!reject && !cutThrough) {
                        meshPt(rb[0]);
                        localPt(nLoc);
                        localPt(li);
                        localPt(lb);
                        meshPt(rb[2]);
                        airRing(rb);
                    }
                    else if (!reject) {
                        reject = !ring_loop(*air, vi, ri);
                        // loops sharing an air vertex are abandoned (TriMesh.cpp:2700-2706)
                        if (!reject) {
                            std::vector<int> x(rb), y(ri);
                            std::sort(x.begin(), x.end());
                            std::sort(y.begin(), y.end());
                            std::vector<int> both;
                            std::set_intersection(x.begin(), x.end(), y.begin(), y.end(), std::back_inserter(both));
                            reject = !both.empty();
                        }
                        if (!reject) {
                            meshPt(rb[0]);
                            localPt(nLoc);
                            localPt(li);
                            meshPt(ri[2]);
                            airRing(ri);
                            meshPt(ri[0]);
                            localPt(nLoc + 1);
                            localPt(lb);
                            meshPt(rb[2]);
                            airRing(rb);
                        }
                    }
                    emit_air(B, al, ap, local_air_thres(in.Vrest, in.F, tris), reject);
                }
            });
        }
        else {
            // computeLocalLDec interior branch (TriMesh.cpp:2200-2259): all
            // paths (p0, vI, p2) through two umbrella edges; one work item
            // per candidate
            build_parallel(in, cands.size(), B, [&](BuildCtx& X, size_t ci) {
                if ((int)(ci % in.shardCount) != in.shardRank) return;   // another shard's candidate
                auto& triMark = X.triMark;
                auto& L = X.L;
                Batch& B = X.B;
                const int vI = cands[ci];
                const int nbMin = T.nb[T.nbPtr[vI]];
                std::vector<int> umbrella;
                T.walk(vI, nbMin, false, umbrella);
                const int n = static_cast<int>(umbrella.size());
                auto after = [&](int t) {
                    for (int k = 0; k < 3; ++k)
                        if (T.F[3 * t + k] == vI) return T.F[3 * t + (k + 1) % 3];
                    return -1;
                };
                L.build(T, umbrella);
                const int lv = L.find(vI);
                const int nLoc = static_cast<int>(L.gv.size());
                for (int s = 0; s + 1 < n; ++s) {
                    const int p0 = after(umbrella[s]);
                    for (int e = s + 1; e < n; ++e) {
                        const int p2 = after(umbrella[e]);
                        // TriMesh::cutPath interior branch (TriMesh.cpp:1449-1475):
                        // the triangles from edge (vI, p0) round to p2 get the copy
                        std::vector<int> left;
                        int vNew = p0;
                        bool ok = true;
                        for (int guard = 0; guard <= n; ++guard) {
                            const int f = T.edge_tri(vI, vNew);
                            if (f < 0) { ok = false; break; }
                            left.push_back(f);
                            vNew = T.third(f, vI, vNew);
                            if (vNew == p2) break;
                            if (vNew == p0) { ok = false; break; }
                        }
                        if (!ok) continue;
                        LocalMesh Lc;
                        Lc.gv = L.gv;
                        Lc.corner = L.corner;
                        for (int t : left) triMark[t] = 1;
                        for (int k = 0; k < n; ++k) {
                            if (!triMark[umbrella[k]]) continue;
                            for (int c = 0; c < 3; ++c)
                                if (Lc.corner[3 * k + c] == lv) Lc.corner[3 * k + c] = nLoc;
                        }
                        for (int t : left) triMark[t] = 0;
                        std::vector<double2> extra{make_double2(in.UV[2 * (size_t)vI], in.UV[2 * (size_t)vI + 1])};
                        // newVertPos rows: the copy, then vI
                        std::vector<int> slot(nLoc + 1, -1);
                        slot[nLoc] = 0;
                        slot[lv] = 1;
                        Batch::Tag tg;
                        tg.cand = static_cast<int>(ci);
                        tg.a = p0;
                        tg.b = vI;
                        tg.c = p2;
                        tg.se = (rest_dist(in.Vrest, p0, vI) * (1.0 + 1.0) + rest_dist(in.Vrest, vI, p2) * (1.0 + 1.0)) /
                                R / 2.0;   // seInc (TriMesh.cpp:2246-2247)
                        tg.nRows = 2;
                        emit(B, T, in.rest, in.UV, umbrella, Lc, extra, slot, 2, nLoc - 1, tg);
                        if (air) {
                            // separate the copies; the opened slit is the air
                            // loop (p2, vI, p0, copy) (TriMesh.cpp:2322-2372)
                            const LocalProblem& P = B.prob.back();
                            std::vector<double2> lp(B.lvPos.begin() + P.vertOff,
                                                    B.lvPos.begin() + P.vertOff + P.nVert);
                            Topo LT;
                            LT.build(P.nVert, Lc.corner.data(), n);
                            const double dx = in.UV[2 * (size_t)vI] - in.UV[2 * (size_t)p0];
                            const double dy = in.UV[2 * (size_t)vI + 1] - in.UV[2 * (size_t)p0 + 1];
                            separate_copies(LT, lp, Lc.corner, lv, nLoc, (dx * dx + dy * dy) * 1.0e-4);
                            for (int l = 0; l < P.nVert; ++l) B.lvPos[P.vertOff + l] = lp[l];
                            const int l2 = L.find(p2), l0 = L.find(p0);
                            const std::vector<int> al{l2, lv, l0, nLoc};
                            const std::vector<double2> ap{lp[l2], lp[lv], lp[l0], lp[nLoc]};
                            emit_air(B, al, ap, local_air_thres(in.Vrest, in.F, umbrella), l2 < 0 || l0 < 0);
                        }
                    }
                }
            });
        }
    }
    else if (opType == kOpMerge) {
        // TriMesh::queryMerge (TriMesh.cpp:800-930): zipper-bottom pairs
        std::vector<double> V(in.UV, in.UV + 2 * (size_t)in.nV);
        const double eps_IC = 1.0e-6 * in.avgEdgeLen;
        for (int ci = 0; ci < in.nCohE; ++ci) {
            const int* ce = in.cohE + 4 * (size_t)ci;
            int fork;
            if (ce[0] == ce[2]) fork = 0;
            else if (ce[1] == ce[3]) fork = 1;
            else continue;
            if (in.mergeFork != -2 && ce[fork] != in.mergeFork) continue;   // propagation (TriMesh.cpp:828-833)
            const int va = ce[1 - fork], vb = ce[3 - fork];
            std::vector<int> triangles;
            int firstAmt = 0;
            for (int m2 = 0; m2 < 2; ++m2) {
                const int v = m2 == 0 ? va : vb;
                for (int p = T.nbPtr[v]; p < T.nbPtr[v + 1]; ++p) {
                    const int f = T.edge_tri(v, T.nb[p]);
                    if (f >= 0) triangles.push_back(f);
                }
                if (m2 == 0) firstAmt = static_cast<int>(triangles.size());
            }
            double mp[2] = {(V[2 * va] + V[2 * vb]) / 2.0, (V[2 * va + 1] + V[2 * vb + 1]) / 2.0};
            const double b0[2] = {V[2 * va], V[2 * va + 1]}, b1[2] = {V[2 * vb], V[2 * vb + 1]};
            auto place = [&](const double* p) {
                V[2 * va] = p[0]; V[2 * va + 1] = p[1];
                V[2 * vb] = p[0]; V[2 * vb + 1] = p[1];
            };
            auto restore = [&]() {
                V[2 * va] = b0[0]; V[2 * va + 1] = b0[1];
                V[2 * vb] = b1[0]; V[2 * vb + 1] = b1[1];
            };
            place(mp);
            if (!inverted_any(T, V, triangles)) {
                restore();
            }
            else {
                // relaxation projection onto the non-inversion half-planes
                std::vector<double> cm, cv;
                for (size_t k = 0; k < triangles.size(); ++k) {
                    const int t = triangles[k];
                    const int vm = (int)k < firstAmt ? va : vb;
                    for (int i = 0; i < 3; ++i)
                        if (T.F[3 * t + i] == vm) {
                            const int i1 = T.F[3 * t + (i + 1) % 3], i2 = T.F[3 * t + (i + 2) % 3];
                            const double v1x = V[2 * i1], v1y = V[2 * i1 + 1], v2x = V[2 * i2], v2y = V[2 * i2 + 1];
                            const double cx = v2y - v1y, cy = v1x - v2x;
                            const double nrm = std::sqrt(cx * cx + cy * cy);
                            cm.push_back(cx / nrm);
                            cm.push_back(cy / nrm);
                            cv.push_back((v1x * v2y - v1y * v2x) / nrm);
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
                        if (res > maxRes) maxRes = res;
                    }
                    if (maxRes < 0.0) break;
                }
                place(mp);
                const bool bad = inverted_any(T, V, triangles);
                restore();
                if (bad) continue;   // no feasible merged position
            }
            const int p0 = fork ? ce[0] : ce[3], p1 = fork ? ce[1] : ce[2], p2 = fork ? ce[2] : ce[1];
            // seam decrease, closing a split diamond (TriMesh.cpp:2121-2135)
            double seDec = rest_dist(in.Vrest, p0, p1) / R * (1.0 + 1.0) / 2.0;
            bool closeup = false;
            for (int p = T.nbPtr[p0]; p < T.nbPtr[p0 + 1]; ++p) {
                const int nbv = T.nb[p];
                if (nbv != p1 && T.bnd[nbv] && T.adjacent(p2, nbv)) {
                    seDec += rest_dist(in.Vrest, p0, nbv) / R * (1.0 + 1.0) / 2.0;
                    closeup = true;
                    break;
                }
            }
            // local mesh with p0 and p2 as one vertex at the merged position
            L.build(T, triangles, p0, p2);
            const int lm = L.find(p0);
            std::vector<int> slot(L.gv.size(), -1);
            slot[lm] = 0;
            Batch::Tag tg;
            tg.cand = static_cast<int>(out.size());
            tg.a = p0;
            tg.b = p1;
            tg.c = p2;
            tg.se = seDec;
            tg.nRows = 1;
            TopoCandidate C;
            C.path = {p0, p1, p2};
            C.EwDec = -DBL_MAX;
            if ((int)(out.size() % in.shardCount) != in.shardRank) {   // another shard's candidate
                C.ec0 = C.ec1 = DBL_MAX;
                out.push_back(C);
                continue;
            }
            out.push_back(C);
            const size_t before = B.lvPos.size();
            emit(B, T, in.rest, in.UV, triangles, L, {}, slot, 1, static_cast<int>(L.gv.size()) - 1, tg);
            B.lvPos[before + lm] = make_double2(mp[0], mp[1]);   // initMergedPos
            if (air && !closeup) {
                // the corner loop with the merged vertex at initMergedPos
                // (TriMesh.cpp:2406, 2480-2497); closing up a diamond needs none
                std::vector<int> loop, al;
                std::vector<double2> pts;
                const int cm[3] = {p0, p1, p2};
                bool reject = !corner_loop(*air, cm, make_double2(mp[0], mp[1]), loop, pts);
                if (!reject)
                    for (size_t i = 0; i < loop.size(); ++i) {
                        int l = -1;
                        if (i < 3) {
                            const int g = air->mesh_of(loop[i]);
                            l = g == p2 ? lm : L.find(g);
                            if (l < 0) reject = true;
                        }
                        al.push_back(l);
                        if (l >= 0) pts[i] = B.lvPos[before + l];
                    }
                emit_air(B, al, pts, local_air_thres(in.Vrest, in.F, triangles), reject);
            }
        }
        candidatePool = in.nCohE;
    }
    else {
        if (err) *err = "topology query: unknown operation";
        return OC_ERR_INVALID;
    }
    return OC_OK;
}

// Per candidate of one operation: the best of its solved local problems
// (strict >, first wins) over problems [p0, p1) of B; interior splits halved.
void finish_op(int opType, double lambda_t, const Batch& B, size_t p0, size_t p1, const std::vector<LocalResult>& res,
               const std::vector<char>& solved, std::vector<TopoCandidate>& out, int& best, TopoStats& stats,
               TopoExtras* extras)
{
    best = -1;
    if (extras) {
        const size_t n = p1 - p0;
        extras->cand.resize(n);
        extras->ewExact.assign(n, std::nan(""));
        extras->nTri.resize(n);
        extras->nFree.resize(n);
        extras->iters.resize(n);
        extras->trials.resize(n);
        extras->cycles.resize(n);
        for (size_t k = p0; k < p1; ++k) {
            extras->cand[k - p0] = B.tag[k].cand;
            extras->nTri[k - p0] = B.prob[k].nTri;
            extras->nFree[k - p0] = B.prob[k].nFree;
            extras->iters[k - p0] = res[k].iters;
            extras->trials[k - p0] = res[k].trials;
            extras->cycles[k - p0] = res[k].cycles;
        }
    }
    for (size_t k = p0; k < p1; ++k) {
        if (!solved[k]) continue;
        const LocalResult& r = res[k];
        const Batch::Tag& tg = B.tag[k];
        TopoCandidate& C = out[tg.cand];
        if (B.prob[k].nAir != 0) {
            stats.airProblems++;
            if (B.prob[k].nAir < 0) stats.airRejected++;
            stats.airSteinerMax = std::max(stats.airSteinerMax, r.airSteiner);
            if (r.airStatus & (kLoopSteinerCap | kLoopQueueCap)) stats.airCapped++;
        }
        stats.maxIters = std::max(stats.maxIters, r.iters);
        stats.totalIters += r.iters;
        if (r.status != 1) stats.nonConverged++;
        stats.totalTrials += r.trials;
        const double SDDec = r.eDec;
        double EwDec;
        if (opType == kOpMerge) {
            const double SDInc = -SDDec;
            EwDec = lambda_t * tg.se - (1.0 - lambda_t) * SDInc;   // TriMesh.cpp:2157
            if (extras) extras->ewExact[k - p0] = EwDec;
            C.ec0 = SDInc;
            C.ec1 = -tg.se;
            C.EwDec = EwDec;
            C.pos = {r.pos[0].x, r.pos[0].y};
            continue;
        }
        EwDec = (1.0 - lambda_t) * SDDec - lambda_t * tg.se;   // TriMesh.cpp:2187, 2248
        if (extras) extras->ewExact[k - p0] = opType == kOpInteriorSplit ? 0.5 * EwDec : EwDec;
        if (EwDec > C.EwDec) {
            C.EwDec = EwDec;
            C.ec0 = -SDDec;
            C.ec1 = tg.se;
            C.pos.clear();
            for (int row = 0; row < tg.nRows; ++row) {
                C.pos.push_back(r.pos[row].x);
                C.pos.push_back(r.pos[row].y);
            }
            if (opType == kOpBoundarySplit) C.path = {tg.a, tg.b};
            else C.path = {tg.a, tg.b, tg.c};
        }
    }
    if (opType == kOpInteriorSplit)   // querySplit halves interior-split decreases (TriMesh.cpp:702-704)
        for (auto& C : out)
            if (C.EwDec != -DBL_MAX) C.EwDec *= 0.5;
    for (size_t c = 0; c < out.size(); ++c)
        if (best < 0 || out[c].EwDec > out[best].EwDec) best = static_cast<int>(c);
}

} // namespace

int topo_query_ops(const TopoQueryIn& in, const int* ops, int nOps, double lambda_t, double filterExp,
                   const TopoOptions& opts, TopoOpResult* results, std::string* err)
{
    using clk = std::chrono::steady_clock;
    if (!in.F || !in.Vrest || !in.UV || !in.rest || !in.dm || in.nV <= 0 || in.nF <= 0 || nOps <= 0 || !ops ||
        !results) {
        if (err) *err = "topology query: bad arguments";
        return OC_ERR_INVALID;
    }
    for (int i = 0; i < nOps; ++i) results[i] = TopoOpResult{};
    Topo ownT;
    if (!in.adj) ownT.build(in.nV, in.F, in.nF);
    const Topo& T = in.adj ? in.adj->T : ownT;
    if (T.nV != in.nV || T.nF != in.nF || T.F != in.F) {
        if (err) *err = "topology query: adjacency of another mesh";
        return OC_ERR_INVALID;
    }
    // bijective form: the whole-mesh air mesh the local loops come from
    std::unique_ptr<AirSrc> airSrc;
    const auto tAir = clk::now();
    if (in.bijective) {
        if (!in.airV || !in.airF || !in.airBnd || in.nAirF <= 0 || in.nAirBnd <= 0 || in.nAirV < in.nAirBnd) {
            if (err) *err = "topology query: the bijective form needs the scaffold's air mesh";
            return OC_ERR_INVALID;
        }
        airSrc = std::make_unique<AirSrc>();
        airSrc->build(in);
    }
    const double airMs = std::chrono::duration<double, std::milli>(clk::now() - tAir).count();
    // every operation's problems in one batch, op i owning [start[i], start[i + 1])
    Batch B;
    std::vector<size_t> start(nOps + 1, 0);
    std::vector<int> opOf;
    for (int i = 0; i < nOps; ++i) {
        const auto t0 = clk::now();
        Batch Bi;
        const int rc = build_op(in, T, ops[i], filterExp, results[i].cands, results[i].pool, Bi, err,
                                airSrc.get());
        if (rc) return rc;
        append_batch(B, Bi);
        start[i + 1] = B.prob.size();
        opOf.insert(opOf.end(), Bi.prob.size(), ops[i]);
        results[i].stats.nCandidates = static_cast<int>(results[i].cands.size());
        results[i].stats.nProblems = static_cast<int>(Bi.prob.size());
        results[i].stats.buildMs = std::chrono::duration<double, std::milli>(clk::now() - t0).count();
    }
    const auto t1 = clk::now();
    // one batched device solve of all problems (exhaustive), or the learned
    // proposal: a one-step pass over all problems gives their features, the
    // MLP ranks each operation's problems and only the top fraction of each
    // gets the full solve
    const size_t n = B.prob.size();
    std::vector<LocalResult> res(n);
    std::vector<char> solved(n, 1);
    const unsigned long long batchId = in.ws ? in.ws->nextBatch++ : 0;
    const bool learned = (opts.flags & kTopoLearned) && opts.mlp;
    const int fp32 = opts.flags & kTopoFp32Hessian;
    const bool tune = (opts.flags & kTopoAutotune) != 0;
    double probeMs = 0.0, exactMs = 0.0, rankMs = 0.0;
    if (n) {
        std::string e2;
        std::vector<int> all(n);
        for (size_t k = 0; k < n; ++k) all[k] = static_cast<int>(k);
        if (learned) {
            int rc = solve_batch(in, B, batchId, all, 1, fp32, res, &e2, tune);
            if (rc) { if (err) *err = e2; return rc; }
            const auto tA = clk::now();
            probeMs = std::chrono::duration<double, std::milli>(tA - t1).count();
            // features -> predicted fraction of excess energy removed -> E_w decrease
            std::vector<float> X(n * kTopoNumFeatures), r(n);
            host_parallel_for(n, 1024, [&](size_t k0, size_t k1) {
                for (size_t k = k0; k < k1; ++k)
                    topo_features(B.prob[k], res[k], opOf[k], in, &X[k * kTopoNumFeatures]);
            });
            rc = mlp_predict_host(*opts.mlp, X.data(), static_cast<int>(n), r.data());
            if (rc) { if (err) *err = "topology query: MLP inference failed"; return rc; }
            std::fill(solved.begin(), solved.end(), 0);
            std::vector<int> sel;
            for (int i = 0; i < nOps; ++i) {
                const int op = ops[i];
                const int ni = static_cast<int>(start[i + 1] - start[i]);
                if (!ni) continue;
                std::vector<std::pair<double, int>> pred(ni);
                for (int j = 0; j < ni; ++j) {
                    const size_t k = start[i] + j;
                    const double sdd = static_cast<double>(r[k]) * excess_global(B.prob[k], res[k], in.surfaceArea);
                    const double ew = op == kOpMerge ? lambda_t * B.tag[k].se + (1.0 - lambda_t) * sdd
                                                     : (1.0 - lambda_t) * sdd - lambda_t * B.tag[k].se;
                    pred[j] = {-ew, j};
                }
                TopoExtras& ex = results[i].extras;
                ex.ewPred.resize(ni);
                for (int j = 0; j < ni; ++j) ex.ewPred[j] = -pred[j].first * (op == kOpInteriorSplit ? 0.5 : 1.0);
                // the top fraction, and never fewer than kMinExact problems
                // (an operation with few candidates, a step's merges
                // typically, is solved exhaustively): the kTop smallest
                // (-decrease, index) pairs, a total order, so the set is the
                // first kTop of the sorted list
                constexpr int kMinExact = 32;
                int kTop = static_cast<int>(std::ceil(opts.topFrac * ni));
                kTop = std::max(std::min(ni, kMinExact), std::min(ni, kTop));
                if (kTop < ni) std::nth_element(pred.begin(), pred.begin() + kTop, pred.end());
                for (int q = 0; q < kTop; ++q) {
                    solved[start[i] + pred[q].second] = 1;
                    sel.push_back(static_cast<int>(start[i] + pred[q].second));
                }
                results[i].stats.nSelected = kTop;
                ex.X.assign(X.begin() + start[i] * kTopoNumFeatures, X.begin() + start[i + 1] * kTopoNumFeatures);
                ex.predicted.assign(r.begin() + start[i], r.begin() + start[i + 1]);
            }
            std::sort(sel.begin(), sel.end());
            std::vector<LocalResult> full(n);
            const auto tB = clk::now();
            rankMs = std::chrono::duration<double, std::milli>(tB - tA).count();
            rc = solve_batch(in, B, batchId, sel, -1, fp32, full, &e2, tune);
            if (rc) { if (err) *err = e2; return rc; }
            for (int k : sel) res[k] = full[k];
            exactMs = std::chrono::duration<double, std::milli>(clk::now() - tB).count();
        }
        else {
            const int rc = solve_batch(in, B, batchId, all, -1, fp32, res, &e2, tune);
            if (rc) { if (err) *err = e2; return rc; }
            for (int i = 0; i < nOps; ++i) {
                results[i].stats.nSelected = static_cast<int>(start[i + 1] - start[i]);
                if (!(opts.flags & kTopoRecordFeatures)) continue;
                TopoExtras& ex = results[i].extras;
                const size_t ni = start[i + 1] - start[i];
                ex.X.assign(ni * kTopoNumFeatures, 0.0f);
                ex.target.assign(ni, 0.0f);
                host_parallel_for(ni, 1024, [&](size_t j0, size_t j1) {
                    for (size_t j = j0; j < j1; ++j) {
                        const size_t k = start[i] + j;
                        topo_features(B.prob[k], res[k], ops[i], in, &ex.X[j * kTopoNumFeatures]);
                        const double xs = excess_global(B.prob[k], res[k], in.surfaceArea);
                        const double t = xs > 0.0 ? res[k].eDec / xs : 0.0;
                        ex.target[j] = static_cast<float>(std::max(-1.0, std::min(1.0, t)));
                    }
                });
            }
        }
    }
    const auto t2 = clk::now();
    const double solveMs = std::chrono::duration<double, std::milli>(t2 - t1).count();
    for (int i = 0; i < nOps; ++i) {
        TopoOpResult& R = results[i];
        R.stats.solveMs = solveMs;   // shared by the operations solved together
        R.stats.probeMs = probeMs;
        R.stats.exactMs = exactMs;
        R.stats.rankMs = rankMs;
        R.stats.airMs = airMs;
        finish_op(ops[i], lambda_t, B, start[i], start[i + 1], res, solved, R.cands, R.best, R.stats, &R.extras);
    }
    const double finishMs = std::chrono::duration<double, std::milli>(clk::now() - t2).count();
    for (int i = 0; i < nOps; ++i) results[i].stats.finishMs = finishMs;
    return OC_OK;
}

int topo_query(const TopoQueryIn& in, int opType, double lambda_t, double filterExp, const TopoOptions& opts,
               std::vector<TopoCandidate>& out, int& best, int& candidatePool, TopoStats& stats, std::string* err,
               TopoExtras* extras)
{
    out.clear();
    best = -1;
    candidatePool = 0;
    stats = TopoStats{};
    TopoOpResult r;
    const int rc = topo_query_ops(in, &opType, 1, lambda_t, filterExp, opts, &r, err);
    if (rc) return rc;
    out.swap(r.cands);
    best = r.best;
    candidatePool = r.pool;
    stats = r.stats;
    if (extras) *extras = std::move(r.extras);
    return OC_OK;
}

} // namespace oc
