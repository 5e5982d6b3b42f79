// Air mesh of the bijectivity scaffold, built on the host without Triangle.
//
// The reference's Scaffold constructor (src/Scaffold.cpp:27-205, whole-mesh
// branch) collects the UV boundary loops of the mesh, adds a segmented
// bounding box at margin 4 * avgEdgeLen with segments of 9 * avgEdgeLen
// (scaleFactor 3, bandAmt 2, :63-95), marks one hole point inside every
// connected component (:97-158) and calls Triangle with "qYQ" (:167).
//
// This file computes a constrained Delaunay triangulation of the same input
// (boundary loops + box) and removes the outside of the box and every mesh
// component's interior by flood fill from a seed inside the component, the
// same region Triangle's hole points carve out.  Like "Y", no point is added
// on a boundary segment.  Vertex rows:
//   rows 0 .. nBnd-1        mesh boundary vertices, loop by loop
//   next                    box points, counter-clockwise from (minX, minY)
//   last                    interior Steiner points of the refinement
//
// Method: incremental Delaunay insertion with Lawson flips inside a super
// triangle, constraint recovery by edge flips (Sloan, "A fast algorithm for
// generating constrained Delaunay triangulations", Computers & Structures
// 47(3), 1993), then Lawson flips of the recovered region's free edges, and
// optionally Delaunay refinement of the air region to a minimum angle (the
// counterpart of "q", 20 degrees there) by circumcenter insertion without
// splitting any segment (as "Y" forbids).  Orientation and in-circle tests
// are plain double-precision determinants.

#include "oc_airmesh.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <utility>
#include <vector>

namespace oc {
namespace {

struct P2 {
    double x, y;
};

inline double orient(const P2& a, const P2& b, const P2& c)
{
    return (b.x - a.x) * (c.y - a.y) - (b.y - a.y) * (c.x - a.x);
}

// > 0 when d lies inside the circumcircle of the counter-clockwise (a, b, c)
inline double incircle(const P2& a, const P2& b, const P2& c, const P2& d)
{
    const double adx = a.x - d.x, ady = a.y - d.y;
    const double bdx = b.x - d.x, bdy = b.y - d.y;
    const double cdx = c.x - d.x, cdy = c.y - d.y;
    const double ad = adx * adx + ady * ady, bd = bdx * bdx + bdy * bdy, cd = cdx * cdx + cdy * cdy;
    return adx * (bdy * cd - bd * cdy) - ady * (bdx * cd - bd * cdx) + ad * (bdx * cdy - bdy * cdx);
}

// Triangle t: counter-clockwise v[0..2]; n[i] is the neighbour across the
// edge opposite v[i] (v[i+1], v[i+2]); c[i] marks that edge constrained.
struct Tri {
    int v[3];
    int n[3];
    bool c[3];
};

class Cdt {
public:
    explicit Cdt(const std::vector<P2>& pts) : P(pts) {}

    int nReal() const { return nReal_; }

    bool build(int nRealPoints)
    {
        nReal_ = nRealPoints;
        double lo[2] = {P[0].x, P[0].y}, hi[2] = {P[0].x, P[0].y};
        for (int i = 0; i < nReal_; ++i) {
            lo[0] = std::min(lo[0], P[i].x); hi[0] = std::max(hi[0], P[i].x);
            lo[1] = std::min(lo[1], P[i].y); hi[1] = std::max(hi[1], P[i].y);
        }
        const double cx = 0.5 * (lo[0] + hi[0]), cy = 0.5 * (lo[1] + hi[1]);
        const double r = std::max(hi[0] - lo[0], hi[1] - lo[1]) + 1.0;
        P.resize(nReal_ + 3);
        P[nReal_] = {cx - 20.0 * r, cy - 10.0 * r};
        P[nReal_ + 1] = {cx + 20.0 * r, cy - 10.0 * r};
        P[nReal_ + 2] = {cx, cy + 20.0 * r};
        T.clear();
        T.push_back(Tri{{nReal_, nReal_ + 1, nReal_ + 2}, {-1, -1, -1}, {false, false, false}});
        dead.assign(1, 0);
        vt.assign(nReal_ + 3, 0);
        last = 0;
        for (int k = 0; k < nReal_; ++k)
            if (!insert(k, last)) return false;
        return true;
    }

    // Delaunay refinement inside the carved domain (Ruppert's circumcenter
    // insertion, "A Delaunay refinement algorithm for quality 2-dimensional
    // mesh generation", J. Algorithms 18(3), 1995) without splitting any
    // segment: a skinny triangle whose circumcenter is not visible from it
    // or encroaches a segment's diametral circle is left as it is.  New
    // points are appended after the input points.
    void refine(double minAngleDeg, int maxSteiner)
    {
        const double cosMax = std::cos(minAngleDeg * M_PI / 180.0);
        std::vector<int> queue;
        for (size_t t = 0; t < T.size(); ++t)
            if (!dead[t]) queue.push_back(static_cast<int>(t));
        std::vector<char> hopeless(T.size(), 0);
        int added = 0;
        size_t head = 0;
        while (head < queue.size() && added < maxSteiner) {
            const int t = queue[head++];
            if (dead[t] || (t < (int)hopeless.size() && hopeless[t]) || !skinny(t, cosMax)) continue;
            P2 c;
            if (!circumcenter(t, c)) continue;
            const int s = walk_visible(c, t);
            if (s < 0 || encroaches(s, c)) {
                if (t >= (int)hopeless.size()) hopeless.resize(T.size(), 0);
                hopeless[t] = 1;
                continue;
            }
            const int k = static_cast<int>(P.size());
            P.push_back(c);
            vt.push_back(s);
            touched.clear();
            recording = true;
            const bool ok = insert(k, s);
            recording = false;
            if (!ok) {
                P.pop_back();
                vt.pop_back();
                if (t >= (int)hopeless.size()) hopeless.resize(T.size(), 0);
                hopeless[t] = 1;
                continue;
            }
            ++added;
            if (hopeless.size() < T.size()) hopeless.resize(T.size(), 0);
            for (int u : touched) {
                hopeless[u] = 0;
                queue.push_back(u);
            }
            if (head > 65536 && head * 2 > queue.size()) {
                queue.erase(queue.begin(), queue.begin() + head);
                head = 0;
            }
        }
    }

    // Makes (a, b) an edge and marks it constrained; false on a vertex lying
    // on the open segment or a failure to converge.
    bool constrain(int a, int b)
    {
        int t, i;
        if (find_edge(a, b, t, i)) {
            mark(t, i, true);
            return true;
        }
        std::vector<std::pair<int, int>> cross;
        if (!crossed_edges(a, b, cross)) return false;
        std::vector<std::pair<int, int>> fresh;
        size_t guard = 0;
        const size_t limit = 64 * (cross.size() + 8) * (cross.size() + 8);
        size_t head = 0;
        while (head < cross.size()) {
            if (++guard > limit) return false;
            const std::pair<int, int> e = cross[head++];
            if (!find_edge(e.first, e.second, t, i)) return false;
            const int u = T[t].n[i];
            if (u < 0) return false;
            const int p = T[t].v[i];
            const int j = opposite_index(u, t);
            const int q = T[u].v[j];
            const int ea = T[t].v[(i + 1) % 3], eb = T[t].v[(i + 2) % 3];
            if (!(orient(P[p], P[ea], P[q]) > 0.0 && orient(P[q], P[eb], P[p]) > 0.0)) {
                cross.push_back(e);   // not strictly convex: retry after the others
                continue;
            }
            flip(t, i);
            if (proper_cross(a, b, p, q)) cross.push_back({p, q});
            else fresh.push_back({p, q});
            if (head > 4096 && head * 2 > cross.size()) {   // compact the processed prefix
                cross.erase(cross.begin(), cross.begin() + head);
                head = 0;
            }
        }
        if (!find_edge(a, b, t, i)) return false;
        mark(t, i, true);
        // restore the Delaunay property among the new free edges
        bool changed = true;
        int rounds = 0;
        while (changed && rounds++ < 64) {
            changed = false;
            for (auto& e : fresh) {
                if ((e.first == a && e.second == b) || (e.first == b && e.second == a)) continue;
                if (!find_edge(e.first, e.second, t, i)) continue;
                if (T[t].c[i]) continue;
                const int u = T[t].n[i];
                if (u < 0) continue;
                const int j = opposite_index(u, t);
                const int q = T[u].v[j];
                if (incircle(P[T[t].v[0]], P[T[t].v[1]], P[T[t].v[2]], P[q]) > 0.0) {
                    const int p = T[t].v[i];
                    const int ea = T[t].v[(i + 1) % 3], eb = T[t].v[(i + 2) % 3];
                    if (orient(P[p], P[ea], P[q]) > 0.0 && orient(P[q], P[eb], P[p]) > 0.0) {
                        flip(t, i);
                        e = {p, q};
                        changed = true;
                    }
                }
            }
        }
        return true;
    }

    // Removes every triangle reachable from `seed` without crossing a
    // constrained edge.
    void carve(int seed)
    {
        if (seed < 0 || dead[seed]) return;
        std::vector<int> stack{seed};
        dead[seed] = 1;
        while (!stack.empty()) {
            const int t = stack.back();
            stack.pop_back();
            for (int i = 0; i < 3; ++i) {
                const int u = T[t].n[i];
                if (u >= 0 && !T[t].c[i] && !dead[u]) {
                    dead[u] = 1;
                    stack.push_back(u);
                }
            }
        }
    }

    int triangle_with_super_vertex() const
    {
        for (size_t t = 0; t < T.size(); ++t)
            for (int k = 0; k < 3; ++k)
                if (T[t].v[k] >= nReal_) return static_cast<int>(t);
        return -1;
    }

    int locate(const P2& p) const { return walk(p, last); }

    std::vector<P2> P;
    std::vector<Tri> T;
    std::vector<char> dead;   // carved away (outside the box or inside the mesh)

private:
    std::vector<int> vt;   // a triangle incident to each vertex
    std::vector<int> touched;
    bool recording = false;
    int last = 0;
    int nReal_ = 0;

    void touch(int t)
    {
        for (int k = 0; k < 3; ++k) vt[T[t].v[k]] = t;
        if (recording) touched.push_back(t);
    }

    bool skinny(int t, double cosMax) const
    {
        const P2 &a = P[T[t].v[0]], &b = P[T[t].v[1]], &c = P[T[t].v[2]];
        const double la = (b.x - c.x) * (b.x - c.x) + (b.y - c.y) * (b.y - c.y);
        const double lb = (a.x - c.x) * (a.x - c.x) + (a.y - c.y) * (a.y - c.y);
        const double lc = (a.x - b.x) * (a.x - b.x) + (a.y - b.y) * (a.y - b.y);
        // smallest angle is opposite the shortest edge
        double s = la, o1 = lb, o2 = lc;
        if (lb < s) { s = lb; o1 = la; o2 = lc; }
        if (lc < s) { s = lc; o1 = la; o2 = lb; }
        const double cosA = (o1 + o2 - s) / (2.0 * std::sqrt(o1 * o2));
        return cosA > cosMax;
    }

    bool circumcenter(int t, P2& c) const
    {
        const P2 &a = P[T[t].v[0]], &b = P[T[t].v[1]], &d = P[T[t].v[2]];
        const double bx = b.x - a.x, by = b.y - a.y, dx = d.x - a.x, dy = d.y - a.y;
        const double den = 2.0 * (bx * dy - by * dx);
        if (!(den > 0.0)) return false;
        const double b2 = bx * bx + by * by, d2 = dx * dx + dy * dy;
        c = {a.x + (dy * b2 - by * d2) / den, a.y + (bx * d2 - dx * b2) / den};
        return std::isfinite(c.x) && std::isfinite(c.y);
    }

    // Walk from t towards p without crossing a constrained edge; -1 if p is
    // not reachable that way or lies on a vertex or a constrained edge.
    int walk_visible(const P2& p, int t) const
    {
        const int limit = 4 * static_cast<int>(T.size()) + 16;
        for (int step = 0; step < limit; ++step) {
            int next = -1;
            for (int i = 0; i < 3; ++i) {
                const P2& a = P[T[t].v[(i + 1) % 3]];
                const P2& b = P[T[t].v[(i + 2) % 3]];
                const double o = orient(a, b, p);
                if (o < 0.0) {
                    if (T[t].c[i] || T[t].n[i] < 0) return -1;
                    next = T[t].n[i];
                    break;
                }
                if (o == 0.0 && T[t].c[i]) return -1;
            }
            if (next < 0) return dead[t] ? -1 : t;
            t = next;
        }
        return -1;
    }

    // p strictly inside the diametral circle of a constrained edge of s or
    // of its neighbours
    bool encroaches(int s, const P2& p) const
    {
        int ts[4] = {s, T[s].n[0], T[s].n[1], T[s].n[2]};
        for (int u : ts) {
            if (u < 0) continue;
            for (int i = 0; i < 3; ++i) {
                if (!T[u].c[i]) continue;
                const P2& a = P[T[u].v[(i + 1) % 3]];
                const P2& b = P[T[u].v[(i + 2) % 3]];
                if ((p.x - a.x) * (p.x - b.x) + (p.y - a.y) * (p.y - b.y) < 0.0) return true;
            }
        }
        return false;
    }

    int opposite_index(int u, int t) const
    {
        for (int j = 0; j < 3; ++j)
            if (T[u].n[j] == t) return j;
        return -1;
    }

    void set_back(int nb, int from, int to)
    {
        if (nb < 0) return;
        for (int j = 0; j < 3; ++j)
            if (T[nb].n[j] == from) {
                T[nb].n[j] = to;
                return;
            }
    }

    void mark(int t, int i, bool c)
    {
        T[t].c[i] = c;
        const int u = T[t].n[i];
        if (u >= 0) {
            const int j = opposite_index(u, t);
            if (j >= 0) T[u].c[j] = c;
        }
    }

    // Walk towards p; falls back to a scan if the walk does not settle.
    int walk(const P2& p, int start) const
    {
        int t = start;
        const int limit = 4 * static_cast<int>(T.size()) + 16;
        for (int step = 0; step < limit; ++step) {
            bool moved = false;
            for (int i = 0; i < 3; ++i) {
                const P2& a = P[T[t].v[(i + 1) % 3]];
                const P2& b = P[T[t].v[(i + 2) % 3]];
                if (orient(a, b, p) < 0.0 && T[t].n[i] >= 0) {
                    t = T[t].n[i];
                    moved = true;
                    break;
                }
            }
            if (!moved) return t;
        }
        for (size_t s = 0; s < T.size(); ++s) {
            bool in = true;
            for (int i = 0; i < 3 && in; ++i)
                in = orient(P[T[s].v[(i + 1) % 3]], P[T[s].v[(i + 2) % 3]], p) >= 0.0;
            if (in) return static_cast<int>(s);
        }
        return -1;
    }

    // Flip the edge opposite T[t].v[i]: (p, a, b) + (q, b, a) -> (p, a, q) + (q, b, p).
    void flip(int t, int i)
    {
        const int u = T[t].n[i];
        const int j = opposite_index(u, t);
        const int p = T[t].v[i], a = T[t].v[(i + 1) % 3], b = T[t].v[(i + 2) % 3];
        const int q = T[u].v[j];
        const int tA = T[t].n[(i + 1) % 3], tB = T[t].n[(i + 2) % 3];
        const bool cA = T[t].c[(i + 1) % 3], cB = T[t].c[(i + 2) % 3];
        const int uB = T[u].n[(j + 1) % 3], uA = T[u].n[(j + 2) % 3];
        const bool cuB = T[u].c[(j + 1) % 3], cuA = T[u].c[(j + 2) % 3];
        T[t] = Tri{{p, a, q}, {uB, u, tB}, {cuB, false, cB}};
        T[u] = Tri{{q, b, p}, {tA, t, uA}, {cA, false, cuA}};
        set_back(uB, u, t);
        set_back(tA, t, u);
        touch(t);
        touch(u);
    }

    void legalize(int t, int i)
    {
        std::vector<std::pair<int, int>> stack{{t, i}};
        size_t guard = 0;
        while (!stack.empty() && guard++ < 64 * T.size() + 1024) {
            const auto [s, k] = stack.back();
            stack.pop_back();
            if (T[s].c[k]) continue;
            const int u = T[s].n[k];
            if (u < 0) continue;
            const int j = opposite_index(u, s);
            const int q = T[u].v[j];
            if (incircle(P[T[s].v[0]], P[T[s].v[1]], P[T[s].v[2]], P[q]) > 0.0) {
                flip(s, k);
                stack.push_back({s, 0});   // (p, a, q): edge (a, q) opposite p
                stack.push_back({u, 2});   // (q, b, p): edge (q, b) opposite p
            }
        }
    }

    bool insert(int k, int start)
    {
        const P2 p = P[k];
        int t = walk(p, start);
        if (t < 0) return false;
        double o[3];
        for (int i = 0; i < 3; ++i) o[i] = orient(P[T[t].v[(i + 1) % 3]], P[T[t].v[(i + 2) % 3]], p);
        int onEdge = -1;
        for (int i = 0; i < 3; ++i) {
            if (o[i] == 0.0) {
                if (onEdge >= 0) return false;   // coincides with a vertex
                onEdge = i;
            }
        }
        if (onEdge < 0) {
            // split into three: t0 = (p, v1, v2), t1 = (p, v2, v0), t2 = (p, v0, v1)
            const Tri old = T[t];
            const int t1 = static_cast<int>(T.size()), t2 = t1 + 1;
            T.push_back(Tri{});
            T.push_back(Tri{});
            dead.push_back(dead[t]);
            dead.push_back(dead[t]);
            T[t] = Tri{{k, old.v[1], old.v[2]}, {old.n[0], t1, t2}, {old.c[0], false, false}};
            T[t1] = Tri{{k, old.v[2], old.v[0]}, {old.n[1], t2, t}, {old.c[1], false, false}};
            T[t2] = Tri{{k, old.v[0], old.v[1]}, {old.n[2], t, t1}, {old.c[2], false, false}};
            set_back(old.n[1], t, t1);
            set_back(old.n[2], t, t2);
            touch(t); touch(t1); touch(t2);
            legalize(t, 0);
            legalize(t1, 0);
            legalize(t2, 0);
        }
        else {
            // p on the edge (a, b) opposite vi: split t and its neighbour u into four
            const int i = onEdge;
            const int u = T[t].n[i];
            if (u < 0) return false;
            const int j = opposite_index(u, t);
            const int vi = T[t].v[i], a = T[t].v[(i + 1) % 3], b = T[t].v[(i + 2) % 3];
            const int q = T[u].v[j];
            const int tA = T[t].n[(i + 1) % 3], tB = T[t].n[(i + 2) % 3];
            const bool ctA = T[t].c[(i + 1) % 3], ctB = T[t].c[(i + 2) % 3], cab = T[t].c[i];
            const int uB = T[u].n[(j + 1) % 3], uA = T[u].n[(j + 2) % 3];
            const bool cuB = T[u].c[(j + 1) % 3], cuA = T[u].c[(j + 2) % 3];
            if (T[t].c[i] && recording) return false;   // no point on a segment
            const int t2 = static_cast<int>(T.size()), u2 = t2 + 1;
            T.push_back(Tri{});
            T.push_back(Tri{});
            dead.push_back(dead[t]);
            dead.push_back(dead[u]);
            T[t] = Tri{{vi, a, k}, {u2, t2, tB}, {cab, false, ctB}};
            T[t2] = Tri{{vi, k, b}, {u, tA, t}, {cab, ctA, false}};
            T[u] = Tri{{q, b, k}, {t2, u2, uA}, {cab, false, cuA}};
            T[u2] = Tri{{q, k, a}, {t, uB, u}, {cab, cuB, false}};
            set_back(tA, t, t2);
            set_back(uB, u, u2);
            touch(t); touch(t2); touch(u); touch(u2);
            legalize(t, 2);
            legalize(t2, 1);
            legalize(u, 2);
            legalize(u2, 1);
        }
        last = t;
        return true;
    }

    // Triangle t and index i with {a, b} the edge opposite T[t].v[i].
    bool find_edge(int a, int b, int& t, int& i) const
    {
        const int start = vt[a];
        int s = start;
        for (int guard = 0; guard < 4096; ++guard) {
            int k = -1;
            for (int m = 0; m < 3; ++m)
                if (T[s].v[m] == a) k = m;
            if (k < 0) return find_edge_scan(a, b, t, i);
            const int x = T[s].v[(k + 1) % 3], y = T[s].v[(k + 2) % 3];
            if (x == b) { t = s; i = (k + 2) % 3; return true; }
            if (y == b) { t = s; i = (k + 1) % 3; return true; }
            s = T[s].n[(k + 2) % 3];   // next triangle counter-clockwise around a
            if (s < 0) return find_edge_scan(a, b, t, i);
            if (s == start) return false;
        }
        return find_edge_scan(a, b, t, i);
    }

    bool find_edge_scan(int a, int b, int& t, int& i) const
    {
        for (size_t s = 0; s < T.size(); ++s)
            for (int k = 0; k < 3; ++k) {
                const int x = T[s].v[(k + 1) % 3], y = T[s].v[(k + 2) % 3];
                if ((x == a && y == b) || (x == b && y == a)) {
                    t = static_cast<int>(s);
                    i = k;
                    return true;
                }
            }
        return false;
    }

    bool proper_cross(int a, int b, int x, int y) const
    {
        const double o1 = orient(P[a], P[b], P[x]), o2 = orient(P[a], P[b], P[y]);
        const double o3 = orient(P[x], P[y], P[a]), o4 = orient(P[x], P[y], P[b]);
        return ((o1 > 0.0 && o2 < 0.0) || (o1 < 0.0 && o2 > 0.0)) && ((o3 > 0.0 && o4 < 0.0) || (o3 < 0.0 && o4 > 0.0));
    }

    // Edges crossed by the open segment (a, b), in order from a.
    bool crossed_edges(int a, int b, std::vector<std::pair<int, int>>& out) const
    {
        // the triangle around a whose opposite edge the segment leaves through
        const int start = vt[a];
        int s = start, r = -1, l = -1, t = -1;
        for (int guard = 0; guard < 4096; ++guard) {
            int k = -1;
            for (int m = 0; m < 3; ++m)
                if (T[s].v[m] == a) k = m;
            if (k < 0) return false;
            const int x = T[s].v[(k + 1) % 3], y = T[s].v[(k + 2) % 3];
            const double ox = orient(P[a], P[b], P[x]), oy = orient(P[a], P[b], P[y]);
            if (ox == 0.0 && orient(P[a], P[x], P[b]) == 0.0 &&
                (P[x].x - P[a].x) * (P[b].x - P[a].x) + (P[x].y - P[a].y) * (P[b].y - P[a].y) > 0.0)
                return false;   // a vertex on the segment
            if (ox < 0.0 && oy > 0.0) { t = s; r = x; l = y; break; }
            s = T[s].n[(k + 2) % 3];
            if (s < 0 || s == start) return false;
        }
        if (t < 0) return false;
        for (size_t guard = 0; guard < 4 * T.size() + 16; ++guard) {
            out.push_back({r, l});
            // neighbour of t across (r, l)
            int i = -1;
            for (int m = 0; m < 3; ++m) {
                const int x = T[t].v[(m + 1) % 3], y = T[t].v[(m + 2) % 3];
                if ((x == r && y == l) || (x == l && y == r)) i = m;
            }
            if (i < 0) return false;
            const int u = T[t].n[i];
            if (u < 0) return false;
            const int j = opposite_index(u, t);
            const int z = T[u].v[j];
            if (z == b) return true;
            const double oz = orient(P[a], P[b], P[z]);
            if (oz == 0.0) return false;   // a vertex on the segment
            if (oz < 0.0) r = z;
            else l = z;
            t = u;
        }
        return false;
    }
};

} // namespace

int air_mesh_boundary(int nV, const int* F, int nF, std::vector<int>& bnd, std::vector<int>& loopStart,
                      std::vector<int>& seedTris, std::string* err)
{
    auto bad = [&](const char* m) {
        if (err) *err = m;
        return OC_ERR_INVALID;
    };
    if (!F || nV <= 0 || nF <= 0) return bad("air mesh: bad arguments");
    for (long long i = 0; i < 3LL * nF; ++i)
        if (F[i] < 0 || F[i] >= nV) return bad("air mesh: vertex index out of range");
    // outgoing half-edges per vertex (CSR); (a, b) is on the boundary when
    // b has no half-edge back to a
    std::vector<int> hp(nV + 1, 0), hto(3 * (size_t)nF);
    for (long long i = 0; i < 3LL * nF; ++i) hp[F[i] + 1]++;
    for (int v = 0; v < nV; ++v) hp[v + 1] += hp[v];
    {
        std::vector<int> fill(hp.begin(), hp.end() - 1);
        for (int t = 0; t < nF; ++t)
            for (int k = 0; k < 3; ++k) hto[fill[F[3 * t + k]]++] = F[3 * t + (k + 1) % 3];
    }
    std::vector<int> next(nV, -1);
    for (int a = 0; a < nV; ++a)
        for (int p = hp[a]; p < hp[a + 1]; ++p) {
            const int b = hto[p];
            bool twin = false;
            for (int q = hp[b]; q < hp[b + 1] && !twin; ++q) twin = hto[q] == a;
            if (twin) continue;
            if (next[a] >= 0) return bad("air mesh: non-manifold boundary vertex");
            next[a] = b;
        }
    bnd.clear();
    loopStart.clear();
    std::vector<char> used(nV, 0);
    for (int v = 0; v < nV; ++v) {
        if (next[v] < 0 || used[v]) continue;
        loopStart.push_back(static_cast<int>(bnd.size()));
        int w = v;
        while (!used[w]) {
            used[w] = 1;
            bnd.push_back(w);
            w = next[w];
            if (w < 0) return bad("air mesh: open boundary chain");
        }
        if (w != v) return bad("air mesh: boundary chains merge");
    }
    loopStart.push_back(static_cast<int>(bnd.size()));
    if (bnd.size() < 3) return bad("air mesh: the mesh has no boundary");
    // the first triangle of each connected component (union-find over
    // vertices), whose centroid seeds the removal of the mesh's own region
    seedTris.clear();
    std::vector<int> root(nV);
    for (int v = 0; v < nV; ++v) root[v] = v;
    auto find = [&](int v) {
        while (root[v] != v) v = root[v] = root[root[v]];
        return v;
    };
    for (int t = 0; t < nF; ++t) {
        const int r0 = find(F[3 * t]);
        for (int k = 1; k < 3; ++k) {
            const int r = find(F[3 * t + k]);
            if (r != r0) root[r] = r0;
        }
    }
    std::vector<char> seeded(nV, 0);
    for (int t = 0; t < nF; ++t) {
        const int r = find(F[3 * t]);
        if (seeded[r]) continue;
        seeded[r] = 1;
        seedTris.insert(seedTris.end(), F + 3 * t, F + 3 * t + 3);
    }
    return OC_OK;
}

int air_mesh_build(const double* UV, int nV, const int* F, int nF, double avgEdgeLen, AirMesh& out, std::string* err,
                   double minAngleDeg)
{
    std::vector<int> bnd, loopStart, seedTris;
    const int rc = air_mesh_boundary(nV, F, nF, bnd, loopStart, seedTris, err);
    if (rc) return rc;
    return air_mesh_build_loops(UV, nV, bnd, loopStart, seedTris, avgEdgeLen, out, err, minAngleDeg);
}

int air_mesh_build_loops(const double* UV, int nV, const std::vector<int>& bnd, const std::vector<int>& loopStart,
                         const std::vector<int>& seedTris, double avgEdgeLen, AirMesh& out, std::string* err,
                         double minAngleDeg)
{
    auto bad = [&](const char* m) {
        if (err) *err = m;
        return OC_ERR_INVALID;
    };
    if (!UV || nV <= 0 || !(avgEdgeLen > 0.0) || bnd.size() < 3 || loopStart.size() < 2)
        return bad("air mesh: bad arguments");
    for (int b : bnd)
        if (b < 0 || b >= nV) return bad("air mesh: boundary vertex out of range");
    for (int v : seedTris)
        if (v < 0 || v >= nV) return bad("air mesh: seed vertex out of range");
    out = AirMesh{};
    out.bnd = bnd;
    std::vector<std::pair<int, int>> segs;
    for (size_t l = 0; l + 1 < loopStart.size(); ++l) {
        const int first = loopStart[l], last = loopStart[l + 1] - 1;
        for (int i = first; i < last; ++i) segs.push_back({i, i + 1});
        segs.push_back({last, first});
    }
    const int nBnd = static_cast<int>(out.bnd.size());
    // bounding box and its segmentation (Scaffold.cpp:63-95)
    double minX = UV[0], maxX = UV[0], minY = UV[1], maxY = UV[1];
    for (int v = 1; v < nV; ++v) {
        minX = std::min(minX, UV[2 * v]); maxX = std::max(maxX, UV[2 * v]);
        minY = std::min(minY, UV[2 * v + 1]); maxY = std::max(maxY, UV[2 * v + 1]);
    }
    const double scaleFactor = 3.0;
    const int bandAmt = 2;
    const double segLen = avgEdgeLen * std::pow(scaleFactor, bandAmt);
    const double margin = (avgEdgeLen - segLen) / (1.0 - scaleFactor);
    minX -= margin; maxX += margin; minY -= margin; maxY += margin;
    const int segX = static_cast<int>(std::ceil((maxX - minX) / segLen));
    const int segY = static_cast<int>(std::ceil((maxY - minY) / segLen));
    const double stepX = (maxX - minX) / segX, stepY = (maxY - minY) / segY;
    std::vector<P2> pts(nBnd);
    for (int i = 0; i < nBnd; ++i) pts[i] = {UV[2 * out.bnd[i]], UV[2 * out.bnd[i] + 1]};
    for (int i = 0; i < segX; ++i) pts.push_back({minX + i * stepX, minY});
    for (int i = 0; i < segY; ++i) pts.push_back({maxX, minY + i * stepY});
    for (int i = 0; i < segX; ++i) pts.push_back({maxX - i * stepX, maxY});
    for (int i = 0; i < segY; ++i) pts.push_back({minX, maxY - i * stepY});
    const int nPts = static_cast<int>(pts.size());
    for (int i = nBnd; i + 1 < nPts; ++i) segs.push_back({i, i + 1});
    segs.push_back({nPts - 1, nBnd});

    Cdt cdt(pts);
    if (!cdt.build(nPts)) return bad("air mesh: coincident boundary points");
    for (const auto& sg : segs)
        if (!cdt.constrain(sg.first, sg.second)) return bad("air mesh: boundary segments cross or touch");
    cdt.carve(cdt.triangle_with_super_vertex());
    // one seed per connected component: the centroid of its first triangle
    for (size_t i = 0; i + 2 < seedTris.size(); i += 3) {
        const int* f = seedTris.data() + i;
        const P2 c = {(UV[2 * f[0]] + UV[2 * f[1]] + UV[2 * f[2]]) / 3.0,
                      (UV[2 * f[0] + 1] + UV[2 * f[1] + 1] + UV[2 * f[2] + 1]) / 3.0};
        cdt.carve(cdt.locate(c));
    }
    if (minAngleDeg > 0.0) cdt.refine(minAngleDeg, 4 * nPts + 1024);
    // output: input points, then Steiner points (stored after the three
    // super-triangle vertices)
    const int nAll = static_cast<int>(cdt.P.size()) - 3;
    auto outId = [&](int v) { return v < nPts ? v : v - 3; };
    out.V.resize(2 * (size_t)nAll);
    for (int i = 0; i < nAll; ++i) {
        const P2& q = cdt.P[i < nPts ? i : i + 3];
        out.V[2 * (size_t)i] = q.x;
        out.V[2 * (size_t)i + 1] = q.y;
    }
    out.nBnd = nBnd;
    for (size_t t = 0; t < cdt.T.size(); ++t) {
        if (cdt.dead[t]) continue;
        const Tri& tr = cdt.T[t];
        bool super = false;
        for (int k = 0; k < 3; ++k) super = super || (tr.v[k] >= nPts && tr.v[k] < nPts + 3);
        if (super) continue;
        out.F.insert(out.F.end(), {outId(tr.v[0]), outId(tr.v[1]), outId(tr.v[2])});
    }
    if (out.F.empty()) return bad("air mesh: no air triangle left");
    return OC_OK;
}

} // namespace oc

struct oc_air_mesh {
    oc::AirMesh m;
};

#define OC_EXPORT extern "C" __attribute__((visibility("default")))

OC_EXPORT int oc_air_mesh_build(const double* UV, int nV, const int* F, int nF, double avgEdgeLen, double minAngleDeg,
                                oc_air_mesh** out)
{
    if (!out) return OC_ERR_INVALID;
    *out = nullptr;
    oc_air_mesh* a = new (std::nothrow) oc_air_mesh;
    if (!a) return OC_ERR_NOMEM;
    const int rc = oc::air_mesh_build(UV, nV, F, nF, avgEdgeLen, a->m, nullptr, minAngleDeg);
    if (rc != OC_OK) {
        delete a;
        return rc;
    }
    *out = a;
    return OC_OK;
}

OC_EXPORT int oc_air_mesh_sizes(const oc_air_mesh* a, int* nAirV, int* nAirF, int* nBnd)
{
    if (!a || !nAirV || !nAirF || !nBnd) return OC_ERR_INVALID;
    *nAirV = static_cast<int>(a->m.V.size() / 2);
    *nAirF = static_cast<int>(a->m.F.size() / 3);
    *nBnd = a->m.nBnd;
    return OC_OK;
}

OC_EXPORT int oc_air_mesh_get(const oc_air_mesh* a, double* airV, int* airF, int* bnd)
{
    if (!a) return OC_ERR_INVALID;
    if (airV) std::memcpy(airV, a->m.V.data(), sizeof(double) * a->m.V.size());
    if (airF) std::memcpy(airF, a->m.F.data(), sizeof(int) * a->m.F.size());
    if (bnd) std::memcpy(bnd, a->m.bnd.data(), sizeof(int) * a->m.bnd.size());
    return OC_OK;
}

OC_EXPORT int oc_air_mesh_destroy(oc_air_mesh* a)
{
    if (!a) return OC_ERR_INVALID;
    delete a;
    return OC_OK;
}
