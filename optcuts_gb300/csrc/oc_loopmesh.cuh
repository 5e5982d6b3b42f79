// Mesher for the local air loops of the bijective topology solves: the
// region inside one simple polygon (a candidate's opened slit, the air ring
// around a boundary vertex, the corner loop of a merge) triangulated as
// Triangle does it for the reference's local Scaffold (switches "qYQ",
// src/Scaffold.cpp:150-170): the constrained Delaunay triangulation of the
// polygon, then Delaunay refinement towards a 20 degree minimum angle that
// never puts a Steiner point on the polygon ("Y"), so bad triangles next to
// it may stay.
//
// The refinement restates the published method Triangle implements
// (Shewchuk, "Delaunay refinement algorithms for triangular mesh
// generation", 2002; off-centers after Ungor, 2004): bad triangles are
// taken shortest edge first in half-octave bins (first in, first out
// within a bin); each is split at its circumcenter, or at the off-center on
// the bisector of its shortest edge when that is closer (0.475 sqrt((1 +
// cos t) / (1 - cos t)) edge lengths from the edge, t = 20 degrees, the
// constant Triangle uses); a point outside the polygon, on its
// boundary, or inside the diametral lens (apex angle above 140 degrees) of
// a polygon edge is not inserted and its triangle is given up.
//
// One thread runs it (__host__ __device__: the same code serves the
// kernels and the host entry point the tests call).  Orientation tests are
// exact (error-free products and expansion sums when the filtered double
// result is not certain); the in-circle test falls back to double-double
// arithmetic.  Sizes are bounded (kLoopMax*); the caller rejects larger
// loops.
#pragma once

#include <cmath>
#include <cuda_runtime.h>

namespace oc {

constexpr int kLoopMaxPts = 48;                          // polygon vertices
constexpr int kLoopMaxSteiner = 12;                      // Steiner points
constexpr int kLoopMaxV = kLoopMaxPts + kLoopMaxSteiner;
constexpr int kLoopMaxTri = kLoopMaxPts - 2 + 2 * kLoopMaxSteiner;
constexpr int kLoopMaxQueue = 4 * kLoopMaxTri;

// status bits of loop_mesh
constexpr int kLoopOk = 0;
constexpr int kLoopBadInput = 1;      // too many points, or fewer than 3
constexpr int kLoopNoEar = 2;         // not a simple polygon (no ear found)
constexpr int kLoopFlipCap = 4;       // flip loop bound reached
constexpr int kLoopSteinerCap = 8;    // refinement stopped at kLoopMaxSteiner (mesh valid)
constexpr int kLoopQueueCap = 16;     // bad-triangle queue full (mesh valid)

struct LoopMesh {
    int nV = 0, nT = 0;
    double2 P[kLoopMaxV];
    short T[kLoopMaxTri][3];   // counter-clockwise
    short N[kLoopMaxTri][3];   // triangle across edge (T[k], T[k+1]); -1 on the polygon
};

namespace loopmesh {

// ---- exact orientation: error-free transforms and expansion sums
// (Shewchuk, "Adaptive precision floating-point arithmetic and fast robust
// geometric predicates", 1997)
__host__ __device__ inline void two_sum(double a, double b, double& s, double& e)
{
    s = a + b;
    const double bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

__host__ __device__ inline void two_prod(double a, double b, double& p, double& e)
{
    p = a * b;
    e = fma(a, b, -p);
}

// sign of the exact sum of x[0..n): grow a nonoverlapping expansion
__host__ __device__ inline int expansion_sign(const double* x, int n)
{
    double e[16];
    int m = 0;
    for (int i = 0; i < n; ++i) {
        double q = x[i];
        int k = 0;
        for (int j = 0; j < m; ++j) {
            double s, h;
            two_sum(q, e[j], s, h);
            q = s;
            if (h != 0.0) e[k++] = h;
        }
        if (q != 0.0) e[k++] = q;
        m = k;
    }
    if (m == 0) return 0;
    return e[m - 1] > 0.0 ? 1 : -1;
}

// > 0 when a, b, c turn counter-clockwise
__host__ __device__ inline int orient(double2 a, double2 b, double2 c)
{
    const double l = (b.x - a.x) * (c.y - a.y);
    const double r = (b.y - a.y) * (c.x - a.x);
    const double det = l - r;
    const double bound = 3.3306690738754716e-16 * (fabs(l) + fabs(r));   // (3 + 16 eps) eps
    if (det > bound) return 1;
    if (-det > bound) return -1;
    // det = bx cy - bx ay - ax cy - by cx + by ax + ay cx, each product exact
    double t[12];
    two_prod(b.x, c.y, t[0], t[1]);
    two_prod(-b.x, a.y, t[2], t[3]);
    two_prod(-a.x, c.y, t[4], t[5]);
    two_prod(-b.y, c.x, t[6], t[7]);
    two_prod(b.y, a.x, t[8], t[9]);
    two_prod(a.y, c.x, t[10], t[11]);
    return expansion_sign(t, 12);
}

// ---- in-circle with a double-double fallback
struct dd {
    double hi, lo;
};
__host__ __device__ inline dd dd_from(double a) { return {a, 0.0}; }
__host__ __device__ inline dd dd_add(dd a, dd b)
{
    double s, e;
    two_sum(a.hi, b.hi, s, e);
    e += a.lo + b.lo;
    double h, l;
    two_sum(s, e, h, l);
    return {h, l};
}
__host__ __device__ inline dd dd_neg(dd a) { return {-a.hi, -a.lo}; }
__host__ __device__ inline dd dd_mul(dd a, dd b)
{
    double p, e;
    two_prod(a.hi, b.hi, p, e);
    e += a.hi * b.lo + a.lo * b.hi;
    double h, l;
    two_sum(p, e, h, l);
    return {h, l};
}
__host__ __device__ inline dd dd_diff(double a, double b)
{
    double s, e;
    two_sum(a, -b, s, e);
    return {s, e};
}

// > 0 when d lies inside the circle through the counter-clockwise a, b, c
__host__ __device__ inline int incircle(double2 a, double2 b, double2 c, double2 d)
{
    const double adx = a.x - d.x, ady = a.y - d.y;
    const double bdx = b.x - d.x, bdy = b.y - d.y;
    const double cdx = c.x - d.x, cdy = c.y - d.y;
    const double alift = adx * adx + ady * ady;
    const double blift = bdx * bdx + bdy * bdy;
    const double clift = cdx * cdx + cdy * cdy;
    const double t1 = bdx * cdy - bdy * cdx, t2 = cdx * ady - cdy * adx, t3 = adx * bdy - ady * bdx;
    const double det = alift * t1 + blift * t2 + clift * t3;
    const double perm = (fabs(bdx * cdy) + fabs(bdy * cdx)) * alift + (fabs(cdx * ady) + fabs(cdy * adx)) * blift +
                        (fabs(adx * bdy) + fabs(ady * bdx)) * clift;
    const double bound = 1.2e-15 * perm;   // above (10 + 96 eps) eps
    if (det > bound) return 1;
    if (-det > bound) return -1;
    const dd ax = dd_diff(a.x, d.x), ay = dd_diff(a.y, d.y);
    const dd bx = dd_diff(b.x, d.x), by = dd_diff(b.y, d.y);
    const dd cx = dd_diff(c.x, d.x), cy = dd_diff(c.y, d.y);
    const dd al = dd_add(dd_mul(ax, ax), dd_mul(ay, ay));
    const dd bl = dd_add(dd_mul(bx, bx), dd_mul(by, by));
    const dd cl = dd_add(dd_mul(cx, cx), dd_mul(cy, cy));
    const dd u1 = dd_add(dd_mul(bx, cy), dd_neg(dd_mul(by, cx)));
    const dd u2 = dd_add(dd_mul(cx, ay), dd_neg(dd_mul(cy, ax)));
    const dd u3 = dd_add(dd_mul(ax, by), dd_neg(dd_mul(ay, bx)));
    const dd r = dd_add(dd_add(dd_mul(al, u1), dd_mul(bl, u2)), dd_mul(cl, u3));
    const double v = r.hi + r.lo;
    if (fabs(v) <= 1e-28 * perm) return 0;
    return v > 0.0 ? 1 : -1;
}

__host__ __device__ inline double sqd(double2 a, double2 b)
{
    const double dx = a.x - b.x, dy = a.y - b.y;
    return dx * dx + dy * dy;
}

// cos^2 of the minimum angle (20 degrees) and the off-center constant
constexpr double kGoodAngle = 0.8830222215594891;     // cos(20 deg)^2
constexpr double kOffConstant = 2.6938588643184125;   // 0.475 sqrt((1 + cos 20) / (1 - cos 20))

__host__ __device__ inline int edge_of(const LoopMesh& M, int t, int a, int b)
{
    for (int k = 0; k < 3; ++k)
        if (M.T[t][k] == a && M.T[t][(k + 1) % 3] == b) return k;
    return -1;
}

// neighbour links of every triangle from scratch (small meshes)
__host__ __device__ inline void link_all(LoopMesh& M)
{
    for (int t = 0; t < M.nT; ++t)
        for (int k = 0; k < 3; ++k) {
            const int a = M.T[t][k], b = M.T[t][(k + 1) % 3];
            int nb = -1;
            for (int u = 0; u < M.nT && nb < 0; ++u)
                if (u != t && edge_of(M, u, b, a) >= 0) nb = u;
            M.N[t][k] = static_cast<short>(nb);
        }
}

// point the neighbour of t across (a, b) -- now u -- at u
__host__ __device__ inline void relink(LoopMesh& M, int t, int a, int b, int u)
{
    if (t < 0) return;
    const int k = edge_of(M, t, b, a);
    if (k >= 0) M.N[t][k] = static_cast<short>(u);
}

// flips edge k of t (shared with triangle s): (a b c) + (b a d) -> (d c a) + (c d b)
__host__ __device__ inline void flip(LoopMesh& M, int t, int k)
{
    const int s = M.N[t][k];
    const int a = M.T[t][k], b = M.T[t][(k + 1) % 3], c = M.T[t][(k + 2) % 3];
    const int ks = edge_of(M, s, b, a);
    const int d = M.T[s][(ks + 2) % 3];
    const int nBC = M.N[t][(k + 1) % 3], nCA = M.N[t][(k + 2) % 3];
    const int nAD = M.N[s][(ks + 1) % 3], nDB = M.N[s][(ks + 2) % 3];
    M.T[t][0] = static_cast<short>(d); M.T[t][1] = static_cast<short>(c); M.T[t][2] = static_cast<short>(a);
    M.T[s][0] = static_cast<short>(c); M.T[s][1] = static_cast<short>(d); M.T[s][2] = static_cast<short>(b);
    // t = (d c a): edges dc -> s, ca -> nCA, ad -> nAD
    M.N[t][0] = static_cast<short>(s); M.N[t][1] = static_cast<short>(nCA); M.N[t][2] = static_cast<short>(nAD);
    // s = (c d b): edges cd -> t, db -> nDB, bc -> nBC
    M.N[s][0] = static_cast<short>(t); M.N[s][1] = static_cast<short>(nDB); M.N[s][2] = static_cast<short>(nBC);
    relink(M, nAD, a, d, t);
    relink(M, nBC, b, c, s);
}

// edge k of t is interior and not locally Delaunay (strictly convex quad)
__host__ __device__ inline bool illegal(const LoopMesh& M, int t, int k)
{
    const int s = M.N[t][k];
    if (s < 0) return false;
    const int a = M.T[t][k], b = M.T[t][(k + 1) % 3], c = M.T[t][(k + 2) % 3];
    const int ks = edge_of(M, s, b, a);
    const int d = M.T[s][(ks + 2) % 3];
    if (incircle(M.P[a], M.P[b], M.P[c], M.P[d]) <= 0) return false;
    return orient(M.P[c], M.P[a], M.P[d]) > 0 && orient(M.P[d], M.P[b], M.P[c]) > 0;
}

// Triangle's quality test (minimum angle below 20 degrees); key: squared
// length of the shortest edge
__host__ __device__ inline bool bad_triangle(const LoopMesh& M, int t, double& key)
{
    const double2 o = M.P[M.T[t][0]], d = M.P[M.T[t][1]], a = M.P[M.T[t][2]];
    const double dxod = o.x - d.x, dyod = o.y - d.y;
    const double dxda = d.x - a.x, dyda = d.y - a.y;
    const double dxao = a.x - o.x, dyao = a.y - o.y;
    const double apexlen = dxod * dxod + dyod * dyod;
    const double orglen = dxda * dxda + dyda * dyda;
    const double destlen = dxao * dxao + dyao * dyao;
    double angle;
    if (apexlen < orglen && apexlen < destlen) {
        key = apexlen;
        angle = dxda * dxao + dyda * dyao;
        angle = angle * angle / (orglen * destlen);
    }
    else if (orglen < destlen) {
        key = orglen;
        angle = dxod * dxao + dyod * dyao;
        angle = angle * angle / (apexlen * destlen);
    }
    else {
        key = destlen;
        angle = dxod * dxda + dyod * dyda;
        angle = angle * angle / (apexlen * orglen);
    }
    return angle > kGoodAngle;
}

// queue bin of a squared shortest edge: half-octaves, shortest first
__host__ __device__ inline int queue_bin(double key)
{
    int e = 0;
    (void)frexp(key, &e);
    const double m = ldexp(key, -e);   // [0.5, 1)
    return 2 * e + (m > 0.70710678118654752 ? 1 : 0);
}

struct BadQueue {
    int n = 0, seq = 0;
    short v[kLoopMaxQueue][3];
    int bin[kLoopMaxQueue], order[kLoopMaxQueue];
};

__host__ __device__ inline bool enqueue(BadQueue& Q, const LoopMesh& M, int t, double key)
{
    if (Q.n >= kLoopMaxQueue) return false;
    for (int k = 0; k < 3; ++k) Q.v[Q.n][k] = M.T[t][k];
    Q.bin[Q.n] = queue_bin(key);
    Q.order[Q.n] = Q.seq++;
    ++Q.n;
    return true;
}

// smallest bin first, then insertion order
__host__ __device__ inline int dequeue(BadQueue& Q, short out[3])
{
    if (Q.n == 0) return 0;
    int best = 0;
    for (int i = 1; i < Q.n; ++i)
        if (Q.bin[i] < Q.bin[best] || (Q.bin[i] == Q.bin[best] && Q.order[i] < Q.order[best])) best = i;
    for (int k = 0; k < 3; ++k) out[k] = Q.v[best][k];
    --Q.n;
    for (int k = 0; k < 3; ++k) Q.v[best][k] = Q.v[Q.n][k];
    Q.bin[best] = Q.bin[Q.n];
    Q.order[best] = Q.order[Q.n];
    return 1;
}

// triangle with exactly this (org, dest, apex), or -1
__host__ __device__ inline int find_tri(const LoopMesh& M, const short v[3])
{
    for (int t = 0; t < M.nT; ++t)
        if (M.T[t][0] == v[0] && M.T[t][1] == v[1] && M.T[t][2] == v[2]) return t;
    return -1;
}

// circumcenter, or Triangle's off-center when that is closer to the
// shortest edge (findcircumcenter with offcenter on)
__host__ __device__ inline double2 split_point(double2 o, double2 d, double2 a)
{
    const double xdo = d.x - o.x, ydo = d.y - o.y;
    const double xao = a.x - o.x, yao = a.y - o.y;
    const double dodist = xdo * xdo + ydo * ydo;
    const double aodist = xao * xao + yao * yao;
    const double dadist = (d.x - a.x) * (d.x - a.x) + (d.y - a.y) * (d.y - a.y);
    const double den = 0.5 / (xdo * yao - xao * ydo);
    double dx = (yao * dodist - ydo * aodist) * den;
    double dy = (xdo * aodist - xao * dodist) * den;
    if (dodist < aodist && dodist < dadist) {
        const double ox = 0.5 * xdo - kOffConstant * ydo, oy = 0.5 * ydo + kOffConstant * xdo;
        if (ox * ox + oy * oy < dx * dx + dy * dy) { dx = ox; dy = oy; }
    }
    else if (aodist < dadist) {
        const double ox = 0.5 * xao + kOffConstant * yao, oy = 0.5 * yao - kOffConstant * xao;
        if (ox * ox + oy * oy < dx * dx + dy * dy) { dx = ox; dy = oy; }
    }
    else {
        const double ox = 0.5 * (a.x - d.x) - kOffConstant * (a.y - d.y);
        const double oy = 0.5 * (a.y - d.y) + kOffConstant * (a.x - d.x);
        if (ox * ox + oy * oy < (dx - xdo) * (dx - xdo) + (dy - ydo) * (dy - ydo)) { dx = xdo + ox; dy = ydo + oy; }
    }
    return make_double2(o.x + dx, o.y + dy);
}

// polygon edge (a, b) encroached by apex p: inside its diametral lens
__host__ __device__ inline bool encroaches(double2 a, double2 b, double2 p)
{
    const double dot = (a.x - p.x) * (b.x - p.x) + (a.y - p.y) * (b.y - p.y);
    if (!(dot < 0.0)) return false;
    const double g = 2.0 * kGoodAngle - 1.0;
    return dot * dot >= g * g * sqd(a, p) * sqd(b, p);
}

} // namespace loopmesh

// Triangulates the simple polygon pts[0..L) (either orientation) into M:
// M.P starts with the polygon's points in their order, Steiner points
// follow; triangles counter-clockwise.  Returns kLoopOk or status bits
// (kLoopBadInput / kLoopNoEar / kLoopFlipCap: no mesh; kLoopSteinerCap /
// kLoopQueueCap: a valid mesh whose refinement stopped early).  Q and B are
// the caller's scratch (a bad-triangle queue and an undo copy).
__host__ __device__ inline int loop_mesh(const double2* pts, int L, int maxSteiner, LoopMesh& M, LoopMesh& B,
                                         loopmesh::BadQueue& Q)
{
    using namespace loopmesh;
    M.nV = 0;
    M.nT = 0;
    if (L < 3 || L > kLoopMaxPts) return kLoopBadInput;
    if (maxSteiner > kLoopMaxSteiner) maxSteiner = kLoopMaxSteiner;
    for (int i = 0; i < L; ++i) M.P[i] = pts[i];
    M.nV = L;
    // polygon orientation (shoelace, relative to the first point)
    double area2 = 0.0;
    for (int i = 1; i + 1 < L; ++i)
        area2 += (pts[i].x - pts[0].x) * (pts[i + 1].y - pts[0].y) - (pts[i].y - pts[0].y) * (pts[i + 1].x - pts[0].x);
    const bool ccw = area2 > 0.0;
    // ear clipping over a counter-clockwise index ring; only vertices that
    // are not strictly convex can lie in an ear, so only they are tested
    short ring[kLoopMaxPts];
    signed char convex[kLoopMaxPts];   // by ring position
    int n = L;
    for (int i = 0; i < L; ++i) ring[i] = static_cast<short>(ccw ? i : L - 1 - i);
    for (int i = 0; i < n; ++i)
        convex[i] = orient(M.P[ring[(i + n - 1) % n]], M.P[ring[i]], M.P[ring[(i + 1) % n]]) > 0 ? 1 : 0;
    int guard = 0;
    while (n > 3) {
        bool clipped = false;
        for (int i = 0; i < n && !clipped; ++i) {
            if (!convex[i]) continue;   // reflex or flat
            const int ip = ring[(i + n - 1) % n], iv = ring[i], in = ring[(i + 1) % n];
            const double2 p = M.P[ip], v = M.P[iv], q = M.P[in];
            bool ear = true;
            for (int j = 0; j < n && ear; ++j) {
                if (convex[j]) continue;
                const int w = ring[j];
                if (w == ip || w == iv || w == in) continue;
                const double2 x = M.P[w];
                if (orient(p, v, x) >= 0 && orient(v, q, x) >= 0 && orient(q, p, x) >= 0) ear = false;
            }
            if (!ear) continue;
            M.T[M.nT][0] = static_cast<short>(ip);
            M.T[M.nT][1] = static_cast<short>(iv);
            M.T[M.nT][2] = static_cast<short>(in);
            ++M.nT;
            for (int j = i; j + 1 < n; ++j) {
                ring[j] = ring[j + 1];
                convex[j] = convex[j + 1];
            }
            --n;
            // the two neighbours' corners changed
            const int a = (i + n - 1) % n, b = i % n;
            convex[a] = orient(M.P[ring[(a + n - 1) % n]], M.P[ring[a]], M.P[ring[(a + 1) % n]]) > 0 ? 1 : 0;
            convex[b] = orient(M.P[ring[(b + n - 1) % n]], M.P[ring[b]], M.P[ring[(b + 1) % n]]) > 0 ? 1 : 0;
            clipped = true;
        }
        if (!clipped || ++guard > kLoopMaxPts) return kLoopNoEar;
    }
    if (orient(M.P[ring[0]], M.P[ring[1]], M.P[ring[2]]) <= 0) return kLoopNoEar;
    M.T[M.nT][0] = ring[0];
    M.T[M.nT][1] = ring[1];
    M.T[M.nT][2] = ring[2];
    ++M.nT;
    link_all(M);
    // Lawson flips to the constrained Delaunay triangulation (the polygon's
    // edges have no neighbour and are never flipped): every interior edge
    // once, then the outer edges of each flipped quad again
    {
        short stk[6 * kLoopMaxTri][2];   // (triangle, its lower-numbered vertex of the edge)
        int sp = 0;
        for (int t = 0; t < M.nT; ++t)
            for (int k = 0; k < 3; ++k)
                if (M.N[t][k] > t) {
                    stk[sp][0] = static_cast<short>(t);
                    stk[sp][1] = M.T[t][k];
                    ++sp;
                }
        int flips = 0;
        while (sp > 0) {
            --sp;
            const int t = stk[sp][0], a = stk[sp][1];
            int k = -1;
            for (int q = 0; q < 3; ++q)
                if (M.T[t][q] == a) k = q;
            if (k < 0 || M.N[t][k] < 0 || !illegal(M, t, k)) continue;
            const int s2 = M.N[t][k];
            flip(M, t, k);
            if (++flips > 4 * kLoopMaxTri * kLoopMaxTri) return kLoopFlipCap;
            // t = (d c a), s2 = (c d b): their edges other than (d, c)
            if (sp + 4 > 6 * kLoopMaxTri) return kLoopFlipCap;
            for (int q = 1; q < 3; ++q) {
                stk[sp][0] = static_cast<short>(t);
                stk[sp][1] = M.T[t][q];
                ++sp;
                stk[sp][0] = static_cast<short>(s2);
                stk[sp][1] = M.T[s2][q];
                ++sp;
            }
        }
    }
    if (maxSteiner <= 0) return kLoopOk;
    // refinement
    int status = kLoopOk;
    Q.n = 0;
    Q.seq = 0;
    for (int t = 0; t < M.nT; ++t) {
        double key;
        if (bad_triangle(M, t, key) && !enqueue(Q, M, t, key)) status |= kLoopQueueCap;
    }
    short tv[3];
    int steps = 0;
    while (dequeue(Q, tv)) {
        if (++steps > 64 * kLoopMaxQueue) break;
        const int t0 = find_tri(M, tv);
        if (t0 < 0) continue;   // no longer there
        if (M.nV - L >= maxSteiner) {
            status |= kLoopSteinerCap;
            break;
        }
        const double2 o = M.P[tv[0]], d = M.P[tv[1]], a = M.P[tv[2]];
        const double2 x = split_point(o, d, a);
        bool dup = false;
        for (int v = 0; v < M.nV && !dup; ++v) dup = M.P[v].x == x.x && M.P[v].y == x.y;
        if (dup) continue;   // an existing vertex is there
        // locate x by walking from t0; leaving through a polygon edge or
        // landing on one rejects it
        int t = t0, onEdge = -1;
        bool outside = false;
        for (int w = 0; w <= 2 * kLoopMaxTri; ++w) {
            int exitK = -1;
            onEdge = -1;
            for (int k = 0; k < 3 && exitK < 0; ++k) {
                const int s = orient(M.P[M.T[t][k]], M.P[M.T[t][(k + 1) % 3]], x);
                if (s < 0) exitK = k;
                else if (s == 0) onEdge = k;
            }
            if (exitK < 0) break;
            if (M.N[t][exitK] < 0) {
                outside = true;
                break;
            }
            t = M.N[t][exitK];
            if (w == 2 * kLoopMaxTri) outside = true;
        }
        if (outside) continue;
        if (onEdge >= 0 && M.N[t][onEdge] < 0) continue;   // on the polygon
        B = M;
        const int xv = M.nV++;
        M.P[xv] = x;
        // split: 1 -> 3 inside a triangle, 2 -> 4 on an interior edge
        int stack[3 * kLoopMaxTri];
        int sp = 0;
        if (onEdge < 0) {
            const int A = M.T[t][0], Bv = M.T[t][1], C = M.T[t][2];
            const int nAB = M.N[t][0], nBC = M.N[t][1], nCA = M.N[t][2];
            const int t1 = M.nT, t2 = M.nT + 1;
            M.nT += 2;
            M.T[t][0] = static_cast<short>(A); M.T[t][1] = static_cast<short>(Bv); M.T[t][2] = static_cast<short>(xv);
            M.T[t1][0] = static_cast<short>(Bv); M.T[t1][1] = static_cast<short>(C); M.T[t1][2] = static_cast<short>(xv);
            M.T[t2][0] = static_cast<short>(C); M.T[t2][1] = static_cast<short>(A); M.T[t2][2] = static_cast<short>(xv);
            M.N[t][0] = static_cast<short>(nAB); M.N[t][1] = static_cast<short>(t1); M.N[t][2] = static_cast<short>(t2);
            M.N[t1][0] = static_cast<short>(nBC); M.N[t1][1] = static_cast<short>(t2); M.N[t1][2] = static_cast<short>(t);
            M.N[t2][0] = static_cast<short>(nCA); M.N[t2][1] = static_cast<short>(t); M.N[t2][2] = static_cast<short>(t1);
            relink(M, nBC, Bv, C, t1);
            relink(M, nCA, C, A, t2);
            stack[sp++] = t;
            stack[sp++] = t1;
            stack[sp++] = t2;
        }
        else {
            const int k = onEdge;
            const int s = M.N[t][k];
            const int A = M.T[t][k], Bv = M.T[t][(k + 1) % 3], C = M.T[t][(k + 2) % 3];
            const int ks = edge_of(M, s, Bv, A);
            const int D = M.T[s][(ks + 2) % 3];
            const int nBC = M.N[t][(k + 1) % 3], nCA = M.N[t][(k + 2) % 3];
            const int nAD = M.N[s][(ks + 1) % 3], nDB = M.N[s][(ks + 2) % 3];
            const int t1 = M.nT, s1 = M.nT + 1;
            M.nT += 2;
            // t = (x C A), t1 = (x B C), s = (x A D), s1 = (x D B)
            M.T[t][0] = static_cast<short>(xv); M.T[t][1] = static_cast<short>(C); M.T[t][2] = static_cast<short>(A);
            M.T[t1][0] = static_cast<short>(xv); M.T[t1][1] = static_cast<short>(Bv); M.T[t1][2] = static_cast<short>(C);
            M.T[s][0] = static_cast<short>(xv); M.T[s][1] = static_cast<short>(A); M.T[s][2] = static_cast<short>(D);
            M.T[s1][0] = static_cast<short>(xv); M.T[s1][1] = static_cast<short>(D); M.T[s1][2] = static_cast<short>(Bv);
            M.N[t][0] = static_cast<short>(t1); M.N[t][1] = static_cast<short>(nCA); M.N[t][2] = static_cast<short>(s);
            M.N[t1][0] = static_cast<short>(s1); M.N[t1][1] = static_cast<short>(nBC); M.N[t1][2] = static_cast<short>(t);
            M.N[s][0] = static_cast<short>(t); M.N[s][1] = static_cast<short>(nAD); M.N[s][2] = static_cast<short>(s1);
            M.N[s1][0] = static_cast<short>(s); M.N[s1][1] = static_cast<short>(nDB); M.N[s1][2] = static_cast<short>(t1);
            relink(M, nBC, Bv, C, t1);
            relink(M, nDB, D, Bv, s1);
            stack[sp++] = t;
            stack[sp++] = t1;
            stack[sp++] = s;
            stack[sp++] = s1;
        }
        // legalize the edges opposite x
        int flips = 0;
        bool rejected = false;
        while (sp > 0 && !rejected) {
            const int u = stack[--sp];
            int k = -1;
            for (int q = 0; q < 3; ++q)
                if (M.T[u][q] == xv) k = (q + 1) % 3;   // edge opposite x
            if (k < 0) continue;
            if (M.N[u][k] < 0) {
                // a polygon edge: not flipped; x must not encroach it
                if (encroaches(M.P[M.T[u][k]], M.P[M.T[u][(k + 1) % 3]], x)) rejected = true;
                continue;
            }
            if (illegal(M, u, k)) {
                const int s = M.N[u][k];
                flip(M, u, k);
                // u = (d c a) with c == x: the new outer edges are in u and s
                stack[sp++] = u;
                stack[sp++] = s;
                if (++flips > 8 * kLoopMaxTri) rejected = true;
            }
        }
        if (rejected) {
            M = B;
            continue;
        }
        // the triangles around x: enqueue the bad ones
        for (int u = 0; u < M.nT; ++u) {
            if (M.T[u][0] != xv && M.T[u][1] != xv && M.T[u][2] != xv) continue;
            double key;
            if (bad_triangle(M, u, key) && !enqueue(Q, M, u, key)) status |= kLoopQueueCap;
        }
    }
    return status;
}

} // namespace oc
