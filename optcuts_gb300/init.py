"""Initial cut and Tutte embedding -- the caller that produces the geometry
step's starting state.

Restates the "no input UV" initialisation of the reference's src/main.cpp
(lines 1379-1534) for the cases this library handles:

* a closed genus-0 single-component mesh: one-point cut at the first
  vertex of the first triangle (TriMesh::onePointCut, TriMesh.cpp:1054-1074,
  through the interior branch of TriMesh::cutPath, TriMesh.cpp:1449-1500);
* a single component of genus >= 1: the reference's cut_to_disk loop
  (main.cpp:1397-1484, cut_to_disk below, TriMesh::cutPath through the
  library's topology operations);
* a topological disk: no cut.

then the boundary loop (igl::boundary_loop: smallest boundary vertex first,
following boundary half-edges), arc-length placement on the unit circle
(igl::map_vertices_to_circle) and the harmonic map with the reference's
uniform Laplacian (IglUtils::computeUniformLaplacian, IglUtils.cpp:39-60).
The result is the TriMesh the reference builds with
``TriMesh(V, F, UV_Tutte, F_cut, false)`` (main.cpp:1534, TriMesh.cpp:122-189):
the rest positions are re-indexed to the cut mesh and vertex 0 is fixed.

Several components are handled as the reference handles them: each cut by
its own Euler characteristic, their UV disks on a grid.
"""
from __future__ import annotations

import numpy as np


class InitState:
    def __init__(self, V_rest, UV, F, fixed, cut_path, bnd, cohE):
        self.V_rest = V_rest
        self.UV = UV
        self.F = F
        self.fixedVert = fixed
        self.cut_path = cut_path
        self.bnd = bnd
        self.cohE = cohE


def cohesive_edges(F_mesh, F_uv):
    """Cohesive-edge pairs of a cut mesh (TriMesh.cpp:128-166): for every
    UV-boundary half-edge (a, b) of F_uv whose surface half-edge is interior,
    the row (a, b, c, d) with (c, d) the opposite side's UV vertices; each
    surface edge is recorded once, in triangle / edge order."""
    F_mesh = np.asarray(F_mesh)
    F_uv = np.asarray(F_uv)
    he_uv = set()
    he = {}
    for t in range(len(F_uv)):
        for e in range(3):
            he_uv.add((int(F_uv[t, e]), int(F_uv[t, (e + 1) % 3])))
            he[(int(F_mesh[t, e]), int(F_mesh[t, (e + 1) % 3]))] = (t, e)
    rows = []
    for t in range(len(F_uv)):
        for e in range(3):
            a, b = int(F_uv[t, e]), int(F_uv[t, (e + 1) % 3])
            if (b, a) in he_uv:
                continue
            key = (int(F_mesh[t, (e + 1) % 3]), int(F_mesh[t, e]))
            if key in he:
                t2, e2 = he[key]
                rows.append([a, b, int(F_uv[t2, (e2 + 1) % 3]), int(F_uv[t2, e2])])
                he.pop((int(F_mesh[t, e]), int(F_mesh[t, (e + 1) % 3])), None)
    return np.asarray(rows, np.int32).reshape(-1, 4)


def seam_sparsity(V_rest, UV, cohE, avg_edge_len, init_seam_len=0.0, tri_soup=False):
    """TriMesh::computeSeamSparsity (TriMesh.cpp:1542-1558): total rest length
    of the interior cohesive edges (in tri-soup mode only those whose UV
    copies separated by more than 1% of the average edge length), plus the
    initial seam length.  Divide by virtualRadius for E_se."""
    V_rest = np.asarray(V_rest)
    cohE = np.asarray(cohE).reshape(-1, 4)
    s = 0.0
    for row in cohE:
        if row.min() < 0:
            continue
        if tri_soup:
            UVa = np.asarray(UV)
            if not (np.linalg.norm(UVa[row[0]] - UVa[row[2]]) / avg_edge_len > 1e-2 or
                    np.linalg.norm(UVa[row[1]] - UVa[row[3]]) / avg_edge_len > 1e-2):
                continue
        s += float(np.linalg.norm(V_rest[row[0]] - V_rest[row[1]]))
    return s + init_seam_len


def euler_characteristic(V, F):
    F = np.asarray(F)
    e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    nE = len(np.unique(e[:, 0].astype(np.int64) * (F.max() + 1) + e[:, 1]))
    nV = len(np.unique(F))
    return nV - nE + len(F)


def one_point_cut(V, F, vI=None):
    """Split vertex vI (default F[0,0]) along path [n0, vI, n2] (n0, n2: its
    first and third neighbours in index order).  Returns (V', F', path)."""
    F = np.array(F, np.int32, copy=True)
    vI = int(F[0, 0]) if vI is None else int(vI)
    nbrs = set()
    inc = np.nonzero((F == vI).any(axis=1))[0]
    for t in inc:
        for v in F[t]:
            if v != vI:
                nbrs.add(int(v))
    nb = sorted(nbrs)
    if len(nb) < 3:
        raise ValueError("one-point cut needs a vertex of valence >= 3")
    path = [nb[0], vI, nb[2]]
    # directed edge (a, b) -> triangle containing it
    e2t = {}
    for t in inc:
        a, b, c = (int(x) for x in F[t])
        e2t[(a, b)] = t
        e2t[(b, c)] = t
        e2t[(c, a)] = t
    tri_left = []
    v_new = path[0]
    for _ in range(len(inc) + 1):
        t = e2t[(vI, v_new)]
        tri_left.append(t)
        v_new = next(int(x) for x in F[t] if x != vI and x != v_new)
        if v_new == path[2]:
            break
        if v_new == path[0]:
            raise ValueError("not a valid cut path")
    nV = len(V)
    V2 = np.vstack([V, V[vI:vI + 1]])
    for t in tri_left:
        F[t][F[t] == vI] = nV
    return V2, F, path


def facet_components(F):
    """Component label of every triangle (triangles sharing an edge are
    connected; igl::facet_components), labels in order of first appearance."""
    F = np.asarray(F)
    n = len(F)
    parent = np.arange(n)

    def root(a):
        while parent[a] != a:
            parent[a] = parent[parent[a]]
            a = parent[a]
        return a
    edge = {}
    for t in range(n):
        for k in range(3):
            a, b = int(F[t, k]), int(F[t, (k + 1) % 3])
            key = (min(a, b), max(a, b))
            if key in edge:
                ra, rb = root(edge[key]), root(t)
                if ra != rb:
                    parent[max(ra, rb)] = min(ra, rb)
            else:
                edge[key] = t
    labels, C = {}, np.zeros(n, np.int64)
    for t in range(n):
        r = root(t)
        if r not in labels:
            labels[r] = len(labels)
        C[t] = labels[r]
    return C


def cut_to_disk(F):
    """The cut graph the reference's initialisation asks for on a surface of
    genus >= 1 (igl::cut_to_disk as vendored in src/Utils/cut_to_disk.cpp):

    1. edges numbered in (min, max) vertex order; faces are peeled from each
       not yet deleted face outwards, a face being deleted through an
       interior edge with exactly one deleted neighbour (a breadth-first
       queue of such edges);
    2. the edges left form a graph whose degree-1 vertices are pruned
       repeatedly (a queue, vertices in index order);
    3. the remaining edges are walked into cycles (a walk that meets its own
       vertex again: the cut is the loop from that vertex, closed) or, after
       a dead end and a walk the other way from the reversed list, chains.

    Returns the cuts as vertex lists (a closed loop repeats its first
    vertex).  Step 3 keeps the source's vertex-position map across the
    reversal, so a cycle found on the second walk is read from the reversed
    list with the first walk's positions.  Computed on the host by the
    library (oc_cut_to_disk)."""
    from optcuts_gb300 import cut_to_disk as lib_cut_to_disk
    F = np.asarray(F)
    if len(F) == 0:
        return []
    return lib_cut_to_disk(F)


def cut_path(path, V_rest, UV, F, cohE):
    """TriMesh::cutPath(path, makeCoh = true) (TriMesh.cpp:1393-1517) as the
    initialisation calls it: from a boundary end, every interior edge of the
    path split on the boundary in turn (cut through where both of its ends
    are on the boundary); for an interior path, the interior cut of its
    first three vertices, then its remaining edges split on the boundary.
    The library's topology operations, applied by topology_cut_path on the
    faces around each edge.  Returns the new arrays and the number of edges
    split."""
    from optcuts_gb300 import topology_cut_path
    return topology_cut_path([int(v) for v in path], V_rest, UV, F, cohE)


def cut_high_genus(V, F):
    """The reference's initial cutting of one component of genus >= 1
    (main.cpp:1397-1484): cut_to_disk on the current mesh, then the first of
    its seams that cuts anything (a closed loop first through the interior
    cut of its last three vertices, then the rest of it), repeated until the
    component is a disk.  Returns (V_rest, F) of the cut mesh."""
    V_rest = np.asarray(V, np.float64)
    F = np.asarray(F, np.int32)
    UV = np.zeros((len(V_rest), 2))
    cohE = np.zeros((0, 4), np.int32)
    for _ in range(10000):
        ec = euler_characteristic(V_rest, F)
        if ec == 1:
            return V_rest, F
        if ec > 1:
            raise NotImplementedError("a component turned closed genus 0 while being cut")
        V_rest, UV, F, cohE, made = cut_component_once(F, V_rest, UV, F, cohE)
        if not made:
            raise ValueError("no cut made while cutting to a disk")
    raise ValueError("cutting to a disk did not finish")


def cut_component_once(F_comp, V_rest, UV, F, cohE):
    """One pass of the reference's cut_to_disk loop for one component
    (main.cpp:1423-1451): the component's cut graph, then the first seam
    that cuts anything applied to the whole mesh."""
    made = 0
    for seam in cut_to_disk(F_comp):
        seam = list(seam)
        if seam[0] == seam[-1]:
            # (an interior cut of three vertices counts no split, as in cutPath)
            V_rest, UV, F, cohE, m = cut_path(seam[-3:], V_rest, UV, F, cohE)
            made += m
            seam = seam[:-2]
        V_rest, UV, F, cohE, m = cut_path(seam, V_rest, UV, F, cohE)
        made += m
        if made:
            break
    return V_rest, UV, F, cohE, made


def boundary_loops(F):
    """igl::boundary_loop's loops: each starts at the smallest boundary
    vertex not yet on a loop and follows the boundary half-edges."""
    F = np.asarray(F)
    he = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    key = he[:, 0].astype(np.int64) * (F.max() + 1) + he[:, 1]
    rkey = he[:, 1].astype(np.int64) * (F.max() + 1) + he[:, 0]
    bhe = he[~np.isin(key, rkey)]
    nxt = {}
    for a, b in bhe.tolist():
        nxt.setdefault(a, b)
    loops, seen = [], set()
    for start in sorted(nxt):
        if start in seen:
            continue
        loop = [start]
        seen.add(start)
        v = nxt[start]
        while v not in seen and v in nxt:
            loop.append(v)
            seen.add(v)
            v = nxt[v]
        loops.append(loop)
    return loops


def boundary_loop(F):
    """igl::boundary_loop for a single-boundary manifold: start at the
    smallest boundary vertex, follow the boundary half-edges."""
    F = np.asarray(F)
    he = np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]])
    key = he[:, 0].astype(np.int64) * (F.max() + 1) + he[:, 1]
    rkey = he[:, 1].astype(np.int64) * (F.max() + 1) + he[:, 0]
    bmask = ~np.isin(key, rkey)
    bhe = he[bmask]
    if len(bhe) == 0:
        return []
    nxt = dict(zip(bhe[:, 0].tolist(), bhe[:, 1].tolist()))
    start = int(min(nxt))
    loop = [start]
    v = nxt[start]
    while v != start and len(loop) <= len(bhe):
        loop.append(v)
        v = nxt[v]
    return loop


def map_vertices_to_circle(V, bnd):
    P = V[bnd]
    seg = np.linalg.norm(P[1:] - P[:-1], axis=1)
    length = np.concatenate([[0.0], np.cumsum(seg)])
    total = length[-1] + np.linalg.norm(P[0] - P[-1])
    frac = length * 2.0 * np.pi / total
    return np.stack([np.cos(frac), np.sin(frac)], 1)


def uniform_laplacian(F, n):
    import scipy.sparse as sp
    F = np.asarray(F)
    r = np.concatenate([F[:, 0], F[:, 1], F[:, 1], F[:, 2], F[:, 2], F[:, 0], F[:, 0], F[:, 1], F[:, 2]])
    c = np.concatenate([F[:, 1], F[:, 0], F[:, 2], F[:, 1], F[:, 0], F[:, 2], F[:, 0], F[:, 1], F[:, 2]])
    w = np.concatenate([np.ones(6 * len(F)), -2.0 * np.ones(3 * len(F))])
    return sp.csr_matrix((w, (r, c)), shape=(n, n))


def harmonic(F, n, bnd, bnd_uv):
    import scipy.sparse.linalg as spl
    L = uniform_laplacian(F, n).tocsr()
    interior = np.setdiff1d(np.arange(n), bnd)
    Lii = L[interior][:, interior].tocsc()
    Lib = L[interior][:, bnd]
    UV = np.zeros((n, 2))
    UV[bnd] = bnd_uv
    rhs = -(Lib @ bnd_uv)
    UV[interior] = spl.splu(Lii).solve(rhs)
    return UV


def init_uv(V, F):
    """Cut every component to a disk and Tutte-embed the whole mesh, as the
    reference's "no input UV" start does (main.cpp:1379-1534): per component
    by its Euler characteristic -- closed genus 0: the one-point cut at its
    first triangle's first vertex; genus >= 1: the cut_to_disk loop; a disk:
    nothing -- repeated until every component is a disk; then per component
    its longest boundary loop on a unit circle, the circles on a grid 2.1
    apart (main.cpp:1503-1527), and one harmonic map with every loop held.
    Returns an InitState."""
    V = np.asarray(V, np.float64)
    F_mesh = np.asarray(F, np.int32)
    C = facet_components(F_mesh)
    nComp = int(C.max()) + 1 if len(C) else 0
    V_rest, F = V, F_mesh
    UV = np.zeros((len(V_rest), 2))
    cohE = np.zeros((0, 4), np.int32)
    path = None
    cut_any = False
    for _ in range(10000):
        todo = []
        for ci in range(nComp):
            Fc = F[C == ci]
            ec = euler_characteristic(V_rest, Fc)
            if ec < 1 or ec == 2:
                todo.append((ci, ec))
            elif ec != 1:
                raise NotImplementedError("component %d: unsupported Euler characteristic %d" % (ci, ec))
        if not todo:
            break
        for ci, ec in todo:
            Fc = F[C == ci]
            if ec == 2:
                V_rest, F, p = one_point_cut(V_rest, F, int(Fc[0, 0]))
                UV = np.vstack([UV, np.zeros((len(V_rest) - len(UV), 2))])
                path = p if nComp == 1 else path
            else:
                V_rest, UV, F, cohE, made = cut_component_once(Fc, V_rest, UV, F, cohE)
                if not made:
                    raise ValueError("no cut made while cutting component %d to a disk" % ci)
                if path is None:
                    path = []
            cut_any = True
    grid = 0
    while grid * grid < nComp:
        grid += 1
    bnd, bnd_uv = [], []
    for ci in range(nComp):
        loops = boundary_loops(F[C == ci])
        if not loops:
            raise ValueError("component %d has no boundary after the cut" % ci)
        longest = max(range(len(loops)), key=lambda i: (len(loops[i]), -i))
        loop = np.asarray(loops[longest], np.int64)
        uv = map_vertices_to_circle(V_rest, loop)
        uv = uv + np.array([ci % grid * 2.1, ci // grid * 2.1])
        bnd.append(loop)
        bnd_uv.append(uv)
    bnd = np.concatenate(bnd)
    UV = harmonic(F, len(V_rest), bnd, np.vstack(bnd_uv))
    # a cut mesh is built from (F_mesh, F_uv) with cohesive edges along the
    # cuts (TriMesh.cpp:122-189); an uncut disk has none (TriMesh.cpp:116-120)
    cohE = cohesive_edges(F_mesh, F) if cut_any else np.zeros((0, 4), np.int32)
    if nComp == 1 and path is None:
        path = None
    return InitState(V_rest, UV, F, np.array([0], np.int32), path, bnd, cohE)
