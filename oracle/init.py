"""Initial state of a closed genus-0 mesh, restated for the oracle -- TEST
INFRASTRUCTURE ONLY (the checker and the CPU arm of the benchmark use it; the
product has its own initialisation and never imports this).

The reference's "no input UV" start for one closed genus-0 component
(src/main.cpp:1379-1534):

* TriMesh::onePointCut(F(0, 0)) (src/TriMesh.cpp:1054-1074): the path is
  (n0, v, n2), n0 and n2 the first and third entries of the vertex's sorted
  neighbour set; TriMesh::cutPath's interior branch (src/TriMesh.cpp:1449-1500)
  walks the triangles around v from the directed edge v->n0 to n2 and gives
  them a copy of v appended as the last vertex;
* the cohesive edges TriMesh(V, F, UV, F_cut) rebuilds from the surface and
  cut triangles (src/TriMesh.cpp:128-166);
* igl::boundary_loop of the cut mesh, igl::map_vertices_to_circle
  (arc length of the rest-space boundary polygon, unit circle);
* igl::harmonic with the reference's uniform Laplacian
  (IglUtils::computeUniformLaplacian, src/Utils/IglUtils.cpp:39-60, twice the
  graph Laplacian on interior rows): the interior UV solve the boundary
  values; vertex 0 is the fixed vertex (src/TriMesh.cpp:325-328).

Pinned against the reference's own dumps of the same meshes
(tests/test_oracle_golden.py)."""
from __future__ import annotations

import numpy as np


def one_point_cut(V, F):
    """(V_cut, F_cut, path) after the reference's one-point cut."""
    F = np.array(F, np.int32)
    v = int(F[0, 0])
    around = np.nonzero((F == v).any(axis=1))[0]
    nbr = sorted({int(x) for t in around for x in F[t] if x != v})
    path = [nbr[0], v, nbr[2]]
    # directed edge v -> w of a triangle around v, keyed by w
    nxt = {}
    for t in around:
        k = int(np.nonzero(F[t] == v)[0][0])
        nxt[int(F[t, (k + 1) % 3])] = (int(t), int(F[t, (k + 2) % 3]))
    left, w = [], path[0]
    while True:
        t, w = nxt[w]
        left.append(t)
        if w == path[2]:
            break
        if w == path[0] or len(left) > len(around):
            raise ValueError("one-point cut: no path around vertex %d" % v)
    copy = len(V)
    for t in left:
        F[t][F[t] == v] = copy
    V_cut = np.vstack([np.asarray(V, np.float64), np.asarray(V, np.float64)[v]])
    return V_cut, F, path


def cohesive_rows(F_mesh, F_uv):
    """Cohesive edges as TriMesh(V, F, UV, F_uv) rebuilds them
    (src/TriMesh.cpp:128-166): triangles and their edges in order, every UV
    half-edge a->b without a UV twin whose surface edge has a twin gives the
    row (a, b, twin's UV end, twin's UV start); the twin's own surface
    half-edge is then struck out so that each seam edge appears once."""
    F_mesh = np.asarray(F_mesh, np.int64)
    F_uv = np.asarray(F_uv, np.int64)
    uv_edges = {(int(r[k]), int(r[(k + 1) % 3])) for r in F_uv for k in range(3)}
    surf = {}
    for t, r in enumerate(F_mesh):
        for k in range(3):
            surf[(int(r[k]), int(r[(k + 1) % 3]))] = (t, k)
    rows = []
    for t in range(len(F_uv)):
        for k in range(3):
            a, b = int(F_uv[t, k]), int(F_uv[t, (k + 1) % 3])
            if (b, a) in uv_edges:
                continue
            s0, s1 = int(F_mesh[t, k]), int(F_mesh[t, (k + 1) % 3])
            twin = surf.get((s1, s0))
            if twin is None:
                continue
            t2, k2 = twin
            rows.append((a, b, int(F_uv[t2, (k2 + 1) % 3]), int(F_uv[t2, k2])))
            surf.pop((s0, s1), None)
    return np.asarray(rows, np.int32).reshape(-1, 4)


def boundary_loop(F):
    """The boundary of a disk: directed boundary half-edges (no twin) walked
    from the smallest boundary vertex."""
    F = np.asarray(F, np.int64)
    succ = {}
    edges = set()
    for a, b, c in F:
        edges.update(((a, b), (b, c), (c, a)))
    for a, b in edges:
        if (b, a) not in edges:
            succ[int(a)] = int(b)
    if not succ:
        return np.zeros(0, np.int64)
    loop = [min(succ)]
    while succ[loop[-1]] != loop[0]:
        loop.append(succ[loop[-1]])
        if len(loop) > len(succ):
            raise ValueError("boundary is not a single loop")
    return np.asarray(loop, np.int64)


def circle(V, loop):
    """Boundary vertices on the unit circle at their arc-length fractions."""
    P = np.asarray(V, np.float64)[loop]
    seg = np.sqrt(((np.roll(P, -1, axis=0) - P) ** 2).sum(1))
    cum = np.concatenate([[0.0], np.cumsum(seg[:-1])])
    ang = 2.0 * np.pi * cum / seg.sum()
    return np.column_stack([np.cos(ang), np.sin(ang)])


def tutte(F, n, loop, loop_uv):
    """Uniform-weight harmonic map with the boundary held."""
    import scipy.sparse as sp
    import scipy.sparse.linalg as spl
    F = np.asarray(F, np.int64)
    i = np.concatenate([F[:, 0], F[:, 1], F[:, 2], F[:, 1], F[:, 2], F[:, 0]])
    j = np.concatenate([F[:, 1], F[:, 2], F[:, 0], F[:, 0], F[:, 1], F[:, 2]])
    A = sp.coo_matrix((np.ones(len(i)), (i, j)), shape=(n, n)).tocsr()
    L = sp.diags(np.asarray(A.sum(axis=1)).ravel()) - A
    free = np.ones(n, bool)
    free[loop] = False
    idx = np.nonzero(free)[0]
    UV = np.zeros((n, 2))
    UV[loop] = loop_uv
    rhs = -(L[idx][:, loop] @ loop_uv)
    UV[idx] = spl.spsolve(L[idx][:, idx].tocsc(), rhs)
    return UV


def init_genus0(V, F):
    """dict(V_rest, UV, F, fixedVert, bnd, cohE) of a closed genus-0 mesh."""
    V_cut, F_cut, path = one_point_cut(V, F)
    loop = boundary_loop(F_cut)
    UV = tutte(F_cut, len(V_cut), loop, circle(V_cut, loop))
    return {"V_rest": V_cut, "UV": UV, "F": F_cut, "fixedVert": np.array([0], np.int32), "bnd": loop,
            "cohE": cohesive_rows(F, F_cut), "path": path}
