"""Initial cut and Tutte embedding -- the caller that produces the geometry
step's starting state.

Restates the "no input UV" initialisation of the reference's src/main.cpp
(lines 1379-1534) for the cases this library handles:

* a closed genus-0 single-component mesh: one-point cut at the first
  vertex of the first triangle (TriMesh::onePointCut, TriMesh.cpp:1054-1074,
  through the interior branch of TriMesh::cutPath, TriMesh.cpp:1449-1500);
* a topological disk: no cut.

then the boundary loop (igl::boundary_loop: smallest boundary vertex first,
following boundary half-edges), arc-length placement on the unit circle
(igl::map_vertices_to_circle) and the harmonic map with the reference's
uniform Laplacian (IglUtils::computeUniformLaplacian, IglUtils.cpp:39-60).
The result is the TriMesh the reference builds with
``TriMesh(V, F, UV_Tutte, F_cut, false)`` (main.cpp:1534, TriMesh.cpp:122-189):
the rest positions are re-indexed to the cut mesh and vertex 0 is fixed.

High-genus meshes (igl::cut_to_disk) are not handled here.
"""
from __future__ import annotations

import numpy as np


class InitState:
    def __init__(self, V_rest, UV, F, fixed, cut_path, bnd):
        self.V_rest = V_rest
        self.UV = UV
        self.F = F
        self.fixedVert = fixed
        self.cut_path = cut_path
        self.bnd = bnd


def euler_characteristic(V, F):
    F = np.asarray(F)
    e = np.sort(np.concatenate([F[:, [0, 1]], F[:, [1, 2]], F[:, [2, 0]]]), axis=1)
    nE = len(np.unique(e[:, 0].astype(np.int64) * (F.max() + 1) + e[:, 1]))
    nV = len(np.unique(F))
    return nV - nE + len(F)


def one_point_cut(V, F):
    """Split vertex vI = F[0,0] along path [n0, vI, n2] (n0, n2: its first and
    third neighbours in index order).  Returns (V', F', path)."""
    F = np.array(F, np.int32, copy=True)
    vI = int(F[0, 0])
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
    """Cut (if closed genus 0) and Tutte-embed; returns an InitState."""
    V = np.asarray(V, np.float64)
    F = np.asarray(F, np.int32)
    ec = euler_characteristic(V, F)
    path = None
    if ec == 2:
        V, F, path = one_point_cut(V, F)
    elif ec != 1:
        raise NotImplementedError("only closed genus-0 meshes and disks are initialised here")
    bnd = boundary_loop(F)
    if not bnd:
        raise ValueError("mesh has no boundary after the cut")
    bnd = np.asarray(bnd, np.int64)
    UV = harmonic(F, len(V), bnd, map_vertices_to_circle(V, bnd))
    return InitState(V, UV, F, np.array([0], np.int32), path, bnd)
