"""The project's air-mesh generator (constrained Delaunay between the UV
boundary loops and the reference's segmented box, no Triangle) on the
reference's own UV layouts.  Host code only: runs without a GPU."""
import numpy as np
import pytest

import optcuts_gb300 as oc
from conftest import golden_scaffolds

CASES = ["sheet_3k", "torus_768", "icosphere_320_scaf", "plane", "triangle"]


def signed_areas(V, F):
    a, b, c = V[F[:, 0]], V[F[:, 1]], V[F[:, 2]]
    return 0.5 * ((b[:, 0] - a[:, 0]) * (c[:, 1] - a[:, 1]) - (b[:, 1] - a[:, 1]) * (c[:, 0] - a[:, 0]))


def box_points(UV, avg):
    """The reference's segmented bounding box (Scaffold.cpp:63-95)."""
    seg = avg * 3.0 ** 2
    margin = (avg - seg) / (1.0 - 3.0)
    x0, x1 = UV[:, 0].min() - margin, UV[:, 0].max() + margin
    y0, y1 = UV[:, 1].min() - margin, UV[:, 1].max() + margin
    nx, ny = int(np.ceil((x1 - x0) / seg)), int(np.ceil((y1 - y0) / seg))
    sx, sy = (x1 - x0) / nx, (y1 - y0) / ny
    pts = [(x0 + i * sx, y0) for i in range(nx)] + [(x1, y0 + i * sy) for i in range(ny)]
    pts += [(x1 - i * sx, y1) for i in range(nx)] + [(x0, y1 - i * sy) for i in range(ny)]
    return np.array(pts)


def boundary_edges(F):
    he = {}
    for t in F:
        for k in range(3):
            he[(int(t[k]), int(t[(k + 1) % 3]))] = he.get((int(t[k]), int(t[(k + 1) % 3])), 0) + 1
    assert max(he.values()) == 1                       # each directed edge once: manifold, consistent
    return {e for e in he if (e[1], e[0]) not in he}


@pytest.mark.parametrize("minAngle", [0.0, 20.0])
@pytest.mark.parametrize("case", CASES)
def test_air_mesh_fills_box_minus_mesh(golden, case, minAngle):
    g = golden(case)
    UV, F = g["UV0"], g["F"]
    sc = oc.Scaffold.build(UV, F, g["scalars"][1], minAngle)
    nb = len(sc.bnd)
    ref = golden_scaffolds(g)[0]
    # the same boundary vertices and the reference's box points, bit for bit
    assert sorted(sc.bnd.tolist()) == sorted(ref[2].tolist())
    box = box_points(UV, g["scalars"][1])
    nbox = len(box)
    np.testing.assert_array_equal(sc.airV[nb:nb + nbox], box)
    np.testing.assert_array_equal(ref[0][nb:nb + nbox], box)
    np.testing.assert_array_equal(sc.airV[:nb], UV[sc.bnd])
    # counter-clockwise, non-degenerate triangles covering box minus mesh
    A = signed_areas(sc.airV, sc.airF)
    assert A.min() > 0.0
    box = sc.airV[nb:]
    box_area = (box[:, 0].max() - box[:, 0].min()) * (box[:, 1].max() - box[:, 1].min())
    mesh_area = signed_areas(UV, F).sum()
    assert A.sum() + mesh_area == pytest.approx(box_area, rel=1e-12)
    # its boundary is exactly the box loop plus the mesh's boundary loops, reversed
    loc = {int(v): i for i, v in enumerate(sc.bnd)}
    mesh_bnd = {(loc[b], loc[a]) for (a, b) in boundary_edges(F)}
    box_loop = {(nb + i, nb + (i + 1) % nbox) for i in range(nbox)}
    assert boundary_edges(sc.airF) == mesh_bnd | box_loop
    # every vertex is used; Steiner points only with refinement, strictly inside
    assert len(np.unique(sc.airF)) == len(sc.airV)
    if minAngle == 0.0:
        assert len(sc.airV) == nb + nbox


def min_angles(V, F):
    a = V[F]
    out = []
    for k in range(3):
        u, w = a[:, (k + 1) % 3] - a[:, k], a[:, (k + 2) % 3] - a[:, k]
        c = (u * w).sum(1) / np.linalg.norm(u, axis=1) / np.linalg.norm(w, axis=1)
        out.append(np.degrees(np.arccos(np.clip(c, -1.0, 1.0))))
    return np.min(out, axis=0)


@pytest.mark.parametrize("case", ["sheet_3k", "torus_768"])
def test_refinement_improves_angles(golden, case):
    g = golden(case)
    raw = oc.Scaffold.build(g["UV0"], g["F"], g["scalars"][1], 0.0)
    ref = oc.Scaffold.build(g["UV0"], g["F"], g["scalars"][1], 20.0)
    a0, a1 = min_angles(raw.airV, raw.airF), min_angles(ref.airV, ref.airF)
    # triangles not touching a segment reach the bound; the rest keep what
    # the boundary (no segment splitting) allows
    assert np.median(a1) > np.median(a0)
    assert np.mean(a1 >= 20.0 - 1e-9) > 0.5


@pytest.mark.parametrize("minAngle", [0.0, 20.0])
@pytest.mark.parametrize("case", ["sheet_3k", "torus_768"])
def test_air_mesh_is_constrained_delaunay(golden, case, minAngle):
    g = golden(case)
    sc = oc.Scaffold.build(g["UV0"], g["F"], g["scalars"][1], minAngle)
    V, F = sc.airV, sc.airF
    nb = len(sc.bnd)
    nbox = len(box_points(g["UV0"], g["scalars"][1]))
    loc = {int(v): i for i, v in enumerate(sc.bnd)}
    constrained = {frozenset((loc[a], loc[b])) for (a, b) in boundary_edges(g["F"])}
    constrained |= {frozenset((nb + i, nb + (i + 1) % nbox)) for i in range(nbox)}
    opp = {}
    for t, tri in enumerate(F):
        for k in range(3):
            opp.setdefault(frozenset((int(tri[(k + 1) % 3]), int(tri[(k + 2) % 3]))), []).append((t, int(tri[k])))
    scale = np.abs(V).max() ** 4
    for e, sides in opp.items():
        if len(sides) != 2 or e in constrained:
            continue
        (t, _), (_, q) = sides
        a, b, c = V[F[t]]
        d = V[q]
        m = np.array([[a[0] - d[0], a[1] - d[1], (a - d) @ (a - d)],
                      [b[0] - d[0], b[1] - d[1], (b - d) @ (b - d)],
                      [c[0] - d[0], c[1] - d[1], (c - d) @ (c - d)]])
        assert np.linalg.det(m) <= 1e-12 * scale


def test_air_mesh_rejects_closed_mesh(golden):
    g = golden("cube")
    from optcuts_gb300 import meshes as M
    V, F = M.cube()
    with pytest.raises(oc.OCError):
        oc.Scaffold.build(V[:, :2], F, 1.0)
