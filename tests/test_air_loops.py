"""The bijective local solves' loop mesher (oc_air_loop_mesh, the same code
the kernels run) against Triangle's own output on the local air loops the
reference meshed during bijective topology queries (tests/golden/
air_loops.npz, recorded from the compiled reference by
oracle/_ref/ref_driver_trilog).  Loops Triangle did not refine must give
the same triangles (the polygon's constrained Delaunay triangulation is
unique); on the loops it refined, the Steiner points must agree in number
and place almost always (the refinement order within a queue bin is
Triangle's internal triangle order, which is not restated)."""
import numpy as np
import pytest

import optcuts_gb300 as oc


@pytest.fixture(scope="module")
def loops():
    g = np.load(__import__("os").path.join(__import__("os").path.dirname(__file__), "golden", "air_loops.npz"))
    out = []
    for i in range(len(g["loop_off"]) - 1):
        pts = g["loop_pts"][g["loop_off"][i]:g["loop_off"][i + 1]]
        tri = g["tri"][g["tri_off"][i]:g["tri_off"][i + 1]]
        st = g["steiner"][g["steiner_off"][i]:g["steiner_off"][i + 1]]
        out.append((pts, tri, st))
    return out


def tri_key(T):
    return sorted(tuple(sorted(int(v) for v in t)) for t in T)


def polygon_area(P):
    x, y = P[:, 0], P[:, 1]
    return 0.5 * abs(np.dot(x, np.roll(y, -1)) - np.dot(y, np.roll(x, -1)))


def test_unrefined_loops_equal_triangle(loops):
    n = 0
    for pts, tri, st in loops:
        if len(st):
            continue
        V, T, status = oc.air_loop_mesh(pts)
        assert status == 0
        assert len(V) == len(pts)
        assert tri_key(T) == tri_key(tri)
        n += 1
    assert n >= 100


def test_refined_loops_match_triangle(loops):
    same_count = close = total = 0
    for pts, tri, st in loops:
        if not len(st):
            continue
        total += 1
        V, T, status = oc.air_loop_mesh(pts)
        assert status == 0
        S = V[len(pts):]
        if len(S) == len(st):
            same_count += 1
            scale = np.abs(pts).max()
            if np.abs(np.sort(S, axis=0) - np.sort(st, axis=0)).max() <= 1e-9 * scale:
                close += 1
    assert total >= 100
    assert same_count >= 0.98 * total and close >= 0.97 * total, (same_count, close, total)


def test_meshes_are_valid_triangulations(loops):
    for pts, tri, st in loops:
        V, T, status = oc.air_loop_mesh(pts)
        a = V[T[:, 1]] - V[T[:, 0]]
        b = V[T[:, 2]] - V[T[:, 0]]
        area = 0.5 * (a[:, 0] * b[:, 1] - a[:, 1] * b[:, 0])
        assert np.all(area > 0.0)
        assert area.sum() == pytest.approx(polygon_area(pts), rel=1e-9)
        assert len(T) == len(pts) - 2 + 2 * (len(V) - len(pts))


def test_orientation_and_limits():
    sq = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1.0], [0.0, 1.0]])
    V1, T1, _ = oc.air_loop_mesh(sq)
    V2, T2, _ = oc.air_loop_mesh(sq[::-1].copy())
    assert len(T1) == len(T2) == 2
    # a thin sliver: no Steiner point may go on the polygon ("Y")
    sl = np.array([[0.0, 0.0], [1.0, 0.0], [1.0, 1e-3], [0.0, 1e-3]])
    V, T, _ = oc.air_loop_mesh(sl)
    assert len(V) == 4
    # with refinement off the mesh is the constrained Delaunay triangulation
    hexagon = np.array([[np.cos(t), np.sin(t)] for t in np.linspace(0, 2 * np.pi, 7)[:-1]])
    V, T, st = oc.air_loop_mesh(hexagon, maxSteiner=0)
    assert len(V) == 6 and len(T) == 4 and st == 0
    with pytest.raises(oc.OCError):
        oc.air_loop_mesh(np.zeros((2, 2)))
    bowtie = np.array([[0.0, 0.0], [1.0, 1.0], [1.0, 0.0], [0.0, 1.0]])
    with pytest.raises(oc.OCError):
        oc.air_loop_mesh(bowtie)
