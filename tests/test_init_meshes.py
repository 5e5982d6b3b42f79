"""Synthetic workloads and the initial cut + Tutte embedding, against the
reference's own initial state (tests/golden)."""
import numpy as np
import pytest

from optcuts_gb300 import init as I
from optcuts_gb300 import meshes as M


@pytest.mark.parametrize("case", ["cube", "icosphere_320", "ellipsoid_2k", "icosphere_5k", "plane", "triangle",
                                  "sheet_3k", "torus_768", "components"])
def test_init_matches_reference(golden, case):
    """The cut mesh (one-point cut for genus 0; for the genus-1 torus the
    reference's cut_to_disk loop; for a mesh of three components each by its
    own Euler characteristic), its boundary loops and cohesive edges, and the
    Tutte embedding (the components' disks on the reference's grid), against
    the reference's own initial state."""
    g = golden(case)
    st = I.init_uv(g["mesh_V"], g["mesh_F"])
    np.testing.assert_array_equal(st.F, g["F"])
    np.testing.assert_array_equal(st.V_rest, g["V_rest"])
    np.testing.assert_array_equal(st.bnd, g["bnd"])
    np.testing.assert_array_equal(st.cohE, g["cohE"].reshape(-1, 4))
    # the harmonic solve differs (SuperLU here, Eigen in the reference)
    assert np.abs(st.UV - g["UV0"]).max() < 1e-10


def test_cut_to_disk_on_a_torus():
    """A closed torus (Euler characteristic 0): the cut graph holds two
    loops through a common vertex; cutting along them leaves a disk."""
    V, F = M.CONFIGS["torus_768"]()
    cuts = I.cut_to_disk(F)
    assert len(cuts) >= 2 and all(len(c) >= 3 for c in cuts)
    Vc, Fc = I.cut_high_genus(V, F)
    assert I.euler_characteristic(Vc, Fc) == 1 and len(I.boundary_loop(Fc)) > 0


def _cut_path_edge_by_edge(path, V_rest, UV, F, cohE):
    """cutPath as a loop of single operations on the whole mesh (each one
    topology_apply, pinned against the reference's splitEdgeOnBoundary and
    cutPath): the sequence topology_cut_path applies on local faces."""
    import optcuts_gb300 as oc

    def fan(F, v):
        rows = F[np.any(F == v, axis=1)]
        k = np.argmax(rows == v, axis=1)
        return rows[np.arange(len(rows)), (k + 1) % 3], rows[np.arange(len(rows)), (k + 2) % 3]

    def boundary(F, v):
        nxt, prv = fan(F, v)
        return sorted(nxt.tolist()) != sorted(prv.tolist())

    def interior_edge(F, a, b):
        nxt, prv = fan(F, a)
        return b in nxt and b in prv

    def split_edges(vs, V_rest, UV, F, cohE, made):
        for a, b in zip(vs[:-1], vs[1:]):
            if not interior_edge(F, a, b):
                continue
            rows = 4 if (boundary(F, a) and boundary(F, b)) else 2
            V_rest, UV, F, cohE = oc.topology_apply(oc.OP_BOUNDARY_SPLIT, [a, b], np.repeat(UV[[a]], rows, axis=0),
                                                    V_rest, UV, F, cohE)
            made += 1
        return V_rest, UV, F, cohE, made

    path = [int(v) for v in path]
    if boundary(F, path[0]) or boundary(F, path[-1]):
        if not boundary(F, path[0]):
            path = path[::-1]
        return split_edges(path, V_rest, UV, F, cohE, 0)
    V_rest, UV, F, cohE = oc.topology_apply(oc.OP_INTERIOR_SPLIT, path[:3], np.repeat(UV[[path[1]]], 2, axis=0),
                                            V_rest, UV, F, cohE)
    return split_edges(path[2:], V_rest, UV, F, cohE, 0)


def test_cut_path_equals_single_operations():
    """topology_cut_path (each edge on the faces around it) leaves the same
    arrays as the same operations applied one by one to the whole mesh, for
    every path the initial cutting of a torus takes."""
    V, F = M.torus(40, 32)
    calls = []
    orig = I.cut_path

    def record(path, V_rest, UV, F, cohE):
        out = orig(path, V_rest, UV, F, cohE)
        calls.append(((list(path), V_rest, UV, F, cohE), out))
        return out

    I.cut_path = record
    try:
        I.cut_high_genus(V, F)
    finally:
        I.cut_path = orig
    assert len(calls) >= 2 and any(out[4] > 0 for _, out in calls)
    for args, out in calls:
        ref = _cut_path_edge_by_edge(*args)
        for a, b in zip(out, ref):
            np.testing.assert_array_equal(np.asarray(a), np.asarray(b))


def test_torus_41k_initialises():
    """The genus-1 41k-triangle torus (the plain-method configuration) gets
    a valid start: a disk whose Tutte map inverts no triangle."""
    V, F = M.CONFIGS["torus_41k"]()
    st = I.init_uv(V, F)
    assert I.euler_characteristic(st.V_rest, st.F) == 1
    U = st.UV[st.F]
    det = (U[:, 1, 0] - U[:, 0, 0]) * (U[:, 2, 1] - U[:, 0, 1]) - (U[:, 1, 1] - U[:, 0, 1]) * (U[:, 2, 0] - U[:, 0, 0])
    assert (det > 0).all()


@pytest.mark.parametrize("key,nf", [("icosphere_5k", 5120), ("torus_41k", 40960), ("ellipsoid_199k", 199080)])
def test_config_sizes_and_orientation(key, nf):
    V, F = M.CONFIGS[key]()
    assert F.shape == (nf, 3)
    vol = np.einsum("ij,ij->i", V[F[:, 0]], np.cross(V[F[:, 1]], V[F[:, 2]])).sum() / 6
    assert vol > 0


def test_knot_size():
    # (2,3) torus-knot tube, 2000 x 512 grid
    V, F = M.torus_knot_tube(200, 64)
    assert F.shape == (2 * 200 * 64, 3) and V.shape == (200 * 64, 3)
    assert 2 * 2000 * 512 == 2_048_000


def test_generators_are_deterministic():
    a = M.CONFIGS["ellipsoid_2k"]()
    b = M.CONFIGS["ellipsoid_2k"]()
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])


def test_obj_roundtrip(tmp_path):
    V, F = M.cube()
    p = tmp_path / "c.obj"
    M.write_obj(str(p), V, F)
    V2, F2 = M.read_obj(str(p))
    np.testing.assert_array_equal(V, V2)
    np.testing.assert_array_equal(F, F2)
    (tmp_path / "t.obj").write_text("v 0 0 0\n")
    with pytest.raises(ValueError):
        M.read_obj(str(tmp_path / "t.obj"))


@pytest.mark.parametrize("case", ["cube", "icosphere_320", "ellipsoid_2k", "icosphere_5k", "plane", "triangle",
                                  "sheet_3k"])
def test_cohesive_edges_and_seam_term_match_reference(golden, case):
    g = golden(case)
    st = I.init_uv(g["mesh_V"], g["mesh_F"])
    np.testing.assert_array_equal(st.cohE.reshape(-1, 4), g["cohE"].reshape(-1, 4))
    # E_se before division by virtualRadius (TriMesh::computeSeamSparsity)
    avg = g["scalars"][1]
    assert I.seam_sparsity(st.V_rest, st.UV, st.cohE, avg) == pytest.approx(g["scalars"][3], rel=1e-15, abs=0)


def test_cut_to_disk_and_cut_path_edge_cases():
    """A closed sphere has no cut graph; on a disk the boundary edges are
    never peeled, so the boundary loop is what remains (the initialisation
    calls it for closed surfaces of genus >= 1 only); the C call reports
    sizes first and refuses short output arrays; a cut path with a vertex
    out of range is an error, not a crash."""
    import ctypes

    import optcuts_gb300 as oc
    V, F = M.icosphere(2)
    assert oc.cut_to_disk(F) == []
    Vp, Fp = M.CONFIGS["plane"]()
    cuts = oc.cut_to_disk(Fp)
    assert len(cuts) == 1 and cuts[0][0] == cuts[0][-1]
    assert sorted(cuts[0][:-1]) == sorted(I.boundary_loop(Fp))
    Vt, Ft = M.torus(12, 10)
    Ft = np.ascontiguousarray(Ft, np.int32)
    nc, nv = ctypes.c_int(), ctypes.c_int()
    P = ctypes.POINTER(ctypes.c_int)
    lib = oc.lib()
    assert lib.oc_cut_to_disk(Ft.ctypes.data_as(P), len(Ft), None, 0, None, 0, ctypes.byref(nc),
                              ctypes.byref(nv)) == oc.OC_OK
    assert nc.value == 2 and nv.value == sum(len(c) for c in oc.cut_to_disk(Ft))
    short = np.zeros(1, np.int32)
    off = np.zeros(nc.value + 1, np.int32)
    assert lib.oc_cut_to_disk(Ft.ctypes.data_as(P), len(Ft), short.ctypes.data_as(P), 1, off.ctypes.data_as(P),
                              len(off), ctypes.byref(nc), ctypes.byref(nv)) != oc.OC_OK
    UV = np.zeros((len(Vt), 2))
    with pytest.raises(oc.OCError):
        oc.topology_cut_path([0, len(Vt) + 5], Vt, UV, Ft, np.zeros((0, 4), np.int32))
