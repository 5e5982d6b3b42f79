"""Synthetic workloads and the initial cut + Tutte embedding, against the
reference's own initial state (tests/golden)."""
import numpy as np
import pytest

from optcuts_gb300 import init as I
from optcuts_gb300 import meshes as M


@pytest.mark.parametrize("case", ["cube", "icosphere_320", "ellipsoid_2k", "icosphere_5k", "plane", "triangle",
                                  "sheet_3k"])
def test_init_matches_reference(golden, case):
    g = golden(case)
    st = I.init_uv(g["mesh_V"], g["mesh_F"])
    np.testing.assert_array_equal(st.F, g["F"])
    np.testing.assert_array_equal(st.V_rest, g["V_rest"])
    np.testing.assert_array_equal(st.bnd, g["bnd"])
    # the harmonic solve differs (SuperLU here, Eigen in the reference)
    assert np.abs(st.UV - g["UV0"]).max() < 1e-10


def test_high_genus_not_handled():
    V, F = M.CONFIGS["torus_768"]()
    with pytest.raises(NotImplementedError):
        I.init_uv(V, F)


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
