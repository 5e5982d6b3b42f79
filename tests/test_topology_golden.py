"""Topology-query candidate selection (the split filter, TriMesh.cpp:561-629)
against the reference's own queries (tests/golden/*_topo: a converged state,
its split filter values and every candidate querySplit / queryMerge
evaluated, bijectivity off).  Host code only."""
import numpy as np
import pytest

import optcuts_gb300 as oc
from conftest import TOPO_CASES, golden_candidates

DBL_MAX = np.finfo(np.float64).max


@pytest.mark.parametrize("case", TOPO_CASES)
def test_interior_split_candidates(golden, case):
    g = golden(case)
    nV = len(g["topo_V"])
    cands, pool = oc.split_candidates(nV, g["topo_F"], g["topo_divGrad"], True)
    ref = golden_candidates(g, "iSplit")
    assert pool == int(g["topo_best"][4])          # inSplitTotalAmt
    assert len(cands) == len(ref)
    for v, r in zip(cands, ref):
        if r["energyChanges"][0] != DBL_MAX:
            assert r["path"][1] == v


@pytest.mark.parametrize("case", TOPO_CASES)
def test_boundary_split_candidates(golden, case):
    g = golden(case)
    nV = len(g["topo_V"])
    cands, pool = oc.split_candidates(nV, g["topo_F"], g["topo_divGrad"], False)
    ref = golden_candidates(g, "bSplit")
    assert len(cands) == len(ref)
    for v, r in zip(cands, ref):
        if r["energyChanges"][0] != DBL_MAX:
            assert r["path"][0] == v


def test_candidate_counts_follow_the_filter_exponents(golden):
    g = golden("sheet_3k_topo")
    nV = len(g["topo_V"])
    c_in, pool_in = oc.split_candidates(nV, g["topo_F"], g["topo_divGrad"], True)
    c_b, pool_b = oc.split_candidates(nV, g["topo_F"], g["topo_divGrad"], False)
    assert len(c_in) == max(2, int(pool_in ** 0.6))
    assert len(c_b) == max(2, int(pool_b ** 0.8))
    c_in2, _ = oc.split_candidates(nV, g["topo_F"], g["topo_divGrad"], True, 0.8)
    assert len(c_in2) == max(2, int(pool_in ** 0.8)) and list(c_in2[:len(c_in)]) == list(c_in)


def state(g, tag):
    return (g["topo_%s_Vrest" % tag], g["topo_%s_V" % tag], g["topo_%s_F" % tag], g["topo_%s_cohE" % tag].reshape(-1, 4))


@pytest.mark.parametrize("case", TOPO_CASES)
def test_boundary_split_apply_matches_reference(golden, case):
    """TriMesh::splitEdgeOnBoundary with the reference's chosen edge and new
    positions: identical F, V_rest, UV and cohesive edges."""
    g = golden(case)
    Vr, UV, F, C = oc.topology_apply(oc.OP_BOUNDARY_SPLIT, g["topo_opB_path"], g["topo_opB_pos"], g["topo_Vrest"],
                                     g["topo_V"], g["topo_F"], g["topo_cohE"])
    rVr, rUV, rF, rC = state(g, "afterB")
    np.testing.assert_array_equal(F, rF)
    np.testing.assert_array_equal(Vr, rVr)
    np.testing.assert_array_equal(UV, rUV)
    np.testing.assert_array_equal(C, rC)


@pytest.mark.parametrize("case", TOPO_CASES)
def test_interior_split_apply_matches_reference(golden, case):
    g = golden(case)
    Vr, UV, F, C = oc.topology_apply(oc.OP_INTERIOR_SPLIT, g["topo_opI_path"], g["topo_opI_pos"], g["topo_Vrest"],
                                     g["topo_V"], g["topo_F"], g["topo_cohE"])
    rVr, rUV, rF, rC = state(g, "afterI")
    np.testing.assert_array_equal(F, rF)
    np.testing.assert_array_equal(Vr, rVr)
    np.testing.assert_array_equal(UV, rUV)
    np.testing.assert_array_equal(C, rC)


@pytest.mark.parametrize("case", TOPO_CASES)
def test_merge_apply_matches_reference(golden, case):
    """TriMesh::mergeBoundaryEdges on the split state, with the reference's
    best merge (vertex removal by moving the last vertex, cohesive rows)."""
    g = golden(case)
    bVr, bUV, bF, bC = state(g, "afterB")
    Vr, UV, F, C = oc.topology_apply(oc.OP_MERGE, g["topo_opM_path"], g["topo_opM_pos"], bVr, bUV, bF, bC)
    rVr, rUV, rF, rC = state(g, "afterM")
    np.testing.assert_array_equal(F, rF)
    np.testing.assert_array_equal(Vr, rVr)
    np.testing.assert_array_equal(UV, rUV)
    np.testing.assert_array_equal(C, rC)


def test_bad_operations_rejected(golden):
    g = golden("icosphere_320_topo")
    with pytest.raises(oc.OCError):   # an interior vertex's edge does not touch the boundary
        v = int(g["topo_opI_path"][1])
        nb = int(g["topo_opI_path"][0])
        oc.topology_apply(oc.OP_BOUNDARY_SPLIT, [v, nb], np.zeros((2, 2)), g["topo_Vrest"], g["topo_V"],
                          g["topo_F"], g["topo_cohE"])
    with pytest.raises(oc.OCError):
        oc.topology_apply(oc.OP_INTERIOR_SPLIT, [0, 1], np.zeros((2, 2)), g["topo_Vrest"], g["topo_V"],
                          g["topo_F"], g["topo_cohE"])


@pytest.mark.parametrize("op,tag", [(0, "bSplit"), (1, "iSplit"), (2, "merge")])
@pytest.mark.parametrize("case", TOPO_CASES)
def test_oracle_topology_query(golden, case, op, tag):
    """The CPU restatement of the topology queries against the reference's."""
    import oracle as O
    g = golden(case)
    cands, _ = O.topology_query(g["topo_Vrest"], g["topo_V"], g["topo_F"], g["topo_cohE"], op, g["topo_best"][3],
                                threads=4)
    ref = golden_candidates(g, tag)
    assert len(cands) == len(ref)
    for c, r in zip(cands, ref):
        if r["energyChanges"][0] == DBL_MAX:
            assert c["EwDec"] == -DBL_MAX
            continue
        assert c["path"] == r["path"]
        for a, b in zip(c["energyChanges"], r["energyChanges"]):
            assert a == pytest.approx(b, rel=1e-6, abs=1e-12)


@pytest.mark.parametrize("case", TOPO_CASES)
def test_oracle_merge_query_after_split(golden, case):
    import oracle as O
    g = golden(case)
    cands, _ = O.topology_query(g["topo_afterB_Vrest"], g["topo_afterB_V"], g["topo_afterB_F"], g["topo_afterB_cohE"],
                                2, g["topo_best"][3])
    ref = golden_candidates(g, "mergeB")
    assert len(cands) == len(ref)
    for c, r in zip(cands, ref):
        assert c["path"] == r["path"]
        assert c["energyChanges"][0] == pytest.approx(r["energyChanges"][0], rel=1e-6, abs=1e-12)
