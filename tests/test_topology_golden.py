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
