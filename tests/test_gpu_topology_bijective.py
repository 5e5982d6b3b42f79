"""Bijective topology queries on the GPU (OC_TOPO_BIJECTIVE: split copies
separated, every local solve with its air loop re-meshed each local Newton
iteration) against the reference's own queries with bijectivity on, on the
same converged state and the same whole-mesh air mesh
(tests/golden/*_bij_topo)."""
from types import SimpleNamespace

import numpy as np
import pytest

import optcuts_gb300 as oc
from conftest import golden_candidates

pytestmark = pytest.mark.gpu
DBL_MAX = np.finfo(np.float64).max
BIJ_CASES = ["icosphere_320_bij_topo", "sheet_3k_bij_topo", "torus_768_bij_topo"]


def bij_state(g, tag=""):
    """The topology state with the reference's air mesh as the scaffold of
    an Optimizer of the mesh (the loops the queries take)."""
    p = "topo_" + (tag + "_" if tag else "")
    m = oc.TriMesh(g[p + "Vrest"], g[p + "V"], g[p + "F"], g["topo_fixed"])
    m.setCohesiveEdges(g[p + "cohE"])
    opt = oc.Optimizer(m, [1.0 - float(g["topo_best"][3])])
    opt.setScaffold(SimpleNamespace(airV=g[p + "airV"], airF=g[p + "airF"], bnd=g[p + "airBnd"]))
    return m, opt


def compare(ours, ref, rel=1e-6, frac=0.9, rel_all=1e-3):
    """The same candidates and paths, abandoned problems (-DBL_MAX) where
    the reference abandoned them; every energy change within rel_all and a
    fraction frac of them within rel.  The air meshes of the local solves
    come from this project's mesher: Triangle's own triangles on every loop
    it does not refine, its Steiner points on almost every loop it does;
    the few boundary splits whose loops were refined differently differ by
    up to ~1e-4 relative."""
    assert len(ours["candidates"]) == len(ref)
    good = n = 0
    for c, r in zip(ours["candidates"], ref):
        if r["energyChanges"][0] == DBL_MAX:
            assert c["energyChanges"][0] == DBL_MAX
            continue
        n += 1
        assert c["path"] == r["path"]
        for a, b in zip(c["energyChanges"], r["energyChanges"]):
            assert a == pytest.approx(b, rel=rel_all, abs=1e-12)
        good += all(a == pytest.approx(b, rel=rel, abs=1e-12) for a, b in zip(c["energyChanges"], r["energyChanges"]))
    assert good >= frac * n, (good, n)
    return n


@pytest.mark.parametrize("case", BIJ_CASES)
def test_boundary_split_query_bijective(golden, case):
    g = golden(case)
    m, opt = bij_state(g)
    q = m.querySplit(g["topo_best"][3], splitInterior=False, bijective=True)
    assert q["air"]["problems"] == q["local_problems"] and q["air"]["capped"] == 0
    compare(q, golden_candidates(g, "bSplit"))
    assert q["EwDec_max"] == pytest.approx(g["topo_best"][0], rel=1e-6)


@pytest.mark.parametrize("case", BIJ_CASES)
def test_interior_split_query_bijective(golden, case):
    g = golden(case)
    m, opt = bij_state(g)
    q = m.querySplit(g["topo_best"][3], splitInterior=True, bijective=True)
    assert q["air"]["problems"] == q["local_problems"]
    compare(q, golden_candidates(g, "iSplit"), frac=1.0)
    assert q["EwDec_max"] == pytest.approx(g["topo_best"][2], rel=1e-6)


@pytest.mark.parametrize("case", BIJ_CASES)
def test_merge_query_after_split_bijective(golden, case):
    g = golden(case)
    if "topo_afterB_airV" not in g:
        pytest.skip("no boundary split applied in this case")
    m, opt = bij_state(g, "afterB")
    q = m.queryMerge(g["topo_best"][3], bijective=True)
    compare(q, golden_candidates(g, "mergeB"), frac=1.0)
    assert q["EwDec_max"] == pytest.approx(float(g["topo_mergeB_best"][0]), rel=1e-6)


def test_bijective_differs_from_unconstrained(golden):
    """The air loops change the answer: the bijective interior-split
    decreases are not the bijectivity-off ones."""
    g = golden("icosphere_320_bij_topo")
    m, opt = bij_state(g)
    lam = g["topo_best"][3]
    qb = m.querySplit(lam, splitInterior=True, bijective=True)
    qf = m.querySplit(lam, splitInterior=True)
    a = np.array([c["energyChanges"][0] for c in qb["candidates"]])
    b = np.array([c["energyChanges"][0] for c in qf["candidates"]])
    ok = (a < DBL_MAX) & (b < DBL_MAX)
    assert np.any(np.abs(a[ok] - b[ok]) > 1e-6 * np.abs(b[ok]))


def test_bijective_needs_a_scaffold(golden):
    g = golden("icosphere_320_bij_topo")
    m = oc.TriMesh(g["topo_Vrest"], g["topo_V"], g["topo_F"], g["topo_fixed"])
    m.setCohesiveEdges(g["topo_cohE"])
    with pytest.raises(oc.OCError):
        m.querySplit(g["topo_best"][3], bijective=True)


def test_learned_bijective_probe_features_and_full_fraction(golden):
    """The learned proposal on bijective queries: its probe is the bijective
    solve's own first iteration, so the one-step pass sees exactly the
    features an exhaustive bijective query records; with the whole fraction
    solved exactly it reproduces the exhaustive query."""
    g = golden("sheet_3k_bij_topo")
    m, opt = bij_state(g)
    lam = g["topo_best"][3]
    ex = m.querySplit(lam, splitInterior=True, features=True, bijective=True)
    mlp = oc.MLP(32, 128, seed=3)
    le = m.querySplit(lam, splitInterior=True, mlp=mlp, topFrac=0.1, bijective=True)
    np.testing.assert_array_equal(le["features"], ex["features"])
    assert le["selected"] == max(min(ex["local_problems"], 32), int(np.ceil(0.1 * ex["local_problems"])))
    full = m.querySplit(lam, splitInterior=True, mlp=mlp, topFrac=1.0, bijective=True)
    assert [c["EwDec"] for c in full["candidates"]] == [c["EwDec"] for c in ex["candidates"]]
    # trained on the exhaustive pairs, the learned pass keeps the best candidate
    mlp.train(ex["features"], ex["target"], epochs=40, batch=256, lr=2e-3, seed=3)
    le = m.querySplit(lam, splitInterior=True, mlp=mlp, topFrac=0.2, bijective=True)
    assert le["EwDec_max"] == pytest.approx(ex["EwDec_max"], rel=1e-12)
