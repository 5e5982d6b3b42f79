"""Topology queries on the GPU (every candidate's local projected-Newton
solve in one batched launch) against the reference's own queries on the
same converged state (tests/golden/*_topo, bijectivity off)."""
import numpy as np
import pytest

import optcuts_gb300 as oc
from conftest import TOPO_CASES, golden_candidates

pytestmark = pytest.mark.gpu
DBL_MAX = np.finfo(np.float64).max


def topo_mesh(g):
    m = oc.TriMesh(g["topo_Vrest"], g["topo_V"], g["topo_F"], g["topo_fixed"])
    m.setCohesiveEdges(g["topo_cohE"])
    return m


@pytest.mark.parametrize("case", TOPO_CASES)
def test_split_filter_bit_exact(golden, case):
    g = golden(case)
    np.testing.assert_array_equal(topo_mesh(g).splitFilter(), g["topo_divGrad"])


def compare(ours, ref, rel=1e-6):
    """Same candidates, paths and energy changes; the same new vertex
    positions except for cut-through boundary splits (4 rows): their local
    mesh falls apart into two pieces, and a piece held by a single fixed
    vertex can rotate about it at no energy cost, so where its vertices end
    up depends on how each LDL^T rounds that singular direction."""
    assert len(ours["candidates"]) == len(ref)
    for c, r in zip(ours["candidates"], ref):
        if r["energyChanges"][0] == DBL_MAX:
            assert c["EwDec"] == -DBL_MAX
            continue
        assert c["path"] == r["path"]
        for a, b in zip(c["energyChanges"], r["energyChanges"]):
            assert a == pytest.approx(b, rel=rel, abs=1e-12)
        assert c["newVertPos"].shape == r["newVertPos"].shape
        if len(r["newVertPos"]) == 4:
            continue
        scale = np.abs(r["newVertPos"]).max() + 1e-12
        assert np.abs(c["newVertPos"] - r["newVertPos"]).max() <= 1e-5 * scale


@pytest.mark.parametrize("case", TOPO_CASES)
def test_boundary_split_query(golden, case):
    g = golden(case)
    lam_t = g["topo_best"][3]
    q = topo_mesh(g).querySplit(lam_t, splitInterior=False)
    compare(q, golden_candidates(g, "bSplit"))
    assert q["EwDec_max"] == pytest.approx(g["topo_best"][0], rel=1e-6)


@pytest.mark.parametrize("case", TOPO_CASES)
def test_interior_split_query(golden, case):
    g = golden(case)
    lam_t = g["topo_best"][3]
    q = topo_mesh(g).querySplit(lam_t, splitInterior=True)
    compare(q, golden_candidates(g, "iSplit"))
    assert q["EwDec_max"] == pytest.approx(g["topo_best"][2], rel=1e-6)
    assert q["pool"] == int(g["topo_best"][4])
    assert q["local_problems"] > len(q["candidates"])


@pytest.mark.parametrize("case", TOPO_CASES)
def test_fp32_projection_option(golden, case):
    """FP32 projection of the local element Hessians: the same candidates and
    paths; energy changes within 1e-3 relative (the local solves stop at a
    gradient tolerance, so a differently rounded Hessian stops at another
    point of that tolerance band)."""
    g = golden(case)
    lam_t = g["topo_best"][3]
    for interior, tag in ((False, "bSplit"), (True, "iSplit")):
        q = topo_mesh(g).querySplit(lam_t, splitInterior=interior, fp32=True)
        ref = golden_candidates(g, tag)
        assert len(q["candidates"]) == len(ref)
        for c, r in zip(q["candidates"], ref):
            if r["energyChanges"][0] == DBL_MAX:
                continue
            assert c["path"] == r["path"]
            assert c["energyChanges"][0] == pytest.approx(r["energyChanges"][0], rel=1e-3, abs=1e-9)


@pytest.mark.parametrize("case", TOPO_CASES)
def test_merge_query(golden, case):
    g = golden(case)
    q = topo_mesh(g).queryMerge(g["topo_best"][3])
    assert len(q["candidates"]) == len(golden_candidates(g, "merge"))


@pytest.mark.parametrize("case", TOPO_CASES)
def test_merge_query_after_split(golden, case):
    """queryMerge on the state after the reference applied its best boundary
    split: the new zipper-bottom pair (undoing that split) and any others."""
    g = golden(case)
    m = oc.TriMesh(g["topo_afterB_Vrest"], g["topo_afterB_V"], g["topo_afterB_F"], g["topo_fixed"])
    m.setCohesiveEdges(g["topo_afterB_cohE"])
    q = m.queryMerge(g["topo_best"][3])
    compare(q, golden_candidates(g, "mergeB"))
    assert q["EwDec_max"] == pytest.approx(float(g["topo_mergeB_best"][0]), rel=1e-6)


@pytest.mark.parametrize("case", ["icosphere_320_topo", "sheet_3k_topo"])
def test_create_fracture_through_the_optimizer(golden, case):
    """Optimizer::createFracture with a queried boundary split: the mesh
    takes the reference's new topology, the energy is recomputed, and Newton
    continues without inverting anything."""
    g = golden(case)
    m = topo_mesh(g)
    par = 1.0 - g["topo_best"][3]
    opt = oc.Optimizer(m, [par])
    opt.precompute()
    q = m.querySplit(g["topo_best"][3], splitInterior=False)
    c = q["candidates"][q["best"]]
    assert c["path"] == list(g["topo_opB_path"])
    opt.createFracture(oc.OP_BOUNDARY_SPLIT, g["topo_opB_path"], g["topo_opB_pos"])
    np.testing.assert_array_equal(m.F, g["topo_afterB_F"])
    np.testing.assert_array_equal(m.cohE, g["topo_afterB_cohE"].reshape(-1, 4))
    np.testing.assert_array_equal(m.V, g["topo_afterB_V"])
    e = opt.getLastEnergyVal()
    assert e == pytest.approx(par * oc.SymDirichletEnergy().computeEnergyVal(m), rel=1e-13)
    for _ in range(5):
        opt.solve(1)
        assert opt.getLastEnergyVal() <= e
        e = opt.getLastEnergyVal()
    assert m.checkInversion()


@pytest.mark.parametrize("case", ["icosphere_320_topo", "sheet_3k_topo"])
@pytest.mark.parametrize("learned", [False, True])
def test_split_or_merge(golden, case, learned):
    """Optimizer::createFracture(thres, 0, ...) -> TriMesh::splitOrMerge: the
    larger of the best boundary split and the best merge, applied when above
    the threshold; the reference's applied boundary split comes out (its
    topology bit-exact, positions to the candidates' tolerance). The learned
    form with every problem selected takes the same decision."""
    g = golden(case)
    par = 1.0 - g["topo_best"][3]
    m = topo_mesh(g)
    opt = oc.Optimizer(m, [par])
    opt.precompute()
    F0 = m.F.copy()
    mlp = oc.MLP(32, 128, seed=3) if learned else None
    changed, op, ew = opt.splitOrMerge(1e300, mlp=mlp, topFrac=1.0)
    assert not changed and op == oc.OP_BOUNDARY_SPLIT
    assert ew == pytest.approx(g["topo_best"][0], rel=1e-6)
    np.testing.assert_array_equal(m.F, F0)
    changed, op, ew = opt.splitOrMerge(-1e300, mlp=mlp, topFrac=1.0)
    assert changed and op == oc.OP_BOUNDARY_SPLIT
    np.testing.assert_array_equal(m.F, g["topo_afterB_F"])
    np.testing.assert_array_equal(m.cohE, g["topo_afterB_cohE"].reshape(-1, 4))
    ref = g["topo_afterB_V"]
    assert np.abs(m.V - ref).max() <= 1e-5 * np.abs(ref).max()
    e = opt.getLastEnergyVal()
    assert e == pytest.approx(par * oc.SymDirichletEnergy().computeEnergyVal(m), rel=1e-13)


@pytest.mark.parametrize("nlon,nlat", [(24, 8), (72, 10), (200, 10)])
def test_problem_size_classes_match_oracle(nlon, nlat):
    """Pole fans of 24, 72 and 200 triangles put boundary-split problems in
    every threads-per-problem class (8, 32, 128, 256 threads); each class
    sums in triangle order, so every candidate's E_w decrease agrees with
    the oracle's to 1e-8 and, where its local solves converged, its new
    positions to 1e-5 of their scale at the converged state
    (the local solves project the element Hessians in the translation-free
    4x4 form, the oracle with the reference's 6x6 eigen-clamp)."""
    import os

    import oracle as O
    from optcuts_gb300 import init as I
    from optcuts_gb300 import meshes as M
    V, F = M.ellipsoid(nlon, nlat, (1.0, 0.6, 0.4), 8, 6, 0.02, 2)
    st = I.init_uv(V, F)
    mesh = oc.TriMesh(st.V_rest, st.UV, st.F, st.fixedVert)
    opt = oc.Optimizer(mesh, [0.001])
    opt.precompute()
    opt.solve(300)
    mesh.setCohesiveEdges(st.cohE)
    sizes = set()
    checked = 0
    for op in (oc.OP_BOUNDARY_SPLIT, oc.OP_INTERIOR_SPLIT):
        q = mesh.querySplit(0.999, splitInterior=op == oc.OP_INTERIOR_SPLIT)
        ref, _ = O.topology_query(mesh.V_rest, mesh.V, mesh.F, st.cohE, op, 0.999, threads=os.cpu_count() or 1)
        assert len(q["candidates"]) == len(ref)
        # a local solve that stops at the 100-iteration cap (the largest pole
        # fans, slow along a nearly flat direction) ends where its rounding
        # led it: there only the E_w decrease is compared
        pr = q["problems"]
        capped = set(pr["cand"][pr["iters"] >= 100].tolist())
        for ci, (c, r) in enumerate(zip(q["candidates"], ref)):
            assert c["EwDec"] == pytest.approx(r["EwDec"], rel=1e-8, abs=1e-12)
            assert c["path"] == r["path"]
            if len(r["newVertPos"]) != 4 and ci not in capped:   # cut-through splits: see compare()
                scale = np.abs(r["newVertPos"]).max() + 1e-12
                assert np.abs(c["newVertPos"] - r["newVertPos"]).max() <= 1e-5 * scale
                checked += 1
        sizes.update(int(n) for n in q["problems"]["nTri"])
    assert checked > 0
    assert max(sizes) >= nlon and min(sizes) <= 8
    # a learned query solves few problems exactly, so its large fans run on
    # clusters of blocks: the same decreases as the exhaustive pass
    mlp = oc.MLP(32, 128, seed=3)
    for op in (oc.OP_BOUNDARY_SPLIT, oc.OP_INTERIOR_SPLIT):
        ex = mesh.querySplit(0.999, splitInterior=op == oc.OP_INTERIOR_SPLIT)
        le = mesh.querySplit(0.999, splitInterior=op == oc.OP_INTERIOR_SPLIT, mlp=mlp, topFrac=0.05)
        sel = np.isfinite(le["problems"]["EwDec"])
        assert sel.sum() == le["selected"]
        np.testing.assert_allclose(le["problems"]["EwDec"][sel], ex["problems"]["EwDec"][sel], rtol=1e-8, atol=1e-12)


@pytest.mark.parametrize("case", ["icosphere_320_topo", "ellipsoid_2k_topo"])
@pytest.mark.parametrize("world", [2, 3])
def test_sharded_step_equals_unsharded(golden, case, world):
    """Each shard solves only its candidates; merged (optcuts_gb300.shard),
    the lists equal the unsharded step's bit for bit."""
    from optcuts_gb300 import shard
    g = golden(case)
    m = topo_mesh(g)
    lam = float(g["topo_best"][3])
    full = [q for q in m.topologyStep(lam)]
    merged = shard.merge([m.topologyStepShard(lam, r, world) for r in range(world)])
    for q, s in zip(full, merged):
        np.testing.assert_array_equal(np.array([c["EwDec"] for c in q["candidates"]]), s["EwDec"])
        np.testing.assert_array_equal(np.array([c["energyChanges"] for c in q["candidates"]]).reshape(-1, 2),
                                      s["energyChanges"])
        assert q["best"] == s["best"]


def test_autotuned_schedules_same_candidates(golden):
    """The measured schedule autotuner: the step with the tuned schedules
    reports the same candidates (energy changes to 1e-8 relative: clustered
    sums may group differently) and fills the table with timings."""
    g = golden("ellipsoid_2k_topo")
    m = topo_mesh(g)
    lam = float(g["topo_best"][3])
    ref = m.topologyStep(lam)
    for _ in range(2):   # the first call tunes, the second reuses the table
        got = m.topologyStep(lam, autotune=True)
        for q, r in zip(got, ref):
            assert len(q["candidates"]) == len(r["candidates"]) and q["best"] == r["best"]
            for a, b in zip(q["candidates"], r["candidates"]):
                if b["EwDec"] > -1e300:
                    assert abs(a["EwDec"] - b["EwDec"]) <= 1e-8 * abs(b["EwDec"]) + 1e-14
    table = oc.topology_schedules()
    assert table and all(t["chosen"]["ms"] > 0.0 and t["candidates"] >= 2 for t in table)
    assert all(t["chosen"]["ms"] <= t["rule"]["ms"] + 1e-6 for t in table if t["rule"]["ms"] > 0.0)
