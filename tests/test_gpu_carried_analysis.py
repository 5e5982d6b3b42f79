"""The direct solver's symbolic analysis carried through topology
operations (oc_optimizer_config.carryAnalysis): after a split the copy joins
its source vertex's dissection node, after a merge the merged vertex the two
nodes' common ancestor, and only the front structures are rebuilt.  The
elimination order then differs from a fresh dissection's, so the Newton
runs after the operations must agree with the runs that re-analyse from
scratch to rounding (the states are converged, not chaotic), and the
analyses must have been carried."""
import numpy as np
import pytest

import optcuts_gb300 as oc

pytestmark = pytest.mark.gpu
CASES = [("torus_768_topo", False), ("sheet_3k_topo", False), ("icosphere_320_bij_topo", True),
         ("torus_768_bij_topo", True)]


def run(g, carry, scaf, newton=3, exact=False):
    """The reference's best boundary split, then its best merge of the new
    state (a vertex appended, then one merged away with the last vertex
    moved into its slot), each followed by Newton iterations.  exact: the
    scaffold's exact air pattern instead of the dense clique (the form of
    scaffolds too large for the clique), whose carried analyses keep the
    air-only vertices in the root front."""
    lam = float(g["topo_best"][3])
    m = oc.TriMesh(g["topo_Vrest"], g["topo_V"], g["topo_F"], g["topo_fixed"])
    m.setCohesiveEdges(g["topo_cohE"])
    opt = oc.Optimizer(m, [1.0 - lam], carryAnalysis=1 if carry else 0, scaffoldPattern=1 if exact else 0)
    if scaf:
        opt.rebuildScaffold()
    opt.precompute()
    E, info = [], []
    ops = [(oc.OP_BOUNDARY_SPLIT, g["topo_opB_path"], g["topo_opB_pos"])]
    if "topo_opM_path" in g:
        ops.append((oc.OP_MERGE, g["topo_opM_path"], g["topo_opM_pos"]))
    for op, path, pos in ops:
        opt.createFracture(op, path, pos)
        info.append(opt.analysisInfo())
        for _ in range(newton):
            r = opt.solve(1)
            E.append(opt.getLastEnergyVal())
            if r == 1:
                break
            if scaf:
                opt.rebuildScaffold()
    return np.array(E), info, m


@pytest.mark.parametrize("case,scaf", CASES)
def test_carried_analysis_equals_full(golden, case, scaf):
    g = golden(case)
    Ec, ic, mc = run(g, True, scaf)
    Ef, if_, mf = run(g, False, scaf)
    assert len(Ec) == len(Ef)
    np.testing.assert_allclose(Ec, Ef, rtol=1e-10)
    np.testing.assert_allclose(mc.V, mf.V, rtol=0, atol=1e-9 * np.abs(mf.V).max())
    assert all(i["carried"] >= 1 and i["nd_ms"] == 0.0 for i in ic), ic
    assert all(i["carried"] == 0 for i in if_), if_
    for a, b in zip(ic, if_):
        assert a["flops"] <= 1.3 * a["full_flops"]


@pytest.mark.parametrize("case", ["icosphere_320_bij_topo", "torus_768_bij_topo"])
def test_carried_analysis_exact_air_pattern(golden, case):
    """A scaffold with its exact air pattern: the operations' analyses and
    those of the rebuilt air meshes between Newton steps are carried (the
    air-only vertices as the root front), and the runs agree with the runs
    that re-analyse from scratch to rounding."""
    g = golden(case)
    Ec, ic, mc = run(g, True, True, exact=True)
    Ef, if_, mf = run(g, False, True, exact=True)
    assert len(Ec) == len(Ef)
    np.testing.assert_allclose(Ec, Ef, rtol=1e-10)
    np.testing.assert_allclose(mc.V, mf.V, rtol=0, atol=1e-9 * np.abs(mf.V).max())
    assert all(i["carried"] >= 1 and i["nd_ms"] == 0.0 for i in ic), ic
    assert all(i["carried"] == 0 for i in if_), if_
