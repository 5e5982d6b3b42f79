"""The projected-Newton Optimizer on the GPU against the reference's traces.

The reference solves each Newton system exactly (SimplicialLDLT); the GPU
path solves it exactly too, with a multifrontal LDL^T under its own
nested-dissection ordering (block-Jacobi PCG remains an option).  At a
Tutte start the Newton matrix has condition numbers near 1e14, so two exact
factorizations with different orderings give directions that differ at
cond x eps; the trajectories accumulate that and separate by up to ~10-20%
in the first iterations, while both runs converge to the same stationary
energy, which is what these tests pin (relative 1e-6 .. 5e-3), together with
the invariants: monotone energy, no inverted triangle, determinism.  Single
steps from the reference's own iterates are pinned to 1e-6 in
tests/test_gpu_parity_steps.py."""
import numpy as np
import pytest

import optcuts_gb300 as oc
from conftest import SCAFFOLD_OFF

pytestmark = pytest.mark.gpu


def run(g, iters=400, **cfg):
    m = oc.TriMesh(g["V_rest"], g["UV0"], g["F"], g["fixedVert"])
    par = 1.0 - g["scalars"][4]
    opt = oc.Optimizer(m, [par], **cfg)
    opt.precompute()
    E = [opt.getLastEnergyVal()]
    steps = []
    status = 0
    for _ in range(iters):
        status = opt.solve(1)
        E.append(opt.getLastEnergyVal())
        steps.append(opt.last_step())
        if status == 1:
            break
    return m, opt, np.array(E), steps, status


@pytest.mark.parametrize("case,tol", [("cube", 1e-6), ("icosphere_320", 1e-4), ("ellipsoid_2k", 5e-3),
                                      ("icosphere_5k", 1e-3)])
def test_converged_energy_matches_reference(golden, case, tol):
    g = golden(case)
    m, opt, E, steps, status = run(g)
    assert status == 1
    assert E[0] == pytest.approx(g["trace_E"][0], rel=1e-14)
    assert abs(E[-1] - g["trace_E"][-1]) / g["trace_E"][-1] < tol
    assert np.all(np.diff(E) <= 0.0)                 # line search never accepts an increase
    assert m.checkInversion()                        # zero flipped triangles
    assert all(s["pcgRelRes"] <= 1e-8 for s in steps if s["pcgIters"] > 0)


@pytest.mark.parametrize("case", SCAFFOLD_OFF)
def test_first_iterations_track_reference(golden, case):
    g = golden(case)
    _, _, E, _, _ = run(g, iters=10)
    m = min(len(E), len(g["trace_E"]))
    rel = np.abs(E[:m] - g["trace_E"][:m]) / g["trace_E"][:m]
    assert rel[0] < 1e-14
    assert rel.max() < 0.25, rel


def test_deterministic(golden):
    g = golden("icosphere_320")
    m1, _, E1, _, _ = run(g, iters=6)
    m2, _, E2, _, _ = run(g, iters=6)
    np.testing.assert_array_equal(E1, E2)
    np.testing.assert_array_equal(m1.V, m2.V)


def test_converged_gradient_below_target(golden):
    g = golden("icosphere_320")
    m, opt, E, steps, status = run(g)
    par = 1.0 - g["scalars"][4]
    grad = par * oc.SymDirichletEnergy().computeGradient(m)
    nV = len(g["UV0"])
    target = par * (nV - 1) / nV * 1e-12
    # stopped either by ||g||^2 < targetGRes or by the relative-decrease test
    assert grad @ grad < target or steps[-1]["stepSize"] > 1e-3


def test_inverted_start_rejected(golden):
    g = golden("icosphere_320")
    uv = g["UV0"].copy()
    t = g["F"][3]
    uv[t[0]], uv[t[1]] = g["UV0"][t[1]], g["UV0"][t[0]]
    m = oc.TriMesh(g["V_rest"], uv, g["F"], g["fixedVert"])
    opt = oc.Optimizer(m, [0.001])
    with pytest.raises(oc.OCError) as e:
        opt.precompute()
    assert e.value.status == 2


def test_energy_param_update(golden):
    g = golden("icosphere_320")
    m = oc.TriMesh(g["V_rest"], g["UV0"], g["F"], g["fixedVert"])
    opt = oc.Optimizer(m, [0.001])
    opt.precompute()
    e1 = opt.getLastEnergyVal()
    opt.energyParams[0] = 0.002
    opt.updateEnergyData()
    assert opt.getLastEnergyVal() == pytest.approx(2 * e1, rel=1e-15)


def test_pcg_solver_option_runs(golden):
    """The block-Jacobi PCG solver behind the same Optimizer (the iterative option)."""
    g = golden("icosphere_320")
    m, opt, E, steps, status = run(g, iters=5, linearSolver=oc.SOLVER_PCG, pcgMaxIter=50000)
    assert np.all(np.diff(E) <= 0.0) and m.checkInversion()
    assert all(s["pcgIters"] > 0 for s in steps)


def test_phase_timing_and_launch_count(golden):
    g = golden("icosphere_320")
    m = oc.TriMesh(g["V_rest"], g["UV0"], g["F"], g["fixedVert"])
    opt = oc.Optimizer(m, [0.001], timing=1)
    opt.precompute()
    opt.solve(2)
    ph = opt.phase_ms()
    assert set(ph) == set(oc.Optimizer.PHASES) and all(v >= 0.0 for v in ph.values())
    assert ph["factorize"] > 0.0 and ph["solve"] > 0.0
    assert opt.launch_count() > 10


def test_energy_w_trace_matches_reference(golden):
    """E_w = (1-lambda) E_SD + lambda E_se per iteration (Optimizer.cpp:706-716)."""
    from optcuts_gb300 import init as I
    g = golden("icosphere_320")
    lam = g["scalars"][4]
    seam = I.seam_sparsity(g["V_rest"], g["UV0"], g["cohE"], g["scalars"][1])
    m, opt, E, steps, status = run(g)
    Ew = [oc.energy_w(e, seam, g["scalars"][2], lam) for e in E]
    Ew_ref = g["trace_E"][-1] + lam * g["scalars"][3] / g["scalars"][2]
    assert abs(Ew[-1] - Ew_ref) / Ew_ref < 1e-4
    assert np.all(np.diff(Ew) <= 0.0)


@pytest.mark.parametrize("case", ["icosphere_320", "ellipsoid_2k"])
def test_hessian_projection_forms_agree(golden, case):
    """The Newton step with the 6x6 Jacobi projection (default), the
    translation-free 4x4 form and the hybrid of the two: the same projection
    up to rounding, so the runs converge to the same stationary energy."""
    g = golden(case)
    out = {}
    for proj in (oc.HESSIAN_REDUCED, oc.HESSIAN_JACOBI6, oc.HESSIAN_HYBRID):
        m, opt, E, steps, status = run(g, hessianProjection=proj)
        assert status == 1 and np.all(np.diff(E) <= 0.0) and m.checkInversion()
        out[proj] = E
    # both stop at the gradient tolerance, not at the same iterate
    b = out[oc.HESSIAN_JACOBI6][-1]
    for proj in (oc.HESSIAN_REDUCED, oc.HESSIAN_HYBRID):
        assert abs(out[proj][-1] - b) / b < 1e-4
        assert out[proj][0] == out[oc.HESSIAN_JACOBI6][0]   # the same start energy


def test_deterministic_multiwave_factorization():
    """Two runs at ~20k triangles with the scaffold (leaf-level panel and
    update launches of several waves, 32x32 update blocks at the top levels)
    are bit-identical: every diagonal tile is factored exactly once, by a
    launch that ends before any block reads it."""
    from optcuts_gb300 import init as I
    from optcuts_gb300 import meshes as M
    V, F = M.ellipsoid(100, 100, (1.0, 0.6, 0.4), 8, 6, 0.02, 2)
    st = I.init_uv(V, F)
    runs = []
    for _ in range(2):
        m = oc.TriMesh(st.V_rest, st.UV, st.F, st.fixedVert)
        opt = oc.Optimizer(m, [0.001])
        opt.rebuildScaffold()
        opt.precompute()
        E = []
        for _ in range(12):
            opt.solve(1)
            opt.rebuildScaffold()
            E.append(opt.getLastEnergyVal())
        runs.append((np.array(E), m.V.copy()))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])


def test_zero_pivot_is_an_error(golden):
    """A vertex no triangle references leaves a zero diagonal block in the
    Newton matrix, a zero pivot: the step ends with OC_ERR_NOT_SPD (the
    reference dumps the matrix and exits, Optimizer.cpp:548-554) and the
    mesh keeps its UV."""
    g = golden("icosphere_320")
    Vr = np.vstack([g["V_rest"], [[0.0, 0.0, 2.0]]])
    uv = np.vstack([g["UV0"], [[3.0, 3.0]]])
    m = oc.TriMesh(Vr, uv, g["F"], g["fixedVert"])
    opt = oc.Optimizer(m, [0.001])
    opt.precompute()
    with pytest.raises(oc.OCError) as e:
        opt.solve(1)
    assert e.value.status == oc.OC_ERR_NOT_SPD
    assert opt.badPivots() >= 1
    np.testing.assert_array_equal(m.V, uv)
