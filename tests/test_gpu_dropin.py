"""The reference's LinSysSolver interface on the GPU, driven the way the
reference's Optimizer drives it (Optimizer.cpp:154-201, 505-652):
set_pattern(vNeighbor, fixedVert), then per Newton iteration update_a with
the triplet Hessian (energyParams[0] x the PSD-projected per-triangle blocks
and the unit fixed-vertex diagonal, SymDirichletEnergy.cpp:429-549),
factorize, solve(-gradient), the injective bound x 0.99 and the halving
line search.  The neighbour-list pattern must give the same run, bit for
bit, as the pattern derived from the triangles, and its first step the
reference's energy."""
import numpy as np
import pytest

import optcuts_gb300 as oc

pytestmark = pytest.mark.gpu


def vneighbor(nV, F):
    """TriMesh::vNeighbor: per vertex the set of vertices sharing an edge."""
    nb = [set() for _ in range(nV)]
    for a, b, c in F:
        for u, v in ((a, b), (b, c), (c, a)):
            nb[u].add(int(v))
            nb[v].add(int(u))
    return nb


def triplets(blocks, F, fixed, param):
    I, J, V = [], [], []
    fx = set(int(v) for v in fixed)
    for t, tri in enumerate(F):
        idx = [(a, int(v)) for a, v in enumerate(tri) if int(v) not in fx]
        for a, va in idx:
            for b, vb in idx:
                for p in range(2):
                    for q in range(2):
                        I.append(2 * va + p)
                        J.append(2 * vb + q)
                        V.append(blocks[t, 2 * a + p, 2 * b + q])
    for v in sorted(fx):
        for p in range(2):
            I.append(2 * v + p)
            J.append(2 * v + p)
            V.append(1.0)
    return np.array(I), np.array(J), param * np.array(V)


def run(g, neighbors, iters):
    par = 1.0 - g["scalars"][4]
    m = oc.TriMesh(g["V_rest"], g["UV0"], g["F"], g["fixedVert"])
    sd = oc.SymDirichletEnergy()
    ls = oc.LinSysSolver(solver=oc.SOLVER_DIRECT)
    nV = len(g["UV0"])
    if neighbors:
        ls.set_pattern_neighbors(vneighbor(nV, g["F"]), g["fixedVert"])
    else:
        ls.set_pattern(nV, g["F"], g["fixedVert"])
    E = [par * sd.computeEnergyVal(m)]
    for _ in range(iters):
        grad = par * sd.computeGradient(m)
        ls.update_a(*triplets(sd.computeHessian(m), g["F"], g["fixedVert"], par))
        assert ls.factorize()
        d = ls.solve(-grad)
        alpha = sd.initStepSize(m, d) * 0.99
        uv0 = m.V.copy()
        while True:
            m.V = uv0 + alpha * d.reshape(-1, 2)
            e = par * sd.computeEnergyVal(m)
            if not e > E[-1] or alpha == 0.0:
                break
            alpha /= 2.0
        E.append(e)
    return np.array(E), m.V


@pytest.mark.parametrize("case", ["icosphere_320", "torus_768"])
def test_neighbor_pattern_equals_mesh_pattern(golden, case):
    g = golden(case)
    E1, uv1 = run(g, True, 5)
    E2, uv2 = run(g, False, 5)
    np.testing.assert_array_equal(E1, E2)
    np.testing.assert_array_equal(uv1, uv2)
    assert np.all(np.diff(E1) <= 0.0)


def test_neighbor_pattern_first_step_matches_reference(golden):
    g = golden("icosphere_320")
    E, _ = run(g, True, 1)
    assert E[0] == pytest.approx(g["trace_E"][0], rel=1e-14)
    assert abs(E[1] - g["trace_E"][1]) <= 1e-6 * g["trace_E"][1]
