"""The direct solver's cluster substitutions (the top tree levels' pivot
parts solved by a thread-block cluster per front) against the one-CTA-per-
front kernels: the same bits, standalone and through Newton steps."""
import numpy as np
import pytest

import optcuts_gb300 as oc

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def state():
    from optcuts_gb300 import init as I
    from optcuts_gb300 import meshes as M
    V, F = M.ellipsoid(224, 224, (1.0, 0.6, 0.4), 8, 6, 0.02, 2)
    return I.init_uv(V, F)


def _spd_triplets(F, nV, fixed, seed):
    """A random SPD system on the mesh's vertex pattern: per triangle a 6x6
    block B B^T over its free vertices, plus the identity (the fixed
    vertices' diagonal blocks)."""
    rng = np.random.default_rng(seed)
    B = rng.standard_normal((len(F), 6, 6))
    K = np.einsum("tij,tkj->tik", B, B)
    dof = np.stack([2 * F[:, a] + c for a in range(3) for c in range(2)], axis=1)
    I = np.repeat(dof, 6, axis=1).reshape(-1)
    J = np.tile(dof, (1, 6)).reshape(-1)
    V = K.reshape(-1)
    fx = np.zeros(2 * nV, bool)
    for v in fixed:
        fx[2 * v:2 * v + 2] = True
    keep = ~(fx[I] | fx[J])
    I = np.concatenate([I[keep], np.arange(2 * nV)])
    J = np.concatenate([J[keep], np.arange(2 * nV)])
    return I, J, np.concatenate([V[keep], np.ones(2 * nV)])


def test_cluster_solve_bit_identical_standalone(state):
    F = np.asarray(state.F, np.int32)
    nV = len(state.UV)
    ls = oc.LinSysSolver(solver=oc.SOLVER_DIRECT)
    ls.set_pattern(nV, F, [0])
    I, J, V = _spd_triplets(F, nV, [0], 3)
    ls.update_a(I, J, V)
    assert ls.factorize()
    levels, largest = ls.solve_clusters()
    assert levels >= 1 and largest >= 2, (levels, largest)
    b = np.random.default_rng(4).standard_normal(2 * nV)
    x = {}
    for C in (1, 2, 4, 8):
        ls.set_solve_cluster(C)
        x[C] = ls.solve(b)
    for C in (2, 4, 8):
        np.testing.assert_array_equal(x[C], x[1])
    # and a solution: residual at rounding level
    r = ls.multiply(x[8]) - b
    assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(b)
    with pytest.raises(oc.OCError):
        ls.set_solve_cluster(0)
    with pytest.raises(oc.OCError):
        ls.set_solve_cluster(9)


def test_cluster_solve_bit_identical_newton(state):
    """Newton steps with the scaffold (the air-mesh clique as the root front)
    take the same path with clusters of up to 8 CTAs as with one CTA per
    front."""
    runs = []
    for C in (1, 8):
        m = oc.TriMesh(state.V_rest, state.UV, state.F, state.fixedVert)
        opt = oc.Optimizer(m, [0.001])
        opt.rebuildScaffold()
        opt.precompute()
        opt.set_solve_cluster(C)
        levels, largest = opt.solve_clusters()
        assert (levels == 0) if C == 1 else (levels >= 1 and largest == 8), (C, levels, largest)
        E = []
        for _ in range(4):
            opt.solve(1)
            opt.rebuildScaffold()
            E.append(opt.getLastEnergyVal())
        runs.append((np.array(E), m.V.copy()))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
