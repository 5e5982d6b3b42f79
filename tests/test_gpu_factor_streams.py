"""The direct solver's factorization with its independent subtrees on
several CUDA streams (joined by events inside the captured graph) against
one stream: the same factor bits, so the same solutions.  Streams are used
from 4 GFLOP per factorization on, so both cases are large enough."""
import numpy as np
import pytest

import optcuts_gb300 as oc
from test_gpu_cluster_solve import _spd_triplets

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def state():
    from optcuts_gb300 import init as I
    from optcuts_gb300 import meshes as M
    V, F = M.ellipsoid(224, 224, (1.0, 0.6, 0.4), 8, 6, 0.02, 2)
    return I.init_uv(V, F)


def _solve(state, streams, fixed, rhs_seed=4):
    F = np.asarray(state.F, np.int32)
    nV = len(state.UV)
    ls = oc.LinSysSolver(solver=oc.SOLVER_DIRECT)
    ls.set_factor_streams(streams)
    ls.set_pattern(nV, F, fixed)
    I, J, V = _spd_triplets(F, nV, fixed, 3)
    ls.update_a(I, J, V)
    assert ls.factorize()
    b = np.random.default_rng(rhs_seed).standard_normal(2 * nV)
    x = ls.solve(b)
    # a second factorization of new values through the same graph
    ls.update_a(I, J, 2.0 * V)
    assert ls.factorize()
    x2 = ls.solve(b)
    return ls, x, x2, b


def test_factor_streams_bit_identical(state):
    runs = {s: _solve(state, s, [0]) for s in (1, 2, 4, 8)}
    assert runs[1][0].factor_streams() == (1, 1)
    s2, g2 = runs[2][0].factor_streams()
    s4, g4 = runs[4][0].factor_streams()
    assert s2 == 2 and g2 == 3, (s2, g2)
    assert 3 <= s4 <= 4 and s4 < g4 <= 2 * s4 - 1, (s4, g4)
    s8, g8 = runs[8][0].factor_streams()
    assert s4 <= s8 <= 8 and s8 < g8 <= 2 * s8 - 1, (s8, g8)
    for s in (2, 4, 8):
        np.testing.assert_array_equal(runs[s][1], runs[1][1])
        np.testing.assert_array_equal(runs[s][2], runs[1][2])
    ls, x, x2, b = runs[8]   # the solver holds the second (doubled) matrix
    assert np.linalg.norm(ls.multiply(x2) - b) <= 1e-10 * np.linalg.norm(b)
    np.testing.assert_allclose(x2, 0.5 * x, rtol=1e-9, atol=1e-12)
    with pytest.raises(oc.OCError):
        ls.set_factor_streams(0)
    with pytest.raises(oc.OCError):
        ls.set_factor_streams(9)


def test_factor_streams_bit_identical_newton():
    """Newton steps with the scaffold (the air mesh as the root front above
    the dissected mesh) at 199k triangles take the same path on eight streams
    as on one."""
    from optcuts_gb300 import init as I
    from optcuts_gb300 import meshes as M
    state = I.init_uv(*M.CONFIGS["ellipsoid_199k"]())
    runs = []
    for s in (1, 8):
        m = oc.TriMesh(state.V_rest, state.UV, state.F, state.fixedVert)
        opt = oc.Optimizer(m, [0.001])
        opt.set_factor_streams(s)
        opt.rebuildScaffold()
        opt.precompute()
        E = []
        for _ in range(4):
            opt.solve(1)
            opt.rebuildScaffold()
            E.append(opt.getLastEnergyVal())
        used = opt.factor_streams()[0]
        assert (used == 1) if s == 1 else (used >= 2), (s, used, opt.solver_stats()["flops"])
        runs.append((np.array(E), m.V.copy()))
    np.testing.assert_array_equal(runs[0][0], runs[1][0])
    np.testing.assert_array_equal(runs[0][1], runs[1][1])
