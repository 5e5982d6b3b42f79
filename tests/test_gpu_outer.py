"""The OptCuts outer loop on the GPU against whole runs of the reference.

The reference driver (oracle/ref/ref_outer.cpp restating src/main.cpp's
offline preDrawFunc, updateLambda_stationaryV and converge_preDrawFunc)
ran each mesh from its Tutte start to the end of the outer loop with
b_d = 4.1 and bijectivity off (tests/golden/*_outer.npz).  The GPU run
starts from the same state and must end the same way: finished, E_SD at the
bound (b_d - 1e-3 <= E_SD <= b_d, or the oscillation stop below it), E_SD,
E_se and lambda within 0.5% of the reference's, and no inverted triangle.
The sequence of operations is compared up to the first divergence: the
runs are the same discrete process, and a topology decision taken on energy
changes that agree to 1e-6 may still flip on a near-tie."""
import numpy as np
import pytest

import optcuts_gb300 as oc

pytestmark = pytest.mark.gpu

CASES = ["icosphere_320_outer", "icosphere_1k_outer", "icosphere_5k_outer"]


def run_outer(g, **kw):
    m = oc.TriMesh(g["V_rest"], g["UV0"], g["F"], g["fixedVert"])
    m.setCohesiveEdges(g["cohE"])
    opt = oc.Optimizer(m, [1.0 - g["scalars"][4]])
    opt.precompute()
    o = oc.OptCuts(opt, upperBound=4.1, **kw)
    finished = o.run()
    return m, opt, o, finished


@pytest.mark.parametrize("case", CASES)
def test_outer_loop_matches_reference(golden, case):
    g = golden(case)
    m, opt, o, finished = run_outer(g)
    ref = g["outer_final"]
    st = o.state()
    assert finished and ref[5] == 1
    assert m.checkInversion()
    assert st["E_SD"] <= 4.1 + 1e-12
    for k, i in (("E_SD", 0), ("E_se", 1), ("lambda", 2)):
        assert abs(st[k] - ref[i]) <= 5e-3 * abs(ref[i]), (k, st[k], ref[i])
    ev, rev = o.events(), g["outer_events"]
    assert len(ev) > 0 and ev[0, 5] == 0 and rev[0, 5] == 0
    # the first inner loop converges to the same state before any topology change
    assert abs(ev[0, 1] - rev[0, 1]) <= 1e-3 * rev[0, 1]


def test_outer_loop_first_decisions_match(golden):
    """On the 1k icosphere the first topology steps (the dual update, the
    first boundary split and the critical-lambda splits after it) are the
    reference's: same event codes and vertex counts until the first
    divergence, which must not come before the third operation."""
    g = golden("icosphere_1k_outer")
    _, _, o, _ = run_outer(g)
    ev, rev = o.events(), g["outer_events"]
    n = min(len(ev), len(rev))
    same = 0
    while same < n and ev[same, 5] == rev[same, 5] and ev[same, 4] == rev[same, 4]:
        same += 1
    assert same >= 6, (ev[:8], rev[:8])


def test_outer_loop_trace_and_state(golden):
    g = golden("icosphere_320_outer")
    m, opt, o, finished = run_outer(g)
    tr = o.trace()
    st = o.state()
    assert finished and len(tr) > 0
    assert tr[-1, 0] <= st["newton_iterations"]
    assert st["topology_steps"] >= 1 and st["vertices"] == m.nV
    assert st["total_ms"] >= st["newton_ms"] >= 0.0
    # E_w of every row is lambda-weighted: (1 - lambda) E_SD + lambda E_se
    assert tr.shape[1] == 7 and np.all(tr[:, 6] >= 0.0)
    lam = tr[:, 4]
    np.testing.assert_allclose(tr[:, 1], (1 - lam) * tr[:, 2] + lam * tr[:, 3], rtol=1e-12)


def test_outer_loop_writes_reference_outputs(golden, tmp_path):
    """energyValPerIter.txt, gradientPerIter.txt, info.txt and
    finalResult_mesh.obj as the reference writes them (Optimizer.cpp:706-740,
    main.cpp:346-387, TriMesh.cpp:1758-1969)."""
    g = golden("icosphere_320_outer")
    m, opt, o, finished = run_outer(g)
    tr = o.trace()
    o.write(str(tmp_path), F0=g["mesh_F"], nV0=len(g["mesh_V"]), lambdaInit=0.999)
    E = np.loadtxt(tmp_path / "energyValPerIter.txt")
    G = np.loadtxt(tmp_path / "gradientPerIter.txt")
    assert E.shape == (len(tr), 4) and G.shape == (len(tr), 2)
    np.testing.assert_allclose(E[:, 1], tr[:, 2], rtol=1e-5)          # E_SD, six digits
    np.testing.assert_allclose(E[:, 3], 1.0 - tr[:, 4], rtol=1e-5)    # energyParams[0]
    info = (tmp_path / "info.txt").read_text().splitlines()
    assert info[0].split() == [str(len(g["mesh_V"])), str(len(g["mesh_F"]))]
    st = o.state()
    assert int(info[1].split()[0]) == int(st["newton_iterations"])
    dist, seam = (float(x) for x in info[3].split())
    assert dist == pytest.approx(st["E_SD"], rel=1e-5) and seam == pytest.approx(st["E_se"], rel=1e-5)
    stretch = [float(x) for x in info[4].split()]
    assert len(stretch) == 4 and stretch[0] >= 1.0 - 1e-9 and stretch[3] <= 1.0 + 1e-9
    assert info[5] == "initialSeams %d" % len(g["cohE"])
    lines = (tmp_path / "finalResult_mesh.obj").read_text().splitlines()
    v = np.array([[float(x) for x in l.split()[1:]] for l in lines if l.startswith("v ")])
    vt = [l for l in lines if l.startswith("vt ")]
    f = [l for l in lines if l.startswith("f ")]
    assert len(v) == len(g["mesh_V"]) and len(vt) == m.nV and len(f) == len(g["mesh_F"])
    np.testing.assert_allclose(v, g["mesh_V"], rtol=1e-6, atol=1e-6)   # rest positions in the input numbering
    first = [int(x.split("/")[0]) - 1 for x in f[0].split()[1:]]
    assert first == g["mesh_F"][0].tolist()


BIJ_CASES = ["icosphere_320_bij_outer", "icosphere_1k_bij_outer"]


def boundary_self_intersections(UV, F):
    """Pairs of non-adjacent boundary edges of the UV layout that cross (0
    for a bijective map)."""
    from collections import Counter
    cnt = Counter()
    for a, b, c in F:
        for u, v in ((a, b), (b, c), (c, a)):
            cnt[(int(u), int(v))] += 1
    bnd = [(u, v) for (u, v) in cnt if (v, u) not in cnt]
    P = np.asarray(UV)

    def cross(o, a, b):
        return (a[0] - o[0]) * (b[1] - o[1]) - (a[1] - o[1]) * (b[0] - o[0])

    n = 0
    for i in range(len(bnd)):
        a, b = P[bnd[i][0]], P[bnd[i][1]]
        for j in range(i + 1, len(bnd)):
            if set(bnd[i]) & set(bnd[j]):
                continue
            c, d = P[bnd[j][0]], P[bnd[j][1]]
            if cross(a, b, c) * cross(a, b, d) < 0 and cross(c, d, a) * cross(c, d, b) < 0:
                n += 1
    return n


@pytest.mark.parametrize("case", BIJ_CASES)
def test_outer_loop_bijective_matches_reference(golden, case):
    """Bijectivity on (the reference's default): the scaffold starts after
    the first inner loop, every topology query is bijective, no exact final
    solve.  The whole-mesh air meshes come from this project's generator,
    not Triangle, so the trajectories separate at rounding level over the
    run; the end state must still agree within 1%, stay within the bound,
    and the final UV layout must not overlap itself."""
    g = golden(case)
    m, opt, o, finished = run_outer(g, bijective=True)
    ref = g["outer_final"]
    st = o.state()
    assert finished and ref[5] == 1
    assert m.checkInversion()
    assert st["E_SD"] <= 4.1 + 1e-12
    for k, i in (("E_SD", 0), ("E_se", 1), ("lambda", 2)):
        assert abs(st[k] - ref[i]) <= 1e-2 * abs(ref[i]), (k, st[k], ref[i])
    assert boundary_self_intersections(m.V, m.F) == 0
    ev, rev = o.events(), g["outer_events"]
    assert abs(ev[0, 1] - rev[0, 1]) <= 1e-3 * rev[0, 1]
