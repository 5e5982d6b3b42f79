"""CUDA kernels against the reference's golden vectors and the CPU oracle,
through the C ABI (each call below is one oc_* entry point)."""
import numpy as np
import pytest

import optcuts_gb300 as oc
import oracle as O
from conftest import GOLDEN_CASES, SCAFFOLD_OFF

pytestmark = pytest.mark.gpu


def mesh_of(g):
    return oc.TriMesh(g["V_rest"], g["UV0"], g["F"], g["fixedVert"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_rest_constants_bit_exact(golden, case):
    g = golden(case)
    rest, sc = mesh_of(g).rest_constants()
    np.testing.assert_array_equal(rest, g["rest"])
    np.testing.assert_array_equal(sc, g["scalars"][:3])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_energy_per_elem_bit_exact(golden, case):
    # FP64, no FMA contraction, IEEE division: identical rounding to the reference
    g = golden(case)
    e = oc.SymDirichletEnergy().getEnergyValPerElem(mesh_of(g))
    np.testing.assert_array_equal(e, g["E_elem0"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_energy_total(golden, case):
    g = golden(case)
    E = oc.SymDirichletEnergy().computeEnergyVal(mesh_of(g))
    ref = g["E_elem0"].sum()
    assert abs(E - ref) <= 1e-14 * abs(ref) * max(1.0, np.log2(len(g["F"])))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_gradient_bit_exact(golden, case):
    g = golden(case)
    grad = oc.SymDirichletEnergy().computeGradient(mesh_of(g))
    np.testing.assert_array_equal(grad, g["grad0"])


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_uniform_weight_energy_and_gradient(golden, case):
    g = golden(case)
    m = mesh_of(g)
    sd = oc.SymDirichletEnergy()
    np.testing.assert_array_equal(sd.getEnergyValPerElem(m, True), O.energy_elem(g["rest"], g["F"], g["UV0"], True))
    np.testing.assert_array_equal(sd.computeGradient(m, True),
                                  O.gradient(g["rest"], g["F"], g["UV0"], g["fixedVert"], True))


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_hessian_psd_projection(golden, case):
    """FP64 6x6 eigen-clamp.  Against the CPU oracle (the same cyclic Jacobi,
    same operation order, no FMA on either side) the upper triangle is
    bit-identical; against the reference (Eigen's tridiagonal QR eigensolver)
    it agrees to rounding relative to each block's largest entry."""
    g = golden(case)
    H = oc.SymDirichletEnergy().computeHessian(mesh_of(g))
    ref_all = O.hessian_blocks(g["rest"], g["F"], g["UV0"])
    iu = np.triu_indices(6)
    np.testing.assert_array_equal(H[:, iu[0], iu[1]], ref_all[:, iu[0], iu[1]])
    scale = np.abs(ref_all).reshape(len(ref_all), -1).max(axis=1)[:, None, None]
    err = np.abs(H - ref_all) / scale
    assert err.max() < 1e-14, err.max()
    # against the reference's own blocks (fixed rows/cols removed there)
    ref = g["H0_blocks"]
    fixed = set(g["fixedVert"].tolist())
    Hm = H[: len(ref)].copy()
    for t in range(len(ref)):
        keep = np.array([int(g["F"][t, k // 2]) not in fixed for k in range(6)])
        Hm[t][~keep, :] = 0.0
        Hm[t][:, ~keep] = 0.0
    assert (np.abs(Hm - ref) / scale[: len(ref)]).max() < 1e-10
    # every projected block is PSD to rounding
    ev = np.linalg.eigvalsh(H)
    assert (ev.min(axis=1) / scale[:, 0, 0]).min() > -1e-12


@pytest.mark.parametrize("case", SCAFFOLD_OFF)
def test_init_step_size_exact(golden, case):
    g = golden(case)
    s = oc.SymDirichletEnergy().initStepSize(mesh_of(g), g["dir0"], 1.0)
    assert s == O.init_step_size(g["F"], g["UV0"], g["dir0"], 1.0)


def test_init_step_size_keeps_smaller_input(golden):
    g = golden("icosphere_320")
    s = oc.SymDirichletEnergy().initStepSize(mesh_of(g), g["dir0"], 1e-6)
    assert s == 1e-6


def test_check_inversion(golden):
    g = golden("icosphere_320")
    m = mesh_of(g)
    assert m.checkInversion()
    uv = g["UV0"].copy()
    t = g["F"][7]
    uv[t[0]], uv[t[1]] = g["UV0"][t[1]], g["UV0"][t[0]]   # flip one triangle
    m.V = uv
    assert not m.checkInversion()


def _assembled_dense(g, par):
    """Dense reference matrix from the oracle's blocks (fixed rows = par * I)."""
    n = 2 * len(g["UV0"])
    B = O.hessian_blocks(g["rest"], g["F"], g["UV0"])
    A = np.zeros((n, n))
    fixed = set(g["fixedVert"].tolist())
    for t, tri in enumerate(g["F"]):
        for a in range(3):
            for b in range(3):
                if tri[a] in fixed or tri[b] in fixed:
                    continue
                A[2 * tri[a]:2 * tri[a] + 2, 2 * tri[b]:2 * tri[b] + 2] += par * B[t, 2 * a:2 * a + 2, 2 * b:2 * b + 2]
    for v in fixed:
        A[2 * v:2 * v + 2, 2 * v:2 * v + 2] = par * np.eye(2)
    return A


def _reference_triplets(g, par):
    """Triplets in the reference's order (IglUtils::addBlockToMatrix + the
    fixed-vertex diagonal, SymDirichletEnergy.cpp:536-548), scaled by par."""
    B = O.hessian_blocks(g["rest"], g["F"], g["UV0"])
    fixed = set(g["fixedVert"].tolist())
    I, J, V = [], [], []
    for t, tri in enumerate(g["F"]):
        idx = [a for a in range(3) if int(tri[a]) not in fixed]
        for a in idx:
            for b in idx:
                for i in range(2):
                    for j in range(2):
                        I.append(2 * tri[a] + i)
                        J.append(2 * tri[b] + j)
                        V.append(par * B[t, 2 * a + i, 2 * b + j])
    for v in sorted(fixed):
        I += [2 * v, 2 * v + 1]
        J += [2 * v, 2 * v + 1]
        V += [par, par]
    return np.array(I), np.array(J), np.array(V)


@pytest.mark.parametrize("case", ["cube", "icosphere_320", "ellipsoid_2k", "icosphere_5k"])
def test_direct_solver_matches_reference_direction(golden, case):
    """Multifrontal Cholesky vs the reference's SimplicialLDLT direction."""
    g = golden(case)
    par = 1.0 - g["scalars"][4]
    I, J, V = _reference_triplets(g, par)
    ls = oc.LinSysSolver(solver=oc.SOLVER_DIRECT)
    ls.set_pattern(len(g["UV0"]), g["F"], g["fixedVert"])
    ls.update_a(I, J, V)
    assert ls.factorize()
    b = -par * g["grad0"]
    d = ls.solve(b)
    assert ls.last_relres < 1e-9, ls.last_relres
    # two exact FP64 LDL^T factorisations with different orderings agree to
    # ~cond(A) * eps in the near-null modes (the CPU oracle sees the same)
    rel = np.linalg.norm(d - g["dir0"]) / np.linalg.norm(g["dir0"])
    assert rel < 5e-3, rel
    st = ls.stats()
    assert st["dof"] == 2 * len(g["UV0"]) and st["fronts"] >= 1


@pytest.mark.parametrize("case", ["cube", "icosphere_320"])
def test_direct_solver_dense_check(golden, case):
    g = golden(case)
    par = 1.0 - g["scalars"][4]
    A = _assembled_dense(g, par)
    I, J = np.nonzero(A)
    ls = oc.LinSysSolver(solver=oc.SOLVER_DIRECT)
    ls.set_pattern(len(g["UV0"]), g["F"], g["fixedVert"])
    ls.update_a(I, J, A[I, J])
    ls.factorize()
    rng = np.random.default_rng(1)
    b = rng.standard_normal(A.shape[0])
    x = ls.solve(b)
    x_ref = np.linalg.solve(A, b)
    cond = np.linalg.cond(A)
    assert np.linalg.norm(x - x_ref) <= 1e-13 * cond * np.linalg.norm(x_ref)
    # backward stable: residual at rounding level of ||A|| ||x||
    assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(A, 2) * np.linalg.norm(x)


@pytest.mark.parametrize("case", ["cube", "icosphere_320"])
def test_linsys_update_a_multiply_solve(golden, case):
    g = golden(case)
    par = 1.0 - g["scalars"][4]
    A = _assembled_dense(g, par)
    I, J = np.nonzero(A)
    ls = oc.LinSysSolver(solver=oc.SOLVER_PCG)
    ls.set_pattern(len(g["UV0"]), g["F"], g["fixedVert"])
    ls.update_a(I, J, A[I, J])
    assert ls.factorize()
    rng = np.random.default_rng(0)
    x = rng.standard_normal(A.shape[0])
    y = ls.multiply(x)
    assert np.linalg.norm(y - A @ x) <= 1e-14 * np.linalg.norm(A) * np.linalg.norm(x)
    b = -par * g["grad0"]
    d = ls.solve(b, tol=1e-10, maxIter=50000)
    assert ls.last_converged
    # recursive PCG residual 1e-10; the true residual within rounding of it
    assert np.linalg.norm(A @ d - b) <= 1e-9 * np.linalg.norm(b) + 1e-13 * np.linalg.norm(A, 2) * np.linalg.norm(d)


def test_linsys_iteration_cap_reports_not_converged(golden):
    g = golden("icosphere_320")
    par = 1.0 - g["scalars"][4]
    A = _assembled_dense(g, par)
    I, J = np.nonzero(A)
    ls = oc.LinSysSolver(solver=oc.SOLVER_PCG)
    ls.set_pattern(len(g["UV0"]), g["F"], g["fixedVert"])
    ls.update_a(I, J, A[I, J])
    ls.factorize()
    ls.solve(-par * g["grad0"], tol=1e-12, maxIter=3)
    assert not ls.last_converged and ls.last_iters == 3


def test_invalid_inputs_rejected(golden):
    g = golden("cube")
    F = g["F"].copy()
    F[0, 0] = 10_000
    with pytest.raises(oc.OCError):
        oc.TriMesh(g["V_rest"], g["UV0"], F, g["fixedVert"])
    Vr = g["V_rest"].copy()
    t = g["F"][0]
    Vr[t[1]] = Vr[t[0]]                       # zero-area rest triangle
    with pytest.raises(oc.OCError) as e:
        oc.TriMesh(Vr, g["UV0"], g["F"], g["fixedVert"])
    assert e.value.status == 7


@pytest.mark.parametrize("case", GOLDEN_CASES)
def test_hessian_reduced_projection(golden, case):
    """The translation-free 4x4 form of the eigen-clamp (the optimizer's
    default) against the oracle's 6x6 Jacobi: the same projection up to
    rounding relative to each block's largest entry."""
    g = golden(case)
    ref_all = O.hessian_blocks(g["rest"], g["F"], g["UV0"])
    scale = np.abs(ref_all).reshape(len(ref_all), -1).max(axis=1)[:, None, None]
    H = oc.SymDirichletEnergy().computeHessian(mesh_of(g), projection=oc.HESSIAN_REDUCED)
    assert (np.abs(H - ref_all) / scale).max() < 1e-12
    assert np.array_equal(H, np.transpose(H, (0, 2, 1)))
    # translations stay in the null space
    t = np.tile([1.0, 0.0], 3)
    assert (np.abs(H @ t) / scale[:, :, 0]).max() < 1e-12
    # the hybrid: the 4x4 form or the 6x6 one per element, both to rounding
    Hh = oc.SymDirichletEnergy().computeHessian(mesh_of(g), projection=oc.HESSIAN_HYBRID)
    assert (np.abs(Hh - ref_all) / scale).max() < 1e-12
