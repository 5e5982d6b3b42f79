"""The bijectivity scaffold restated on the CPU from oracle primitives,
against the reference's own scaffold runs (tests/golden: the air mesh each
iteration used, the augmented gradient of iteration 0, energies with and
without the scaffold term).

Scaffold terms (Optimizer.cpp:764-797, Scaffold.cpp:179-230):
  E      = (1 - lambda) E_SD(mesh) + w_scaf / |F_air| * E_SD(air, uniform)
  g[v]   = (1 - lambda) g_mesh[v] + w_scaf / |F_air| * g_air[air id of v]
  w_scaf = 0.01 (1 - lambda); the air mesh's rest shape is its own layout
  (z = 0) with the degenerate clamp areaThres_AM = sqrt(3)/4 (avgEdgeLen/2)^2.
"""
import numpy as np
import pytest

import oracle as O
from conftest import SCAFFOLD_DUMPS, golden_scaffolds


def air_setup(g, k=0):
    airV, airF, bnd, fixed = golden_scaffolds(g)[k]
    avg = g["scalars"][1]
    thres = np.sqrt(3.0) / 4.0 * (0.5 * avg) ** 2
    V3 = np.concatenate([airV, np.zeros((len(airV), 1))], 1)
    rest, _ = O.rest_constants(V3, airF, thres)
    return airV, airF, bnd, fixed, rest


@pytest.mark.parametrize("case", SCAFFOLD_DUMPS)
def test_air_mesh_structure(golden, case):
    g = golden(case)
    nV = len(g["UV0"])
    for airV, airF, bnd, fixed in golden_scaffolds(g):
        assert len(bnd) > 0 and airF.min() >= 0 and airF.max() < len(airV)
        # boundary rows are the mesh's vertices; air fixed = fixed mesh vertices on the boundary
        assert bnd.min() >= 0 and bnd.max() < nV and len(np.unique(bnd)) == len(bnd)
        want = sorted(i for i, v in enumerate(bnd) if v in set(g["fixedVert"].tolist()))
        assert sorted(fixed.tolist()) == want


@pytest.mark.parametrize("case", SCAFFOLD_DUMPS)
def test_initial_energy_with_scaffold(golden, case):
    g = golden(case)
    par = 1.0 - g["scalars"][4]
    airV, airF, bnd, fixed, rest = air_setup(g)
    np.testing.assert_array_equal(airV[: len(bnd)], g["UV0"][bnd])
    e_mesh = par * O.energy(g["rest"], g["F"], g["UV0"])
    e_air = O.energy(rest, airF, airV, uniform=True) * (0.01 * par / len(airF))
    assert e_mesh + e_air == pytest.approx(g["trace_Etot"][0], rel=1e-14)
    assert g["trace_Etot"][0] - e_air == pytest.approx(g["trace_E"][0], rel=1e-14)


@pytest.mark.parametrize("case", SCAFFOLD_DUMPS)
def test_augmented_gradient_bit_exact(golden, case):
    g = golden(case)
    par = 1.0 - g["scalars"][4]
    nV = len(g["UV0"])
    airV, airF, bnd, fixed, rest = air_setup(g)
    gm = par * O.gradient(g["rest"], g["F"], g["UV0"], g["fixedVert"])
    ga = O.gradient(rest, airF, airV, fixed, uniform=True)
    w = 0.01 * par / len(airF)
    nb = len(bnd)
    whole = np.zeros(2 * (nV + len(airV) - nb))
    whole[: 2 * nV] = gm
    for i, v in enumerate(bnd):                       # Scaffold::augmentGradient
        whole[2 * v] += w * ga[2 * i]
        whole[2 * v + 1] += w * ga[2 * i + 1]
    whole[2 * nV:] = w * ga[2 * nb:]
    np.testing.assert_array_equal(whole, g["gradw0"])
    assert len(g["dir0"]) == len(whole)


@pytest.mark.parametrize("case", ["sheet_3k", "torus_768", "icosphere_320_scaf"])
def test_port_first_iteration_with_scaffold(golden, case):
    """The CPU restatement's scaffolding branches, one Newton iteration on the
    reference's own first air mesh."""
    g = golden(case)
    par = 1.0 - g["scalars"][4]
    airV, airF, bnd, _ = golden_scaffolds(g)[0]
    _, tr, _ = O.newton(g["V_rest"], g["F"], g["fixedVert"], g["UV0"], par, 1, scaffold=(airV, airF, bnd),
                        avg_edge_len=g["scalars"][1])
    assert tr["E"][0] == pytest.approx(g["trace_Etot"][0], rel=1e-14)
    assert tr["E"][1] == pytest.approx(g["trace_Etot"][1], rel=1e-3)
    assert tr["gsq"][0] == pytest.approx(float(g["gradw0"] @ g["gradw0"]), rel=1e-12)
    if g["trace_alpha"][0] > 0:
        assert tr["alpha"][0] == pytest.approx(g["trace_alpha"][0], rel=1e-3)


def test_port_scaffold_run_is_monotone(golden):
    g = golden("sheet_3k")
    par = 1.0 - g["scalars"][4]
    airV, airF, bnd, _ = golden_scaffolds(g)[0]
    _, tr, st = O.newton(g["V_rest"], g["F"], g["fixedVert"], g["UV0"], par, 40, scaffold=(airV, airF, bnd),
                         avg_edge_len=g["scalars"][1])
    assert st == 1 and np.all(np.diff(tr["E"]) <= 0.0)
