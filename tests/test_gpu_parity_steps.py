"""Per-iteration parity of one Newton step, without accumulation.

Every iteration k < 20 of the reference's own run is restarted on the GPU
from the reference's iterate (UV after its iteration k-1, and for scaffold
cases the air mesh its iteration k used), one Optimizer::solve(1) is taken,
and the energy after the step is compared with the reference's energy after
its iteration k (Optimizer.cpp:505-652, the trace written by
writeEnergyValToFile, Optimizer.cpp:706-728).  The trajectory itself is not
compared here: it accumulates the rounding of ill-conditioned solves
(tests/test_gpu_optimizer.py pins its converged end).

Tolerance: 1e-6 relative on E_SD and E_w.  The exception is the first three
iterations of the 5,120-triangle icosphere from its Tutte start, where the
Newton matrix spans ~1e14 in scale: any two exact FP64 factorizations of it
(Eigen's AMD-ordered SimplicialLDLT, the CPU oracle's nested dissection, the
GPU's multifrontal LDL^T) give directions that differ at cond x eps, and the
energy after the step by up to ~3e-5 (measured for the CPU oracle against the
reference as well); those three steps are held to 2e-4.  The CPU oracle's
column of the same table is asserted in tests/test_oracle_golden.py."""
import numpy as np
import pytest

import optcuts_gb300 as oc
from conftest import golden_scaffolds

pytestmark = pytest.mark.gpu

STEPS = 20
ILL_CONDITIONED = {"icosphere_5k": 3}   # leading iterations held to 2e-4


def tolerance(case, k):
    return 2e-4 if k < ILL_CONDITIONED.get(case, 0) else 1e-6


def start_uv(g, k):
    return g["UV0"] if k == 0 else g["UV_iters"][k - 1]


def gpu_step(g, k, scaf=None):
    m = oc.TriMesh(g["V_rest"], start_uv(g, k), g["F"], g["fixedVert"])
    opt = oc.Optimizer(m, [1.0 - g["scalars"][4]])
    if scaf is not None:
        opt.setScaffold(oc.Scaffold(*scaf[:3]))
    opt.precompute()
    opt.solve(1)
    return opt.getLastEnergyVal(), opt.getLastEnergyVal(excludeScaffold=True)


def steps(g):
    return min(STEPS, len(g["UV_iters"]), len(g["trace_E"]) - 1)


def energy_w(g, e_sd_param):
    """E_w from the weighted SD energy (energyParams[0] * E_SD) and the seam
    term, constant during the Newton step (Optimizer.cpp:706-716)."""
    lam = g["scalars"][4]
    return e_sd_param + lam * g["scalars"][3] / g["scalars"][2]


@pytest.mark.parametrize("case", ["cube", "icosphere_320", "icosphere_5k"])
def test_one_step_from_reference_iterate(golden, case):
    g = golden(case)
    errs = []
    for k in range(steps(g)):
        e, _ = gpu_step(g, k)
        ref = g["trace_E"][k + 1]
        rel_sd = abs(e - ref) / ref
        rel_w = abs(energy_w(g, e) - energy_w(g, ref)) / energy_w(g, ref)
        errs.append(rel_sd)
        assert rel_sd <= tolerance(case, k), (k, rel_sd)
        assert rel_w <= tolerance(case, k), (k, rel_w)
    assert len(errs) == steps(g)


@pytest.mark.parametrize("case", ["sheet_3k", "icosphere_320_scaf"])
def test_one_step_from_reference_iterate_scaffold(golden, case):
    g = golden(case)
    scafs = golden_scaffolds(g)
    for k in range(min(steps(g), len(scafs))):
        etot, e = gpu_step(g, k, scafs[k])
        rel_tot = abs(etot - g["trace_Etot"][k + 1]) / g["trace_Etot"][k + 1]
        rel_sd = abs(e - g["trace_E"][k + 1]) / g["trace_E"][k + 1]
        assert rel_tot <= tolerance(case, k), (k, rel_tot)
        assert rel_sd <= tolerance(case, k), (k, rel_sd)
