"""The allocation-free energy entry point, oc_sd_energy_trials_noalloc.

Some callers cannot allocate device memory themselves: a host framework that
owns every device allocation and hands out buffers, or work recorded into a
CUDA graph that someone else manages.  For them the line-search energy
evaluation is offered on caller-owned device buffers, with its block partial
sums in a static device array of the library instead of an allocation.

Checked here through the C ABI against the mesh-based entry point
(oc_sd_energy, which allocates its own scratch), on two calls in a row.  This
file is collected last so a failure here leaves every other test already run.
"""
import numpy as np
import pytest

import optcuts_gb300 as oc

pytestmark = pytest.mark.gpu

REL_TOL = 1e-14   # the same per-triangle arithmetic and reduction order: agreement to rounding


def test_noalloc_energy_matches_mesh_entry_point(golden):
    torch = pytest.importorskip("torch")
    g = golden("icosphere_5k")
    mesh = oc.TriMesh(g["V_rest"], g["UV0"], g["F"], g["fixedVert"])
    rest, sc = mesh.rest_constants()
    sd = oc.SymDirichletEnergy()
    dev = torch.device("cuda", 0)
    F = torch.tensor(g["F"], dtype=torch.int32, device=dev)
    uv = torch.tensor(g["UV0"], dtype=torch.float64, device=dev)
    d = torch.tensor(g["dir0"].reshape(-1, 2), dtype=torch.float64, device=dev)
    R = torch.tensor(rest, dtype=torch.float64, device=dev)
    out = torch.full((8,), float("nan"), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    alphas = np.array([0.5, 0.25, 0.125, 1e-2, 1e-3], np.float64)
    nF = len(g["F"])
    L = oc.lib()
    for _call in range(2):
        # energy at UV (dir = NULL)
        rc = L.oc_sd_energy_trials_noalloc(F.data_ptr(), uv.data_ptr(), None, R.data_ptr(), float(sc[0]), nF, None,
                                           1, 0, out.data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc == 0
        mesh.V = g["UV0"]
        ref = sd.computeEnergyVal(mesh)
        assert abs(out[0].item() - ref) <= REL_TOL * abs(ref)
        # the line-search trials E(UV + alpha_k * dir)
        a = np.ascontiguousarray(alphas)
        rc = L.oc_sd_energy_trials_noalloc(F.data_ptr(), uv.data_ptr(), d.data_ptr(), R.data_ptr(), float(sc[0]), nF,
                                           a.ctypes.data_as(oc._d), len(a), 0, out.data_ptr(), stream)
        torch.cuda.synchronize()
        assert rc == 0
        got = out[: len(a)].cpu().numpy()
        for k, alpha in enumerate(alphas):
            mesh.V = g["UV0"] + alpha * g["dir0"].reshape(-1, 2)
            ref_k = sd.computeEnergyVal(mesh)
            assert abs(got[k] - ref_k) <= REL_TOL * abs(ref_k), (k, got[k], ref_k)
        mesh.V = g["UV0"]


def test_noalloc_rejects_sizes_beyond_its_scratch(golden):
    torch = pytest.importorskip("torch")
    g = golden("cube")
    mesh = oc.TriMesh(g["V_rest"], g["UV0"], g["F"], g["fixedVert"])
    rest, sc = mesh.rest_constants()
    dev = torch.device("cuda", 0)
    F = torch.tensor(g["F"], dtype=torch.int32, device=dev)
    uv = torch.tensor(g["UV0"], dtype=torch.float64, device=dev)
    R = torch.tensor(rest, dtype=torch.float64, device=dev)
    out = torch.zeros(16, dtype=torch.float64, device=dev)
    a = np.full(9, 0.5)
    L = oc.lib()
    # more than 8 trial step sizes do not fit the static partials array
    rc = L.oc_sd_energy_trials_noalloc(F.data_ptr(), uv.data_ptr(), uv.data_ptr(), R.data_ptr(), float(sc[0]),
                                       len(g["F"]), a.ctypes.data_as(oc._d), 9, 0, out.data_ptr(), None)
    assert rc == 1
    rc = L.oc_sd_energy_trials_noalloc(F.data_ptr(), uv.data_ptr(), None, R.data_ptr(), float(sc[0]), 0, None, 1, 0,
                                       out.data_ptr(), None)
    assert rc == 1
