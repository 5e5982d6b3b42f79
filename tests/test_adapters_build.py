"""The reference-side adapters compile and link against the reference.

optcuts_gb300/adapters/ holds the C++ drop-ins a maintainer adds to the
reference (GpuSymDirichletEnergy, GpuLinSysSolver, and GpuOptimizer.cpp,
which defines OptCuts::Optimizer's methods on the GPU in place of
src/Optimizer.cpp).  Where the reference's source tree is present, the
recipe oracle/ref/Makefile (target gpu-dropin) builds the reference's own
headless driver with every reference object except Optimizer.o, the
adapters and liboc_gpu.so.  This test runs that build and checks the link:
the Optimizer symbols come from the drop-in and the binary loads the
library.  (Running it needs a GPU and the reference tree on the same host.)"""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
RECIPE = os.path.join(ROOT, "oracle", "ref")
BIN = os.path.join(ROOT, "oracle", "_ref", "ref_driver_gpu")


def have_reference():
    return subprocess.run(["make", "-s", "-C", RECIPE, "have-ref"], stdout=subprocess.DEVNULL,
                          stderr=subprocess.DEVNULL).returncode == 0


@pytest.mark.skipif(not have_reference(), reason="the reference's source tree is not on this host")
def test_gpu_dropin_builds_against_reference():
    from optcuts_gb300 import build as b
    b.build()
    r = subprocess.run(["make", "-s", "-j8", "-C", RECIPE, "gpu-dropin"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert os.path.exists(BIN)
    needed = subprocess.run(["readelf", "-d", BIN], capture_output=True, text=True).stdout
    assert "liboc_gpu.so" in needed
    syms = subprocess.run(["nm", "-C", "--defined-only", BIN], capture_output=True, text=True).stdout
    for m in ("OptCuts::Optimizer::solve(int)", "OptCuts::Optimizer::precompute()",
              "OptCuts::Optimizer::createFracture(double, int, bool, bool)", "oc_adapters_instantiate"):
        assert m in syms, m
    # the reference's own Optimizer.o is not linked: its line search's
    # logging string is absent, the drop-in's diagnostics are present
    strings = open(BIN, "rb").read()
    assert b"GPU optimizer: " in strings
    assert b"(armijo)" not in strings
