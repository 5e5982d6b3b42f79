"""The C-ABI library loads and exports every entry point include/*.h declares
(no compute calls: this runs without a GPU)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

import optcuts_gb300 as oc

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_\s\*]*?\b(oc_[a-z0-9_]+)\s*\(", src, flags=re.M)
    return sorted(set(names))


def test_header_declares_entry_points():
    names = declared_functions()
    assert "oc_optimizer_solve" in names and "oc_sd_gradient" in names and len(names) >= 30


def test_library_exports_every_declared_symbol():
    if not os.path.exists(oc.LIB_PATH):
        from optcuts_gb300 import build
        build.build()
    lib = ctypes.CDLL(oc.LIB_PATH)
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings():
    L = oc.lib()
    assert L.oc_status_string(0) == b"ok"
    assert L.oc_status_string(3) == b"PCG did not converge"


def test_loud_failure_without_library(monkeypatch, tmp_path):
    monkeypatch.setattr(oc, "LIB_PATH", str(tmp_path / "missing.so"))
    monkeypatch.setattr(oc, "_lib", None)
    with pytest.raises(ImportError):
        oc.lib()


def test_symbolic_analysis_host_only():
    """Nested-dissection front structure of the direct solver (no GPU)."""
    from optcuts_gb300 import init as I
    from optcuts_gb300 import meshes as M
    V, F = M.CONFIGS["icosphere_1k"]()
    st = I.init_uv(V, F)
    s = oc.chol_analyze_stats(len(st.UV), st.F, st.fixedVert)
    n = 2 * len(st.UV)
    assert s["dof"] == n
    assert s["fronts"] > 10 and s["levels"] >= 4
    # the factor is sparse: far fewer entries than the dense lower triangle
    assert n < s["factor_entries"] < n * n / 8
    assert s["flops"] > 0 and s["max_front_rows"] <= n


def test_symbolic_analysis_rejects_bad_input():
    F = np.array([[0, 1, 5]], np.int32)
    with pytest.raises(oc.OCError):
        oc.chol_analyze_stats(3, F)
