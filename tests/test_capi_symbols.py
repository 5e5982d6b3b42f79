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


def test_ordering_with_coordinates_handles_an_air_ring():
    """Host-only symbolic analysis of a torus knot's cut mesh with its air
    mesh: BFS level sets wrap around the air ring into separators as long as
    the boundary; with the UV coordinates each dissection node keeps the
    smaller balanced separator of the two, so the tree stays shallow and the
    factorisation several times cheaper.  Without air (and on the one-point
    cut ellipsoid) the choice costs no more than BFS."""
    import optcuts_gb300 as oc
    from optcuts_gb300 import init as I
    from optcuts_gb300 import meshes as M
    V, F = M.torus_knot_tube(200, 64, 2, 3, 0.15, 0.002, 4)
    st = I.init_uv(V, F)
    e = np.concatenate([st.F[:, [0, 1]], st.F[:, [1, 2]], st.F[:, [2, 0]]])
    avg = float(np.linalg.norm(st.V_rest[e[:, 0]] - st.V_rest[e[:, 1]], axis=1).mean())
    am = oc.Scaffold.build(st.UV, st.F, avg)
    nV = len(st.UV)
    Fa = am.localVI2Global(nV)[am.airF]
    Fall = np.vstack([st.F, Fa])
    xy = np.vstack([st.UV, am.airV[len(am.bnd):]])
    n = len(xy)
    bfs = oc.chol_analyze_stats(n, Fall, st.fixedVert)
    geo = oc.chol_analyze_stats(n, Fall, st.fixedVert, xy=xy)
    assert geo["dof"] == bfs["dof"] == 2 * n
    assert geo["flops"] < 0.5 * bfs["flops"] and geo["levels"] < bfs["levels"]
    for V2, F2 in (M.torus_knot_tube(200, 64, 2, 3, 0.15, 0.002, 4), M.ellipsoid(60, 60)):
        s2 = I.init_uv(V2, F2)
        b = oc.chol_analyze_stats(len(s2.UV), s2.F, s2.fixedVert)
        g = oc.chol_analyze_stats(len(s2.UV), s2.F, s2.fixedVert, xy=s2.UV)
        assert g["flops"] <= 1.05 * b["flops"]
    # a non-finite coordinate: BFS alone
    bad = s2.UV.copy()
    bad[3, 1] = np.nan
    assert oc.chol_analyze_stats(len(s2.UV), s2.F, s2.fixedVert, xy=bad) == b
