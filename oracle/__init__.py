"""Oracle for the OptCuts geometry step -- TEST INFRASTRUCTURE ONLY.

Two layers:

* ``oracle/ref``  -- a recipe (Makefile + headless driver) that compiles the
  reference's own sources into ``oracle/_ref/ref_driver``.  It exists only
  where the reference source tree is present and is used to generate the
  golden vectors under ``tests/golden/``.
* ``oracle/port`` -- a CPU restatement of the same path in plain C++
  (``liboc_oracle.so``), pinned against those golden vectors.  It is the
  checker for the CUDA path and the timed CPU baseline.

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may import this package.  The product never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_BUILD = os.path.join(_HERE, "_build")
_SO = os.path.join(_BUILD, "liboc_oracle.so")
_lib = None


def build(force=False):
    srcs = [os.path.join(_HERE, "port", f) for f in ("oc_oracle.cpp", "oc_topo_oracle.cpp")]
    inputs = srcs + [os.path.join(_HERE, "port", "oc_oracle.h"), os.path.abspath(__file__)]
    if not force and os.path.exists(_SO) and all(os.path.getmtime(_SO) >= os.path.getmtime(p) for p in inputs):
        return _SO
    os.makedirs(_BUILD, exist_ok=True)
    tmp = _SO + ".tmp%d" % os.getpid()
    # -ffp-contract=off: aarch64 GCC would fuse multiply-adds and change rounding
    subprocess.check_call(["g++", "-O3", "-std=c++17", "-ffp-contract=off", "-fPIC", "-shared", "-pthread", *srcs,
                           "-o", tmp])
    os.replace(tmp, _SO)
    return _SO


_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)


class ScaffoldArgs(ctypes.Structure):
    _fields_ = [("airV", ctypes.POINTER(ctypes.c_double)), ("nAirV", ctypes.c_int),
                ("airF", ctypes.POINTER(ctypes.c_int)), ("nAirF", ctypes.c_int),
                ("bnd", ctypes.POINTER(ctypes.c_int)), ("nBnd", ctypes.c_int), ("areaThres", ctypes.c_double)]


class NewtonOpts(ctypes.Structure):
    _fields_ = [("energyParam", ctypes.c_double), ("relGL2Tol", ctypes.c_double),
                ("maxIter", ctypes.c_int), ("nThreads", ctypes.c_int)]


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(build())
        L.ocr_rest_constants.argtypes = [_d, ctypes.c_int, _i, ctypes.c_int, ctypes.c_double, _d, _d]
        L.ocr_energy_elem.argtypes = [_d, _i, ctypes.c_int, _d, ctypes.c_int, _d]
        L.ocr_energy.argtypes = [_d, _i, ctypes.c_int, _d, ctypes.c_int]
        L.ocr_energy.restype = ctypes.c_double
        L.ocr_gradient.argtypes = [_d, _i, ctypes.c_int, _d, ctypes.c_int, _i, ctypes.c_int, ctypes.c_int, _d]
        L.ocr_hessian_blocks.argtypes = [_d, _i, ctypes.c_int, _d, ctypes.c_int, _d]
        L.ocr_init_step_size.argtypes = [_i, ctypes.c_int, _d, _d, _d]
        L.ocr_solver_create.argtypes = [ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int, _d]
        L.ocr_solver_create.restype = ctypes.c_void_p
        L.ocr_solver_destroy.argtypes = [ctypes.c_void_p]
        L.ocr_solver_factorize.argtypes = [ctypes.c_void_p, _d, ctypes.c_double]
        L.ocr_solver_solve.argtypes = [ctypes.c_void_p, _d, _d]
        L.ocr_solver_nnz_L.argtypes = [ctypes.c_void_p]
        L.ocr_solver_nnz_L.restype = ctypes.c_longlong
        L.ocr_newton.argtypes = [_d, ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int, _d,
                                 ctypes.POINTER(NewtonOpts), _d, _d, _d, _d, _i]
        L.ocr_newton_scaffold.argtypes = [_d, ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int, _d,
                                          ctypes.POINTER(NewtonOpts), ctypes.POINTER(ScaffoldArgs), _d, _d, _d, _d, _i]
        L.ocr_topology_query.argtypes = [ctypes.c_int, _i, ctypes.c_int, _d, _d, _i, ctypes.c_int, ctypes.c_int,
                                         ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int, _d, _d, _i, _d,
                                         _i, _i, _d]
        _lib = L
    return _lib


def _pd(a):
    return a.ctypes.data_as(_d)


def _pi(a):
    return a.ctypes.data_as(_i)


def _f8(a):
    return np.ascontiguousarray(a, np.float64)


def _i4(a):
    return np.ascontiguousarray(a, np.int32)


def rest_constants(V_rest, F, area_thres=0.0):
    V_rest, F = _f8(V_rest), _i4(F)
    rest = np.empty((len(F), 8))
    sc = np.empty(3)
    rc = lib().ocr_rest_constants(_pd(V_rest), len(V_rest), _pi(F), len(F), area_thres, _pd(rest), _pd(sc))
    if rc != 0:
        raise ValueError("zero-area rest triangle")
    return rest, sc


def energy_elem(rest, F, UV, uniform=False):
    rest, F, UV = _f8(rest), _i4(F), _f8(UV)
    out = np.empty(len(F))
    lib().ocr_energy_elem(_pd(rest), _pi(F), len(F), _pd(UV), int(uniform), _pd(out))
    return out


def energy(rest, F, UV, uniform=False):
    rest, F, UV = _f8(rest), _i4(F), _f8(UV)
    return lib().ocr_energy(_pd(rest), _pi(F), len(F), _pd(UV), int(uniform))


def gradient(rest, F, UV, fixed, uniform=False):
    rest, F, UV, fixed = _f8(rest), _i4(F), _f8(UV), _i4(fixed)
    g = np.empty(2 * len(UV))
    lib().ocr_gradient(_pd(rest), _pi(F), len(F), _pd(UV), len(UV), _pi(fixed), len(fixed), int(uniform), _pd(g))
    return g


def hessian_blocks(rest, F, UV, uniform=False):
    rest, F, UV = _f8(rest), _i4(F), _f8(UV)
    out = np.empty((len(F), 6, 6))
    lib().ocr_hessian_blocks(_pd(rest), _pi(F), len(F), _pd(UV), int(uniform), _pd(out))
    return out


def init_step_size(F, UV, d, step=1.0):
    F, UV, d = _i4(F), _f8(UV), _f8(d)
    s = np.array([step], np.float64)
    lib().ocr_init_step_size(_pi(F), len(F), _pd(UV), _pd(d), _pd(s))
    return float(s[0])


class Solver:
    """Sparse LDL^T of the assembled Newton matrix (EigenLibSolver stand-in)."""

    def __init__(self, nV, F, fixed, V_rest):
        self._F, self._fixed, self._Vr = _i4(F), _i4(fixed), _f8(V_rest)
        self.n = 2 * nV
        self._h = lib().ocr_solver_create(nV, _pi(self._F), len(self._F), _pi(self._fixed), len(self._fixed),
                                          _pd(self._Vr))

    def factorize(self, blocks, param):
        b = _f8(blocks)
        if lib().ocr_solver_factorize(self._h, _pd(b), param) != 0:
            raise ArithmeticError("LDL^T: zero or non-finite pivot")

    def solve(self, rhs):
        rhs = _f8(rhs)
        x = np.empty(self.n)
        lib().ocr_solver_solve(self._h, _pd(rhs), _pd(x))
        return x

    def nnz_L(self):
        return lib().ocr_solver_nnz_L(self._h)

    def __del__(self):
        if getattr(self, "_h", None):
            lib().ocr_solver_destroy(self._h)
            self._h = None


def newton(V_rest, F, fixed, UV, energy_param, iters, rel_gl2_tol=1e-12, threads=1, scaffold=None,
           area_thres=None, avg_edge_len=None):
    """Projected-Newton loop; returns (UV, traces dict, status).  scaffold =
    (airV, airF, bnd) runs the scaffolding branches with that air mesh moved
    along each step (areaThres_AM from avg_edge_len unless area_thres)."""
    V_rest, F, fixed = _f8(V_rest), _i4(F), _i4(fixed)
    UV = np.array(UV, np.float64, copy=True, order="C")
    o = NewtonOpts(energy_param, rel_gl2_tol, iters, threads)
    tE = np.zeros(iters + 1)
    tG = np.zeros(iters)
    tA = np.zeros(iters)
    tS = np.zeros(iters)
    st = np.zeros(1, np.int32)
    if scaffold is not None:
        aV, aF, bnd = _f8(scaffold[0]), _i4(scaffold[1]), _i4(scaffold[2])
        if area_thres is None:
            area_thres = np.sqrt(3.0) / 4.0 * (0.5 * avg_edge_len) ** 2
        sa = ScaffoldArgs(_pd(aV), len(aV), _pi(aF), len(aF), _pi(bnd), len(bnd), float(area_thres))
        n = lib().ocr_newton_scaffold(_pd(V_rest), len(V_rest), _pi(F), len(F), _pi(fixed), len(fixed), _pd(UV),
                                      ctypes.byref(o), ctypes.byref(sa), _pd(tE), _pd(tG), _pd(tA), _pd(tS), _pi(st))
    else:
        n = lib().ocr_newton(_pd(V_rest), len(V_rest), _pi(F), len(F), _pi(fixed), len(fixed), _pd(UV),
                             ctypes.byref(o), _pd(tE), _pd(tG), _pd(tA), _pd(tS), _pi(st))
    if n < 0:
        raise ArithmeticError("factorization failed")
    return UV, {"E": tE[:n + 1], "gsq": tG[:n], "alpha": tA[:n], "seconds": tS[:n]}, int(st[0])


def topology_query(V_rest, UV, F, cohE, op, lambda_t, filter_exp=0.6, threads=1, max_cand=100000):
    """CPU restatement of querySplit (op 0 boundary, 1 interior) / queryMerge
    (op 2), bijectivity off: list of candidate dicts and the seconds taken."""
    V_rest, UV, F = _f8(V_rest), _f8(UV), _i4(F)
    c = _i4(np.asarray(cohE).reshape(-1, 4))
    ew = np.zeros(max_cand)
    ec = np.zeros(2 * max_cand)
    path = np.zeros(3 * max_cand, np.int32)
    pos = np.zeros(8 * max_cand)
    rows = np.zeros(max_cand, np.int32)
    n = np.zeros(1, np.int32)
    sec = np.zeros(1)
    lib().ocr_topology_query(len(V_rest), _pi(F), len(F), _pd(V_rest), _pd(UV), _pi(c), len(c), op, lambda_t,
                             filter_exp, threads, max_cand, _pd(ew), _pd(ec), _pi(path), _pd(pos), _pi(rows), _pi(n),
                             _pd(sec))
    out = []
    for k in range(min(int(n[0]), max_cand)):
        p = [int(x) for x in path[3 * k:3 * k + 3] if x >= 0]
        out.append({"EwDec": ew[k], "energyChanges": (ec[2 * k], ec[2 * k + 1]), "path": p,
                    "newVertPos": pos[8 * k:8 * k + 2 * rows[k]].reshape(-1, 2)})
    return out, float(sec[0])
