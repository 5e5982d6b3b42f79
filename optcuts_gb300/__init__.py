"""optcuts_gb300 -- the OptCuts geometry step on one GB300 (sm_103a).

Python mirror of the reference's interfaces for the path, over the C ABI in
include/optcuts_gpu.h (library: optcuts_gb300/_lib/liboc_gpu.so):

    TriMesh             -- device-resident mesh state (src/TriMesh.hpp:28-63)
    SymDirichletEnergy  -- computeEnergyVal / getEnergyValPerElem /
                           computeGradient / computeHessian / initStepSize
                           (src/Energy/Energy.hpp:27-44)
    LinSysSolver        -- set_pattern / update_a / factorize / solve /
                           multiply (src/LinSysSolver/LinSysSolver.hpp:22-187)
    Optimizer           -- precompute / solve / getLastEnergyVal / ...
                           (src/Optimizer.hpp:74-142)

There is no CPU fallback: if the CUDA library is missing or no GPU is
visible, construction raises.
"""
from __future__ import annotations

import ctypes
import time
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_lib", "liboc_gpu.so")

_lib = None

OC_OK = 0
OC_ERR_INVALID = 1
OC_ERR_INVERTED = 2
OC_ERR_NOT_CONVERGED = 3
OC_ERR_TIMEOUT = 4
OC_ERR_NOT_SPD = 8


class OCError(RuntimeError):
    def __init__(self, status, msg):
        super().__init__("%s (status %d)" % (msg, status))
        self.status = status


_d = ctypes.POINTER(ctypes.c_double)
_i = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p


class OptimizerConfig(ctypes.Structure):
    _fields_ = [("pcgTol", ctypes.c_double), ("pcgMaxIter", ctypes.c_int), ("relGL2Tol", ctypes.c_double),
                ("lineSearchBatch", ctypes.c_int), ("timing", ctypes.c_int), ("linearSolver", ctypes.c_int),
                ("scaffoldPattern", ctypes.c_int), ("hessianProjection", ctypes.c_int), ("ordering", ctypes.c_int),
                ("carryAnalysis", ctypes.c_int)]


class OptCutsConfig(ctypes.Structure):
    _fields_ = [("upperBound", ctypes.c_double), ("bijective", ctypes.c_int), ("topoLineSearch", ctypes.c_int),
                ("filterExp", ctypes.c_double), ("topoOptions", ctypes.c_int), ("mlp", _vp),
                ("topFrac", ctypes.c_double), ("maxNewtonIters", ctypes.c_int), ("recordFeatures", ctypes.c_int)]


SOLVER_DIRECT = 0
SOLVER_PCG = 1
HESSIAN_REDUCED, HESSIAN_JACOBI6, HESSIAN_HYBRID = 0, 1, 2
ORDER_AUTO, ORDER_BFS = 0, 1
OP_BOUNDARY_SPLIT, OP_INTERIOR_SPLIT, OP_MERGE = 0, 1, 2


_SIGS = {
    "oc_ctx_create": [ctypes.c_int, _vp, ctypes.POINTER(_vp)],
    "oc_ctx_destroy": [_vp],
    "oc_ctx_synchronize": [_vp],
    "oc_mesh_create": [_vp, _d, _d, ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int, ctypes.c_double,
                       ctypes.POINTER(_vp)],
    "oc_mesh_destroy": [_vp],
    "oc_mesh_set_uv": [_vp, _d],
    "oc_mesh_get_uv": [_vp, _d],
    "oc_mesh_rest_constants": [_vp, _d, _d],
    "oc_mesh_check_inversion": [_vp, _i],
    "oc_sd_energy": [_vp, ctypes.c_int, _d],
    "oc_sd_energy_per_elem": [_vp, ctypes.c_int, _d],
    "oc_sd_gradient": [_vp, ctypes.c_int, _d],
    "oc_sd_hessian_blocks": [_vp, ctypes.c_int, _d],
    "oc_sd_hessian_blocks_projected": [_vp, ctypes.c_int, ctypes.c_int, _d],
    "oc_sd_init_step_size": [_vp, _d, _d],
    "oc_linsys_create": [_vp, ctypes.POINTER(_vp)],
    "oc_linsys_destroy": [_vp],
    "oc_linsys_set_type": [_vp, ctypes.c_int],
    "oc_linsys_analyze_pattern": [_vp],
    "oc_linsys_stats": [_vp, _d],
    "oc_chol_analyze_stats": [ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int, ctypes.c_int, _d],
    "oc_chol_analyze_stats_xy": [ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int, ctypes.c_int, _d, _d],
    "oc_chol_analyze_groups": [ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i],
    "oc_linsys_set_pattern": [_vp, ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int],
    "oc_linsys_update_a": [_vp, _i, _i, _d, ctypes.c_int],
    "oc_linsys_factorize": [_vp],
    "oc_linsys_solve": [_vp, _d, _d, ctypes.c_double, ctypes.c_int, _i, _d],
    "oc_linsys_multiply": [_vp, _d, _d],
    "oc_optimizer_default_config": [ctypes.POINTER(OptimizerConfig)],
    "oc_optimizer_create": [_vp, ctypes.c_double, ctypes.POINTER(OptimizerConfig), ctypes.POINTER(_vp)],
    "oc_optimizer_destroy": [_vp],
    "oc_optimizer_precompute": [_vp],
    "oc_optimizer_solve": [_vp, ctypes.c_int, _i],
    "oc_optimizer_get_last_energy": [_vp, _d],
    "oc_optimizer_get_iter_num": [_vp, _i],
    "oc_optimizer_set_rel_gl2_tol": [_vp, ctypes.c_double],
    "oc_optimizer_set_energy_param": [_vp, ctypes.c_double],
    "oc_optimizer_last_step": [_vp, _d, _i, _d, _i, _d],
    "oc_optimizer_phase_ms": [_vp, _d],
    "oc_optimizer_launch_count": [_vp, ctypes.POINTER(ctypes.c_longlong)],
    "oc_optimizer_solver_stats": [_vp, _d],
    "oc_optimizer_set_solve_cluster": [_vp, ctypes.c_int],
    "oc_linsys_set_solve_cluster": [_vp, ctypes.c_int],
    "oc_linsys_set_factor_streams": [_vp, ctypes.c_int],
    "oc_linsys_factor_streams": [_vp, _i, _i],
    "oc_topo_result_host_phases": [_vp, _d],
    "oc_tc_set_wait_polls": [ctypes.c_int],
    "oc_linsys_solve_clusters": [_vp, _i, _i],
    "oc_optimizer_solve_clusters": [_vp, _i, _i],
    "oc_optimizer_set_factor_streams": [_vp, ctypes.c_int],
    "oc_optimizer_factor_streams": [_vp, _i, _i],
    "oc_optimizer_set_scaffold": [_vp, _d, ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int, ctypes.c_double],
    "oc_optimizer_clear_scaffold": [_vp],
    "oc_optimizer_rebuild_scaffold": [_vp],
    "oc_air_mesh_build": [_d, ctypes.c_int, _i, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.POINTER(_vp)],
    "oc_air_mesh_sizes": [_vp, _i, _i, _i],
    "oc_air_mesh_get": [_vp, _d, _i, _i],
    "oc_air_mesh_destroy": [_vp],
    "oc_mesh_set_cohesive_edges": [_vp, _i, ctypes.c_int],
    "oc_mesh_drop_adjacency": [_vp],
    "oc_mesh_split_filter": [_vp, _d],
    "oc_topology_query": [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.POINTER(_vp)],
    "oc_topo_result_info": [_vp, _i, _i, _i, _i, _i, _d, _d],
    "oc_topo_result_candidate": [_vp, ctypes.c_int, _d, _d, _i, _i, _d, _i],
    "oc_topo_result_destroy": [_vp],
    "oc_topo_result_air": [_vp, _i, _i, _i, _i],
    "oc_optimizer_analysis_info": [_vp, _i, _d, _d, _d, _d],
    "oc_air_loop_mesh": [_vp, ctypes.c_int, ctypes.c_int, _i, _vp, _i, _vp, _i],
    "oc_topo_result_iterations": [_vp, _i, _i, ctypes.POINTER(ctypes.c_longlong)],
    "oc_optimizer_create_fracture": [_vp, ctypes.c_int, _i, ctypes.c_int, _d, ctypes.c_int],
    "oc_optimizer_apply_timing": [_vp, _d],
    "oc_optimizer_split_or_merge": [_vp, ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int, _vp,
                                    ctypes.c_double, _i, _i, _d],
    "oc_mesh_apply_topology": [_vp, ctypes.c_int, _i, ctypes.c_int, _d, ctypes.c_int],
    "oc_mesh_get_topology": [_vp, _i, _i, _i, _i, _d, _i],
    "oc_topology_apply": [ctypes.c_int, _i, ctypes.c_int, _d, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i, _d, _d,
                          ctypes.c_int, _i, _i, _d, _d, _i, _i, _i],
    "oc_cut_to_disk": [_i, ctypes.c_int, _i, ctypes.c_int, _i, ctypes.c_int, _i, _i],
    "oc_topology_cut_path": [_i, ctypes.c_int, ctypes.c_int, ctypes.c_int, _i, _d, _d, ctypes.c_int, _i, _i, _d, _d,
                             _i, _i, _i, _i],
    "oc_topology_query_learned": [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _vp,
                                  ctypes.c_double, ctypes.POINTER(_vp)],
    "oc_topo_result_features": [_vp, _i, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float),
                                ctypes.POINTER(ctypes.c_float)],
    "oc_topo_result_timing": [_vp, _i, _d, _d],
    "oc_topo_result_problems": [_vp, _i, _vp, _vp, _vp],
    "oc_topo_result_candidates": [_vp, _vp, _vp, _vp, _vp, _vp],
    "oc_topology_step": [_vp, ctypes.c_double, ctypes.c_double, ctypes.c_int, _vp, ctypes.c_double,
                         ctypes.POINTER(_vp), ctypes.POINTER(_vp), ctypes.POINTER(_vp)],
    "oc_topo_result_problem_stats": [_vp, _i, _vp, _vp, _vp, _vp, _vp],
    "oc_mlp_create": [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_uint, ctypes.POINTER(_vp)],
    "oc_mlp_destroy": [_vp],
    "oc_mlp_num_params": [_vp, _i],
    "oc_mlp_get_params": [_vp, ctypes.POINTER(ctypes.c_float)],
    "oc_mlp_set_params": [_vp, ctypes.POINTER(ctypes.c_float)],
    "oc_mlp_predict": [_vp, ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.POINTER(ctypes.c_float)],
    "oc_mlp_gradient": [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ctypes.c_int,
                        ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float)],
    "oc_mlp_set_tensor_cores": [_vp, ctypes.c_int],
    "oc_bf16_gemm": [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_float), ctypes.c_longlong,
                     ctypes.c_longlong, ctypes.POINTER(ctypes.c_float), ctypes.c_longlong, ctypes.c_longlong,
                     ctypes.POINTER(ctypes.c_float), ctypes.c_int],
    "oc_mlp_train": [_vp, ctypes.POINTER(ctypes.c_float), ctypes.POINTER(ctypes.c_float), ctypes.c_int, ctypes.c_int,
                     ctypes.c_int, ctypes.c_float, ctypes.c_uint, ctypes.POINTER(ctypes.c_float)],
    "oc_topology_split_candidates": [ctypes.c_int, _i, ctypes.c_int, _d, ctypes.c_int, ctypes.c_double, _i, _i, _i],
    "oc_optimizer_get_scaffold": [_vp, _i, _i, _i, _d, _i, _i],
    "oc_optimizer_get_last_energy_scaffold": [_vp, _d],
    "oc_optimizer_system_size": [_vp, _i],
    "oc_optimizer_last_vectors": [_vp, _d, _d],
    "oc_optimizer_bad_pivots": [_vp, _i],
    "oc_linsys_set_pattern_neighbors": [_vp, ctypes.c_int, _i, _i, _i, ctypes.c_int],
    "oc_topology_schedules": [_i, _i, _vp],
    "oc_topology_queries": [_vp, _i, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _vp,
                            ctypes.c_double, ctypes.POINTER(_vp)],
    "oc_topology_query_tail": [_vp, ctypes.c_int, ctypes.c_double, ctypes.c_int, ctypes.POINTER(_vp)],
    "oc_topology_queries_sharded": [_vp, _i, ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_int, _vp,
                                    ctypes.c_double, ctypes.c_int, ctypes.c_int, ctypes.POINTER(_vp)],
    "oc_mesh_fracture_tails": [_vp, _i],
    "oc_mesh_set_fracture_tails": [_vp, _i],
    "oc_mesh_seam_length": [_vp, _d],
    "oc_optimizer_last_edec": [_vp, _d],
    "oc_optimizer_set_allow_edec_rel_tol": [_vp, ctypes.c_int],
    "oc_optimizer_get_energy_param": [_vp, _d],
    "oc_optimizer_set_state": [_vp, ctypes.c_int, _d, _d, ctypes.c_int, _i, ctypes.c_int, _i, _i, ctypes.c_int],
    "oc_optcuts_default_config": [_vp],
    "oc_optcuts_create": [_vp, _vp, _vp, ctypes.POINTER(_vp)],
    "oc_optcuts_destroy": [_vp],
    "oc_optcuts_run": [_vp, ctypes.c_int, _i],
    "oc_optcuts_state": [_vp, _d],
    "oc_optcuts_events": [_vp, _i, _d],
    "oc_optcuts_trace": [_vp, _i, _d],
    "oc_optcuts_write": [_vp, ctypes.c_char_p, _i, ctypes.c_int, ctypes.c_double],
    "oc_optcuts_mesh": [_vp, ctypes.POINTER(_vp)],
    "oc_optcuts_features": [_vp, _i, _vp, _vp],
    "oc_optcuts_initial_seams": [_vp, _i, _i],
    "oc_mesh_write_obj": [_vp, ctypes.c_char_p, _i, ctypes.c_int, ctypes.c_int],
    "oc_sd_energy_trials_noalloc": [_vp, _vp, _vp, _vp, ctypes.c_double, ctypes.c_int, _d, ctypes.c_int, ctypes.c_int,
                                    _vp, _vp],
}


def lib():
    """Loads the CUDA library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("liboc_gpu.so is not built (run: python -m optcuts_gb300.build); "
                              "there is no CPU fallback")
        L = ctypes.CDLL(LIB_PATH)
        for name, args in _SIGS.items():
            fn = getattr(L, name)
            fn.argtypes = args
            fn.restype = ctypes.c_int
        L.oc_last_error.argtypes = [_vp]
        L.oc_last_error.restype = ctypes.c_char_p
        L.oc_status_string.argtypes = [ctypes.c_int]
        L.oc_status_string.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _pd(a):
    return a.ctypes.data_as(_d)


def _pi(a):
    return a.ctypes.data_as(_i)


def _f8(a):
    return np.ascontiguousarray(a, np.float64)


def _f4(a):
    return np.ascontiguousarray(a, np.float32)


def _pf(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


def _i4(a):
    return np.ascontiguousarray(a, np.int32)


class Context:
    """One GPU and one CUDA stream (the caller's cudaStream_t handle as an
    int, e.g. torch.cuda.current_stream().cuda_stream, or a new stream)."""

    def __init__(self, device=0, stream=None):
        h = _vp()
        rc = lib().oc_ctx_create(device, _vp(stream) if stream else None, ctypes.byref(h))
        if rc != OC_OK:
            raise OCError(rc, "oc_ctx_create failed (no usable GPU?)")
        self.h = h

    def check(self, rc, what, allow=(OC_OK,)):
        if rc not in allow:
            msg = lib().oc_last_error(self.h).decode() or lib().oc_status_string(rc).decode()
            raise OCError(rc, "%s: %s" % (what, msg))
        return rc

    def synchronize(self):
        self.check(lib().oc_ctx_synchronize(self.h), "synchronize")

    def close(self):
        if getattr(self, "h", None):
            lib().oc_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context():
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


class TriMesh:
    """Device-resident TriMesh state (V_rest, V = UV, F, fixedVert)."""

    def __init__(self, V_rest, UV, F, fixedVert=(0,), areaThres=0.0, ctx=None):
        self.ctx = ctx or default_context()
        self.V_rest = _f8(V_rest)
        self.F = _i4(F)
        self.fixedVert = _i4(np.asarray(fixedVert).reshape(-1))
        uv = _f8(UV)
        if self.V_rest.ndim != 2 or self.V_rest.shape[1] != 3 or uv.shape != (len(self.V_rest), 2):
            raise ValueError("V_rest must be (n, 3) and UV (n, 2)")
        if self.F.ndim != 2 or self.F.shape[1] != 3:
            raise ValueError("F must be (m, 3)")
        self.nV, self.nF = len(self.V_rest), len(self.F)
        h = _vp()
        self.ctx.check(lib().oc_mesh_create(self.ctx.h, _pd(self.V_rest), _pd(uv), self.nV, _pi(self.F), self.nF,
                                            _pi(self.fixedVert), len(self.fixedVert), float(areaThres),
                                            ctypes.byref(h)), "TriMesh")
        self.h = h

    @property
    def V(self):
        out = np.empty((self.nV, 2))
        self.ctx.check(lib().oc_mesh_get_uv(self.h, _pd(out)), "get UV")
        return out

    @V.setter
    def V(self, uv):
        uv = _f8(uv)
        if uv.shape != (self.nV, 2):
            raise ValueError("UV shape")
        self.ctx.check(lib().oc_mesh_set_uv(self.h, _pd(uv)), "set UV")

    def rest_constants(self):
        rest = np.empty((self.nF, 8))
        sc = np.empty(3)
        self.ctx.check(lib().oc_mesh_rest_constants(self.h, _pd(rest), _pd(sc)), "rest constants")
        return rest, sc

    @property
    def surfaceArea(self):
        return self.rest_constants()[1][0]

    def checkInversion(self):
        ok = ctypes.c_int()
        self.ctx.check(lib().oc_mesh_check_inversion(self.h, ctypes.byref(ok)), "checkInversion")
        return bool(ok.value)

    # ---- topology (TriMesh::querySplit / queryMerge) ----
    def setCohesiveEdges(self, cohE):
        c = _i4(np.asarray(cohE).reshape(-1, 4))
        self.ctx.check(lib().oc_mesh_set_cohesive_edges(self.h, _pi(c), len(c)), "setCohesiveEdges")

    def dropAdjacency(self):
        """Forget the cached vertex adjacency: the next topology query
        rebuilds it, as the first query after an applied operation does."""
        self.ctx.check(lib().oc_mesh_drop_adjacency(self.h), "dropAdjacency")

    def splitFilter(self):
        """SymDirichletEnergy::computeDivGradPerVert at the current UV."""
        out = np.zeros(self.nV)
        self.ctx.check(lib().oc_mesh_split_filter(self.h, _pd(out)), "splitFilter")
        return out

    def _query(self, op, lambda_t, filterExp, fp32, features=False, mlp=None, topFrac=0.1, bijective=False):
        h = _vp()
        opt = (1 if fp32 else 0) | (2 if features else 0) | (16 if bijective else 0)
        t0 = time.perf_counter()
        if mlp is not None:
            self.ctx.check(lib().oc_topology_query_learned(self.h, op, float(lambda_t), float(filterExp), opt, mlp.h,
                                                           float(topFrac), ctypes.byref(h)), "learned topology query")
        else:
            self.ctx.check(lib().oc_topology_query(self.h, op, float(lambda_t), float(filterExp), opt,
                                                   ctypes.byref(h)), "topology query")
        query_ms = 1000.0 * (time.perf_counter() - t0)
        return self._result(h, features, mlp, query_ms)

    def topologyStep(self, lambda_t, filterExp=0.6, fp32=False, features=False, mlp=None, topFrac=0.1,
                     autotune=False, bijective=False):
        """The three queries of one topology step on the current state —
        boundary split, merge, interior split — built together and solved in
        the same launches (each result equals its own query's); with mlp the
        learned proposal (top fraction topFrac of each operation's problems
        solved exactly).  Returns (split, merge, interior); query_ms of each is
        the whole step's library time.  bijective: the reference's form with
        its scaffold on (the air loops of the scaffold last given to an
        Optimizer of this mesh)."""
        hs = [_vp(), _vp(), _vp()]
        opt = (1 if fp32 else 0) | (2 if features else 0) | (8 if autotune else 0) | (16 if bijective else 0)
        t0 = time.perf_counter()
        self.ctx.check(lib().oc_topology_step(self.h, float(lambda_t), float(filterExp), opt,
                                              mlp.h if mlp is not None else None, float(topFrac),
                                              *(ctypes.byref(h) for h in hs)), "topology step")
        step_ms = 1000.0 * (time.perf_counter() - t0)
        return tuple(self._result(h, features, mlp, step_ms) for h in hs)

    def topologyStepShard(self, lambda_t, rank, world, filterExp=0.6, fp32=False, ops=(0, 2, 1)):
        """One topology step's queries with only this shard's candidates
        solved (candidate c belongs to shard c % world); returns one raw
        list per op for optcuts_gb300.shard.merge."""
        o = _i4(list(ops))
        hs = (_vp * len(o))()
        self.ctx.check(lib().oc_topology_queries_sharded(self.h, _pi(o), len(o), float(lambda_t), float(filterExp),
                                                         1 if fp32 else 0, None, 0.1, int(rank), int(world), hs),
                       "sharded topology step")
        out = []
        for h in hs:
            try:
                n, pool = ctypes.c_int(), ctypes.c_int()
                lib().oc_topo_result_info(h, ctypes.byref(n), None, ctypes.byref(pool), None, None, None, None)
                nc = n.value
                d = {"EwDec": np.zeros(nc), "energyChanges": np.zeros((nc, 2)), "path": np.zeros((nc, 3), np.int32),
                     "newVertPos": np.zeros((nc, 8)), "posRows": np.zeros(nc, np.int32), "pool": pool.value}
                if nc:
                    lib().oc_topo_result_candidates(h, *(d[k].ctypes.data_as(_vp) for k in
                                                         ("EwDec", "energyChanges", "path", "newVertPos", "posRows")))
                out.append(d)
            finally:
                lib().oc_topo_result_destroy(h)
        return out

    def _result(self, h, features, mlp, query_ms):
        try:
            n, best, pool, nprob, mit = (ctypes.c_int() for _ in range(5))
            bms, sms = ctypes.c_double(), ctypes.c_double()
            lib().oc_topo_result_info(h, ctypes.byref(n), ctypes.byref(best), ctypes.byref(pool), ctypes.byref(nprob),
                                      ctypes.byref(mit), ctypes.byref(bms), ctypes.byref(sms))
            tot, cap, tri = ctypes.c_int(), ctypes.c_int(), ctypes.c_longlong()
            lib().oc_topo_result_iterations(h, ctypes.byref(tot), ctypes.byref(cap), ctypes.byref(tri))
            nsel, pms, ems = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
            lib().oc_topo_result_timing(h, ctypes.byref(nsel), ctypes.byref(pms), ctypes.byref(ems))
            hph = np.zeros(4)
            lib().oc_topo_result_host_phases(h, _pd(hph))
            X = tgt = prd = None
            if features or mlp is not None:
                nrow = ctypes.c_int()
                lib().oc_topo_result_features(h, ctypes.byref(nrow), None, None, None)
                X = np.zeros((nrow.value, 32), np.float32)
                tgt = np.zeros(nrow.value, np.float32) if features else None
                prd = np.zeros(nrow.value, np.float32) if mlp is not None else None
                if nrow.value:
                    lib().oc_topo_result_features(h, ctypes.byref(nrow), _pf(X), None if tgt is None else _pf(tgt),
                                                  None if prd is None else _pf(prd))
            npb = ctypes.c_int()
            lib().oc_topo_result_problems(h, ctypes.byref(npb), None, None, None)
            pc = np.zeros(npb.value, np.int32)
            pe, pp = np.zeros(npb.value), np.zeros(npb.value)
            pstat = {k: np.zeros(npb.value, np.int32) for k in ("nTri", "nFree", "iters", "trials")}
            pstat["cycles"] = np.zeros(npb.value, np.int64)
            if npb.value:
                lib().oc_topo_result_problems(h, ctypes.byref(npb), pc.ctypes.data_as(_vp), pe.ctypes.data_as(_vp),
                                              pp.ctypes.data_as(_vp))
                lib().oc_topo_result_problem_stats(h, ctypes.byref(npb), *(pstat[k].ctypes.data_as(_vp) for k in
                                                   ("nTri", "nFree", "iters", "trials", "cycles")))
            ap, ar, asx, acap = (ctypes.c_int() for _ in range(4))
            lib().oc_topo_result_air(h, ctypes.byref(ap), ctypes.byref(ar), ctypes.byref(asx), ctypes.byref(acap))
            nc = n.value
            ew, ec = np.zeros(nc), np.zeros((nc, 2))
            paths, pos, rows = np.zeros((nc, 3), np.int32), np.zeros((nc, 8)), np.zeros(nc, np.int32)
            if nc:
                lib().oc_topo_result_candidates(h, ew.ctypes.data_as(_vp), ec.ctypes.data_as(_vp),
                                                paths.ctypes.data_as(_vp), pos.ctypes.data_as(_vp),
                                                rows.ctypes.data_as(_vp))
            # (plain lists first: per-element numpy indexing costs more than
            # the query's own bookkeeping at ten thousand candidates)
            ewl, ecl, pl, rl = ew.tolist(), ec.tolist(), paths.tolist(), rows.tolist()
            p3 = pos.reshape(nc, 4, 2)
            cands = [{"EwDec": ewl[c], "energyChanges": (ecl[c][0], ecl[c][1]),
                      "path": [x for x in pl[c] if x >= 0], "newVertPos": p3[c, :rl[c]]} for c in range(nc)]
        finally:
            lib().oc_topo_result_destroy(h)
        b = best.value
        return {"EwDec_max": cands[b]["EwDec"] if b >= 0 else 0.0, "best": b,
                "path_max": cands[b]["path"] if b >= 0 else [], "candidates": cands, "pool": pool.value,
                "local_problems": nprob.value, "max_local_iters": mit.value, "build_ms": bms.value,
                "solve_ms": sms.value, "local_iters_total": tot.value, "local_capped": cap.value,
                "local_trials_total": tri.value, "selected": nsel.value, "probe_ms": pms.value,
                "exact_ms": ems.value, "features": X, "target": tgt, "predicted": prd,
                "host_ms": dict(zip(("prep", "air", "rank", "finish"), hph.tolist())),
                "problems": dict(cand=pc, EwDec=pe, EwDec_pred=pp, **pstat), "query_ms": query_ms,
                "air": {"problems": ap.value, "rejected": ar.value, "steiner_max": asx.value, "capped": acap.value}}

    def querySplit(self, lambda_t, splitInterior=False, filterExp=0.6, fp32=False, features=False, mlp=None,
                   topFrac=0.1, bijective=False):
        """TriMesh::querySplit(lambda_t, false, splitInterior) with every local
        solve batched on the GPU (bijective: with the local air loops of the
        scaffold last given to an Optimizer of this mesh); fp32 projects the local
        element Hessians in FP32; features records each local problem's
        features and exact target; mlp selects the learned proposal (only the
        top fraction topFrac of the problems is solved exactly)."""
        return self._query(OP_INTERIOR_SPLIT if splitInterior else OP_BOUNDARY_SPLIT, lambda_t, filterExp, fp32,
                           features, mlp, topFrac, bijective)

    def applyTopology(self, op, path, newVertPos):
        """splitEdgeOnBoundary / cutPath / mergeBoundaryEdges on this mesh."""
        path, pos = _i4(path), _f8(newVertPos).reshape(-1, 2)
        self.ctx.check(lib().oc_mesh_apply_topology(self.h, op, _pi(path), len(path), _pd(pos), len(pos)),
                       "applyTopology")
        self._sync_topology()

    def saveAsMesh(self, path, F0=None, nV0=0, scaleUV=False):
        """TriMesh::saveAsMesh: OBJ with rest positions (in F0's input
        numbering, or the copies glued along the seams) and the UV."""
        f0 = _i4(F0) if F0 is not None else None
        self.ctx.check(lib().oc_mesh_write_obj(self.h, os.fsencode(path), _pi(f0) if f0 is not None else None,
                                               int(nV0), int(bool(scaleUV))), "saveAsMesh")

    def _sync_topology(self):
        nv, nf, nc = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        lib().oc_mesh_get_topology(self.h, ctypes.byref(nv), ctypes.byref(nf), ctypes.byref(nc), None, None, None)
        F = np.zeros((nf.value, 3), np.int32)
        Vr = np.zeros((nv.value, 3))
        C = np.zeros((nc.value, 4), np.int32)
        lib().oc_mesh_get_topology(self.h, None, None, None, _pi(F), _pd(Vr), _pi(C))
        self.nV, self.nF, self.F, self.V_rest, self.cohE = nv.value, nf.value, F, Vr, C

    def queryMerge(self, lambda_t, fp32=False, features=False, mlp=None, topFrac=0.1, bijective=False):
        """TriMesh::queryMerge(lambda_t, false)."""
        return self._query(OP_MERGE, lambda_t, 0.6, fp32, features, mlp, topFrac, bijective)

    def close(self):
        if getattr(self, "h", None):
            lib().oc_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class SymDirichletEnergy:
    """src/Energy/SymDirichletEnergy.hpp:15-42, on the device."""

    needRefactorize = True

    def computeEnergyVal(self, data, uniformWeight=False):
        e = ctypes.c_double()
        data.ctx.check(lib().oc_sd_energy(data.h, int(uniformWeight), ctypes.byref(e)), "computeEnergyVal")
        return e.value

    def getEnergyValPerElem(self, data, uniformWeight=False):
        out = np.empty(data.nF)
        data.ctx.check(lib().oc_sd_energy_per_elem(data.h, int(uniformWeight), _pd(out)), "getEnergyValPerElem")
        return out

    def computeGradient(self, data, uniformWeight=False):
        g = np.empty(2 * data.nV)
        data.ctx.check(lib().oc_sd_gradient(data.h, int(uniformWeight), _pd(g)), "computeGradient")
        return g

    def computeHessian(self, data, uniformWeight=False, projection=HESSIAN_JACOBI6):
        """Per-triangle PSD-projected 6x6 blocks, shape (nF, 6, 6).
        projection: HESSIAN_JACOBI6 (the 6x6 eigen-clamp, the optimizer's
        default), HESSIAN_REDUCED (the same projection over the
        translation-free 4x4 form) or HESSIAN_HYBRID (4x4 where the element's
        energy density is at most 1e3)."""
        out = np.empty((data.nF, 6, 6))
        data.ctx.check(lib().oc_sd_hessian_blocks_projected(data.h, int(uniformWeight), int(projection), _pd(out)),
                       "computeHessian")
        return out

    def initStepSize(self, data, searchDir, stepSize=1.0):
        d = _f8(searchDir)
        if d.size != 2 * data.nV:
            raise ValueError("searchDir size")
        s = ctypes.c_double(stepSize)
        data.ctx.check(lib().oc_sd_init_step_size(data.h, _pd(d), ctypes.byref(s)), "initStepSize")
        return s.value


class LinSysSolver:
    """GPU block-CSR matrix + block-Jacobi PCG behind the reference's
    LinSysSolver interface (LinSysSolver.hpp:22-187)."""

    def __init__(self, ctx=None, solver=SOLVER_DIRECT):
        self.ctx = ctx or default_context()
        h = _vp()
        self.ctx.check(lib().oc_linsys_create(self.ctx.h, ctypes.byref(h)), "LinSysSolver")
        self.h = h
        self.ctx.check(lib().oc_linsys_set_type(h, int(solver)), "set_type")
        self.numRows = 0
        self.last_iters = 0
        self.last_relres = 0.0

    def set_pattern(self, nV, F, fixedVert):
        F, fx = _i4(F), _i4(np.asarray(fixedVert).reshape(-1))
        self.ctx.check(lib().oc_linsys_set_pattern(self.h, nV, _pi(F), len(F), _pi(fx), len(fx)), "set_pattern")
        self.numRows = 2 * nV

    def set_pattern_neighbors(self, vNeighbor, fixedVert):
        """set_pattern(vNeighbor, fixedVert) as the reference's Optimizer calls
        it: vNeighbor a list of neighbour-index lists, one per vertex."""
        nV = len(vNeighbor)
        ptr = np.zeros(nV + 1, np.int32)
        ptr[1:] = np.cumsum([len(n) for n in vNeighbor])
        idx = _i4(np.concatenate([np.asarray(list(n), np.int32) for n in vNeighbor]) if nV else np.zeros(0))
        fx = _i4(np.asarray(list(fixedVert)).reshape(-1))
        self.ctx.check(lib().oc_linsys_set_pattern_neighbors(self.h, nV, _pi(ptr), _pi(idx), _pi(fx), len(fx)),
                       "set_pattern")
        self.numRows = 2 * nV

    def update_a(self, I, J, V):
        I, J, V = _i4(I), _i4(J), _f8(V)
        self.ctx.check(lib().oc_linsys_update_a(self.h, _pi(I), _pi(J), _pd(V), len(V)), "update_a")

    def analyze_pattern(self):
        self.ctx.check(lib().oc_linsys_analyze_pattern(self.h), "analyze_pattern")

    def stats(self):
        out = np.zeros(8)
        self.ctx.check(lib().oc_linsys_stats(self.h, _pd(out)), "stats")
        return symbolic_stats_dict(out)

    def set_solve_cluster(self, maxCluster):
        """Largest thread-block cluster per front (1..8) in the direct
        solver's substitutions; the solution is the same bits for every value."""
        self.ctx.check(lib().oc_linsys_set_solve_cluster(self.h, int(maxCluster)), "set_solve_cluster")

    def solve_clusters(self):
        """(tree levels whose substitutions run as clusters, largest cluster)"""
        a, b = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(lib().oc_linsys_solve_clusters(self.h, ctypes.byref(a), ctypes.byref(b)), "solve_clusters")
        return a.value, b.value

    def set_factor_streams(self, streams):
        """Most CUDA streams (1..8) for the factorization's independent
        subtrees, from the next set_pattern on; the factor is the same bits
        for every value."""
        self.ctx.check(lib().oc_linsys_set_factor_streams(self.h, int(streams)), "set_factor_streams")

    def factor_streams(self):
        """(streams, subtree groups) of the current plan's factorization"""
        a, b = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(lib().oc_linsys_factor_streams(self.h, ctypes.byref(a), ctypes.byref(b)), "factor_streams")
        return a.value, b.value

    def factorize(self):
        return self.ctx.check(lib().oc_linsys_factorize(self.h), "factorize") == OC_OK

    def solve(self, rhs, tol=1e-8, maxIter=20000):
        rhs = _f8(rhs)
        x = np.empty(self.numRows)
        it = ctypes.c_int()
        rr = ctypes.c_double()
        rc = self.ctx.check(lib().oc_linsys_solve(self.h, _pd(rhs), _pd(x), tol, maxIter, ctypes.byref(it),
                                                  ctypes.byref(rr)), "solve", allow=(OC_OK, OC_ERR_NOT_CONVERGED))
        self.last_iters, self.last_relres, self.last_converged = it.value, rr.value, rc == OC_OK
        return x

    def multiply(self, x):
        x = _f8(x)
        y = np.empty(self.numRows)
        self.ctx.check(lib().oc_linsys_multiply(self.h, _pd(x), _pd(y)), "multiply")
        return y

    def close(self):
        if getattr(self, "h", None):
            lib().oc_linsys_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def energy_w(last_energy, seam_length, virtual_radius, lam):
    """E_w = (1 - lambda) E_SD + lambda E_se, with E_se = seam length /
    virtualRadius -- the value Optimizer::writeEnergyValToFile records per
    iteration in fracture mode (Optimizer.cpp:706-716).  `last_energy` is
    Optimizer.getLastEnergyVal() = (1 - lambda) E_SD; the seam length comes
    from optcuts_gb300.init.seam_sparsity and is constant during a Newton
    phase (it changes only with the topology)."""
    return last_energy + lam * seam_length / virtual_radius


def topology_apply(op, path, newVertPos, V_rest, UV, F, cohE):
    """Host-only topology operation (TriMesh::splitEdgeOnBoundary / cutPath /
    mergeBoundaryEdges) on plain arrays: returns (V_rest, UV, F, cohE)."""
    path, pos = _i4(path), _f8(newVertPos).reshape(-1, 2)
    Vr, uv, F = _f8(V_rest), _f8(UV), _i4(F)
    c = _i4(np.asarray(cohE).reshape(-1, 4))
    nV = len(Vr)
    Fo, Vo, Uo = np.zeros_like(F), np.zeros((nV + 2, 3)), np.zeros((nV + 2, 2))
    Co = np.zeros((len(c) + 2, 4), np.int32)
    nvo, nco = ctypes.c_int(), ctypes.c_int()
    rc = lib().oc_topology_apply(op, _pi(path), len(path), _pd(pos), len(pos), nV, len(F), _pi(F), _pd(Vr), _pd(uv),
                                 len(c), _pi(c), _pi(Fo), _pd(Vo), _pd(Uo), _pi(Co), ctypes.byref(nvo), ctypes.byref(nco))
    if rc != OC_OK:
        raise OCError(rc, "topology_apply")
    return Vo[:nvo.value], Uo[:nvo.value], Fo, Co[:nco.value]


def cut_to_disk(F):
    """Host-only igl::cut_to_disk as the reference vendors it: the cut graph
    of a genus >= 1 surface as vertex lists (a closed loop repeats its first
    vertex)."""
    F = _i4(F)
    nc, nv = ctypes.c_int(), ctypes.c_int()
    rc = lib().oc_cut_to_disk(_pi(F), len(F), None, 0, None, 0, ctypes.byref(nc), ctypes.byref(nv))
    if rc != OC_OK:
        raise OCError(rc, "cut_to_disk")
    verts = np.zeros(max(nv.value, 1), np.int32)
    off = np.zeros(nc.value + 1, np.int32)
    rc = lib().oc_cut_to_disk(_pi(F), len(F), _pi(verts), len(verts), _pi(off), len(off), ctypes.byref(nc),
                              ctypes.byref(nv))
    if rc != OC_OK:
        raise OCError(rc, "cut_to_disk")
    return [verts[off[i]:off[i + 1]].tolist() for i in range(nc.value)]


def topology_cut_path(path, V_rest, UV, F, cohE):
    """Host-only TriMesh::cutPath(path, makeCoh = true) as the initial cutting
    of a genus >= 1 mesh calls it (boundary splits along the path; an
    interior path first cut through its first three vertices): returns
    (V_rest, UV, F, cohE, edges split)."""
    path = _i4(path)
    Vr, uv, F = _f8(V_rest), _f8(UV), _i4(F)
    c = _i4(np.asarray(cohE).reshape(-1, 4))
    nV, extra = len(Vr), 2 * len(path)
    Fo, Vo, Uo = np.zeros_like(F), np.zeros((nV + extra, 3)), np.zeros((nV + extra, 2))
    Co = np.zeros((len(c) + extra, 4), np.int32)
    nvo, nco, made = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rc = lib().oc_topology_cut_path(_pi(path), len(path), nV, len(F), _pi(F), _pd(Vr), _pd(uv), len(c), _pi(c),
                                    _pi(Fo), _pd(Vo), _pd(Uo), _pi(Co), ctypes.byref(nvo), ctypes.byref(nco),
                                    ctypes.byref(made))
    if rc != OC_OK:
        raise OCError(rc, "topology_cut_path")
    return Vo[:nvo.value], Uo[:nvo.value], Fo, Co[:nco.value], made.value


def split_candidates(nV, F, divGrad, interior, filterExp=0.6):
    """Host-only split filter (TriMesh.cpp:561-629): candidate vertices in
    the reference's order and the filtered pool size."""
    F, dg = _i4(F), _f8(divGrad)
    out = np.zeros(nV, np.int32)
    n, pool = ctypes.c_int(), ctypes.c_int()
    rc = lib().oc_topology_split_candidates(nV, _pi(F), len(F), _pd(dg), int(interior), float(filterExp), _pi(out),
                                            ctypes.byref(n), ctypes.byref(pool))
    if rc != OC_OK:
        raise OCError(rc, "split_candidates")
    return out[:n.value], pool.value


def symbolic_stats_dict(out):
    keys = ["fronts", "levels", "max_front_rows", "pool_doubles", "flops", "launches", "factor_entries", "dof"]
    return dict(zip(keys, [float(x) for x in out]))


def chol_analyze_stats(nV, F, fixedVert=(0,), leafSize=16, xy=None):
    """Symbolic analysis of the direct solver, host only (no GPU needed);
    with vertex coordinates xy (nV x 2) the geometric nested dissection."""
    F = _i4(F)
    fx = _i4(np.asarray(fixedVert).reshape(-1))
    out = np.zeros(8)
    if xy is not None:
        xy = _f8(xy).reshape(-1, 2)
        if len(xy) != nV:
            raise ValueError("xy: one row per vertex")
        rc = lib().oc_chol_analyze_stats_xy(int(nV), _pi(F), len(F), _pi(fx), len(fx), int(leafSize), _pd(xy),
                                            _pd(out))
        if rc != OC_OK:
            raise OCError(rc, "oc_chol_analyze_stats_xy")
        return symbolic_stats_dict(out)
    rc = lib().oc_chol_analyze_stats(int(nV), _pi(F), len(F), _pi(fx), len(fx), int(leafSize), _pd(out))
    if rc != OC_OK:
        raise OCError(rc, "oc_chol_analyze_stats")
    return symbolic_stats_dict(out)


def chol_analyze_groups(nV, F, fixedVert=(0,), leafSize=16, maxStreams=8):
    """The direct solver's factorization streams for this pattern, host only:
    (streams used, subtree groups, whether every front's children finish
    before it under the plan's streams and waits)."""
    F = _i4(F)
    fx = _i4(np.asarray(fixedVert).reshape(-1))
    out = np.zeros(3, np.int32)
    rc = lib().oc_chol_analyze_groups(int(nV), _pi(F), len(F), _pi(fx), len(fx), int(leafSize), int(maxStreams),
                                      _pi(out))
    if rc != OC_OK:
        raise OCError(rc, "oc_chol_analyze_groups")
    return int(out[0]), int(out[1]), bool(out[2])


def air_loop_mesh(pts, maxSteiner=12):
    """The bijective local solves' loop mesher on the host (oc_air_loop_mesh:
    Triangle's "qYQ" on a simple polygon): returns (V, T, status) -- the
    polygon's points then the Steiner points, counter-clockwise triangles,
    and the mesher's status bits (8 / 16: refinement stopped at a limit)."""
    p = _f8(pts).reshape(-1, 2)
    n = len(p)
    V = np.zeros((n + 12, 2))
    T = np.zeros((n + 22, 3), np.int32)
    nV, nT, st = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rc = lib().oc_air_loop_mesh(p.ctypes.data_as(_vp), n, int(maxSteiner), ctypes.byref(nV), V.ctypes.data_as(_vp),
                                ctypes.byref(nT), T.ctypes.data_as(_vp), ctypes.byref(st))
    if rc != OC_OK:
        raise OCError(rc, "air_loop_mesh: not a simple polygon of 3..48 points")
    return V[:nV.value], T[:nT.value], st.value


def topology_schedules():
    """The local-solve schedule autotuner's table (OC_TOPO_AUTOTUNE queries):
    one dict per key with the chosen and the fixed rule's schedule and their
    measured milliseconds."""
    n = ctypes.c_int()
    lib().oc_topology_schedules(ctypes.byref(n), None, None)
    rows = np.zeros((n.value, 11), np.int32)
    ms = np.zeros((n.value, 2), np.float32)
    if n.value:
        lib().oc_topology_schedules(ctypes.byref(n), _pi(rows), ms.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
    out = []
    for r, t in zip(rows, ms):
        out.append({"class": int(r[1]) % 4, "probe": bool(r[1] >= 4), "count_log2": int(r[2]), "tri_log2": int(r[3]),
                    "chosen": {"tpp": int(r[4]), "cluster": int(r[5]), "block": int(r[6]), "ms": float(t[0])},
                    "rule": {"tpp": int(r[7]), "cluster": int(r[8]), "block": int(r[9]), "ms": float(t[1])},
                    "candidates": int(r[10])})
    return out


def default_config(**kw):
    c = OptimizerConfig()
    lib().oc_optimizer_default_config(ctypes.byref(c))
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def bf16_gemm(A, B, tensor_cores=True, a_transposed=False, b_transposed=False, ctx=None):
    """C = op(A) @ op(B) with BF16 operands and FP32 accumulation on the
    device (the MLP's product), on the tensor cores or the CUDA cores.
    a_transposed: A holds op(A) transposed (K x M, row-major), read through
    strides (1, M) as the network's backward products read theirs; likewise
    b_transposed (B is N x K)."""
    ctx = ctx or default_context()
    A = _f4(A)
    B = _f4(B)
    M, K = (A.shape[1], A.shape[0]) if a_transposed else A.shape
    N = B.shape[0] if b_transposed else B.shape[1]
    sam, sak = (1, M) if a_transposed else (K, 1)
    sbk, sbn = (1, K) if b_transposed else (N, 1)
    C = np.zeros((M, N), np.float32)
    ctx.check(lib().oc_bf16_gemm(ctx.h, M, N, K, _pf(A), sam, sak, _pf(B), sbk, sbn, _pf(C),
                                 1 if tensor_cores else 0), "bf16_gemm")
    return C


class OptCuts:
    """The OptCuts outer loop (src/main.cpp:538-1086, offline preDrawFunc with
    updateLambda_stationaryV and converge_preDrawFunc) over a precomputed
    Optimizer: inner Newton loops with fracture propagation, topology steps,
    dual lambda updates, oscillation rollback, convergence at b_d.  The
    optimizer's mesh must carry the cohesive edges of its initial cut."""

    STATE = ["E_SD", "E_se", "lambda", "E_w", "newton_iterations", "topology_steps", "finished", "vertices",
             "newton_ms", "query_ms", "apply_ms", "total_ms"]
    EVENTS = {0: "inner converged", 1: "split or merge", 2: "interior split", 3: "interior split (wider filter)",
              4: "critical-lambda split", 5: "critical-lambda interior split", 6: "critical-lambda merge",
              10: "oscillation", 11: "converged at bound", 12: "no merge left"}

    def __init__(self, optimizer, upperBound=4.1, bijective=False, topoLineSearch=True, filterExp=0.6, fp32=False,
                 mlp=None, topFrac=0.1, maxNewtonIters=100000, recordFeatures=False):
        self.opt = optimizer
        self.ctx = optimizer.ctx
        cfg = OptCutsConfig()
        lib().oc_optcuts_default_config(ctypes.byref(cfg))
        cfg.upperBound, cfg.bijective, cfg.topoLineSearch = float(upperBound), int(bool(bijective)), int(topoLineSearch)
        cfg.filterExp, cfg.topoOptions = float(filterExp), 1 if fp32 else 0
        cfg.mlp = mlp.h if mlp is not None else None
        cfg.topFrac, cfg.maxNewtonIters = float(topFrac), int(maxNewtonIters)
        cfg.recordFeatures = int(bool(recordFeatures))
        self._mlp = mlp
        h = _vp()
        self.ctx.check(lib().oc_optcuts_create(optimizer.h, optimizer.data.h, ctypes.byref(cfg), ctypes.byref(h)),
                       "OptCuts")
        self.h = h

    def run(self, maxSteps=1000000):
        """Outer passes until the loop ends; returns whether it finished."""
        f = ctypes.c_int()
        self.ctx.check(lib().oc_optcuts_run(self.h, int(maxSteps), ctypes.byref(f)), "OptCuts.run")
        self.opt.data._sync_topology()
        return bool(f.value)

    def state(self):
        out = np.zeros(12)
        self.ctx.check(lib().oc_optcuts_state(self.h, _pd(out)), "OptCuts.state")
        return dict(zip(self.STATE, out.tolist()))

    def _rows(self, fn, cols):
        n = ctypes.c_int()
        self.ctx.check(fn(self.h, ctypes.byref(n), None), "OptCuts")
        out = np.zeros((n.value, cols))
        self.ctx.check(fn(self.h, ctypes.byref(n), _pd(out)), "OptCuts")
        return out

    def events(self):
        """rows: Newton iterations, E_SD, E_se, lambda, vertices, event code"""
        return self._rows(lib().oc_optcuts_events, 6)

    def trace(self):
        """rows per Newton iteration: iterations, E_w, E_SD, E_se, lambda,
        vertices, ||gradient||^2"""
        return self._rows(lib().oc_optcuts_trace, 7)

    def features(self):
        """(X, target) pairs the exhaustive queries of the run recorded
        (recordFeatures=True): the learned proposal's training data."""
        n = ctypes.c_int()
        self.ctx.check(lib().oc_optcuts_features(self.h, ctypes.byref(n), None, None), "OptCuts.features")
        X = np.zeros((n.value, 32), np.float32)
        t = np.zeros(n.value, np.float32)
        if n.value:
            self.ctx.check(lib().oc_optcuts_features(self.h, ctypes.byref(n), _pf(X), _pf(t)), "OptCuts.features")
        return X, t

    def write(self, folder, F0=None, nV0=0, lambdaInit=0.999):
        """The reference's output files of the run into folder:
        energyValPerIter.txt, gradientPerIter.txt, info.txt and
        finalResult_mesh.obj (F0: the input mesh's triangles)."""
        f0 = _i4(F0) if F0 is not None else None
        self.ctx.check(lib().oc_optcuts_write(self.h, os.fsencode(folder), _pi(f0) if f0 is not None else None,
                                              int(nV0), float(lambdaInit)), "OptCuts.write")

    def close(self):
        if getattr(self, "h", None):
            lib().oc_optcuts_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MLP:
    """The learned proposal's network: nIn -> nHidden -> nHidden -> 1 (ReLU),
    BF16 weights and activations, FP32 accumulation, trained on the GPU."""

    def __init__(self, nIn=32, nHidden=128, seed=0, ctx=None):
        self.ctx = ctx or default_context()
        self.nIn, self.nHidden = nIn, nHidden
        h = _vp()
        self.ctx.check(lib().oc_mlp_create(self.ctx.h, nIn, nHidden, seed, ctypes.byref(h)), "MLP")
        self.h = h

    def num_params(self):
        n = ctypes.c_int()
        lib().oc_mlp_num_params(self.h, ctypes.byref(n))
        return n.value

    def params(self):
        p = np.zeros(self.num_params(), np.float32)
        self.ctx.check(lib().oc_mlp_get_params(self.h, _pf(p)), "MLP params")
        return p

    def set_params(self, p):
        p = _f4(p)
        self.ctx.check(lib().oc_mlp_set_params(self.h, _pf(p)), "MLP set_params")

    def predict(self, X):
        X = _f4(X).reshape(-1, self.nIn)
        y = np.zeros(len(X), np.float32)
        self.ctx.check(lib().oc_mlp_predict(self.h, _pf(X), len(X), _pf(y)), "MLP predict")
        return y

    def gradient(self, X, t):
        X, t = _f4(X).reshape(-1, self.nIn), _f4(t)
        g = np.zeros(self.num_params(), np.float32)
        loss = ctypes.c_float()
        self.ctx.check(lib().oc_mlp_gradient(self.h, _pf(X), _pf(t), len(X), _pf(g), ctypes.byref(loss)),
                       "MLP gradient")
        return g, loss.value

    def train(self, X, t, epochs=30, batch=512, lr=1e-3, seed=0):
        X, t = _f4(X).reshape(-1, self.nIn), _f4(t)
        loss = ctypes.c_float()
        self.ctx.check(lib().oc_mlp_train(self.h, _pf(X), _pf(t), len(X), epochs, batch, lr, seed,
                                          ctypes.byref(loss)), "MLP train")
        return loss.value

    def set_tensor_cores(self, on=True):
        """Hidden-layer products on the tensor cores (tcgen05) or the CUDA cores."""
        self.ctx.check(lib().oc_mlp_set_tensor_cores(self.h, 1 if on else 0), "MLP set_tensor_cores")

    def close(self):
        if getattr(self, "h", None):
            lib().oc_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Scaffold:
    """Air mesh of the bijectivity scaffold as Scaffold's constructor leaves it
    (Scaffold.hpp:18-24): airMesh.V (nAirV x 2), airMesh.F (nAirF x 3) and bnd
    (air vertex i < len(bnd) is mesh vertex bnd[i])."""

    def __init__(self, airV, airF, bnd):
        self.airV = np.ascontiguousarray(airV, np.float64).reshape(-1, 2)
        self.airF = np.ascontiguousarray(airF, np.int32).reshape(-1, 3)
        self.bnd = np.ascontiguousarray(bnd, np.int32).ravel()

    @classmethod
    def build(cls, UV, F, avgEdgeLen, minAngle=20.0):
        """The project's own air mesh for a UV layout (constrained Delaunay
        between the boundary loops and the reference's segmented box, refined
        towards minAngle degrees; no Triangle).  Host only."""
        UV, F = _f8(UV), _i4(F)
        h = _vp()
        rc = lib().oc_air_mesh_build(_pd(UV), len(UV), _pi(F), len(F), float(avgEdgeLen), float(minAngle),
                                     ctypes.byref(h))
        if rc != OC_OK:
            raise OCError(rc, "air mesh: " + lib().oc_status_string(rc).decode())
        try:
            nv, nf, nb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
            lib().oc_air_mesh_sizes(h, ctypes.byref(nv), ctypes.byref(nf), ctypes.byref(nb))
            V = np.zeros((nv.value, 2))
            Fa = np.zeros((nf.value, 3), np.int32)
            b = np.zeros(nb.value, np.int32)
            lib().oc_air_mesh_get(h, _pd(V), _pi(Fa), _pi(b))
        finally:
            lib().oc_air_mesh_destroy(h)
        return cls(V, Fa, b)

    def localVI2Global(self, nV):
        nb = len(self.bnd)
        return np.concatenate([self.bnd, nV + np.arange(len(self.airV) - nb, dtype=np.int32)])


class Optimizer:
    """Projected Newton with the injective line search (Optimizer.hpp:74-142),
    with or without a scaffold.  energyParams = [1 - lambda] as in
    main.cpp:1569."""

    def __init__(self, data0, energyParams, config=None, **kw):
        self.data = data0
        self.ctx = data0.ctx
        self.energyParams = list(energyParams)
        cfg = config if config is not None else default_config(**kw)
        h = _vp()
        self.ctx.check(lib().oc_optimizer_create(data0.h, float(self.energyParams[0]), ctypes.byref(cfg),
                                                 ctypes.byref(h)), "Optimizer")
        self.h = h

    def precompute(self):
        self.ctx.check(lib().oc_optimizer_precompute(self.h), "precompute")

    def solve(self, maxIter=100):
        r = ctypes.c_int()
        self.ctx.check(lib().oc_optimizer_solve(self.h, maxIter, ctypes.byref(r)), "solve",
                       allow=(OC_OK, OC_ERR_NOT_CONVERGED))
        return r.value

    def getLastEnergyVal(self, excludeScaffold=False):
        e = ctypes.c_double()
        self.ctx.check(lib().oc_optimizer_get_last_energy(self.h, ctypes.byref(e)), "getLastEnergyVal")
        if excludeScaffold:
            es = ctypes.c_double()
            self.ctx.check(lib().oc_optimizer_get_last_energy_scaffold(self.h, ctypes.byref(es)), "getLastEnergyVal")
            return e.value - es.value
        return e.value

    def setScaffold(self, scaffold, areaThres=-1.0):
        """Installs the air mesh for the next solve() (the reference rebuilds it
        after every iteration, Optimizer.cpp:251-257)."""
        self.ctx.check(lib().oc_optimizer_set_scaffold(
            self.h, _pd(scaffold.airV), len(scaffold.airV), _pi(scaffold.airF), len(scaffold.airF),
            _pi(scaffold.bnd), len(scaffold.bnd), float(areaThres)), "setScaffold")

    def createFracture(self, op, path, newVertPos):
        """Optimizer::createFracture(opType, path, newVertPos) (Optimizer.cpp:373-440)."""
        path, pos = _i4(path), _f8(newVertPos).reshape(-1, 2)
        self.ctx.check(lib().oc_optimizer_create_fracture(self.h, op, _pi(path), len(path), _pd(pos), len(pos)),
                       "createFracture")
        self.data._sync_topology()

    def analysisInfo(self):
        """The direct solver's last symbolic analysis: carried analyses since
        the last full one (0: full), host ms of the dissection and of the
        front structures, factor flops and those of the last full analysis."""
        c = ctypes.c_int()
        d = [ctypes.c_double() for _ in range(4)]
        self.ctx.check(lib().oc_optimizer_analysis_info(self.h, ctypes.byref(c), *(ctypes.byref(x) for x in d)),
                       "analysisInfo")
        return {"carried": c.value, "nd_ms": d[0].value, "sym_ms": d[1].value, "flops": d[2].value,
                "full_flops": d[3].value}

    def applyTiming(self):
        """Phase durations (ms) of the last createFracture: mesh edit, device
        mesh, scaffold, pattern + symbolic analysis (host), their device
        allocation and upload, energy."""
        out = np.zeros(6)
        self.ctx.check(lib().oc_optimizer_apply_timing(self.h, _pd(out)), "applyTiming")
        keys = ["mesh_edit", "device_mesh", "scaffold", "pattern_host", "pattern_device", "energy"]
        return dict(zip(keys, [float(x) for x in out]))

    def splitOrMerge(self, EDecThres, splitInterior=False, filterExp=0.6, fp32=False, mlp=None, topFrac=0.1):
        """Optimizer::createFracture(EDecThres, 0, false, splitInterior)
        (Optimizer.cpp:440-503) -> TriMesh::splitOrMerge (TriMesh.cpp:978-1052):
        query, pick the larger E_w decrease of split and merge, apply it when
        above EDecThres.  Returns (changed, opType, EwDec_max)."""
        ch, op, ew = ctypes.c_int(), ctypes.c_int(), ctypes.c_double()
        self.ctx.check(lib().oc_optimizer_split_or_merge(self.h, float(EDecThres), 1 if splitInterior else 0,
                                                         float(filterExp), 1 if fp32 else 0,
                                                         mlp.h if mlp is not None else None, float(topFrac),
                                                         ctypes.byref(ch), ctypes.byref(op), ctypes.byref(ew)),
                       "splitOrMerge")
        if ch.value:
            self.data._sync_topology()
        return bool(ch.value), op.value, ew.value

    def rebuildScaffold(self):
        """Scaffold(result) for the current UV with the project's air-mesh
        generator (what the reference does after every iteration)."""
        self.ctx.check(lib().oc_optimizer_rebuild_scaffold(self.h), "rebuildScaffold")
        return self.getScaffold()

    def getScaffold(self):
        """The current air mesh (airMesh.V as the last step moved it)."""
        nv, nf, nb = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
        self.ctx.check(lib().oc_optimizer_get_scaffold(self.h, ctypes.byref(nv), ctypes.byref(nf), ctypes.byref(nb),
                                                       None, None, None), "getScaffold")
        V = np.zeros((nv.value, 2))
        F = np.zeros((nf.value, 3), np.int32)
        b = np.zeros(nb.value, np.int32)
        self.ctx.check(lib().oc_optimizer_get_scaffold(self.h, None, None, None, _pd(V), _pi(F), _pi(b)),
                       "getScaffold")
        return Scaffold(V, F, b)

    def clearScaffold(self):
        self.ctx.check(lib().oc_optimizer_clear_scaffold(self.h), "clearScaffold")

    def scaffoldV(self):
        """Current air-mesh UV (Scaffold::airMesh.V after the last step)."""
        return self.getScaffold().airV

    def systemSize(self):
        n = ctypes.c_int()
        self.ctx.check(lib().oc_optimizer_system_size(self.h, ctypes.byref(n)), "systemSize")
        return n.value

    def lastVectors(self):
        """(gradient, searchDir) of the last iteration, interleaved u, v."""
        n = self.systemSize()
        g, d = np.zeros(2 * n), np.zeros(2 * n)
        self.ctx.check(lib().oc_optimizer_last_vectors(self.h, _pd(g), _pd(d)), "lastVectors")
        return g, d

    def badPivots(self):
        """Zero or non-finite pivots of the last factorization (a solve that
        met any raised OCError with status OC_ERR_NOT_SPD)."""
        n = ctypes.c_int()
        self.ctx.check(lib().oc_optimizer_bad_pivots(self.h, ctypes.byref(n)), "badPivots")
        return n.value

    def getIterNum(self):
        n = ctypes.c_int()
        self.ctx.check(lib().oc_optimizer_get_iter_num(self.h, ctypes.byref(n)), "getIterNum")
        return n.value

    def setRelGL2Tol(self, tol):
        self.ctx.check(lib().oc_optimizer_set_rel_gl2_tol(self.h, tol), "setRelGL2Tol")

    def updateEnergyData(self):
        self.ctx.check(lib().oc_optimizer_set_energy_param(self.h, float(self.energyParams[0])), "updateEnergyData")

    def getResult(self):
        return self.data

    def last_step(self):
        s, r, g = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
        it, ls = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(lib().oc_optimizer_last_step(self.h, ctypes.byref(s), ctypes.byref(it), ctypes.byref(r),
                                                    ctypes.byref(ls), ctypes.byref(g)), "last_step")
        return {"stepSize": s.value, "pcgIters": it.value, "pcgRelRes": r.value, "lineSearchLaunches": ls.value,
                "gradSqNorm": g.value}

    PHASES = ["gradient", "hessian", "assembly", "factorize", "solve", "injective", "linesearch"]

    def phase_ms(self):
        out = np.zeros(7)
        self.ctx.check(lib().oc_optimizer_phase_ms(self.h, _pd(out)), "phase_ms")
        return dict(zip(self.PHASES, out.tolist()))

    def solver_stats(self):
        out = np.zeros(8)
        self.ctx.check(lib().oc_optimizer_solver_stats(self.h, _pd(out)), "solver_stats")
        return symbolic_stats_dict(out)

    def set_solve_cluster(self, maxCluster):
        """LinSysSolver.set_solve_cluster on this optimizer's own solver."""
        self.ctx.check(lib().oc_optimizer_set_solve_cluster(self.h, int(maxCluster)), "set_solve_cluster")

    def solve_clusters(self):
        """LinSysSolver.solve_clusters on this optimizer's own solver."""
        a, b = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(lib().oc_optimizer_solve_clusters(self.h, ctypes.byref(a), ctypes.byref(b)), "solve_clusters")
        return a.value, b.value

    def set_factor_streams(self, streams):
        """LinSysSolver.set_factor_streams on this optimizer's own solver
        (before precompute, to cover every analysis)."""
        self.ctx.check(lib().oc_optimizer_set_factor_streams(self.h, int(streams)), "set_factor_streams")

    def factor_streams(self):
        """LinSysSolver.factor_streams on this optimizer's own solver."""
        a, b = ctypes.c_int(), ctypes.c_int()
        self.ctx.check(lib().oc_optimizer_factor_streams(self.h, ctypes.byref(a), ctypes.byref(b)), "factor_streams")
        return a.value, b.value

    def launch_count(self):
        n = ctypes.c_longlong()
        self.ctx.check(lib().oc_optimizer_launch_count(self.h, ctypes.byref(n)), "launch_count")
        return n.value

    def close(self):
        if getattr(self, "h", None):
            lib().oc_optimizer_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
