#!/usr/bin/env python
"""Newton iterations per second of the OptCuts geometry step on one GB300.

Workload (default): the lat-long ellipsoid, axes (1, 0.6, 0.4), 316 x 316
grid with 8 random spherical-harmonic bumps (199,080 triangles, seed 2),
one-point cut + Tutte embedding, lambda = 0.999, bijectivity scaffold on.
A step is what the reference's Optimizer::solve(1) does with the scaffold
on: one Newton iteration (gradient, PSD-projected Hessian, block assembly,
multifrontal LDL^T factorisation and solve, injective bound, line search)
over mesh + air mesh, then the scaffold rebuilt for the new UV
(Optimizer.cpp:251-257; here the project's own air-mesh generator).
--scaffold off times the scaffold-free Newton phase instead.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Under torchrun (N > 1) every rank runs an independent replica of the same
workload (the Newton solve does not shard); value = iterations of all ranks
divided by the slowest rank's time.  --impl reference times the CPU
restatement of the reference path (oracle/port, the reference's own
sources are not present on the GPU host) on all host cores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Newton iter/s @200k tris"
UNIT = "iter/s"
FP64_PEAK_TFLOPS = 1.25     # GB300 FP64, nominal


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=10)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="ellipsoid_199k")
    p.add_argument("--lam", type=float, default=0.999)
    p.add_argument("--cpu-sample-iters", type=int, default=1)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--scaffold", default="on", choices=["on", "off"])
    p.add_argument("--no-topology", action="store_true")
    p.add_argument("--topo-newton-iters", type=int, default=400,
                   help="Newton iterations (to convergence) after the outer loop's last operation")
    p.add_argument("--outer-steps", type=int, default=5,
                   help="topology operations of the outer loop before the topology step is timed")
    p.add_argument("--outer-newton-cap", type=int, default=4000,
                   help="Newton iterations the outer loop may spend reaching that state")
    p.add_argument("--top-frac", type=float, default=0.1, help="fraction of local problems solved exactly (learned)")
    p.add_argument("--train-epochs", type=int, default=30, help="MLP training epochs over the exhaustive pairs")
    p.add_argument("--topo-bijective", default="on", choices=["on", "off"],
                   help="outer loop and timed topology step with bijectivity on (the reference's default) or off")
    return p.parse_args()


def dist_setup(n):
    rank, world = int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, world):
    if world <= 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def workload(name):
    from optcuts_gb300 import init as I
    from optcuts_gb300 import meshes as M
    V, F = M.CONFIGS[name]()
    return I.init_uv(V, F)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(device), "--query-gpu=" + self.FIELDS,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        time.sleep(0.25)
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.p.kill()
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return None
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower() == "active"})
        loaded = [s for s in sm if mx and s > 0.5 * max(mx)] or sm
        return {"sm_mhz": statistics.median(loaded) if loaded else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def fp64_peak_tflops():
    """FP64 throughput of this GPU measured in place: cuBLAS DGEMM 4096^3
    (torch.matmul), best of 5; the nominal figure where that fails."""
    try:
        import torch
        a = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
        b = torch.randn(4096, 4096, dtype=torch.float64, device="cuda")
        best = None
        for _ in range(6):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        return 2.0 * 4096 ** 3 / (best / 1000.0) / 1e12, "measured (cuBLAS DGEMM 4096^3, best of 6, this run)"
    except Exception:
        return FP64_PEAK_TFLOPS, "nominal"


def avg_edge_len(st):
    V, F = st.V_rest, st.F
    return float(np.mean(np.linalg.norm(V[F[:, [1, 2, 0]]] - V[F], axis=2)))


# The reference's own run of the default workload from its Tutte start with
# the scaffold on (oracle/_ref, tests/golden/make_golden.py): its air mesh
# (Triangle) of the start state and its first Newton iteration's energies.
START_FIXTURE = {"ellipsoid_199k": os.path.join(ROOT, "tests", "golden", "ellipsoid_199k_start.npz")}
# Measured on one host (x86-64, 8 threads, the 199k ellipsoid): the CPU
# restatement takes 10.5 s per Newton iteration, the reference's own code
# 7.0-8.5 s (15% more fill than Eigen's AMD ordering).
PORT_VS_REFERENCE = "the oracle port runs 1.2-1.5x slower than the reference's own code on the same host"


def reference_start(name, UV):
    """The reference's air mesh of the start state and its energies after
    iteration 0 and 1 (total and SD-only), after checking that UV is the
    start state the fixture was made from."""
    path = START_FIXTURE.get(name)
    if path is None or not os.path.exists(path):
        return None
    with np.load(path) as z:
        g = {k: z[k] for k in z.files}
    chk = np.concatenate([UV.sum(0), UV[0], UV[-1]])
    if len(UV) != int(g["uv0_check"][6]) or np.abs(chk - g["uv0_check"][:6]).max() > 1e-8 * len(UV):
        raise RuntimeError("start state differs from the reference's (%s)" % path)
    n = g["scaf_off"][0]
    return {"airV": g["scaf_V"][:n[0]], "airF": g["scaf_F"][:n[1]], "bnd": g["scaf_bnd"][:n[2]],
            "E_tot": g["trace_Etot"][:2], "E": g["trace_E"][:2]}


def oracle_workload(name):
    """The start state for the CPU arm, from the oracle's own restatement of
    the reference's initialisation (closed genus-0 meshes)."""
    from optcuts_gb300 import meshes as M
    from oracle import init as OI
    V, F = M.CONFIGS[name]()
    s = OI.init_genus0(V, F)

    class St:
        pass
    st = St()
    st.V_rest, st.UV, st.F, st.fixedVert, st.cohE = s["V_rest"], s["UV"], s["F"], s["fixedVert"], s["cohE"]
    return st


def cpu_port_run(st, lam, iters, threads, air, avg_len):
    """iters Newton iterations of the oracle port from st.UV; air = (airV,
    airF, bnd) runs the scaffolding branches with that air mesh moved along
    each step.  Returns (per-iteration seconds, energies incl. the start)."""
    import oracle as O
    kw = dict(scaffold=air, avg_edge_len=avg_len) if air is not None else {}
    _, tr, _ = O.newton(st.V_rest, st.F, st.fixedVert, st.UV, 1.0 - lam, iters, threads=threads, **kw)
    return tr["seconds"], tr["E"]


def run_reference(args, rank, world):
    """The reference arm: the CPU restatement of the reference path
    (oracle/port; the reference's own sources do not exist on the GPU host)
    on every host core, from the oracle's own initial state with the
    reference's own air mesh of that state, over the same iterations the GPU
    arm runs: warm-up + 1 ... warm-up + steps are timed.  Nothing of the
    product (its library, initialisation or air-mesh generator) is used."""
    if rank != 0:
        return
    scaf = args.scaffold == "on"
    try:
        st = oracle_workload(args.workload)
    except Exception as e:   # genus >= 1 workloads: the oracle restates the genus-0 start only
        print(json.dumps({"impl": "reference", "unavailable": "no oracle initial state for %s (%s)" % (
            args.workload, e)}), flush=True)
        return
    ref = reference_start(args.workload, st.UV)
    if scaf and ref is None:
        print(json.dumps({"impl": "reference", "unavailable": "no reference air mesh for %s" % args.workload}),
              flush=True)
        return
    threads = os.cpu_count() or 1
    air = (ref["airV"], ref["airF"], ref["bnd"]) if scaf else None
    secs, E = cpu_port_run(st, args.lam, args.warmup + args.steps, threads, air, avg_edge_len(st))
    timed = secs[args.warmup:]
    v = len(timed) / float(np.sum(timed))
    sample = ("Newton iterations %d..%d of %s from the Tutte start (iterations 1..%d untimed)%s; %s" % (
        args.warmup + 1, args.warmup + args.steps, args.workload, args.warmup,
        ", the reference's air mesh of the start moved with each step" if scaf else "", PORT_VS_REFERENCE))
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000.0 / v, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "triangles": len(st.F), "lambda": args.lam, "scaffold": scaf},
        "same_config": True,
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "energy_after": {"iterations": args.warmup + args.steps, "E": float(E[-1])},
        "first_step": {"E_port": float(E[1]), "E_reference": float(ref["E_tot"][1]) if ref else None,
                       "rel_diff": abs(E[1] - ref["E_tot"][1]) / ref["E_tot"][1] if ref else None},
    }), flush=True)


def spearman(a, b):
    """Rank correlation of two equally long arrays (average ranks for ties)."""
    from scipy.stats import spearmanr
    if len(a) < 3:
        return None
    r = spearmanr(a, b).correlation
    return None if r != r else float(r)


def ranking(ex, le, top_frac):
    """How the learned pass ranked the exhaustive pass's local problems:
    recall of the exact top-k problems among those it solved exactly (k =
    the number it solved), whether each op's best problem was among them,
    and the rank correlation of predicted and exact E_w decreases."""
    pe, pl = ex["problems"], le["problems"]
    exact, pred = pe["EwDec"], pl["EwDec_pred"]
    sel = ~np.isnan(pl["EwDec"])
    n, k = len(exact), int(sel.sum())
    ok = np.isfinite(exact) & (exact > -1e300)
    out = {"problems": n, "solved_exactly": k, "spearman": spearman(pred[ok], exact[ok])}
    if n and k:
        top = np.argsort(-np.where(ok, exact, -np.inf), kind="stable")[:k]
        out["recall_at_k"] = float(sel[top].mean())
        out["best_selected"] = bool(sel[int(np.argmax(np.where(ok, exact, -np.inf)))])
    return out


def topology_section(args, oc, ctx, opt, mesh, st, rank):
    """The topology step on the state the outer loop reaches after
    args.outer_steps topology operations (the library's outer loop: dual
    updates, propagation; its first inner loop converges the Newton phase),
    with bijectivity on by default (the reference's default: scaffold on,
    every local solve with its air loop).  Timed: the exhaustive step, the
    learned proposal trained on the (features, target) pairs the outer
    loop's own exhaustive queries recorded on the way, and the
    bijectivity-off step on the same state (with its FP32-projection and
    autotuned variants and the CPU port beside it)."""
    bij = args.topo_bijective == "on"
    if not bij:
        opt.clearScaffold()            # bijectivity off: no air mesh
    mesh.setCohesiveEdges(st.cohE)
    outer = oc.OptCuts(opt, bijective=bij, recordFeatures=True, maxNewtonIters=args.outer_newton_cap)
    ctx.synchronize()
    t0 = time.perf_counter()
    passes, finished = 0, False
    while outer.state()["topology_steps"] < args.outer_steps and passes < 400 and not finished:
        finished = outer.run(1)
        passes += 1
    converged = False
    for _ in range(args.topo_newton_iters):   # the inner loop after the last operation
        if opt.solve(1) == 1:
            converged = True
            break
        if bij:
            opt.rebuildScaffold()          # Optimizer.cpp:251-257
    ctx.synchronize()
    outer_s = time.perf_counter() - t0
    so = outer.state()
    X, t = outer.features()
    lam_t = so["lambda"]

    def queries(**kw):
        # one topology step: boundary splits, merges and interior splits
        # solved together; the first query rebuilds the vertex adjacency as
        # it does after an applied operation
        mesh.dropAdjacency()
        return mesh.topologyStep(lam_t, **kw)

    def timed_step(**kw):
        ctx.synchronize()
        t1 = time.perf_counter()
        qs = queries(**kw)
        ctx.synchronize()
        return time.perf_counter() - t1, qs

    def summary(qs):
        qb, qm, qi = qs
        out = {"query_ms": qb["query_ms"], "gpu_solve_ms": qb["solve_ms"], "probe_ms": qb["probe_ms"],
               "exact_ms": qb["exact_ms"],
               "host_ms": {k: round(v, 3) for k, v in qb["host_ms"].items()},
               "host_build_ms": {name: q["build_ms"] for name, q in
                                 zip(("boundary_split", "merge", "interior_split"), qs)},
               "local_problems": sum(q["local_problems"] for q in qs),
               "exact_solves": sum(q["selected"] for q in qs),
               "local_iterations": sum(q["local_iters_total"] for q in qs),
               "max_local_iterations": max(q["max_local_iters"] for q in qs),
               "best": {"boundary_split": qb["EwDec_max"], "merge": qm["EwDec_max"],
                        "interior_split": qi["EwDec_max"]}}
        air = [q["air"] for q in qs]
        if any(a["problems"] for a in air):
            out["air_loops"] = {"problems": sum(a["problems"] for a in air),
                                "abandoned": sum(a["rejected"] for a in air),
                                "steiner_max": max(a["steiner_max"] for a in air),
                                "refinement_capped": sum(a["capped"] for a in air)}
        return out

    queries(bijective=bij)   # warm-up
    t_gpu, qs = timed_step(features=True, bijective=bij)
    t_fp32, qs32 = timed_step(fp32=True, bijective=bij)
    qb, qm, qi = qs
    form = "on (scaffold on, every local solve with its air loop)" if bij else "off (no air meshes)"
    topo = {"metric": "topology-step s (exhaustive candidate evaluation: boundary split, merge and interior split "
                      "queries of one state, solved together)", "value": t_gpu, "unit": "s",
            "higher_is_better": False, "bijectivity": form,
            "state": {"what": "after %d topology operations of the outer loop (bijectivity %s), inner loop converged" %
                              (int(so["topology_steps"]), "on" if bij else "off"),
                      "newton_iterations": opt.getIterNum(), "topology_steps": int(so["topology_steps"]),
                      "converged": converged, "finished": bool(finished), "lambda": lam_t, "E_SD": so["E_SD"],
                      "E_se": so["E_se"], "vertices": int(so["vertices"]), "outer_loop_s": outer_s,
                      "outer_loop_ms": {k: so[k] for k in ("newton_ms", "query_ms", "apply_ms")}},
            "candidates": {"boundary_split": len(qb["candidates"]), "merge": len(qm["candidates"]),
                           "interior_split": len(qi["candidates"])},
            "local_capped": sum(q["local_capped"] for q in qs),
            **summary(qs), "fp32_hessian_option": {"value": t_fp32, "unit": "s", **summary(qs32)}}
    e_w = opt.getLastEnergyVal(excludeScaffold=True) + lam_t * so["E_se"]

    def after(qs_):
        return e_w - max(0.0, *(q["EwDec_max"] for q in qs_))
    if len(X):
        mlp = oc.MLP(32, 128, seed=3, ctx=ctx)
        ctx.synchronize()
        t1 = time.perf_counter()
        loss = mlp.train(X, t, epochs=args.train_epochs, batch=512, lr=2e-3, seed=3)
        ctx.synchronize()
        train_s = time.perf_counter() - t1
        queries(mlp=mlp, topFrac=args.top_frac, bijective=bij)   # warm-up
        t_l, ql = timed_step(mlp=mlp, topFrac=args.top_frac, bijective=bij)
        t_l32, ql32 = timed_step(mlp=mlp, topFrac=args.top_frac, fp32=True, bijective=bij)
        ew_ex, ew_l, ew_ex32, ew_l32 = after(qs), after(ql), after(qs32), after(ql32)
        # the exhaustive pass's own pairs at this state: held out from training
        Xh = np.concatenate([q["features"] for q in qs])
        th = np.concatenate([q["target"] for q in qs])
        ph = mlp.predict(Xh) if len(Xh) else np.zeros(0)
        r2 = 1.0 - float(np.mean((ph - th) ** 2)) / float(np.var(th)) if len(th) > 1 and np.var(th) > 0 else None
        topo["learned"] = {
            "metric": "topology-step s (learned proposal, top %g of local problems solved exactly)" % args.top_frac,
            "value": t_l, "unit": "s", "higher_is_better": False, **summary(ql),
            "speedup_vs_exhaustive": t_gpu / t_l,
            "E_w_before": e_w, "E_w_after": ew_l, "E_w_after_exhaustive": ew_ex,
            "E_w_rel_diff": abs(ew_l - ew_ex) / abs(ew_ex),
            "ranking": {op: ranking(a, b, args.top_frac) for op, a, b in
                        zip(("boundary_split", "merge", "interior_split"), qs, ql)},
            "fp32_hessian_option": {"value": t_l32, "unit": "s", **summary(ql32), "E_w_after": ew_l32,
                                    "E_w_after_exhaustive": ew_ex32,
                                    "E_w_rel_diff": abs(ew_l32 - ew_ex32) / abs(ew_ex32)},
            "mlp": {"layers": [32, 128, 128, 1], "weights": "bf16 (fp32 master, Adam)", "accumulate": "fp32",
                    "pairs": int(len(X)), "pairs_from": "the outer loop's exhaustive queries before this state",
                    "epochs": args.train_epochs, "batch": 512, "seed": 3, "train_s": train_s, "final_mse": loss,
                    "target_var": float(np.var(t)), "train_r2": 1.0 - loss / float(np.var(t)) if np.var(t) else None,
                    "heldout_r2": r2}}
    if bij:
        # the same state's step without air loops, for comparison
        queries()
        t_off, qs_off = timed_step()
        t_off32, qs_off32 = timed_step(fp32=True)
        queries(autotune=True)   # the schedule autotuner measures its candidates on this state
        t_tuned, qs_t = timed_step(autotune=True)
        topo["bijectivity_off"] = {"metric": "topology-step s (exhaustive, bijectivity off, same state)",
                                   "value": t_off, "unit": "s", **summary(qs_off),
                                   "fp32_hessian_option": {"value": t_off32, "unit": "s", **summary(qs_off32)},
                                   "autotuned_schedules": {"value": t_tuned, "unit": "s", **summary(qs_t),
                                                           "table": oc.topology_schedules()}}
    else:
        queries(autotune=True)
        t_tuned, qs_t = timed_step(autotune=True)
        topo["autotuned_schedules"] = {"value": t_tuned, "unit": "s", **summary(qs_t),
                                       "table": oc.topology_schedules()}
    if rank == 0 and not args.no_cpu_baseline:
        import oracle as O
        threads = os.cpu_count() or 1
        uv = mesh.V
        secs = 0.0
        for op in (0, 2, 1):
            _, s_ = O.topology_query(mesh.V_rest, uv, mesh.F, mesh.cohE, op, lam_t, threads=threads)
            secs += s_
        topo["cpu_baseline"] = {"value": secs, "unit": "s", "cores": threads, "kind": "port",
                                "sample": "the same three queries on the same state, bijectivity off (the port "
                                          "has no air loops)"}
    # applying the chosen operation (Optimizer::createFracture: mesh edit,
    # device mesh, Newton pattern and analysis, scaffold, energy), timed once
    cands = [(q["EwDec_max"], op, q) for op, q in ((oc.OP_BOUNDARY_SPLIT, qb), (oc.OP_MERGE, qm)) if q["best"] >= 0]
    if cands:
        ew, op, q = max(cands, key=lambda x: x[0])
        c = q["candidates"][q["best"]]
        ctx.synchronize()
        t1 = time.perf_counter()
        opt.createFracture(op, c["path"], c["newVertPos"])
        ctx.synchronize()
        topo["apply"] = {"value": time.perf_counter() - t1, "unit": "s",
                         "op": {0: "boundary_split", 1: "interior_split", 2: "merge"}[op], "EwDec": ew,
                         "phases_ms": {k: round(v, 2) for k, v in opt.applyTiming().items()},
                         "analysis": {k: (round(v, 2) if isinstance(v, float) and k.endswith("_ms") else v)
                                      for k, v in opt.analysisInfo().items()},
                         "what": "Optimizer::createFracture: mesh edit, device mesh, Newton pattern and analysis, "
                                 "scaffold, energy"}
    return topo


def outer_config0(oc, ctx, bijective=True):
    """The whole OptCuts run (outer loop, b_d = 4.1) on the 5,120-triangle
    icosphere from its Tutte start, with bijectivity on (the reference's
    default, its command line's bijectiveParam 1: scaffold from the first
    topology step on, bijective local solves) or off, against the
    reference's own run of the same input (tests/golden/icosphere_5k_*outer.npz,
    made by the reference's sources on one x86-64 host thread)."""
    name = "icosphere_5k_bij_outer" if bijective else "icosphere_5k_outer"
    path = os.path.join(ROOT, "tests", "golden", name + ".npz")
    if not os.path.exists(path):
        return None
    with np.load(path) as z:
        g = {k: z[k] for k in z.files}
    m = oc.TriMesh(g["V_rest"], g["UV0"], g["F"], g["fixedVert"], ctx=ctx)
    m.setCohesiveEdges(g["cohE"])
    opt = oc.Optimizer(m, [1.0 - g["scalars"][4]])
    ctx.synchronize()
    t0 = time.perf_counter()
    opt.precompute()
    o = oc.OptCuts(opt, upperBound=4.1, bijective=bijective)
    finished = o.run()
    ctx.synchronize()
    secs = time.perf_counter() - t0
    st = o.state()
    ref = g["outer_final"]
    form = "bijectivity on" if bijective else "bijectivity off"
    out = {"metric": "time to converge s (whole OptCuts run, %s, b_d 4.1)" % form, "value": secs, "unit": "s",
           "higher_is_better": False, "workload": "icosphere_5k (5,120 triangles)", "finished": bool(finished),
           "newton_iterations": int(st["newton_iterations"]), "topology_steps": int(st["topology_steps"]),
           "E_SD": st["E_SD"], "E_se": st["E_se"], "lambda": st["lambda"],
           "reference": {"seconds": float(ref[6]), "newton_iterations": int(ref[3]), "topology_steps": int(ref[4]),
                         "E_SD": float(ref[0]), "E_se": float(ref[1]), "lambda": float(ref[2]),
                         "host": "x86-64, one thread (recorded with the golden run)"},
           "rel_diff": {"E_SD": abs(st["E_SD"] - ref[0]) / ref[0], "E_se": abs(st["E_se"] - ref[1]) / ref[1],
                        "lambda": abs(st["lambda"] - ref[2]) / ref[2]},
           "phases_ms": {k: st[k] for k in ("newton_ms", "query_ms", "apply_ms")}}
    o.close()
    opt.close()
    m.close()
    return out


def run_ours(args, rank, world):
    import optcuts_gb300 as oc
    device = int(os.environ.get("LOCAL_RANK", "0"))
    import torch
    torch.cuda.set_device(device)
    st = workload(args.workload)
    nF, nV = len(st.F), len(st.UV)
    scaf = args.scaffold == "on"
    # one stream for the library, the L2 flush and the timing events
    stream = torch.cuda.Stream(device)
    torch.cuda.set_stream(stream)
    ctx = oc.Context(device, stream=stream.cuda_stream)
    mesh = oc.TriMesh(st.V_rest, st.UV, st.F, st.fixedVert, ctx=ctx)
    opt = oc.Optimizer(mesh, [1.0 - args.lam], timing=1)
    if scaf:
        opt.rebuildScaffold()
    opt.precompute()

    def step():
        r = opt.solve(1)
        if scaf:
            opt.rebuildScaffold()   # Optimizer.cpp:251-257
        return r
    flush = torch.empty(64 * 1024 * 1024, dtype=torch.float32, device="cuda")   # 256 MB > 129 MB L2

    def flush_l2():
        ctx.synchronize()
        flush.zero_()
        torch.cuda.synchronize()

    # parity at this workload: one GPU Newton iteration from the start state
    # with the reference's own air mesh of that state, against the
    # reference's first iteration (and, below, the CPU oracle's)
    ref = reference_start(args.workload, st.UV) if scaf else None
    first = None
    if ref is not None:
        m1 = oc.TriMesh(st.V_rest, st.UV, st.F, st.fixedVert, ctx=ctx)
        o1 = oc.Optimizer(m1, [1.0 - args.lam])
        o1.setScaffold(oc.Scaffold(ref["airV"], ref["airF"], ref["bnd"]))
        o1.precompute()
        o1.solve(1)
        first = {"E_gpu": o1.getLastEnergyVal(), "E_reference": float(ref["E_tot"][1])}
        first["rel_diff_gpu"] = abs(first["E_gpu"] - first["E_reference"]) / first["E_reference"]
        o1.close()
        m1.close()

    for _ in range(args.warmup):
        step()
    opt.phase_ms()
    launches0 = opt.launch_count()
    flush_l2()
    barrier(world)
    torch.cuda.synchronize()
    sampler = ClockSampler(device) if rank == 0 else None
    step_ms, phases = [], []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        step_ms.append(e0.elapsed_time(e1))
        phases.append(opt.phase_ms())
        flush_l2()
    torch.cuda.synchronize()
    barrier(world)
    clocks = sampler.stop() if sampler else None
    launches = opt.launch_count() - launches0
    # the symbolic analysis the timed factorizations used (read before the
    # e2e steps and the topology step, which may analyse again)
    sym = opt.solver_stats()
    energy_after = {"iterations": args.warmup + args.steps, "E": opt.getLastEnergyVal()}
    total_s = sum(step_ms) / 1000.0
    total_s_max = allreduce_max(total_s, world)
    value = world * args.steps / total_s_max

    # end to end through the C ABI with host buffers: UV in, solve(1), UV out
    e2e = None
    if not args.no_e2e:
        uv_host = mesh.V
        e2e_steps = max(3, args.steps)
        barrier(world)
        t0 = time.perf_counter()
        for _ in range(e2e_steps):
            mesh.V = uv_host
            step()
            uv_host = mesh.V
        t1 = time.perf_counter()
        e2e_max = allreduce_max(t1 - t0, world)
        e2e = {"value": world * e2e_steps / e2e_max, "unit": UNIT, "h2d_bytes_per_step": 16 * nV,
               "d2h_bytes_per_step": 16 * nV}

    # one topology step of the outer loop at the converged state: the
    # candidate evaluation of TriMesh::splitOrMerge (boundary splits, merges)
    # and of the interior-split query, every local solve on the GPU
    topo = None
    if not args.no_topology:
        topo = topology_section(args, oc, ctx, opt, mesh, st, rank)

    if rank != 0:
        return
    outer0 = None if args.no_topology else outer_config0(oc, ctx, bijective=True)
    outer0_off = None if args.no_topology else outer_config0(oc, ctx, bijective=False)
    # dominant phase: the multifrontal factorisation, FP64-FMA bound; the
    # algorithmic flops are the dense partial-Cholesky counts of its fronts
    ph_mean = {k: statistics.mean(p[k] for p in phases) for k in phases[0]}
    fact_ms = ph_mean["factorize"]
    fp64_peak, fp64_kind = fp64_peak_tflops()
    achieved = sym["flops"] / (fact_ms / 1000.0) / 1e12
    roofline = {"kernel": "chol_factorize (k_ldl_update, k_ldl_panel, k_ldl_diag, k_extend)", "bound": "fp64",
                "achieved": achieved, "peak": fp64_peak, "unit": "TFLOP/s", "frac": achieved / fp64_peak,
                "traffic": None, "peak_kind": fp64_kind, "frac_of_nominal": achieved / FP64_PEAK_TFLOPS,
                "flops_per_factorization": sym["flops"], "factorize_ms_per_step": fact_ms,
                "phase_ms_per_step": ph_mean, "fronts": sym["fronts"], "tree_levels": sym["levels"]}
    # the substitutions (forward + backward through every front): the factor
    # (FP64 entries of L) streamed once per direction
    hbm, hbm_kind = measured_peak()
    solve_ms = ph_mean["solve"]
    solve_bytes = 2.0 * 8.0 * sym["factor_entries"]
    solve_gbs = solve_bytes / (solve_ms / 1000.0) / 1e9
    roofline_solve = {"kernel": "chol_solve (k_fwd, k_fwd_rect, k_bwd_rect, k_bwd)", "bound": "hbm",
                      "achieved": solve_gbs, "peak": hbm, "unit": "GB/s", "frac": solve_gbs / hbm,
                      "peak_kind": hbm_kind, "traffic": None, "bytes_per_solve": solve_bytes,
                      "factor_entries": sym["factor_entries"], "solve_ms_per_step": solve_ms}
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        air = (ref["airV"], ref["airF"], ref["bnd"]) if ref is not None else None
        secs, E = cpu_port_run(st, args.lam, args.cpu_sample_iters, threads, air, avg_edge_len(st))
        cpu = {"value": len(secs) / float(np.sum(secs)), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "%d Newton iteration(s) of %s from the Tutte start%s" % (
                   len(secs), args.workload, ", the reference's air mesh of the start" if air else "")}
        if first is not None and len(E) > 1:
            first["E_port"] = float(E[1])
            first["rel_diff_port"] = abs(E[1] - first["E_reference"]) / first["E_reference"]
    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(step_ms), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": args.workload, "triangles": nF, "vertices": nV, "lambda": args.lam,
                   "scaffold": scaf, "system_vertices": opt.systemSize(),
                   "parallelism": "replicas" if world > 1 else "single",
                   "l2": "flushed between timed steps (256 MB write)", "solver": "multifrontal Cholesky (FP64)",
                   "precision": "fp64 throughout (energy, gradient, Hessian eigen-clamp, LDL^T)"},
        "roofline": roofline, "roofline_solve": roofline_solve, "cpu_baseline": cpu, "e2e": e2e,
        "gpu_launches": launches, "clocks": clocks, "energy_after": energy_after, "first_step": first,
        "topology": topo, "outer_loop": outer0, "outer_loop_bijectivity_off": outer0_off,
    }
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    rank, world = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
    else:
        run_ours(args, rank, world)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
