"""Generates the golden vectors in tests/golden/ from the reference itself.

Runs oracle/_ref/ref_driver -- the reference's own sources compiled by
oracle/ref/Makefile -- on seeded synthetic meshes (optcuts_gb300.meshes) and
packs its dumps into one compressed .npz per case:

    V_rest, UV0, F, fixedVert, bnd     initial state after the reference's
    cohE                               own cut + Tutte initialisation
    rest, scalars                      TriMesh::computeFeatures constants
    E_elem0, grad0                     per-triangle energy, gradient at UV0
    H0_blocks, H0_tris                 per-triangle PSD-projected Hessians
                                       (rebuilt from the reference's triplets)
    dir0                               SimplicialLDLT Newton direction at UV0
    trace_E, trace_gsq, trace_alpha    per-iteration Optimizer::solve(1) trace
    UV_iters (small cases)             UV after every iteration
    trace_Etot                         energy including the scaffold term
    topo_*                             topology cases: the converged state,
                                       split filter and every candidate of
                                       querySplit (boundary, interior) and
                                       queryMerge (paths, newVertPos,
                                       energyChanges)
    scaf_V, scaf_F, scaf_bnd,          scaffold cases: the air mesh each
    scaf_fixed, scaf_off               iteration used (concatenated; scaf_off
                                       rows = nAirV, nAirF, nBnd, nFixed)
    gradw0                             augmented gradient of iteration 0
    topo_airV, topo_airF, topo_airBnd  bijective topology cases: the
                                       scaffold's air mesh of the state

and air_loops.npz: local air loops Triangle meshed during bijective topology
queries (recorded by oracle/_ref/ref_driver_trilog) with Triangle's output.

Usage (needs the reference source tree; not part of the test run):
    make -C oracle/ref all trilog && python tests/golden/make_golden.py [case ...]
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from optcuts_gb300 import meshes  # noqa: E402

DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")

# case -> (mesh generator key, lambda, Newton iterations, max Hessian triangles, dump UV per iteration
#          (True, or the number of leading iterations kept), extra driver flags)
CASES = {
    "triangle": ("triangle", 0.999, 20, None, True, ["scafdump"]),
    "plane": ("plane", 0.999, 20, None, True, ["scafdump"]),
    "cube": ("cube", 0.999, 40, None, True, []),
    "icosphere_320": ("icosphere_320", 0.999, 40, None, True, []),
    "ellipsoid_2k": ("ellipsoid_2k", 0.999, 300, None, False, []),
    "torus_768": ("torus_768", 0.999, 30, None, False, ["scafdump"]),
    # UV of the first 21 iterations: the start points of the one-step parity
    # test (one Newton step from the reference's own iterate k)
    "icosphere_5k": ("icosphere_5k", 0.999, 120, 512, 21, []),
    # scaffold on: an open bumpy sheet (disk, 156 boundary vertices) and a
    # closed sphere after its one-point cut with the scaffold forced on
    "sheet_3k": ("sheet_3k", 0.999, 40, 256, True, ["scafdump"]),
    "icosphere_320_scaf": ("icosphere_320", 0.999, 40, None, True, ["scaf", "scafdump"]),
    # topology queries of one outer iteration after the Newton phase
    # converged, bijectivity off (the reference's bijectivity argument 0)
    "icosphere_320_topo": ("icosphere_320", 0.999, 60, 16, False, ["nobij", "topo"]),
    "sheet_3k_topo": ("sheet_3k", 0.999, 60, 16, False, ["nobij", "topo"]),
    "torus_768_topo": ("torus_768", 0.999, 60, 16, False, ["nobij", "topo"]),
    "ellipsoid_2k_topo": ("ellipsoid_2k", 0.999, 300, 16, False, ["nobij", "topo"]),
    # the same with bijectivity on: the scaffold's air mesh of that state is
    # kept (the local air loops come from it); the sphere after its
    # one-point cut with the scaffold forced on
    "icosphere_320_bij_topo": ("icosphere_320", 0.999, 60, 16, False, ["scaf", "topo"]),
    "sheet_3k_bij_topo": ("sheet_3k", 0.999, 60, 16, False, ["topo"]),
    "torus_768_bij_topo": ("torus_768", 0.999, 60, 16, False, ["topo"]),
    # three components (sphere, torus, sheet): each cut by its own Euler
    # characteristic, their UV disks on a grid; the scaffold holds them apart
    "components": ("components", 0.999, 30, 16, False, ["scafdump"]),
    # slim cases (large meshes: only the traces, scalars and air meshes kept)
    # the 199k-triangle ellipsoid benchmark workload from its Tutte start with
    # the scaffold on: the reference's air mesh of that start and its first
    # Newton iteration
    "ellipsoid_199k_start": ("ellipsoid_199k", 0.999, 1, 16, False, ["scaf", "scafdump", "slim"]),
    # the genus-1 torus workload (cut_to_disk + Tutte, scaffold on) run to
    # convergence
    "torus_41k_conv": ("torus_41k", 0.999, 3000, 16, False, ["slim"]),
    # whole OptCuts runs (outer loop: dual updates, topology steps,
    # propagation, rollback) to b_d = 4.1, bijectivity off
    "icosphere_320_outer": ("icosphere_320", 0.999, 5000, 16, False, ["outer", "nobij"]),
    "icosphere_1k_outer": ("icosphere_1k", 0.999, 5000, 16, False, ["outer", "nobij"]),
    "icosphere_5k_outer": ("icosphere_5k", 0.999, 5000, 16, False, ["outer", "nobij"]),
    # the same with bijectivity on (the reference's default: the scaffold
    # starts after the first inner loop, bijective topology queries)
    "icosphere_320_bij_outer": ("icosphere_320", 0.999, 5000, 16, False, ["outer"]),
    "icosphere_1k_bij_outer": ("icosphere_1k", 0.999, 5000, 16, False, ["outer"]),
    "icosphere_5k_bij_outer": ("icosphere_5k", 0.999, 5000, 16, False, ["outer"]),
}
OUTER_KEYS = ("outer_events", "outer_final", "outer_V", "outer_F", "outer_Vrest", "outer_cohE")
SLIM_KEYS = ("scalars", "trace_E", "trace_Etot", "trace_gsq", "trace_alpha", "trace_status", "scaf_V", "scaf_F",
             "scaf_bnd", "scaf_fixed", "scaf_off", "uv0_check")


def per_tri_blocks(F, fixed, Hv, ntri):
    """Per-triangle 6x6 blocks from the reference's triplet stream
    (IglUtils::addBlockToMatrix appends free x free entries tri by tri)."""
    fixed = set(int(v) for v in fixed)
    out = np.zeros((ntri, 6, 6))
    p = 0
    for t in range(ntri):
        idx = [a for a in range(3) if int(F[t, a]) not in fixed]
        for a in idx:
            for b in idx:
                for i in range(2):
                    for j in range(2):
                        out[t, 2 * a + i, 2 * b + j] = Hv[p]
                        p += 1
    return out


def run_case(name, key, lam, iters, hmax, states, flags):
    V, F = meshes.CONFIGS[key]()
    slim = "slim" in flags
    flags = [f for f in flags if f != "slim"]
    with tempfile.TemporaryDirectory() as td:
        obj = os.path.join(td, "mesh.obj")
        meshes.write_obj(obj, V, F)
        out = os.path.join(td, "out") + "/"
        os.makedirs(out)
        args = [DRIVER, obj, out, repr(lam), str(iters)] + ([] if slim or "outer" in flags else ["hess"]) + \
            (["states"] if states else []) + flags
        subprocess.run(args, check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                       env=dict(os.environ, OC_REF_THREADS="1"))
        ld = lambda n: np.load(out + n + ".npy")  # noqa: E731
        if slim:
            uv0 = ld("UV0")
            # identifies the start state: UV sums, its first and last rows, size
            pack = {"uv0_check": np.concatenate([uv0.sum(0), uv0[0], uv0[-1], [len(uv0), len(ld("F"))]])}
            for k in SLIM_KEYS:
                if k != "uv0_check" and os.path.exists(out + k + ".npy"):
                    pack[k] = ld(k)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **pack)
            pack.update(UV0=uv0, F=ld("F"))
            return pack
        if "outer" in flags:
            pack = dict(V_rest=ld("V_rest"), UV0=ld("UV0"), F=ld("F"), fixedVert=ld("fixedVert"), cohE=ld("cohE"),
                        scalars=ld("scalars"), mesh_V=V, mesh_F=F)
            for k in OUTER_KEYS:
                pack[k] = ld(k)
            np.savez_compressed(os.path.join(HERE, name + ".npz"), **pack)
            pack["trace_E"] = pack["outer_final"][:1]
            return pack
        Fm, fixed = ld("F"), ld("fixedVert")
        nt = len(Fm) if hmax is None else min(hmax, len(Fm))
        blocks = per_tri_blocks(Fm, fixed, ld("H0_V"), nt)
        pack = dict(V_rest=ld("V_rest"), UV0=ld("UV0"), F=Fm, fixedVert=fixed, bnd=ld("bnd"), cohE=ld("cohE"),
                    rest=ld("rest"), scalars=ld("scalars"), E_elem0=ld("E_elem0"), grad0=ld("grad0"),
                    H0_blocks=blocks, dir0=ld("dir0"), trace_E=ld("trace_E"), trace_gsq=ld("trace_gsq"),
                    trace_alpha=ld("trace_alpha"), trace_status=ld("trace_status"),
                    mesh_V=V, mesh_F=F)
        if states:
            pack["UV_iters"] = ld("UV_iters")
            if states is not True:
                pack["UV_iters"] = pack["UV_iters"][:states]
        pack["trace_Etot"] = ld("trace_Etot")
        if "topo" in flags:
            for k in ("V", "F", "Vrest", "cohE", "fixed", "divGrad", "best"):
                pack["topo_" + k] = ld("topo_" + k)
            for op in ("bSplit", "merge", "iSplit", "mergeB"):
                for k in ("pathLen", "path", "posRows", "pos", "energyChanges"):
                    if os.path.exists(out + "topo_%s_%s.npy" % (op, k)):
                        pack["topo_%s_%s" % (op, k)] = ld("topo_%s_%s" % (op, k))
            for k in ("opB_path", "opB_pos", "opI_path", "opI_pos", "opM_path", "opM_pos", "mergeB_best"):
                if os.path.exists(out + "topo_%s.npy" % k):
                    pack["topo_" + k] = ld("topo_" + k)
            for k in ("airV", "airF", "airBnd", "afterB_airV", "afterB_airF", "afterB_airBnd"):
                if os.path.exists(out + "topo_%s.npy" % k):
                    pack["topo_" + k] = ld("topo_" + k)
            for st in ("afterB", "afterI", "afterM"):
                for k in ("V", "F", "Vrest", "cohE"):
                    if os.path.exists(out + "topo_%s_%s.npy" % (st, k)):
                        pack["topo_%s_%s" % (st, k)] = ld("topo_%s_%s" % (st, k))
        if "scafdump" in flags and os.path.exists(out + "scaf_off.npy"):
            for k in ("scaf_V", "scaf_F", "scaf_bnd", "scaf_fixed", "scaf_off", "gradw0"):
                pack[k] = ld(k)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **pack)
    return pack


TRILOG = os.path.join(ROOT, "oracle", "_ref", "ref_driver_trilog")
# local air loops Triangle meshed during bijective topology queries
# (oracle/ref/trilog.c records them): mesh key, Newton iterations, flags
AIR_LOOP_RUNS = [("sheet_3k", 60, ["topo"]), ("torus_768", 60, ["topo"]), ("icosphere_320", 60, ["scaf", "topo"])]


def read_trilog(path):
    """Records of oracle/ref/trilog.c: (points in, segments, points out, triangles)."""
    b = open(path, "rb").read()
    o, recs = 0, []
    while o < len(b):
        nIn, nSeg, nOut, nTri = np.frombuffer(b, "<i4", 4, o)
        o += 16
        pin = np.frombuffer(b, "<f8", 2 * nIn, o).reshape(-1, 2); o += 16 * nIn
        seg = np.frombuffer(b, "<i4", 2 * nSeg, o).reshape(-1, 2); o += 8 * nSeg
        pout = np.frombuffer(b, "<f8", 2 * nOut, o).reshape(-1, 2); o += 16 * nOut
        tri = np.frombuffer(b, "<i4", 3 * nTri, o).reshape(-1, 3); o += 12 * nTri
        recs.append((pin, seg, pout, tri))
    return recs


def air_loops(per_size=40, steiner_max=400):
    """tests/golden/air_loops.npz: loops in ring order (the segments
    followed from point 0), Triangle's triangles in ring numbering and its
    Steiner points; every loop Triangle refined (up to steiner_max) and the
    first per_size loops of each size it did not."""
    keep, seen = [], {}
    for key, iters, flags in AIR_LOOP_RUNS:
        V, F = meshes.CONFIGS[key]()
        with tempfile.TemporaryDirectory() as td:
            obj = os.path.join(td, "mesh.obj")
            meshes.write_obj(obj, V, F)
            out = os.path.join(td, "out") + "/"
            os.makedirs(out)
            log = os.path.join(td, "tri.bin")
            subprocess.run([TRILOG, obj, out, "0.999", str(iters), "nodump"] + flags, check=True,
                           stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL,
                           env=dict(os.environ, OC_REF_THREADS="1", TRI_LOG=log))
            recs = read_trilog(log)
        for pin, seg, pout, tri in recs:
            L = len(pin)
            steiner = len(pout) - L
            if steiner > 0:
                if sum(1 for k in keep if k[3] > 0) >= steiner_max:
                    continue
            else:
                if seen.get(L, 0) >= per_size:
                    continue
                seen[L] = seen.get(L, 0) + 1
            nxt = {int(a): int(b) for a, b in seg}
            ring = [0]
            while len(ring) < L:
                ring.append(nxt[ring[-1]])
            inv = {old: new for new, old in enumerate(ring)}
            inv.update({L + i: L + i for i in range(steiner)})
            keep.append((pin[ring], np.array([[inv[int(v)] for v in t] for t in tri], np.int32), pout[L:], steiner))
    pack = dict(loop_off=np.cumsum([0] + [len(k[0]) for k in keep]), loop_pts=np.concatenate([k[0] for k in keep]),
                tri_off=np.cumsum([0] + [len(k[1]) for k in keep]), tri=np.concatenate([k[1] for k in keep]),
                steiner_off=np.cumsum([0] + [len(k[2]) for k in keep]),
                steiner=np.concatenate([k[2] for k in keep]).reshape(-1, 2))
    np.savez_compressed(os.path.join(HERE, "air_loops.npz"), **pack)
    print("air_loops: %d loops, %d refined" % (len(keep), sum(1 for k in keep if k[3] > 0)))


def main():
    if not os.path.exists(DRIVER):
        sys.exit("build the reference driver first: make -C oracle/ref")
    only = set(sys.argv[1:])
    if not only or "air_loops" in only:
        if not os.path.exists(TRILOG):
            sys.exit("build the recording driver first: make -C oracle/ref trilog")
        air_loops()
    for name, (key, lam, iters, hmax, states, flags) in CASES.items():
        if only and name not in only:
            continue
        p = run_case(name, key, lam, iters, hmax, states, flags)
        print("%-14s nV=%6d nF=%6d iters=%d E0=%.6g Elast=%.6g" % (
            name, len(p["UV0"]), len(p["F"]), len(p["trace_E"]) - 1, p["trace_E"][0], p["trace_E"][-1]))


if __name__ == "__main__":
    main()
