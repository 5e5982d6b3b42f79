"""Builds liboc_gpu.so (the C-ABI library) in-tree with nvcc for sm_103a.

    python -m optcuts_gb300.build [--force] [--verbose]

Translation units are compiled in parallel; oc_fp64.cu is compiled with
-fmad=false so its FP64 arithmetic rounds exactly as the reference's scalar
host code does (oc_local.cu, the local topology solves, contracts FMAs).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "liboc_gpu.so")
NVCC = os.environ.get("NVCC", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# host code: no FMA contraction (aarch64 GCC contracts by default), so the
# host-side rest constants round exactly as the reference's do on x86-64
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden",
          "-Xcompiler", "-ffp-contract=off",
          "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
UNITS = {
    "oc_fp64.cu": ["-fmad=false"],
    "oc_kernels.cu": [],
    "oc_chol.cu": [],
    "oc_api.cu": ["-Xcompiler", "-fvisibility=default"],
    "oc_airmesh.cpp": [],
    "oc_topo.cpp": [],
    "oc_mlp.cu": [],
    "oc_tc.cu": [],
    "oc_local.cu": [],
    "oc_local_bij.cu": [],
    "oc_outer.cpp": ["-Xcompiler", "-fvisibility=default"],
    "oc_output.cpp": ["-Xcompiler", "-fvisibility=default"],
}
HEADERS = ["oc_internal.h", "oc_chol.h", "oc_airmesh.h", "oc_topo.h", "oc_mlp.h", "oc_tc.h", "oc_elem.cuh",
           "oc_loopmesh.cuh"]


def _newest_input():
    paths = [os.path.join(CSRC, u) for u in UNITS] + [os.path.join(CSRC, h) for h in HEADERS]
    paths.append(os.path.join(ROOT, "include", "optcuts_gpu.h"))
    paths.append(os.path.abspath(__file__))
    return max(os.path.getmtime(p) for p in paths)


def _compile(unit, extra, verbose):
    obj = os.path.join(OUT_DIR, os.path.splitext(unit)[0] + ".o")
    cmd = [NVCC, *ARCH, *COMMON, *extra, "-c", os.path.join(CSRC, unit), "-o", obj]
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s%s" % (unit, r.stdout, r.stderr))
    if verbose and r.stderr:
        print(r.stderr, flush=True)
    return obj


def build(force=False, verbose=False):
    os.makedirs(OUT_DIR, exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _newest_input():
        return LIB
    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(lambda kv: _compile(kv[0], kv[1], verbose), UNITS.items()))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [NVCC, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="--verbose" in sys.argv))
