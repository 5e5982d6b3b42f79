import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def load_golden(name):
    with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


GOLDEN_CASES = ["triangle", "plane", "cube", "icosphere_320", "ellipsoid_2k", "torus_768", "icosphere_5k",
                "sheet_3k", "icosphere_320_scaf", "components"]
# closed genus-0 inputs: the reference runs its first Newton phase without the scaffold
SCAFFOLD_OFF = ["cube", "icosphere_320", "ellipsoid_2k", "icosphere_5k"]


@pytest.fixture(scope="session")
def golden():
    cache = {}

    def get(name):
        if name not in cache:
            cache[name] = load_golden(name)
        return cache[name]
    return get


TOPO_CASES = ["icosphere_320_topo", "sheet_3k_topo", "torus_768_topo", "ellipsoid_2k_topo"]


def golden_candidates(g, op):
    """The reference's candidate list of one topology query: list of dicts
    with path, newVertPos (rows x 2) and energyChanges."""
    L = g["topo_%s_pathLen" % op]
    P = g["topo_%s_path" % op]
    R = g["topo_%s_posRows" % op]
    X = g["topo_%s_pos" % op].reshape(-1, 2)
    E = g["topo_%s_energyChanges" % op].reshape(-1, 2)
    out, pp, px = [], 0, 0
    for c in range(len(L)):
        out.append({"path": P[pp:pp + L[c]].tolist(), "newVertPos": X[px:px + R[c]], "energyChanges": tuple(E[c])})
        pp += L[c]
        px += R[c]
    return out


# cases whose golden holds the air mesh of every iteration
SCAFFOLD_DUMPS = ["triangle", "plane", "torus_768", "sheet_3k", "icosphere_320_scaf", "components"]


def golden_scaffolds(g):
    """Per-iteration air meshes of a golden: list of (airV, airF, bnd, fixed)."""
    out = []
    pv = pf = pb = px = 0
    for nv, nf, nb, nx in g["scaf_off"]:
        out.append((g["scaf_V"][pv:pv + nv], g["scaf_F"][pf:pf + nf], g["scaf_bnd"][pb:pb + nb],
                    g["scaf_fixed"][px:px + nx]))
        pv += nv
        pf += nf
        pb += nb
        px += nx
    return out
