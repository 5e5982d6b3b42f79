"""The direct solver's factorization streams, host only: the independent
subtrees the analysis puts on streams of their own, and that every front's
children finish before it under the plan's streams and event waits."""
import numpy as np
import pytest

import optcuts_gb300 as oc
from optcuts_gb300 import meshes as M


@pytest.fixture(scope="module")
def big():
    # ~100k triangles: 4.9 GFLOP per factorization (BFS dissection), above
    # the 4 GFLOP from which the factorization splits into streams
    V, F = M.ellipsoid(224, 224, (1.0, 0.6, 0.4), 8, 6, 0.02, 2)
    return len(V), np.asarray(F, np.int32)


def test_groups_per_stream_limit(big):
    nV, F = big
    seen = []
    for s in (1, 2, 3, 4, 8):
        streams, groups, ordered = oc.chol_analyze_groups(nV, F, [0], maxStreams=s)
        assert ordered, s
        assert 1 <= streams <= s
        assert groups <= 2 * streams - 1
        seen.append(streams)
    assert seen[0] == 1 and seen[1] == 2 and seen[-1] >= 4, seen
    assert oc.chol_analyze_groups(nV, F, [0], maxStreams=1)[1] == 1


def test_groups_forest(big):
    """Two disjoint copies of the mesh (plus the fixed vertex, a tree of its
    own): the cut starts at the forest's roots."""
    nV, F = big
    F2 = np.concatenate([F, F + nV])
    streams, groups, ordered = oc.chol_analyze_groups(2 * nV, F2, [0], maxStreams=8)
    assert ordered and streams >= 4 and groups <= 2 * streams - 1, (streams, groups)
    streams, groups, ordered = oc.chol_analyze_groups(2 * nV, F2, [0], maxStreams=2)
    assert ordered and (streams, groups) == (2, 3)


def test_small_factorization_stays_on_one_stream():
    V, F = M.CONFIGS["sheet_3k"]()
    assert oc.chol_analyze_groups(len(V), np.asarray(F, np.int32), [0], maxStreams=8) == (1, 1, True)


def test_groups_invalid_limit(big):
    nV, F = big
    for s in (0, 9):
        with pytest.raises(oc.OCError):
            oc.chol_analyze_groups(nV, F, [0], maxStreams=s)
