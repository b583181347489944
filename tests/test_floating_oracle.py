"""The floating-polygon oracle equals MCUT's own detection.

oracle/cutpath_oracle.c (oracle_floating) restates kernel.cpp:4078-4200: a
circular cut path (every vertex on two cut-path edges, none on a polygon-soup
border edge) whose intersection vertices all pierce the same face is a
floating polygon in that face; MCUT stops the dispatch there, partitions the
face and runs the front end again. The reference's detection is observed
inside the unmodified mcDispatch (the seam copy's observer), together with
its cut path; the oracle, given that cut path, must find the same polygons:
per face, the same cycles of vertex coordinates (the reference starts each
cycle at a vertex and in a direction its unordered_map iteration picks, so
cycles are compared from their smallest vertex, in either direction).

Skipped where the seam harness is neither built nor buildable (set
MCUT_REF_ROOT).
"""
import numpy as np
import pytest

import golden_cases as G
import oracle
from test_seam_fragments import WITH_CCS, _user_meshes

pytestmark = pytest.mark.skipif(not oracle.seam_available(),
                                reason="seam harness not built and MCUT_REF_ROOT unset")

CASES = G.all_cases()


def canonical_cycle(pts):
    """A cycle of points from its lexicographically smallest point, in the
    direction whose second point is the smaller."""
    pts = [tuple(p) for p in np.asarray(pts, np.float64).tolist()]
    i = pts.index(min(pts))
    fwd = pts[i:] + pts[:i]
    bwd = [fwd[0]] + fwd[1:][::-1]
    return tuple(min(fwd, bwd))


def polygons_of(faces, off, xyz):
    out = []
    for p in range(len(faces)):
        out.append((int(faces[p]), canonical_cycle(xyz[off[p]:off[p + 1]])))
    return sorted(out)


@pytest.mark.parametrize("name", WITH_CCS)
def test_oracle_equals_mcut_floating_detection(name):
    c = CASES[name]
    src, cut, flags = _user_meshes(c)
    _, cps, fls = oracle.observe_floating(src, cut, flags=flags)
    if not fls:
        pytest.skip("the dispatch stopped before the detection")
    assert len(fls) <= len(cps)
    for cp, fl in zip(cps, fls):
        got = oracle.floating(cp["nv"], cp["reg"], cp["want"]["edges"], cp["x"], (cp["soup_off"], cp["soup_idx"]))
        xyz = np.asarray(cp["ivtx_xyz"]).reshape(-1, 3)
        gp = polygons_of(got["faces"], got["off"], xyz[np.asarray(got["vtx"], np.int64) - cp["nv"]])
        assert gp == polygons_of(fl["faces"], fl["off"], fl["xyz"]), name
        # each face's plane, as MCUT hands it on with the polygon
        want = sorted((int(f), tuple(n), int(m)) for f, n, m in zip(fl["faces"], fl["normals"].tolist(), fl["mc"]))
        have = sorted((int(f), tuple(n), int(m)) for f, n, m in zip(got["faces"], got["normals"].tolist(), got["mc"]))
        assert have == want, name


def test_floating_polygons_are_covered():
    """The benchmark pairs MCUT runs twice have floating polygons in their
    first pass, and the oracle finds each."""
    found = 0
    for name in ("bm025", "bm030", "bm040", "bunny_plane"):
        c = CASES[name]
        src, cut, flags = _user_meshes(c)
        _, cps, fls = oracle.observe_floating(src, cut, flags=flags)
        got = oracle.floating(cps[0]["nv"], cps[0]["reg"], cps[0]["want"]["edges"], cps[0]["x"],
                              (cps[0]["soup_off"], cps[0]["soup_idx"]))
        assert len(got["faces"]) == len(fls[0]["faces"]) > 0, name
        found += len(got["faces"])
    assert found > 0
