"""CPU model of how the device forms the edge-face tests (k_pair_tests).

The reference gives every edge of every candidate face the sorted union of
the partner faces of its (at most two) incident candidate faces
(kernel.cpp:1781-1983), then culls each (edge, face) whose edge box misses the
face box (kernel.cpp:1989-2177). The device forms the same set without a map.
For each candidate pair (F, g), each edge (a, b) of F emits its test unless
the edge's other face G is lower-numbered and its box meets g's box: then G
emits it, as its own pair with g. The emitted edge runs the way the lower
face of the two traverses it, which is MCUT's primary halfedge. This module
restates that rule over the oracle's pairs, face boxes and ps coordinates.
On every committed fixture and on seeded random pairs, it must give exactly
the reference's culled test set, each test emitted once.
"""
import numpy as np
import pytest

import fuzz_cases as F
import golden_cases as G
import oracle

CASES = G.all_cases()


def _faces(m, voff):
    f = np.asarray(m["f"], dtype=np.int64) + voff
    fs = m.get("fs")
    if fs is None:
        return [list(f[3 * i:3 * i + 3]) for i in range(len(f) // 3)]
    out, o = [], 0
    for s in np.asarray(fs, dtype=np.int64):
        out.append(list(f[o:o + s]))
        o += s
    return out


def _overlap(a, b):
    return all(a[j] <= b[3 + j] and a[3 + j] >= b[j] for j in range(3))


def model_tests(src, cut, r):
    nsv = len(r["src_xyz"])
    faces = _faces(src, 0) + _faces(cut, nsv)
    nsf = len(_faces(src, 0))
    x = np.concatenate([r["src_xyz"], r["cut_xyz"]])
    box = r["face_boxes"]
    # the other face of each directed edge: the face holding (b, a)
    face_of = {}
    for fi, fv in enumerate(faces):
        for k in range(len(fv)):
            face_of[(int(fv[k]), int(fv[(k + 1) % len(fv)]))] = fi
    out = []
    for s, c in r["pairs"]:
        for Fc, g in ((int(s), nsf + int(c)), (nsf + int(c), int(s))):
            fv = faces[Fc]
            for k in range(len(fv)):
                a, b = int(fv[k]), int(fv[(k + 1) % len(fv)])
                Gf = face_of.get((b, a))
                if Gf is not None and Gf < Fc and _overlap(box[Gf], box[g]):
                    continue  # the lower face emits it with its own pair
                eb = [min(x[a][j], x[b][j]) for j in range(3)] + [max(x[a][j], x[b][j]) for j in range(3)]
                if not _overlap(eb, box[g]):
                    continue
                out.append((b, a, g) if Gf is not None and Gf < Fc else (a, b, g))
    return out


def _check(src, cut, **kw):
    r = oracle.front_end(src, cut, **kw)
    if r["status"] in (oracle.FE_DEGENERATE_SRC_FACE, oracle.FE_DEGENERATE_CUT_FACE, oracle.FE_INVALID_INPUT):
        return 0
    got = model_tests(src, cut, r)
    assert len(got) == len(set(got)), "a test emitted twice"
    want = {tuple(int(v) for v in t) for t in r["tests"]}
    assert set(got) == want
    return len(got)


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_tests_from_the_ownership_rule(name):
    c = CASES[name]
    _check(c["src"], c["cut"], float_input=bool(c["float_input"]))


def test_random_pairs_from_the_ownership_rule():
    n = 0
    for s, c, kw in F.fracture(1, 10) + F.lattice(1, 10) + F.quads(0.05, 5) + F.quads(0.0, 5):
        n += _check(s, c, **kw)
    assert n > 1000
