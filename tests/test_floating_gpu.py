"""The device's floating polygons equal the oracle's (kernel.cpp:4078-4200).

After a single dispatch the device finds, from its own cut path, the
circular cut paths whose intersection vertices all pierce one face: the
polygon MCUT stops the dispatch on to partition that face. Faces, vertex
cycles (from each polygon's smallest vertex), the face normals and their
largest components must equal oracle/cutpath_oracle.c's (pinned against
MCUT's own detection in tests/test_floating_oracle.py) on the same cut path,
bit for bit: on every golden pair (27 of them hold floating polygons) and
seeded families, and none where there are none.
"""
import numpy as np
import pytest

import fuzz_cases as F
import golden_cases as G
import oracle

pytestmark = pytest.mark.gpu

CASES = G.all_cases()


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _check(ctx, s, c, r):
    got = ctx.floating_polygons()
    cp = ctx.cut_path()
    rid = r.record_ids
    nv = len(s["v"]) + len(c["v"])
    want = oracle.floating(nv, rid[:, 2:5], cp["edges"], ctx.vertices(), oracle.soup_faces(s, c))
    for k in ("faces", "off", "vtx", "mc"):
        assert np.array_equal(np.asarray(got[k]).reshape(-1), np.asarray(want[k]).reshape(-1)), k
    assert G.same_bits(np.asarray(got["normals"]).reshape(-1, 3), want["normals"].reshape(-1, 3))
    return got


@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_pairs(ctx, name):
    c = CASES[name]
    r = ctx.dispatch(c["src"], c["cut"])
    if r.status != 0:
        pytest.skip(f"status {r.status_name}")
    _check(ctx, c["src"], c["cut"], r)


def test_floating_polygons_found(ctx):
    found = 0
    for name in ("bm025", "bm030", "bm040", "bunny_plane"):
        c = CASES[name]
        r = ctx.dispatch(c["src"], c["cut"])
        found += len(_check(ctx, c["src"], c["cut"], r)["faces"])
    assert found > 0


def test_random_families(ctx):
    for s, c, _ in F.fracture(0, 10) + F.lattice(0, 6):
        r = ctx.dispatch(s, c)
        if r.status == 0:
            _check(ctx, s, c, r)
