"""The device's cut path equals the oracle's (kernel.cpp:3332-3632).

After a single dispatch the device builds, from its own record hand-over,
the edges MCUT's m0 gets from cutpath_edge_creation_info: the edges in
creation order (first and second vertex), each face's edge list in append
order and each intersection vertex's incoming halfedges. The oracle
(oracle/cutpath_oracle.c, pinned against MCUT's own stage in
tests/test_cutpath_oracle.py) runs on the same hand-over and coordinates;
every array must be equal. Covered: the golden pairs (keys of two
vertices, and of up to six sorted along their line with midpoint tests),
seeded fracture families, a general-position-enforced dispatch, device
inputs and the full-size workloads.
"""
import numpy as np
import pytest

import fuzz_cases as F
import golden_cases as G
import oracle
from mcut_gb300 import meshgen

pytestmark = pytest.mark.gpu

CASES = G.all_cases()
KEYS = ["edges", "face_keys", "face_off", "face_edges", "ivtx_off", "ivtx_he"]


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _check(ctx, s, c, r):
    got = ctx.cut_path()
    hand = ctx.hand_over()
    hand["rec_ids"], hand["rec_pts"] = r.record_ids, r.record_points
    want = oracle.cutpath_of(s, c, ctx.vertices(), hand)
    assert got["status"] == want["status"]
    if want["status"]:
        assert got["bad_key"] == want["bad_key"]
        return got
    for k in KEYS:
        assert np.array_equal(np.asarray(got[k]).reshape(np.asarray(want[k]).shape), want[k]), k
    return got


@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_pairs(ctx, name):
    c = CASES[name]
    r = ctx.dispatch(c["src"], c["cut"])
    if r.status != 0:
        pytest.skip(f"status {r.status_name}")
    _check(ctx, c["src"], c["cut"], r)


def test_sorted_runs_are_covered(ctx):
    longest = 0
    for name in ("bm002", "bm006", "bm034", "bm036", "bm042"):
        c = CASES[name]
        r = ctx.dispatch(c["src"], c["cut"])
        _check(ctx, c["src"], c["cut"], r)
        longest = max(longest, int(np.diff(ctx.hand_over()["cp_off"]).max()))
    assert longest > 2


def test_random_families(ctx):
    for s, c, _ in F.fracture(0, 12) + F.lattice(0, 6) + F.quads(0.05, 6):
        r = ctx.dispatch(s, c)
        if r.status == 0:
            _check(ctx, s, c, r)


def test_enforced_general_position(ctx):
    """The cut path of a perturbed pass reads the perturbed coordinates."""
    for name in sorted(CASES):
        c = CASES[name]
        r = ctx.dispatch(c["src"], c["cut"], enforce_general_position=True)
        if r.perturbations and r.status == 0:
            _check(ctx, c["src"], c["cut"], r)
            return
    pytest.skip("no golden pair needs a perturbation")


def test_full_size(ctx):
    s, c = meshgen.sphere_heightfield(16.0)
    r = ctx.dispatch(s, c)
    got = _check(ctx, s, c, r)
    assert len(got["edges"]) > 10000
