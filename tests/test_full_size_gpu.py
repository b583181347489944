"""The benchmark workloads at their full sizes against the oracle.

* C3x16, the precision stress (a 512^2-per-face lattice cube, 3,145,728
  triangles, against a 256 x 256 grid coincident with its top face, z nudged
  by U(-1e-12, 1e-12), all x16): every candidate pair, every culled test's
  two orient3d signs, type and point-in-polygon char, every record and point
  bit, and the general-position outcome. The escalation counts the bench
  reports for this workload are the ones this test checks.
* C3 as written (scale 1, 2^-9 lattice legs): the reference rejects a
  collapsed face; the device must name the same face.
* C3x16 with general-position enforcement: the device's perturbation is the
  reference's sequence and the perturbed pass equals the oracle's
  (preproc.cpp:2590-2699).
* C4, the fracture batch the bench times (4096 uneven pairs, seed
  0xC0FFEE + 4): every pair of the packed pass against the oracle run on
  that pair alone.
"""
import numpy as np
import pytest

import golden_cases as G
import gp_rng
import oracle
from gpu_util import canonical_records, canonical_tests, sort_rows
from mcut_gb300 import meshgen

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def c3x16():
    return meshgen.cube_coplanar(16.0)


def _same_front_end(r, want):
    assert r.status == int(want["status"]), (r.status_name, int(want["status"]))
    assert r.bad_face == int(want["bad_face"])
    assert G.same_bits(r.cut_eps, want["cut_eps"])
    assert G.same_bits(sort_rows(r.pairs, [0, 1]), want["pairs"])
    t, info = canonical_tests(r.tests, r.test_info)
    assert G.same_bits(t, want["tests"])
    assert G.same_bits(info, want["test_info"])
    ids, pts = canonical_records(r.record_ids, r.record_points)
    assert G.same_bits(ids, want["rec_ids"])
    assert G.same_bits(pts, want["rec_pts"])


def test_c3_x16_full_size(ctx, c3x16):
    s, c = c3x16
    assert meshgen.num_faces(s) == 3_145_728 and meshgen.num_faces(c) == 130_050
    want = oracle.front_end(s, c, impl="port", threads=16)
    r = ctx.dispatch(s, c, keep_tests=True, keep_pairs=True)
    _same_front_end(r, want)
    # every test decides two signs, each at exactly one stage of the cascade
    esc = [int(x) for x in r.escalations]
    assert sum(esc) == 2 * len(want["tests"])
    assert esc[1] > 0 and esc[2] > 0  # the coplanar grid reaches the fp64 and exact stages


def test_c3_as_written_is_degenerate(ctx):
    s, c = meshgen.cube_coplanar(1.0)
    want = oracle.front_end(s, c, impl="port", threads=16)
    assert want["status"] in (2, 3)
    r = ctx.dispatch(s, c)
    assert (r.status, r.bad_face) == (want["status"], want["bad_face"])


def test_c3_x16_enforced_general_position(c3x16):
    from mcut_gb300 import Context
    s, c = c3x16
    cx = Context(0)  # a fresh perturbation sequence
    try:
        plain = cx.dispatch(s, c)
        assert plain.status_name == "GP_VIOLATION"
        r = cx.dispatch(s, c, keep_tests=True, keep_pairs=True, enforce_general_position=True)
        assert r.perturbations >= 1
        assert r.perturbation == gp_rng.perturbations(r.perturbations, r.cut_eps)[-1]
        want = oracle.front_end(s, c, impl="port", threads=16, perturbation=r.perturbation)
        _same_front_end(r, want)
    finally:
        cx.close()


def test_c4_batch_every_pair(ctx):
    from mcut_gb300 import pack_pairs
    pairs = meshgen.batch_pairs(4096)
    sums, ids, pts, off = ctx.dispatch_packed(pack_pairs(pairs))
    assert len(off) == 4097
    total = 0
    for i, (s, c) in enumerate(pairs):
        want = oracle.front_end(s, c, impl="port", threads=16)
        assert sums[i].status == want["status"], i
        assert G.same_bits(sums[i].cut_eps, want["cut_eps"]), i
        if want["status"] in (2, 3):
            continue
        a, b = int(off[i]), int(off[i + 1])
        w_ids, w_pts = canonical_records(want["rec_ids"], want["rec_pts"])
        g_ids, g_pts = canonical_records(ids[a:b], pts[a:b])
        assert G.same_bits(g_ids, w_ids), i
        assert G.same_bits(g_pts, w_pts), i
        total += b - a
    assert total == int(off[-1]) and total > 2_000_000
