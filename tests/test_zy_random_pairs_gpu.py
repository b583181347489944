"""The GPU front end on seeded random pairs, bit for bit against the oracle.

The inputs are the families of fuzz_cases.py, on which the oracle port is
pinned against the unmodified reference (test_oracle_fuzz.py):
fracture pairs, the same snapped to a 1/8 lattice (general-position
violations), to a 1/2 lattice (collapsed faces, the degenerate status),
planar and warped quad meshes, and float32 vertex arrays. Compared: status,
first degenerate face, eps, the pair set, every culled test with both
orient3d signs, type and point-in-polygon char, and the records with their
point bits.

This file is collected after the other GPU files so that a failure here
cannot hide another test.
"""
import pytest

import fuzz_cases as F
import golden_cases as G
import oracle
from gpu_util import canonical_records, canonical_tests, sort_rows

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _check(ctx, src, cut, kw):
    fi = bool(kw.get("float_input", False))
    want = oracle.front_end(src, cut, impl="port", float_input=fi)
    r = ctx.dispatch(src, cut, float_input=fi, keep_tests=True, keep_pairs=True)
    assert r.status == int(want["status"]), (r.status_name, int(want["status"]))
    assert r.bad_face == int(want["bad_face"])
    assert G.same_bits(r.cut_eps, want["cut_eps"])
    assert G.same_bits(sort_rows(r.pairs, [0, 1]), want["pairs"])
    if int(want["status"]) in (2, 3):
        return int(want["status"])  # the reference stops before the narrow phase
    t, info = canonical_tests(r.tests, r.test_info)
    assert G.same_bits(t, want["tests"])
    assert G.same_bits(info, want["test_info"])
    ids, pts = canonical_records(r.record_ids, r.record_points)
    assert G.same_bits(ids, want["rec_ids"])
    assert G.same_bits(pts, want["rec_pts"])
    return int(want["status"])


@pytest.mark.parametrize("seed", range(4))
def test_random_fracture_pairs(ctx, seed):
    for s, c, kw in F.fracture(seed):
        _check(ctx, s, c, kw)


@pytest.mark.parametrize("seed", range(4))
def test_lattice_snapped_pairs(ctx, seed):
    statuses = {_check(ctx, s, c, kw) for s, c, kw in F.lattice(seed)}
    assert oracle.FE_GP_VIOLATION in statuses


def test_collapsed_faces(ctx):
    statuses = {_check(ctx, s, c, kw) for s, c, kw in F.collapsed()}
    assert statuses & {oracle.FE_DEGENERATE_SRC_FACE, oracle.FE_DEGENERATE_CUT_FACE}


@pytest.mark.parametrize("warp", [0.0, 1e-3, 0.05])
def test_quad_meshes(ctx, warp):
    for s, c, kw in F.quads(warp):
        _check(ctx, s, c, kw)


def test_float_input(ctx):
    for s, c, kw in F.float32(False, vary_constant=False):
        _check(ctx, s, c, kw)
