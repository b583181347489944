"""Seeded random pairs: the plain-C port against the unmodified reference.

The fixtures pin the port on the reference's own test meshes; this module
widens the pin to inputs drawn at random, each run by both and compared bit
for bit (status, eps, pairs, tests with their signs / type / point-in-polygon
chars, records, points, face boxes, recentred cut vertices):

* fracture-like pairs (noisy icosphere vs rotated, displaced grid);
* the same snapped to a 1/8 lattice: coplanar faces, vertices on faces and
  edges through edges, so most raise the general-position violation;
* snapped to a 1/2 lattice: faces collapse, the degenerate-face status;
* quad meshes (face sizes given), planar or warped, against an icosphere;
* float32 vertex arrays with the cut-box constant varied, relative and
  absolute.

Skipped on hosts without the reference sources.
"""
import os

import pytest

import fuzz_cases as F
import golden_cases as G
import oracle

pytestmark = pytest.mark.skipif(not oracle.ref_available(),
                                reason="reference harness not built and MCUT_REF_ROOT unset")

KEYS = G.FE_KEYS + ["face_boxes", "cut_xyz"]


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build(ref=True)


def _same(src, cut, **kw):
    a = oracle.front_end(src, cut, impl="ref", **kw)
    b = oracle.front_end(src, cut, impl="port", **kw)
    assert a["status"] == b["status"]
    assert a["bad_face"] == b["bad_face"]
    assert G.same_bits(a["cut_eps"], b["cut_eps"])
    for k in KEYS:
        assert G.same_bits(a[k], b[k]), k
    return a


@pytest.mark.parametrize("seed", range(4))
def test_random_fracture_pairs(seed):
    recs = 0
    for s, c, kw in F.fracture(seed):
        recs += len(_same(s, c, **kw)["rec_ids"])
    assert recs > 0


@pytest.mark.parametrize("seed", range(4))
def test_lattice_snapped_pairs(seed):
    statuses = {_same(s, c, **kw)["status"] for s, c, kw in F.lattice(seed)}
    assert oracle.FE_GP_VIOLATION in statuses


def test_collapsed_faces():
    statuses = {_same(s, c, **kw)["status"] for s, c, kw in F.collapsed()}
    assert statuses & {oracle.FE_DEGENERATE_SRC_FACE, oracle.FE_DEGENERATE_CUT_FACE}


@pytest.mark.parametrize("warp", [0.0, 1e-3, 0.05])
def test_quad_meshes(warp):
    for s, c, kw in F.quads(warp):
        _same(s, c, **kw)


@pytest.mark.parametrize("absolute", [False, True])
def test_float_input_and_cut_box_constant(absolute):
    for s, c, kw in F.float32(absolute):
        _same(s, c, **kw)
