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

import numpy as np
import pytest

import golden_cases as G
import oracle
from mcut_gb300 import meshgen as M

REF_ROOT = os.environ.get("MCUT_REF_ROOT", "/root/reference")
pytestmark = pytest.mark.skipif(not os.path.isdir(os.path.join(REF_ROOT, "source")),
                                reason="reference checkout not present")

KEYS = G.FE_KEYS + ["face_boxes", "cut_xyz"]


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build(ref=True, ref_root=REF_ROOT)


def _same(src, cut, **kw):
    a = oracle.front_end(src, cut, impl="ref", **kw)
    b = oracle.front_end(src, cut, impl="port", **kw)
    assert a["status"] == b["status"]
    assert a["bad_face"] == b["bad_face"]
    assert G.same_bits(a["cut_eps"], b["cut_eps"])
    for k in KEYS:
        assert G.same_bits(a[k], b[k]), k
    return a


def _lattice(m, step):
    return dict(v=np.round(m["v"] / step) * step, f=m["f"], fs=m["fs"])


def _quads(n, h, rng, warp):
    g = M.grid(n, h)
    i = np.arange(n - 1)
    I, J = np.meshgrid(i, i, indexing="xy")
    a = (J * n + I).ravel()
    f = np.stack([a, a + 1, a + n + 1, a + n], 1).astype(np.uint32)
    v = g["v"].copy()
    v[:, 2] += rng.uniform(-warp, warp, len(v))
    return dict(v=v, f=f.ravel(), fs=np.full(len(f), 4, np.uint32))


@pytest.mark.parametrize("seed", range(4))
def test_random_fracture_pairs(seed):
    rng = np.random.default_rng(M.SEED_BASE + 100 + seed)
    recs = 0
    for _ in range(25):
        s, c = M.crack_pair(rng, level=int(rng.integers(1, 4)), n=int(rng.integers(4, 24)))
        recs += len(_same(s, c)["rec_ids"])
    assert recs > 0


@pytest.mark.parametrize("seed", range(4))
def test_lattice_snapped_pairs(seed):
    rng = np.random.default_rng(M.SEED_BASE + 200 + seed)
    statuses = set()
    for _ in range(25):
        s, c = M.crack_pair(rng, level=int(rng.integers(1, 3)), n=int(rng.integers(3, 9)))
        statuses.add(_same(_lattice(s, 0.125), _lattice(c, 0.125))["status"])
    assert oracle.FE_GP_VIOLATION in statuses


def test_collapsed_faces():
    rng = np.random.default_rng(M.SEED_BASE + 300)
    statuses = set()
    for _ in range(40):
        s, c = M.crack_pair(rng, level=int(rng.integers(1, 3)), n=int(rng.integers(3, 9)))
        statuses.add(_same(_lattice(s, 0.5), _lattice(c, 0.5))["status"])
    assert statuses & {oracle.FE_DEGENERATE_SRC_FACE, oracle.FE_DEGENERATE_CUT_FACE}


@pytest.mark.parametrize("warp", [0.0, 1e-3, 0.05])
def test_quad_meshes(warp):
    rng = np.random.default_rng(M.SEED_BASE + 400)
    for _ in range(10):
        s = M.icosphere(int(rng.integers(1, 3)), 1.0)
        c = _quads(int(rng.integers(3, 10)), 1.5, rng, warp)
        c["v"] = c["v"] @ M._rotation(rng).T + rng.uniform(-0.3, 0.3, 3)
        _same(s, c)


@pytest.mark.parametrize("absolute", [False, True])
def test_float_input_and_cut_box_constant(absolute):
    rng = np.random.default_rng(M.SEED_BASE + 500 + int(absolute))
    for _ in range(12):
        s, c = M.crack_pair(rng, level=2, n=int(rng.integers(4, 16)))
        _same(s, c, float_input=True, gp_absolute=absolute,
              gp_constant=float(rng.choice([1e-4, 1e-3, 1e-2])))
