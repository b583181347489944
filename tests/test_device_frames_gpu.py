"""The pair frame computed on the device equals the host recentring, bit for bit.

With user coordinates from host arrays (MCGPU_RECENTRE) the host only sums
each mesh's centroid in vertex order; the raw coordinates are gathered to
the device, whose kernels take the meshes' bounds with the reference's
sequential rule (preproc.cpp:2124-2290: max = (m < x) ? x : m from
-DBL_MAX, min likewise, float input compared in float from the float cast
of DBL_MAX), form t and the cut-box enlargement, and map every vertex. The
coordinates the dispatch used (MCGPU_DATA_VERTICES) and the summary's
cut_eps must equal mcgpu_recentre's host restatement and the oracle's, for
double and float input, for batches, and for bounds that are zeros of
either sign (where the first zero in vertex order gives the sign).
"""
import numpy as np
import pytest

import fuzz_cases as F
import golden_cases as G
import oracle
from mcut_gb300 import meshgen

pytestmark = pytest.mark.gpu

CASES = G.all_cases()


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _host(s, c, float_input=False):
    from mcut_gb300 import recentre
    sx, cx, eps = recentre(s, c, float_input=float_input)
    return np.concatenate([sx, cx]), eps


def _check(ctx, s, c, float_input=False):
    r = ctx.dispatch(s, c, float_input=float_input, fetch=False)
    v, eps = _host(s, c, float_input)
    assert G.same_bits(np.float64(r.cut_eps), np.float64(eps))
    assert G.same_bits(ctx.vertices(), v)
    return r


@pytest.mark.parametrize("name", ["two_spheres", "bm014", "bm052", "quad_pent", "crack1", "bunny_plane"])
def test_golden_pairs(ctx, name):
    c = CASES[name]
    _check(ctx, c["src"], c["cut"])
    want = oracle.front_end(c["src"], c["cut"], impl="port", threads=4)
    assert G.same_bits(ctx.vertices(), np.concatenate([want["src_xyz"].reshape(-1, 3),
                                                        want["cut_xyz"].reshape(-1, 3)]))


@pytest.mark.parametrize("name", ["two_spheres", "bm014", "crack1"])
def test_float_input(ctx, name):
    c = CASES[name]
    f = {k: (dict(m, v=m["v"].astype(np.float32)) if k in ("src", "cut") else m) for k, m in c.items()
         if k in ("src", "cut")}
    _check(ctx, f["src"], f["cut"], float_input=True)


def test_random_families_and_full_size(ctx):
    for s, c, _ in F.fracture(0, 6) + F.lattice(0, 4):
        _check(ctx, s, c)
    _check(ctx, *meshgen.sphere_heightfield(16.0))
    _check(ctx, *meshgen.cube_coplanar(16.0))


def _zero_bounds(m, axis, first_negative):
    """The mesh shifted so that its bound on `axis` is zero, reached by
    several vertices; the first of them in vertex order is -0.0 or +0.0."""
    v = m["v"].copy()
    lo = v[:, axis].min()
    hit = np.nonzero(v[:, axis] == lo)[0]
    v[:, axis] -= lo
    if len(hit) < 2:
        extra = np.argsort(v[:, axis])[1]
        v[extra, axis] = 0.0
        hit = np.sort(np.concatenate([hit, [extra]]))
    v[hit, axis] = 0.0
    v[hit[0], axis] = -0.0 if first_negative else 0.0
    if len(hit) > 1:
        v[hit[1], axis] = 0.0 if first_negative else -0.0
    return dict(m, v=v)


@pytest.mark.parametrize("first_negative", [False, True])
def test_zero_bounds_of_either_sign(ctx, first_negative):
    c = CASES["two_spheres"]
    for axis in range(3):
        s = _zero_bounds(c["src"], axis, first_negative)
        k = _zero_bounds(c["cut"], (axis + 1) % 3, not first_negative)
        _check(ctx, s, k)
        # the negated mesh: the zero is now the maximum
        s2 = dict(s, v=-s["v"])
        _check(ctx, s2, k)


def test_batch_frames(ctx):
    """A batch's pairs: each pair's enlargement and records equal its own
    dispatch's (the frames are computed per pair in one launch)."""
    pairs = [(CASES[k]["src"], CASES[k]["cut"]) for k in ("two_spheres", "bm014", "crack1", "quad_pent")]
    rng = np.random.default_rng(meshgen.SEED_BASE + 91)
    pairs += [meshgen.crack_pair(rng, target_tris=t) for t in (3000, 40000)]
    out = ctx.dispatch_batch(pairs)
    for (s, c), (summ, ids, pts) in zip(pairs, out):
        _, eps = _host(s, c)
        assert G.same_bits(np.float64(summ["cut_eps"]), np.float64(eps))
        r = ctx.dispatch(s, c)
        assert np.array_equal(ids, r.record_ids) and G.same_bits(pts, r.record_points)


def test_absolute_enlargement(ctx):
    """MCGPU_ENFORCE_GENERAL_POSITION_ABSOLUTE: the enlargement is the
    context's constant itself."""
    c = CASES["two_spheres"]
    ctx.set_general_position(2.5e-3, 4)
    try:
        r = ctx.dispatch(c["src"], c["cut"], enforce_general_position="absolute", fetch=False)
        assert r.cut_eps == 2.5e-3
    finally:
        ctx.set_general_position(1e-4, 4)
