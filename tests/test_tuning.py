"""Launch tuning and graph replay change speed only: every tuning and every
replay of a captured launch graph gives bit-identical results."""
import ctypes as C

import numpy as np
import pytest

import golden_cases as G
from mcut_gb300 import _lib as L
from mcut_gb300 import meshgen

TUNINGS = [dict(leaf_size=l, traversal=t, packet_faces=p, stack_depth=d, split_round=r)
           for l in (1, 4, 16) for (t, p, d, r) in ((0, 32, 64, 2), (0, 32, 64, 0), (0, 7, 64, 1), (1, 32, 64, 0),
                                                    (1, 16, 64, 0), (2, 32, 64, 0), (2, 32, 512, 0))]


def test_tuning_arguments_checked_without_a_gpu():
    lib = L.load()
    t = L.Tuning(4, 0, 32, 64, 2)
    assert lib.mcgpu_context_set_tuning(None, C.byref(t)) == L.INVALID_VALUE
    assert lib.mcgpu_context_get_tuning(None, C.byref(t)) == L.INVALID_VALUE
    assert lib.mcgpu_autotune(None, 0, None, 1, None, None) == L.INVALID_VALUE


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _key(r):
    return r.status, r.num_pairs, r.num_tests, r.record_ids.tobytes(), r.record_points.tobytes(), \
        r.pairs.tobytes() if r.pairs is not None else b""


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["crack", "sphere_heightfield"])
def test_every_tuning_gives_the_same_result(ctx, case):
    if case == "crack":
        s, c = meshgen.crack_pair(np.random.default_rng(11), target_tris=60000)
    else:
        s, c = meshgen.sphere_heightfield(16.0, level=5, n=300)
    ctx.set_tuning()
    want = _key(ctx.dispatch(s, c, keep_pairs=True))
    for t in TUNINGS:
        ctx.set_tuning(**t)
        got = _key(ctx.dispatch(s, c, keep_pairs=True))
        assert got[:3] == want[:3], t
        assert got[3:5] == want[3:5], t
        # the pair list is emitted in traversal order; compare as a set
        a = np.frombuffer(got[5], np.uint32).reshape(-1, 2)
        b = np.frombuffer(want[5], np.uint32).reshape(-1, 2)
        assert np.array_equal(np.unique(a, axis=0), np.unique(b, axis=0)), t
    ctx.set_tuning()


@pytest.mark.gpu
def test_graph_replay_is_identical(ctx):
    """Dispatch 1 runs the launches directly, dispatch 2 captures them into
    graphs, later ones replay; a different size in between changes the key."""
    s, c = meshgen.crack_pair(np.random.default_rng(12), target_tris=20000)
    s2, c2 = meshgen.crack_pair(np.random.default_rng(13), target_tris=5000)
    first = ctx.dispatch(s, c)
    for k in range(5):
        r = ctx.dispatch(s, c)
        assert r.status == first.status
        assert np.array_equal(r.record_ids, first.record_ids)
        assert G.same_bits(r.record_points, first.record_points)
        assert r.kernel_launches == first.kernel_launches
        if k == 2:
            ctx.dispatch(s2, c2)


@pytest.mark.gpu
def test_autotune_keeps_results(ctx):
    from mcut_gb300 import pack_pairs
    pairs = meshgen.batch_pairs(32, seed=meshgen.SEED_BASE + 42)
    pk = pack_pairs(pairs)
    sums0, ids0, pts0, off0 = ctx.dispatch_packed(pk)
    best, ms = ctx.autotune(pk, repeats=1)
    assert ms > 0 and ctx.tuning() == best
    sums1, ids1, pts1, off1 = ctx.dispatch_packed(pk)
    assert np.array_equal(off0, off1) and np.array_equal(ids0, ids1) and G.same_bits(pts0, pts1)
    ctx.set_tuning()


@pytest.mark.gpu
def test_profiled_dispatches_repeat(ctx):
    """Stage timing (direct launches) interleaved with graph replays."""
    s, c = meshgen.crack_pair(np.random.default_rng(14), target_tris=20000)
    for k in range(6):
        r = ctx.dispatch(s, c, profile=(k % 2 == 0), fetch=False)
        assert r.status in (0, 1)
        if k % 2 == 0:
            assert sum(r.stage_ms.values()) > 0


@pytest.mark.gpu
def test_split_capacity_overflow_is_harmless():
    """Slow packets hand their remaining walk to a second launch; with the
    entry capacity forced tiny most of them must finish their own walk, with
    the same result."""
    import os
    from mcut_gb300 import Context
    s, c = meshgen.sphere_heightfield(16.0, level=6, n=512)
    a = Context(0)
    want = a.dispatch(s, c, keep_pairs=True)
    os.environ["MCGPU_SPLIT_CAP"] = "3"
    try:
        b = Context(0)
    finally:
        del os.environ["MCGPU_SPLIT_CAP"]
    got = b.dispatch(s, c, keep_pairs=True)
    assert got.num_pairs == want.num_pairs and got.status == want.status
    assert np.array_equal(np.unique(got.pairs, axis=0), np.unique(want.pairs, axis=0))
    assert np.array_equal(got.record_ids, want.record_ids) and G.same_bits(got.record_points, want.record_points)
    a.close()
    b.close()


def _lifted(m, dz):
    return dict(v=m["v"] + np.array([0.0, 0.0, dz]), f=m["f"], fs=m["fs"])


def _same_result(a, b):
    assert (a.status, a.num_pairs, a.num_tests, a.num_records) == (b.status, b.num_pairs, b.num_tests, b.num_records)
    assert np.array_equal(a.record_ids, b.record_ids)
    assert G.same_bits(a.record_points, b.record_points)


@pytest.mark.gpu
def test_fused_call_reorders_records_past_the_one_launch_sort(ctx):
    """A call of the same shape as the one before runs as one graph; when its
    records outnumber the one-launch ordering (24,576), the record segment
    runs again from the host's count. Stage-timed calls take the stage-by-
    stage path: both give the same records."""
    src = meshgen.grid(200, 1.5, lambda X, Y: 0.02 * np.sin(40.0 * X) * np.sin(40.0 * Y))
    cut = meshgen.grid(200, 1.5, lambda X, Y: np.full_like(X, 0.001))
    far = ctx.dispatch(src, _lifted(cut, 1.0))
    assert far.num_records == 0
    fused = ctx.dispatch(src, cut)
    exact = ctx.dispatch(src, cut, profile=True)
    assert exact.num_records > 24576
    _same_result(fused, exact)
    again = ctx.dispatch(src, cut)
    _same_result(again, exact)


@pytest.mark.gpu
def test_fused_call_reruns_on_pair_overflow():
    """A fresh context holds 2 (source + cut faces) pairs; near-coplanar grids
    overlap about 18 faces each, so the fused call after a disjoint one
    overflows and reruns stage by stage (the pair buffer grows)."""
    from mcut_gb300 import Context
    rng = np.random.default_rng(77)
    src = meshgen.grid(80, 1.0)
    src["v"][:, 2] = rng.uniform(-2e-4, 2e-4, size=src["v"].shape[0])
    cut = meshgen.grid(80, 1.0, lambda X, Y: np.full_like(X, 3e-5))
    c = Context(0)
    try:
        far = c.dispatch(src, _lifted(cut, 5.0))
        assert far.num_pairs == 0
        over = c.dispatch(src, cut)
        assert over.num_pairs > 2 * (meshgen.num_faces(src) + meshgen.num_faces(cut))
        exact = c.dispatch(src, cut, profile=True)
        _same_result(over, exact)
        for _ in range(3):  # the grown buffers, then fused calls at that size
            _same_result(c.dispatch(src, cut), exact)
    finally:
        c.close()
