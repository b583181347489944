"""A context's device pool: its byte count, a cap that turns growth past it
into MCGPU_OUT_OF_MEMORY (a forced allocation failure), and trimming.

After either, the context must keep working and give the same records as
before, bit for bit: a failed call leaves no state a later call reads.
"""
import numpy as np
import pytest

import golden_cases as G
from gpu_util import canonical_records

pytestmark = pytest.mark.gpu

CASES = G.all_cases()


@pytest.fixture()
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _check(r, name):
    want = CASES[name]
    assert r.status == int(want["status"])
    a, b = canonical_records(r.record_ids, r.record_points)
    assert G.same_bits(a, want["rec_ids"]) and G.same_bits(b, want["rec_pts"])


def test_pool_bytes_grow_and_trim(ctx):
    assert ctx.memory() == {"device_bytes": 0, "limit_bytes": 0}
    c = CASES["two_spheres"]
    _check(ctx.dispatch(c["src"], c["cut"]), "two_spheres")
    small = ctx.memory()["device_bytes"]
    assert small > 0
    b = CASES["bunny_plane"]
    _check(ctx.dispatch(b["src"], b["cut"]), "bunny_plane")
    assert ctx.memory()["device_bytes"] >= small
    ctx.trim()
    assert ctx.memory()["device_bytes"] == 0
    # the records of the trimmed pool are gone, not stale
    with pytest.raises(RuntimeError, match="INVALID_VALUE"):
        ctx._get(1, np.uint32, 5)
    _check(ctx.dispatch(c["src"], c["cut"]), "two_spheres")
    _check(ctx.dispatch(b["src"], b["cut"]), "bunny_plane")


def test_forced_allocation_failure(ctx):
    """A cap below what the next call needs: the call fails with
    MCGPU_OUT_OF_MEMORY without growing the pool past the cap; with the cap
    lifted the same call gives the golden records, and so do calls of other
    shapes before and after."""
    from mcut_gb300 import meshgen
    c = CASES["two_spheres"]
    _check(ctx.dispatch(c["src"], c["cut"]), "two_spheres")
    held = ctx.memory()["device_bytes"]
    ctx.set_memory_limit(held + (64 << 10))
    s, k = meshgen.sphere_heightfield(16.0, level=5, n=256)
    with pytest.raises(RuntimeError, match="OUT_OF_MEMORY"):
        ctx.dispatch(s, k)
    assert ctx.memory()["device_bytes"] <= held + (64 << 10)
    assert ctx.memory()["limit_bytes"] == held + (64 << 10)
    # the earlier shape still fits and is unaffected
    _check(ctx.dispatch(c["src"], c["cut"]), "two_spheres")
    ctx.set_memory_limit(0)
    r = ctx.dispatch(s, k)
    from mcut_gb300 import Context
    fresh = Context(0)
    w = fresh.dispatch(s, k)
    fresh.close()
    assert r.status == w.status and r.num_records == w.num_records
    assert np.array_equal(r.record_ids, w.record_ids) and G.same_bits(r.record_points, w.record_points)
    _check(ctx.dispatch(c["src"], c["cut"]), "two_spheres")


def test_allocation_failure_in_a_batch(ctx):
    """The same for a batch: the failed batch changes nothing, the next one
    (cap lifted) equals the golden records pair by pair."""
    names = ["crack1", "two_spheres", "bm014"]
    pairs = [(CASES[k]["src"], CASES[k]["cut"]) for k in names]
    ctx.dispatch(*pairs[0])
    ctx.set_memory_limit(ctx.memory()["device_bytes"] + 4096)
    with pytest.raises(RuntimeError, match="OUT_OF_MEMORY"):
        ctx.dispatch_batch(pairs * 8)
    ctx.set_memory_limit(0)
    for k, (summ, ids, pts) in zip(names, ctx.dispatch_batch(pairs)):
        assert summ["status"] == int(CASES[k]["status"])
        a, b = canonical_records(ids, pts)
        assert G.same_bits(a, CASES[k]["rec_ids"]) and G.same_bits(b, CASES[k]["rec_pts"])
