"""Request server (continuous batching): every result identical alone and in
the mix, resident cut meshes identical to uploaded ones, admission by the
HBM budget. Identical means bit for bit (status, record ids, points)."""
import numpy as np
import pytest

import golden_cases as G
import oracle
from gpu_util import canonical_records
from mcut_gb300 import meshgen


def _requests(count, seed):
    rng = np.random.default_rng(seed)
    return [meshgen.crack_pair(rng, target_tris=int(t)) for t in np.exp(rng.uniform(np.log(1e3), np.log(6e4), count))]


def test_server_without_gpu_is_an_error_not_a_crash():
    import ctypes as C
    import torch
    from mcut_gb300 import _lib as L
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    lib = L.load()
    h = C.c_void_p()
    cfg = L.ServerConfig(0, 1, 0, 0, 0, 0, 0)
    assert lib.mcgpu_server_create(C.byref(h), C.byref(cfg)) != L.OK
    assert lib.mcgpu_server_submit(None, None, None, L.NO_CUT, None) == L.INVALID_VALUE
    assert lib.mcgpu_server_wait(None, 1, 0, None, None) == L.INVALID_VALUE


@pytest.fixture(scope="module")
def alone():
    """Each request dispatched alone on a plain context."""
    from mcut_gb300 import Context
    reqs = _requests(24, meshgen.SEED_BASE + 50)
    ctx = Context(0)
    out = [ctx.dispatch(s, c) for s, c in reqs]
    ctx.close()
    return reqs, out


def _same(a_sum, a_ids, a_pts, b):
    assert a_sum.status == b.status
    assert G.same_bits(a_sum.cut_eps, b.cut_eps)
    assert a_ids.shape == b.record_ids.shape
    assert np.array_equal(a_ids, b.record_ids)
    assert G.same_bits(a_pts, b.record_points)


@pytest.mark.gpu
def test_served_same_alone_and_in_the_mix(alone):
    from mcut_gb300 import Server
    reqs, want = alone
    srv = Server(0, workers=3, max_batch_pairs=7)
    tickets = [srv.submit(s, c) for s, c in reqs]
    for t, w in zip(tickets, want):
        sm, lat = srv.wait(t)
        ids, pts = srv.records(t)
        _same(sm, ids, pts, w)
        assert lat > 0
        srv.release(t)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    assert st["batches"] < len(reqs)  # requests were batched together


@pytest.mark.gpu
def test_served_resident_cut_meshes(alone):
    from mcut_gb300 import Server
    reqs, want = alone
    srv = Server(0, workers=2)
    ids_ = [srv.add_cut(c) for _, c in reqs[:6]]
    tickets = []
    for i, (s, c) in enumerate(reqs):
        # every other request names its cut mesh by resident id
        tickets.append(srv.submit(s, cut_id=ids_[i]) if i < 6 and i % 2 == 0 else srv.submit(s, c))
    for t, w in zip(tickets, want):
        sm, _ = srv.wait(t)
        ids, pts = srv.records(t)
        _same(sm, ids, pts, w)
    st = srv.stats()
    srv.close()
    assert st["resident_meshes"] == 6 and st["resident_bytes"] > 0


@pytest.mark.gpu
def test_served_admission_budget(alone):
    """A budget that fits about one request at a time: still every result,
    and the in-flight estimate never passes the budget except for one
    request running alone."""
    from mcut_gb300 import Server
    reqs, want = alone
    budget = 48 << 20
    srv = Server(0, workers=3, hbm_budget_bytes=budget)
    tickets = [srv.submit(s, c) for s, c in reqs]
    for t, w in zip(tickets, want):
        sm, _ = srv.wait(t)
        ids, pts = srv.records(t)
        _same(sm, ids, pts, w)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs)
    # the server's estimate: 1 MiB + 744 B per face + 128 B per vertex
    biggest = max((1 << 20) + 744 * (meshgen.num_faces(s) + meshgen.num_faces(c))
                  + 128 * (s["v"].shape[0] + c["v"].shape[0]) for s, c in reqs)
    assert st["peak_inflight_bytes"] <= max(budget, biggest)


@pytest.mark.gpu
def test_served_records_match_oracle(alone):
    from mcut_gb300 import Server
    reqs, _ = alone
    srv = Server(0)
    tickets = [srv.submit(s, c) for s, c in reqs[:8]]
    for t, (s, c) in zip(tickets, reqs[:8]):
        sm, _ = srv.wait(t)
        ids, pts = srv.records(t)
        w = oracle.front_end(s, c, impl="port", threads=16)
        assert sm.status == w["status"]
        a, b = canonical_records(ids, pts)
        wa, wb = canonical_records(w["rec_ids"], w["rec_pts"])
        assert G.same_bits(a, wa) and G.same_bits(b, wb)
    srv.close()
