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
    assert lib.mcgpu_server_cancel(None, 1) == L.INVALID_VALUE


@pytest.fixture(scope="module")
def alone():
    """Each request dispatched alone on a plain context (its pool freed
    before each, so that the device bytes it holds after are the request's
    own need)."""
    from mcut_gb300 import Context
    reqs = _requests(24, meshgen.SEED_BASE + 50)
    ctx = Context(0)
    out, needs = [], []
    for s, c in reqs:
        ctx.trim()
        out.append(ctx.dispatch(s, c))
        needs.append(ctx.memory()["device_bytes"])
    ctx.close()
    return reqs, out, needs


def _same(a_sum, a_ids, a_pts, b):
    assert a_sum.status == b.status
    # per-request counters: the request's own pairs, tests and escalations
    assert (a_sum.num_pairs, a_sum.num_tests, tuple(a_sum.escalations)) == \
        (b.num_pairs, b.num_tests, tuple(b.escalations))
    assert G.same_bits(a_sum.cut_eps, b.cut_eps)
    assert a_ids.shape == b.record_ids.shape
    assert np.array_equal(a_ids, b.record_ids)
    assert G.same_bits(a_pts, b.record_points)


@pytest.mark.gpu
def test_served_same_alone_and_in_the_mix(alone):
    from mcut_gb300 import Server
    reqs, want, needs = alone
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
    reqs, want, needs = alone
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


def _estimate(s, c):
    """The server's per-request estimate: 1 MiB + 744 B per face + 128 B per vertex."""
    return (1 << 20) + 744 * (meshgen.num_faces(s) + meshgen.num_faces(c)) + 128 * (s["v"].shape[0] + c["v"].shape[0])


@pytest.mark.gpu
@pytest.mark.parametrize("mult", [1.2, 3.0])
def test_served_admission_budget(alone, mult):
    """Budgets that fit one to a few requests at a time: every result is
    still the request's own, and the device bytes the server reserved (the
    resident meshes plus every worker's pool or batch cap, which the pools
    cannot pass) never exceed the budget; idle pools are freed to make room."""
    from mcut_gb300 import Server
    reqs, want, needs = alone
    # the largest request's own pool and estimate (a request whose estimate
    # exceeds the budget is refused at submission) plus the resident mesh
    # (coordinates, indices and its tree) fit, a few requests at most beside
    # each other
    probe = Server(0, workers=1)
    probe.add_cut(reqs[0][1])
    resident = probe.stats()["resident_bytes"]
    probe.close()
    assert resident > 24 * reqs[0][1]["v"].shape[0] + 12 * meshgen.num_faces(reqs[0][1])
    budget = max(int(max(needs) * mult), max(_estimate(s, c) for s, c in reqs)) + resident
    srv = Server(0, workers=3, hbm_budget_bytes=budget)
    cid = srv.add_cut(reqs[0][1])
    tickets = [srv.submit(s, c) for s, c in reqs] + [srv.submit(reqs[0][0], cut_id=cid)]
    for t, w in zip(tickets, want + [want[0]]):
        sm, _ = srv.wait(t)
        ids, pts = srv.records(t)
        _same(sm, ids, pts, w)
    st = srv.stats()
    srv.close()
    assert st["completed"] == len(reqs) + 1
    assert 0 < st["peak_reserved_bytes"] <= budget
    assert st["pool_bytes"] + st["resident_bytes"] <= budget


def _ngon(n, axis):
    """One flat n-gon of radius 1 through the origin, normal along `axis`."""
    t = np.linspace(0.0, 2.0 * np.pi, n, endpoint=False)
    p = np.zeros((n, 3))
    a, b = [k for k in range(3) if k != axis]
    p[:, a], p[:, b] = np.cos(t), np.sin(t)
    return {"v": p, "f": np.arange(n, dtype=np.uint32), "fs": np.array([n], np.uint32)}


@pytest.mark.gpu
def test_served_request_larger_than_the_budget(alone):
    """A request whose estimate passes admission (two 300-gons: 1 MiB + 744 B
    per face + 128 B per vertex) but whose dispatch needs far more device
    memory than the budget (the narrow phase's plane triplets, C(n, 3) per
    polygon) completes with MCGPU_TOO_LARGE after its retries; requests
    around it keep their own results and the budget holds."""
    from mcut_gb300 import Server
    reqs, want, needs = alone
    big = (_ngon(300, 2), _ngon(300, 0))
    assert _estimate(*big) < (2 << 20)
    small = sorted(range(len(reqs)), key=lambda i: needs[i])[:3]
    budget = max(8 << 20, int(max(needs[i] for i in small) * 1.5), max(_estimate(*reqs[i]) for i in small))
    assert budget < 2 * 24 * (300 * 299 * 298 // 6)  # below the two polygons' triplet scratch
    srv = Server(0, workers=2, hbm_budget_bytes=budget)
    ts = [srv.submit(*reqs[small[0]])]
    tb = srv.submit(*big)
    ts += [srv.submit(*reqs[i]) for i in small[1:]]
    with pytest.raises(RuntimeError, match="TOO_LARGE"):
        srv.wait(tb)
    for t, i in zip(ts, small):
        sm, _ = srv.wait(t)
        ids, pts = srv.records(t)
        _same(sm, ids, pts, want[i])
    st = srv.stats()
    srv.close()
    assert st["peak_reserved_bytes"] <= budget and st["pool_trims"] > 0


@pytest.mark.gpu
def test_served_cancel(alone):
    """A queued request can be taken out before a batch holds it; waiting on
    it reports MCGPU_CANCELLED; a completed one cannot be cancelled; the rest
    complete with their own results."""
    from mcut_gb300 import Server
    from mcut_gb300 import _lib as L
    reqs, want, needs = alone
    srv = Server(0, workers=1, max_batch_pairs=1, linger_us=2_000_000)
    tickets = [srv.submit(s, c) for s, c in reqs[:10]]
    rcs = {t: srv.cancel(t) for t in tickets[5:]}
    assert all(rc in (L.OK, L.NOT_READY) for rc in rcs.values())
    assert any(rc == L.OK for rc in rcs.values())
    for i, t in enumerate(tickets):
        if rcs.get(t) == L.OK:
            with pytest.raises(RuntimeError, match="CANCELLED"):
                srv.wait(t)
            continue
        sm, _ = srv.wait(t)
        ids, pts = srv.records(t)
        _same(sm, ids, pts, want[i])
    assert srv.cancel(tickets[0]) == L.INVALID_VALUE
    st = srv.stats()
    srv.close()
    assert st["cancelled"] == sum(rc == L.OK for rc in rcs.values())
    assert st["completed"] == 10 - st["cancelled"]


@pytest.mark.gpu
def test_served_records_match_oracle(alone):
    from mcut_gb300 import Server
    reqs, _, _ = alone
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


def _few_faces(c, k):
    """The first k faces of cut mesh c, with only the vertices they use."""
    f = np.asarray(c["f"], np.uint32).reshape(-1, 3)[:k]
    used, inv = np.unique(f, return_inverse=True)
    return dict(c, v=c["v"][used], f=inv.astype(np.uint32).reshape(-1))


@pytest.mark.gpu
def test_served_resident_trees_only(alone):
    """Batches in which every pair names a resident cut mesh (no batch tree
    at all: every source face walks its resident mesh's own tree), several
    requests per resident mesh, and resident meshes of one face (a one-leaf
    tree) and of a few faces: each result equals the request alone on a
    plain context, pairs, tests and records included."""
    from mcut_gb300 import Context, Server
    reqs, want, needs = alone
    ctx = Context(0)
    cases = []
    for i in range(4):
        s, c = reqs[i]
        cases.append((s, c, want[i]))
    # small resident meshes cut from request 0's cut mesh, against its source
    for k in (1, 5, 40):
        s, c0 = reqs[0]
        c = _few_faces(c0, k)
        cases.append((s, c, ctx.dispatch(s, c)))
    ctx.close()
    srv = Server(0, workers=2, max_batch_pairs=16)
    cids = [srv.add_cut(c) for _, c, _ in cases]
    tickets = [(srv.submit(s, cut_id=cid), w) for (s, _, w), cid in zip(cases, cids)]
    tickets += [(srv.submit(s, cut_id=cid), w) for (s, _, w), cid in zip(cases, cids)]
    for t, w in tickets:
        sm, _ = srv.wait(t)
        ids, pts = srv.records(t)
        _same(sm, ids, pts, w)
    st = srv.stats()
    srv.close()
    assert st["resident_meshes"] == len(cases)
    # the trees are counted with the meshes: more than coordinates and indices alone
    mesh_bytes = sum(24 * c["v"].shape[0] + 12 * meshgen.num_faces(c) for _, c, _ in cases)
    assert st["resident_bytes"] > mesh_bytes
