"""mcgpu_dispatch_noalloc returns exactly what mcgpu_dispatch returns.

That entry point serves callers that must not allocate GPU memory while they
ask for intersection records (a plugin held to its host application's
device-memory arena, a process whose device memory another framework's
caching allocator already holds, a frame loop that cannot wait on the
allocator): its scratch is one static device array, the caller supplies
device inputs and device output buffers. Here it runs twice in a row -- the
second call sees the first call's leftovers in the shared array -- and each
result must equal the allocating entry point's, bit for bit: on intersecting
pairs, on a general-position violation with records, on degenerate faces, on
a record buffer too small for the records, on more candidate pairs than its
fixed capacity and on indices outside their mesh.

This file is collected last so that a failure here cannot hide another test.
"""
import ctypes as C

import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu

CASES = G.all_cases()


def _device_mesh(torch, xyz, f):
    from mcut_gb300 import _lib as L
    dv = torch.from_numpy(np.ascontiguousarray(xyz, dtype=np.float64)).cuda()
    df = torch.from_numpy(np.ascontiguousarray(f, dtype=np.uint32).view(np.int32)).cuda()
    return L.Mesh(dv.data_ptr(), df.data_ptr(), None, xyz.shape[0], f.shape[0] // 3), (dv, df)


def _noalloc(torch, lib, ms, mc, eps, cap):
    """One call; returns (rc, summary, ids [n,5], points [n,3])."""
    from mcut_gb300 import _lib as L
    ids = torch.full((max(cap, 1) * 5,), -1, dtype=torch.int32, device="cuda")
    pts = torch.full((max(cap, 1) * 3,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    sm = L.Summary()
    rc = lib.mcgpu_dispatch_noalloc(None, C.byref(ms), C.byref(mc), eps, ids.data_ptr(), pts.data_ptr(), cap,
                                    C.byref(sm))
    n = int(sm.num_records) if rc == L.OK else 0
    got_ids = ids.cpu().numpy().view(np.uint32)[: n * 5].reshape(-1, 5)
    got_pts = pts.cpu().numpy()[: n * 3].reshape(-1, 3)
    return rc, sm, got_ids, got_pts


def _reference_result(src, cut):
    """Recentred meshes and mcgpu_dispatch's result on them."""
    from mcut_gb300 import Context, recentre
    sx, cx, eps = recentre(src, cut)
    ctx = Context(0)
    want = ctx.dispatch(dict(v=sx, f=src["f"], fs=None), dict(v=cx, f=cut["f"], fs=None), cut_eps=eps,
                        recentre=False)
    ctx.close()
    return sx, cx, eps, want


# intersecting pairs (status OK), a general-position violation that still has
# records (the coplanar cube), degenerate faces (a zero-area source face and a
# benchmark pair with a collapsed face) and a vertex touching a face
@pytest.mark.parametrize("case", ["two_spheres", "crack1", "cube_coplanar_small_x16", "zero_area", "bm061",
                                  "vertex_on_face"])
def test_noalloc_matches_dispatch_twice(case):
    torch = pytest.importorskip("torch")
    from mcut_gb300 import _lib as L
    c = CASES[case]
    assert not int(c["float_input"]) and c["src"]["fs"] is None and c["cut"]["fs"] is None
    sx, cx, eps, want = _reference_result(c["src"], c["cut"])
    assert want.status == int(c["status"])

    lib = L.load()
    ms, keep_s = _device_mesh(torch, sx, c["src"]["f"])
    mc, keep_c = _device_mesh(torch, cx, c["cut"]["f"])
    cap = int(want.num_records) + 16
    for call in range(2):
        rc, sm, got_ids, got_pts = _noalloc(torch, lib, ms, mc, eps, cap)
        assert rc == L.OK, L.last_error()
        assert sm.status == want.status, (call, sm.status)
        assert sm.bad_face == want.bad_face, call
        assert sm.num_pairs == want.num_pairs and sm.num_tests == want.num_tests, call
        assert int(sm.num_records) == want.num_records, (call, sm.num_records)
        assert G.same_bits(got_ids, want.record_ids), call
        assert G.same_bits(got_pts, want.record_points), call
    del keep_s, keep_c


def test_noalloc_record_buffer_too_small():
    """More records than the caller's buffer holds: MCGPU_TOO_LARGE with the
    record count reported, and the next call with room gives the records."""
    torch = pytest.importorskip("torch")
    from mcut_gb300 import _lib as L
    c = CASES["crack1"]
    sx, cx, eps, want = _reference_result(c["src"], c["cut"])
    assert want.num_records > 0
    lib = L.load()
    ms, keep_s = _device_mesh(torch, sx, c["src"]["f"])
    mc, keep_c = _device_mesh(torch, cx, c["cut"]["f"])
    for cap in (0, int(want.num_records) - 1):
        rc, sm, _, _ = _noalloc(torch, lib, ms, mc, eps, cap)
        assert rc == L.TOO_LARGE and sm.status == L.TOO_LARGE
        assert int(sm.num_records) == want.num_records
    rc, sm, got_ids, got_pts = _noalloc(torch, lib, ms, mc, eps, int(want.num_records))
    assert rc == L.OK and sm.status == want.status
    assert G.same_bits(got_ids, want.record_ids) and G.same_bits(got_pts, want.record_points)
    del keep_s, keep_c


def test_noalloc_too_many_pairs():
    """Two overlapping 64 x 64 grids (15,876 faces, within the face limit)
    have more candidate pairs than the 32,768 the fixed array holds: the call
    reports the full pair count and MCGPU_TOO_LARGE."""
    torch = pytest.importorskip("torch")
    from mcut_gb300 import _lib as L
    from mcut_gb300 import meshgen
    src = meshgen.grid(64, 1.0)
    cut = meshgen.grid(64, 1.0)
    cut = dict(cut, v=cut["v"] + np.array([1.0 / 63.0, 1.0 / 63.0, 0.0]))
    sx, cx, eps, want = _reference_result(src, cut)
    assert want.num_pairs > 32768
    lib = L.load()
    ms, keep_s = _device_mesh(torch, sx, src["f"])
    mc, keep_c = _device_mesh(torch, cx, cut["f"])
    for _ in range(2):
        rc, sm, _, _ = _noalloc(torch, lib, ms, mc, eps, 16)
        assert rc == L.TOO_LARGE and sm.status == L.TOO_LARGE
        assert sm.num_pairs == want.num_pairs
    del keep_s, keep_c


@pytest.mark.parametrize("kind", ["cross_mesh", "wrapping", "far"])
def test_noalloc_index_outside_its_mesh(kind):
    """A source index naming a cut vertex, a cut index that wraps when offset
    by the source vertex count, and an index far past both: MCGPU_INVALID_INPUT
    as mcgpu_dispatch and the oracle report it, and the next valid call is
    unaffected."""
    torch = pytest.importorskip("torch")
    import oracle
    from mcut_gb300 import _lib as L
    c = CASES["two_spheres"]
    src = dict(c["src"], f=c["src"]["f"].copy())
    cut = dict(c["cut"], f=c["cut"]["f"].copy())
    vs = src["v"].shape[0]
    if kind == "cross_mesh":
        src["f"][7] = vs + 1
    elif kind == "wrapping":
        cut["f"][4] = 0xFFFFFFFF - vs + 2
    else:
        src["f"][5] = 1_000_000_000
    assert oracle.front_end(src, cut, impl="port")["status"] == oracle.FE_INVALID_INPUT
    from mcut_gb300 import Context, recentre
    sx, cx, eps = recentre(c["src"], c["cut"])  # the coordinates alone set the frame
    ctx = Context(0)
    bad = ctx.dispatch(dict(v=sx, f=src["f"], fs=None), dict(v=cx, f=cut["f"], fs=None), cut_eps=eps,
                       recentre=False)
    ctx.close()
    assert bad.status == L.INVALID_INPUT
    lib = L.load()
    ms, keep_s = _device_mesh(torch, sx, src["f"])
    mc, keep_c = _device_mesh(torch, cx, cut["f"])
    rc, sm, _, _ = _noalloc(torch, lib, ms, mc, eps, 256)
    assert rc == L.OK and sm.status == L.INVALID_INPUT
    ms2, keep_s2 = _device_mesh(torch, sx, c["src"]["f"])
    mc2, keep_c2 = _device_mesh(torch, cx, c["cut"]["f"])
    rc, sm, got_ids, _ = _noalloc(torch, lib, ms2, mc2, eps, 256)
    assert rc == L.OK and sm.status == L.OK and int(sm.num_records) == 169
    del keep_s, keep_c, keep_s2, keep_c2


def test_noalloc_rejects_oversized_input():
    from mcut_gb300 import _lib as L
    from mcut_gb300 import meshgen
    lib = L.load()
    big = meshgen.icosphere(5)  # 20480 faces: beyond the 16384-face limit
    v = np.ascontiguousarray(big["v"])
    f = np.ascontiguousarray(big["f"])
    m = L.Mesh(v.ctypes.data, f.ctypes.data, None, v.shape[0], f.shape[0] // 3)
    sm = L.Summary()
    rc = lib.mcgpu_dispatch_noalloc(None, C.byref(m), C.byref(m), 1e-4, None, None, 0, C.byref(sm))
    assert rc == L.TOO_LARGE and sm.status == L.TOO_LARGE


def test_noalloc_null_argument_sets_status():
    from mcut_gb300 import _lib as L
    lib = L.load()
    sm = L.Summary()
    sm.status = 12345
    rc = lib.mcgpu_dispatch_noalloc(None, None, None, 1e-4, None, None, 0, C.byref(sm))
    assert rc == L.INVALID_VALUE and sm.status == L.INVALID_VALUE


def test_noalloc_refuses_a_capturing_stream():
    """The call waits for its stream between stages, which a stream being
    captured into a CUDA graph cannot do: on such a stream it returns
    MCGPU_INVALID_VALUE before any GPU work, the caller's capture stays valid
    (it ends without error and replays), and the next call outside the
    capture gives the allocating entry point's records."""
    import torch
    from mcut_gb300 import _lib as L
    lib = L.load()
    c = CASES["two_spheres"]
    sx, cx, eps, want = _reference_result(c["src"], c["cut"])
    ms, k1 = _device_mesh(torch, sx, c["src"]["f"])
    mc, k2 = _device_mesh(torch, cx, c["cut"]["f"])
    ids = torch.zeros(5 * 4096, dtype=torch.int32, device="cuda")
    pts = torch.zeros(3 * 4096, dtype=torch.float64, device="cuda")
    x = torch.zeros(8, device="cuda")
    g = torch.cuda.CUDAGraph()
    sm = L.Summary()
    with torch.cuda.graph(g):
        x += 1.0  # the caller's own captured work
        rc = lib.mcgpu_dispatch_noalloc(C.c_void_p(torch.cuda.current_stream().cuda_stream), C.byref(ms),
                                        C.byref(mc), eps, ids.data_ptr(), pts.data_ptr(), 4096, C.byref(sm))
    assert rc == L.INVALID_VALUE and sm.status == L.INVALID_VALUE
    g.replay()
    torch.cuda.synchronize()
    assert float(x[0]) == 1.0
    rc, sm, got_ids, got_pts = _noalloc(torch, lib, ms, mc, eps, 4096)
    assert rc == L.OK and sm.status == want.status
    assert np.array_equal(got_ids, want.record_ids) and G.same_bits(got_pts, want.record_points)
