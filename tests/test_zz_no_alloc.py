"""mcgpu_dispatch_noalloc returns exactly what mcgpu_dispatch returns.

That entry point serves callers that must not allocate GPU memory while they
ask for intersection records (a thread recording a CUDA graph, a plugin held
to its host application's memory arena, a frame loop that cannot wait on the
allocator): its scratch is one static device array, the caller supplies
device inputs and device output buffers. Here it runs twice in a row -- the
second call sees the first call's leftovers in the shared array -- and each
result must equal the allocating entry point's, bit for bit.

This file is collected last so that a failure here cannot hide another test.
"""
import ctypes as C

import numpy as np
import pytest

import golden_cases as G

pytestmark = pytest.mark.gpu


def _device_mesh(torch, xyz, f):
    from mcut_gb300 import _lib as L
    dv = torch.from_numpy(np.ascontiguousarray(xyz, dtype=np.float64)).cuda()
    df = torch.from_numpy(np.ascontiguousarray(f, dtype=np.uint32).view(np.int32)).cuda()
    return L.Mesh(dv.data_ptr(), df.data_ptr(), None, xyz.shape[0], f.shape[0] // 3), (dv, df)


@pytest.mark.parametrize("case", ["two_spheres", "crack1"])
def test_noalloc_matches_dispatch_twice(case):
    torch = pytest.importorskip("torch")
    from mcut_gb300 import Context, recentre
    from mcut_gb300 import _lib as L
    c = G.load("synthetic.npz")[case]
    sx, cx, eps = recentre(c["src"], c["cut"])

    ctx = Context(0)
    want = ctx.dispatch(dict(v=sx, f=c["src"]["f"], fs=None), dict(v=cx, f=c["cut"]["f"], fs=None),
                        cut_eps=eps, recentre=False)
    ctx.close()
    assert want.status == 0 and want.num_records > 0

    lib = L.load()
    ms, keep_s = _device_mesh(torch, sx, c["src"]["f"])
    mc, keep_c = _device_mesh(torch, cx, c["cut"]["f"])
    cap = int(want.num_records) + 16
    for call in range(2):
        ids = torch.full((cap * 5,), -1, dtype=torch.int32, device="cuda")
        pts = torch.full((cap * 3,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        sm = L.Summary()
        rc = lib.mcgpu_dispatch_noalloc(None, C.byref(ms), C.byref(mc), eps, ids.data_ptr(), pts.data_ptr(), cap,
                                        C.byref(sm))
        assert rc == L.OK, L.last_error()
        assert sm.status == want.status
        n = int(sm.num_records)
        assert n == want.num_records, (call, n)
        got_ids = ids.cpu().numpy().view(np.uint32)[: n * 5].reshape(-1, 5)
        got_pts = pts.cpu().numpy()[: n * 3].reshape(-1, 3)
        assert G.same_bits(got_ids, want.record_ids), call
        assert G.same_bits(got_pts, want.record_points), call
    del keep_s, keep_c


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
