"""The connected-component wire format on the device (mcgpu_halfedge_mesh on a
component's faces in corner order, queries 37-41) against the restatement
and against MCUT's own mcGetConnectedComponentData output for every
component of every fixture dispatch (tests/golden/cc_wire.npz)."""
import numpy as np
import pytest

import cc_wire_cases
import oracle
from test_cc_wire_oracle import restate

pytestmark = pytest.mark.gpu

CCS = cc_wire_cases.load()


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _cc(w):
    tri = bool(np.all(w["fsize"] == 3))
    return dict(v=w["vd"], f=oracle.cc_corners(w["face"], w["fsize"]), fs=None if tri else w["fsize"])


def test_device_equals_restatement_and_mcut(ctx):
    same_edges = 0
    for name, k, w in CCS:
        g = ctx.cc_wire(_cc(w))
        r = restate(w)
        for key in ("face", "adjsize", "adj", "edge"):
            assert np.array_equal(g[key], r[key]), (name, k, key)
        assert np.array_equal(g["vf"].reshape(-1).view(np.uint32), r["vf"].reshape(-1).view(np.uint32)), (name, k)
        # MCUT's own arrays
        for key in ("face", "adjsize", "adj"):
            assert np.array_equal(g[key], w[key]), (name, k, key)
        assert np.array_equal(g["vf"].reshape(-1).view(np.uint32), w["vf"].reshape(-1).view(np.uint32)), (name, k)
        same_edges += int(np.array_equal(g["edge"], w["edge"]))
    assert same_edges >= 0.95 * len(CCS)


def test_device_pointers_and_large_component(ctx):
    """A large component from device arrays: the C2x16 cut mesh (a 1024 x 1024
    grid) taken as one component, against the restatement."""
    torch = pytest.importorskip("torch")
    from mcut_gb300 import meshgen
    _, cut = meshgen.sphere_heightfield(16.0)
    f = np.asarray(cut["f"], np.uint32)
    dv = torch.from_numpy(np.ascontiguousarray(cut["v"], np.float64)).cuda()
    df = torch.from_numpy(f.view(np.int32)).cuda()
    g = ctx.cc_wire(dict(v=dv, f=df, fs=None), device=True)
    h = oracle.hmesh(f, None, len(cut["v"]), impl="port")
    r = oracle.cc_wire_of_hmesh(h, np.full(len(f) // 3, 3, np.uint32), cut["v"])
    for key in ("face", "adjsize", "adj", "edge"):
        assert np.array_equal(g[key], r[key]), key
    assert np.array_equal(g["vf"].reshape(-1).view(np.uint32), r["vf"].reshape(-1).view(np.uint32))


def test_queries_need_a_halfedge_mesh():
    from mcut_gb300 import Context
    from mcut_gb300 import _lib as L
    c = Context(0)
    with pytest.raises(RuntimeError, match="INVALID_VALUE"):
        c._get(L.DATA_CC_FACE, np.uint32, 1)
    # no vertices given: the float vertices are not available, the rest is
    m = dict(f=np.arange(3, dtype=np.uint32), fs=None, nv=3)
    c.halfedge_mesh(m)
    assert np.array_equal(c._get(L.DATA_CC_FACE, np.uint32, 1).reshape(-1), [1, 2, 0])
    with pytest.raises(RuntimeError, match="INVALID_VALUE"):
        c._get(L.DATA_CC_VERTEX_FLOAT, np.float32, 1)
    c.close()
