"""The record hand-over built on the device equals the oracle's, bit for bit.

What dispatch()'s host stages read from the narrow phase (kernel.cpp:2599-2655,
merged at 2673-2714): the records in canonical order with their edges' faces
(record i is m0's intersection vertex Vs + Vc + i), ps_intersecting_edges,
cutpath_edge_creation_info, ps_iface_to_ivtx_list,
cm_border_reentrant_ivtx_list and partial_cut_detected. The oracle
(oracle_seam) restates that loop serially over the fixture's records; the
device builds the same arrays with sorts and scans. Order, ids and point bits
must all be equal.
"""
import os

import numpy as np
import pytest

import golden_cases as G
import oracle
from mcut_gb300 import meshgen

pytestmark = pytest.mark.gpu

CASES = G.all_cases()
# every fixture whose front end ran its narrow phase and kept records
WITH_RECORDS = sorted(k for k, c in CASES.items() if int(c["status"]) in (0, 1) and len(c["rec_ids"]) > 0)
MAPS = ["edge_off", "cp_pairs", "cp_off", "cp_vtx", "face_keys", "face_off", "face_vtx", "border"]


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def check(ctx, r, want):
    assert G.same_bits(r.record_ids, want["rec_ids"])
    assert G.same_bits(r.record_points, want["rec_pts"])
    got = ctx.hand_over()
    for k in MAPS:
        assert G.same_bits(got[k].reshape(want[k].shape), want[k]), k
    assert got["partial_cut"] == (len(want["border"]) > 0)


@pytest.mark.parametrize("name", WITH_RECORDS)
def test_hand_over_fixture(ctx, name):
    c = CASES[name]
    r = ctx.dispatch(c["src"], c["cut"], float_input=bool(c["float_input"]))
    assert r.status == int(c["status"])
    check(ctx, r, oracle.seam(c["src"], c["cut"], c["rec_ids"], c["rec_pts"]))


def test_hand_over_mid_size(ctx):
    s, c = meshgen.sphere_heightfield(16.0, level=6, n=256)
    want = oracle.front_end(s, c, impl="port", threads=8)
    r = ctx.dispatch(s, c)
    assert r.status == want["status"] == 0
    check(ctx, r, oracle.seam(s, c, want["rec_ids"], want["rec_pts"]))


def test_hand_over_empty_and_batch(ctx):
    from mcut_gb300 import _lib as L
    c = CASES["disjoint"]
    r = ctx.dispatch(c["src"], c["cut"])
    assert r.num_records == 0
    got = ctx.hand_over()
    assert list(got["edge_off"]) == [0] and list(got["cp_off"]) == [0] and list(got["face_off"]) == [0]
    assert all(len(got[k]) == 0 for k in ("cp_pairs", "cp_vtx", "face_keys", "face_vtx", "border"))
    assert not got["partial_cut"]
    # the maps follow the last dispatch; a batch has none
    ctx.dispatch_batch([(CASES["crack1"]["src"], CASES["crack1"]["cut"])] * 2)
    with pytest.raises(RuntimeError):
        ctx._get(L.DATA_CUTPATH_PAIRS, np.uint32, 2)


PASSES = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "seam_passes.npz"))
REENTRY = sorted((k[: -len("/passes")], p) for k in PASSES.files if k.endswith("/passes")
                 for p in range(1, int(PASSES[k])))


@pytest.mark.parametrize("name,k", REENTRY)
def test_hand_over_reentry_pass(ctx, name, k):
    """The meshes MCUT's host stages send back through the front end after a
    first pass (floating polygons, kernel.cpp:4078-4200 / preproc.cpp
    re-dispatch), recorded at the seam: the device's hand-over equals the
    oracle's on them too."""
    def mesh(side):
        fs = PASSES[f"{name}/p{k}/{side}_fs"]
        return dict(v=PASSES[f"{name}/p{k}/{side}_v"], f=PASSES[f"{name}/p{k}/{side}_f"], fs=fs if fs.size else None)
    s, c = mesh("src"), mesh("cut")
    eps = float(PASSES[f"{name}/p{k}/eps"])
    want = oracle.front_end_internal(s, c, eps)
    r = ctx.dispatch(s, c, cut_eps=eps, recentre=False)
    assert r.status == want["status"]
    if r.status in (0, 1):
        check(ctx, r, oracle.seam(s, c, want["rec_ids"], want["rec_pts"]))
