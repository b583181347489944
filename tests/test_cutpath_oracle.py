"""The cut-path oracle equals MCUT's own cut-path edge creation.

oracle/cutpath_oracle.c restates kernel.cpp:3332-3632: the edges of the cut
path made from cutpath_edge_creation_info (two vertices: one edge; more:
sorted along their line, consecutive pairs joined where the midpoint lies
inside exactly two shared faces), each edge's place in the per-face edge
lists (with the faces across the two faces' edges,
update_neighouring_ps_iface_m0_edge_list) and the halfedges entering each
intersection vertex. The reference's own stage is observed inside the
unmodified mcDispatch (the seam copy's cut-path observer, oracle/make_seam.py)
with its inputs; the oracle, given those inputs, must give its outputs
exactly: edge for edge in creation order, each face's list in order, each
vertex's halfedges in order.

Skipped where the seam harness is neither built nor buildable (set
MCUT_REF_ROOT).
"""
import numpy as np
import pytest

import golden_cases as G
import oracle
from test_seam_fragments import WITH_CCS, _user_meshes

pytestmark = pytest.mark.skipif(not oracle.seam_available(),
                                reason="seam harness not built and MCUT_REF_ROOT unset")

CASES = G.all_cases()
KEYS = ["edges", "face_keys", "face_off", "face_edges", "ivtx_off", "ivtx_he"]


def _run(o):
    return oracle.cutpath(o["nv"], o["x"], o["soup_off"], o["soup_idx"], o["reg"], o["ivtx_xyz"], o["cp_pairs"],
                          o["cp_off"], o["cp_vtx"])


@pytest.mark.parametrize("name", WITH_CCS)
def test_oracle_equals_mcut_cutpath_stage(name):
    c = CASES[name]
    src, cut, flags = _user_meshes(c)
    result, obs = oracle.observe_cutpath(src, cut, flags=flags)
    if not obs:
        pytest.skip(f"the dispatch stopped before the cut path (result {result})")
    for o in obs:
        assert o["bad"] == 0
        got = _run(o)
        assert got["status"] == 0
        for k in KEYS:
            assert np.array_equal(got[k], o["want"][k]), (name, k)


def test_lists_longer_than_two_are_covered():
    """Among the benchmark pairs, keys with more than two intersection
    vertices (sorted along their line, midpoints tested) occur and match."""
    longest = 0
    for name in ("bm002", "bm006", "bm034", "bm036"):
        c = CASES[name]
        src, cut, flags = _user_meshes(c)
        _, obs = oracle.observe_cutpath(src, cut, flags=flags)
        for o in obs:
            longest = max(longest, int(np.diff(o["cp_off"]).max()))
            got = _run(o)
            for k in KEYS:
                assert np.array_equal(got[k], o["want"][k]), (name, k)
    assert longest > 2


def test_fewer_than_two_vertices_stop_the_dispatch():
    """A key holding one intersection vertex: the stage reports it (the
    reference ends the dispatch there)."""
    c = CASES["two_spheres"]
    src, cut, flags = _user_meshes(c)
    _, obs = oracle.observe_cutpath(src, cut, flags=flags)
    o = dict(obs[-1])
    off = np.array(o["cp_off"], np.int64)
    vtx = np.array(o["cp_vtx"], np.int64)
    # drop the second vertex of the first key
    vtx = np.delete(vtx, off[0] + 1)
    off[1:] -= 1
    o["cp_vtx"], o["cp_off"] = vtx.astype(np.uint32), off.astype(np.uint32)
    got = _run(o)
    assert got["status"] == 1 and got["bad_key"] == 0
