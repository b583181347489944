"""A connected component's wire format (mcGetConnectedComponentData,
frontend.cpp:2006-2832), restated from its halfedge mesh.

MCUT serialises a component from its halfedge mesh: each face's vertices as
the targets of its halfedges (get_vertices_around_face, hmesh.cpp:705-733),
the faces across them (get_faces_around_face, hmesh.cpp:796-818) with their
counts, each edge as vertex(e, 0), vertex(e, 1) (hmesh.cpp:234-256), the
vertices as doubles and as static_cast<float>. The restatement
(oracle.cc_wire_of_hmesh) builds the halfedge mesh of the component's faces
in its corner order (each serialised face list rotated back by one,
oracle.cc_corners) with the oracle port and derives the same arrays. Against
the reference's own output for every component of every fixture dispatch
(tests/golden/cc_wire.npz): faces, adjacency, counts and float vertices bit
for bit; edges as the same undirected edges, in MCUT's own order and
direction wherever MCUT's component mesh created its edges face by face (616 of 643; the others
list them in their construction order, or from the face that made each edge
first, neither of which the serialised arrays carry).
"""
import numpy as np
import pytest

import cc_wire_cases
import oracle

CCS = cc_wire_cases.load()


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build()


def restate(w):
    corners = oracle.cc_corners(w["face"], w["fsize"])
    tri = bool(np.all(w["fsize"] == 3))
    h = oracle.hmesh(corners, None if tri else w["fsize"], len(w["vd"]), impl="port")
    assert h["status"] in (oracle.HM_OK, oracle.HM_TOO_SMALL, oracle.HM_COMPONENTS)
    return oracle.cc_wire_of_hmesh(h, w["fsize"], w["vd"])


def test_fixture_components():
    assert len(CCS) > 600 and len({n for n, _, _ in CCS}) > 60


def test_restatement_equals_mcut_serialisation():
    same_order = 0
    for name, k, w in CCS:
        r = restate(w)
        assert np.array_equal(r["face"], w["face"]), (name, k)
        assert np.array_equal(r["adjsize"], w["adjsize"]), (name, k)
        assert np.array_equal(r["adj"], w["adj"]), (name, k)
        assert np.array_equal(r["vf"].view(np.uint32), w["vf"].view(np.uint32)), (name, k)
        a, b = r["edge"].reshape(-1, 2), w["edge"].reshape(-1, 2)
        und = lambda e: sorted(map(lambda x: tuple(sorted(x)), e.tolist()))  # noqa: E731
        assert und(a) == und(b), (name, k)
        same_order += int(np.array_equal(a, b))
    # MCUT's own edge order and direction wherever its component mesh made its
    # edges face by face (616 of the 643 fixture components)
    assert same_order >= 0.95 * len(CCS), same_order


def test_rotation_is_needed():
    """Planted mistake: the serialised face lists taken as the corner order
    (not rotated back) give the faces shifted by one corner."""
    name, k, w = next(c for c in CCS if len(c[2]["fsize"]) > 4)
    tri = bool(np.all(w["fsize"] == 3))
    h = oracle.hmesh(w["face"], None if tri else w["fsize"], len(w["vd"]), impl="port")
    r = oracle.cc_wire_of_hmesh(h, w["fsize"], w["vd"])
    assert not np.array_equal(r["face"], w["face"])
