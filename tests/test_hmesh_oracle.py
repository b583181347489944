"""MCUT's input-mesh conversion and checks: oracle port, reference, and the
data-parallel formulation a device pass would use.

The port (oracle/hmesh_oracle.c) restates how MCUT turns one mesh's arrays
into its halfedge mesh (client_input_arrays_to_hmesh, preproc.cpp:390-460;
hmesh_t::add_face / add_edge, hmesh.cpp:406-651) and what check_input_mesh
rejects (preproc.cpp:505-579). Against the reference's own hmesh_t (harness,
where the reference checkout exists) it must agree on the status, the face
a conversion error stops at, the edge count, and per halfedge its target,
face, next and prev, per face corner its halfedge, per vertex its halfedge
list, the component count and closedness (mesh_is_closed,
preproc.cpp:1957-1994): on every fixture mesh, the polygon soups the
front end numbers its edges in, seeded random meshes, and seeded corruptions
of each kind MCUT rejects.

`parallel_hmesh` restates the same result with sorts, scans and label
propagation only (no face-order loop): the formulation for the device. It
must equal the port everywhere.
"""
import os
import zlib

import numpy as np
import pytest

import fuzz_cases as F
import golden_cases as G
import oracle

HAVE_REF = oracle.ref_available()
CASES = G.all_cases()
ARRAYS = ["he_target", "he_face", "he_next", "he_prev", "corner_he", "v_off", "v_he"]


@pytest.fixture(scope="module", autouse=True)
def _build():
    oracle.build(ref=HAVE_REF)


def _faces(m):
    f = np.asarray(m["f"], dtype=np.int64)
    fs = m.get("fs")
    return f, (None if fs is None else np.asarray(fs, dtype=np.int64))


def soup(src, cut):
    """The front end's polygon soup: source faces as given, then the cut faces
    as the soup re-adds them (vertex lists rotated by one, the targets of each
    face's halfedges, kernel.cpp:1593-1732) with ids offset by the source
    vertex count."""
    fs_s, fs_c = src.get("fs"), cut.get("fs")
    ns = np.full(len(src["f"]) // 3, 3) if fs_s is None else np.asarray(fs_s, dtype=np.int64)
    nc = np.full(len(cut["f"]) // 3, 3) if fs_c is None else np.asarray(fs_c, dtype=np.int64)
    cf = np.asarray(cut["f"], dtype=np.int64) + len(src["v"])
    off = np.concatenate([[0], np.cumsum(nc)])
    rot = [np.roll(cf[off[i]:off[i + 1]], -1) for i in range(len(nc))]
    f = np.concatenate([np.asarray(src["f"], dtype=np.int64)] + rot)
    fs = None if fs_s is None and fs_c is None else np.concatenate([ns, nc])
    return f, fs, len(src["v"]) + len(cut["v"])


def parallel_hmesh(f, fs, nv):
    """The halfedge mesh and checks from sorts, scans and label propagation."""
    f = np.asarray(f, dtype=np.int64)
    nf = len(f) // 3 if fs is None else len(fs)
    n = np.full(nf, 3, np.int64) if fs is None else np.asarray(fs, dtype=np.int64)
    off = np.concatenate([[0], np.cumsum(n)])
    face = np.repeat(np.arange(nf), n)
    slot = np.arange(int(off[-1]))
    # per-face errors, corner by corner: an index out of range, else an index
    # an earlier corner of the face holds (equal (face, index) neighbours in a
    # sort by (face, index, slot)); a face of fewer than 3 corners fails first
    bad_range = f >= nv
    o = np.lexsort((slot, f, face))
    later = np.zeros(len(f), bool)
    later[o[1:]] = (face[o][1:] == face[o][:-1]) & (f[o][1:] == f[o][:-1])
    bad_dup = later & ~bad_range
    bad_face, bad_code = nf, oracle.HM_OK
    small = np.nonzero(n < 3)[0]
    if len(small):
        bad_face, bad_code = int(small[0]), oracle.HM_FACE_SIZE
    err = np.nonzero(bad_range | bad_dup)[0]
    if len(err) and face[err[0]] < bad_face:
        bad_face = int(face[err[0]])
        bad_code = oracle.HM_INDEX_RANGE if bad_range[err[0]] else oracle.HM_DUPLICATE_INDEX
    # halfedges of the faces before the first failing one
    m = int(off[bad_face])
    f, face, slot = f[:m], face[:m], slot[:m]
    nxt = slot + 1
    last = off[1:bad_face + 1] - 1
    nxt[last] = off[:bad_face]  # the corner after a face's last is its first
    v0, v1 = f, f[nxt]
    key = np.minimum(v0, v1) << 32 | np.maximum(v0, v1)
    # first appearance of each undirected edge: a stable sort keeps slot order within a key
    order = np.argsort(key, kind="stable")
    ks = key[order]
    start = np.concatenate([[True], ks[1:] != ks[:-1]]) if m else np.zeros(0, bool)
    grp = np.cumsum(start) - 1
    first_slot = order[start]
    is_first = np.zeros(m, bool)
    is_first[first_slot] = True
    eid_at_slot = np.cumsum(is_first) - 1  # edge id = rank of its first slot in slot order
    first_of = np.empty(m, np.int64)
    first_of[order] = first_slot[grp]
    h = 2 * eid_at_slot[first_of] + (v1 != v1[first_of])
    # a directed halfedge twice: the face of its later slot fails
    oh = np.argsort(h, kind="stable")
    rep = np.zeros(m, bool)
    rep[oh[1:]] = h[oh][1:] == h[oh][:-1]
    if rep.any():
        return dict(status=oracle.HM_NON_MANIFOLD, bad_face=int(face[rep].min()), n_edges=0, n_components=0,
                    closed=False)
    if bad_code != oracle.HM_OK:
        return dict(status=bad_code, bad_face=bad_face, n_edges=0, n_components=0, closed=False)
    ne = int(is_first.sum())
    he_target = np.empty(2 * ne, np.int64)
    he_target[2 * eid_at_slot[first_slot]] = v1[first_slot]
    he_target[2 * eid_at_slot[first_slot] + 1] = v0[first_slot]
    he_face = np.full(2 * ne, -1, np.int64)
    he_face[h] = face
    he_next = np.full(2 * ne, -1, np.int64)
    he_prev = np.full(2 * ne, -1, np.int64)
    he_next[h] = h[nxt]
    he_prev[h[nxt]] = h
    # each vertex's halfedges in creation order = ascending halfedge id per target
    v_off = np.concatenate([[0], np.cumsum(np.bincount(he_target, minlength=nv))])
    out = dict(status=oracle.HM_OK, bad_face=-1, n_edges=ne, n_components=0, closed=bool(np.all(he_face >= 0)),
               he_target=he_target,
               he_face=he_face, he_next=he_next, he_prev=he_prev, corner_he=h, v_off=v_off,
               v_he=np.argsort(he_target, kind="stable"))
    if nv < 3 or nf < 1:
        out["status"] = oracle.HM_TOO_SMALL
        return out
    # connected components: min-label hooking and pointer jumping until stable
    lab = np.arange(nv)
    a, b = he_target[0::2], he_target[1::2]
    while True:
        lo = np.minimum(lab[a], lab[b])
        new = lab.copy()
        np.minimum.at(new, lab[a], lo)
        np.minimum.at(new, lab[b], lo)
        new = new[new]
        if np.array_equal(new, lab):
            break
        lab = new
    nc = int(np.sum(lab == np.arange(nv)))
    out["n_components"] = nc
    if nc != 1:
        out["status"] = oracle.HM_COMPONENTS
    return out


def _same(a, b):
    for k in ("status", "bad_face", "n_edges", "n_components", "closed"):
        assert a[k] == b[k], (k, a[k], b[k])
    for k in ARRAYS:
        if k in a or k in b:
            assert np.array_equal(np.asarray(a[k], np.int64), np.asarray(b[k], np.int64)), k


def _check(f, fs, nv):
    port = oracle.hmesh(f, fs, nv, "port")
    _same(parallel_hmesh(f, fs, nv), port)
    if HAVE_REF:
        _same(oracle.hmesh(f, fs, nv, "ref"), port)
    return port


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_meshes(name):
    c = CASES[name]
    for m in (c["src"], c["cut"]):
        f, fs = _faces(m)
        _check(f, fs, len(m["v"]))


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_polygon_soups(name):
    c = CASES[name]
    f, fs, nv = soup(c["src"], c["cut"])
    r = _check(f, fs, nv)
    assert r["status"] in (oracle.HM_OK, oracle.HM_COMPONENTS)


def test_random_meshes():
    fams = F.fracture(0, 10) + F.lattice(0, 10) + F.quads(0.05, 5)
    for s, c, _ in fams:
        for m in (s, c):
            f, fs = _faces(m)
            _check(f, fs, len(m["v"]))
        _check(*soup(s, c))


def test_records_run_along_primary_halfedges():
    """A record's edge (q, r) is the soup's primary halfedge 2e of its edge e:
    q is the target of 2e+1 and r the target of 2e. That is the reference's
    edge id of each record for the host stages."""
    for name, c in sorted(CASES.items()):
        if not len(c["rec_ids"]):
            continue
        f, fs, nv = soup(c["src"], c["cut"])
        r = oracle.hmesh(f, fs, nv, "port")
        prim = {(int(r["he_target"][2 * e + 1]), int(r["he_target"][2 * e])): e for e in range(r["n_edges"])}
        for q, rr, _ in c["rec_ids"]:
            assert (int(q), int(rr)) in prim, name


def _corruptions(rng, m):
    """Seeded broken copies of one valid mesh, one per kind MCUT rejects."""
    f, fs = _faces(m)
    nv = len(m["v"])
    nf = len(f) // 3 if fs is None else len(fs)
    sizes = np.full(nf, 3) if fs is None else fs
    off = np.concatenate([[0], np.cumsum(sizes)])
    out = []
    g = int(rng.integers(nf))
    # a face of two vertices
    fs2 = sizes.copy()
    fs2[g] -= 1
    keep = np.ones(len(f), bool)
    keep[off[g + 1] - 1] = False
    if fs2[g] < 3:
        out.append(("face_size", f[keep], fs2, nv))
    # an index out of range
    f2 = f.copy()
    f2[off[g] + int(rng.integers(sizes[g]))] = nv + int(rng.integers(1, 5))
    out.append(("index_range", f2, fs, nv))
    # a vertex twice in one face
    f3 = f.copy()
    f3[off[g] + 1] = f3[off[g]]
    out.append(("duplicate", f3, fs, nv))
    # a face turned over: its halfedges now run the same way as its neighbours'
    f4 = f.copy()
    f4[off[g]:off[g + 1]] = f4[off[g]:off[g + 1]][::-1]
    out.append(("flipped", f4, fs, nv))
    # a face repeated at the end
    f5 = np.concatenate([f, f[off[g]:off[g + 1]]])
    fs5 = None if fs is None else np.concatenate([fs, [sizes[g]]])
    out.append(("repeated", f5, fs5, nv))
    # a vertex no face uses
    out.append(("unused_vertex", f, fs, nv + 1))
    # two copies side by side
    f7 = np.concatenate([f, f + nv])
    fs7 = None if fs is None else np.concatenate([fs, fs])
    out.append(("two_components", f7, fs7, 2 * nv))
    # too small
    out.append(("no_face", np.zeros(0, np.int64), None if fs is None else np.zeros(0, np.int64), nv))
    return out


@pytest.mark.parametrize("name", ["two_spheres", "bm014", "bm029", "quad_pent", "crack1", "bunny_plane"])
def test_corrupted_inputs(name):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    kinds = {}
    for m in (CASES[name]["src"], CASES[name]["cut"]):
        for _ in range(3):
            for kind, f, fs, nv in _corruptions(rng, m):
                kinds.setdefault(kind, set()).add(_check(f, fs, nv)["status"])
    assert kinds["index_range"] == {oracle.HM_INDEX_RANGE}
    assert kinds["duplicate"] == {oracle.HM_DUPLICATE_INDEX}
    assert kinds["repeated"] == {oracle.HM_NON_MANIFOLD}
    assert kinds["two_components"] == {oracle.HM_COMPONENTS}
    assert kinds["unused_vertex"] == {oracle.HM_COMPONENTS}
    assert kinds["no_face"] == {oracle.HM_TOO_SMALL}


def test_closedness():
    """A sphere is closed, a height-field grid is not; the soup of the two is
    not (the grid's border halfedges have no face)."""
    c = CASES["sphere_hf_small"]
    for m, want in ((c["src"], True), (c["cut"], False)):
        f, fs = _faces(m)
        assert _check(f, fs, len(m["v"]))["closed"] is want
    assert _check(*soup(c["src"], c["cut"]))["closed"] is False


def test_record_order_key_against_the_soup_edge_numbering():
    """The device orders records by the slot of the edge's first face corner in
    the source-then-cut face arrays (then face). On source-mesh edges that is
    MCUT's edge numbering in the soup. Cut faces re-enter the soup rotated by
    one, so their edges are numbered in a cyclic shift of the corner order.
    This test checks both statements on every fixture with records."""
    for name, c in sorted(CASES.items()):
        if not len(c["rec_ids"]):
            continue
        src, cut = c["src"], c["cut"]
        f, fs, nv = soup(src, cut)
        r = oracle.hmesh(f, fs, nv, "port")
        eid = {(int(r["he_target"][2 * e + 1]), int(r["he_target"][2 * e])): e for e in range(r["n_edges"])}
        nsv = len(src["v"])
        raw = np.concatenate([np.asarray(src["f"], np.int64), np.asarray(cut["f"], np.int64) + nsv])
        n = (np.full(len(raw) // 3, 3) if src.get("fs") is None and cut.get("fs") is None else
             np.concatenate([np.full(len(src["f"]) // 3, 3) if src.get("fs") is None else np.asarray(src["fs"]),
                             np.full(len(cut["f"]) // 3, 3) if cut.get("fs") is None else np.asarray(cut["fs"])]))
        first, o = {}, 0
        for k in n:
            for j in range(int(k)):
                a, b = int(raw[o + j]), int(raw[o + (j + 1) % int(k)])
                first.setdefault((min(a, b), max(a, b)), o + j)
            o += int(k)
        src_recs = [(int(q), int(rr), int(g)) for q, rr, g in c["rec_ids"] if int(q) < nsv]
        by_slot = sorted(src_recs, key=lambda t: (first[(min(t[0], t[1]), max(t[0], t[1]))], t[2]))
        by_edge = sorted(src_recs, key=lambda t: (eid[(t[0], t[1])], t[2]))
        assert by_slot == by_edge, name
