"""GPU front end vs the reference (golden fixtures) and the pinned oracle.

Bit-exact bar: candidate pairs, every culled edge-face test with both
orient3d signs, its type char and point-in-polygon char, the status
(general-position violation / degenerate face), and every intersection
point (compared as raw fp64 bits: 0 ulp).
"""
import numpy as np
import pytest

import golden_cases as G
import oracle
from gpu_util import canonical_records, canonical_tests, sort_rows
from mcut_gb300 import meshgen

pytestmark = pytest.mark.gpu

CASES = G.all_cases()


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def check_against(r, want, nsf):
    assert r.status == int(want["status"]), (r.status_name, int(want["status"]))
    assert r.bad_face == int(want["bad_face"])
    assert G.same_bits(r.cut_eps, want["cut_eps"])
    pairs = sort_rows(r.pairs, [0, 1])
    assert G.same_bits(pairs, want["pairs"])
    if int(want["status"]) in (2, 3):
        return  # the reference stops before the narrow phase
    t, info = canonical_tests(r.tests, r.test_info)
    assert G.same_bits(t, want["tests"])
    assert G.same_bits(info, want["test_info"])
    ids, pts = canonical_records(r.record_ids, r.record_points)
    assert G.same_bits(ids, want["rec_ids"])
    assert G.same_bits(pts, want["rec_pts"])


@pytest.mark.parametrize("name", sorted(CASES))
def test_golden_case(ctx, name):
    c = CASES[name]
    r = ctx.dispatch(c["src"], c["cut"], float_input=bool(c["float_input"]), keep_tests=True, keep_pairs=True)
    check_against(r, c, meshgen.num_faces(c["src"]))


def test_records_carry_edge_faces(ctx):
    c = CASES["two_spheres"]
    r = ctx.dispatch(c["src"], c["cut"], keep_tests=True, keep_pairs=True)
    nsf = meshgen.num_faces(c["src"])
    ids = r.record_ids
    assert len(ids) == 169
    # an edge's faces come from its own mesh, the tested face from the other
    src_edge = ids[:, 3] < nsf
    assert np.all((ids[:, 2] >= nsf) == src_edge)
    assert np.all((ids[:, 4] == 0xFFFFFFFF) | ((ids[:, 4] < nsf) == src_edge))
    f1 = ids[:, 4].astype(np.int64)
    assert np.all(ids[:, 3].astype(np.int64) < np.where(f1 == 0xFFFFFFFF, 2**32, f1))


def test_deterministic_repeat(ctx):
    c = CASES["crack3"]
    a = ctx.dispatch(c["src"], c["cut"])
    b = ctx.dispatch(c["src"], c["cut"])
    assert G.same_bits(a.record_ids, b.record_ids) and G.same_bits(a.record_points, b.record_points)


@pytest.mark.parametrize("level,n", [(6, 256), (5, 700)])
def test_mid_size_against_oracle(ctx, level, n):
    s, c = meshgen.sphere_heightfield(16.0, level=level, n=n)
    want = oracle.front_end(s, c, impl="port", threads=8)
    r = ctx.dispatch(s, c, keep_tests=True, keep_pairs=True)
    check_against(r, want, meshgen.num_faces(s))


@pytest.mark.parametrize("m,n", [(128, 64), (256, 40)])
def test_coplanar_stress_against_oracle(ctx, m, n):
    """The precision-stress config at reduced size: a grid coincident with
    the cube's top face (z nudged by 1e-12): every test's signs, type and
    point-in-polygon char, and the general-position outcome."""
    s, c = meshgen.cube_coplanar(16.0, m=m, n=n)
    want = oracle.front_end(s, c, impl="port", threads=8)
    r = ctx.dispatch(s, c, keep_tests=True, keep_pairs=True)
    check_against(r, want, meshgen.num_faces(s))
    assert r.escalations[1] + r.escalations[2] > 0  # the near-coplanar signs leave the fp32 filter


def test_full_size_sphere_heightfield_x16(ctx):
    """The single-large-pair workload at full size (327,680 vs 2,093,058 tris)."""
    s, c = meshgen.sphere_heightfield(16.0)
    want = oracle.front_end(s, c, impl="port", threads=16)
    r = ctx.dispatch(s, c, keep_pairs=True)
    assert r.status == want["status"] == 0
    assert G.same_bits(sort_rows(r.pairs, [0, 1]), want["pairs"])
    ids, pts = canonical_records(r.record_ids, r.record_points)
    assert G.same_bits(ids, want["rec_ids"]) and G.same_bits(pts, want["rec_pts"])


def test_full_size_as_written_is_degenerate(ctx):
    """At scale 1 the height field's triangles fall under the reference's
    |n|^2 >= 1e-9 threshold: the dispatch must fail the same way."""
    s, c = meshgen.sphere_heightfield(1.0)
    want = oracle.front_end(s, c, impl="port", threads=16)
    r = ctx.dispatch(s, c)
    assert want["status"] in (2, 3)
    assert (r.status, r.bad_face) == (want["status"], want["bad_face"])


def test_batch_equals_single(ctx):
    names = [k for k in sorted(CASES) if k.startswith("crack")] + ["two_spheres", "bm014", "bm052", "zero_area"]
    pairs = [(CASES[k]["src"], CASES[k]["cut"]) for k in names]
    out = ctx.dispatch_batch(pairs)
    for k, (summ, ids, pts) in zip(names, out):
        want = CASES[k]
        assert summ["status"] == int(want["status"]), k
        if int(want["status"]) in (2, 3):
            continue
        a, b = canonical_records(ids, pts)
        assert G.same_bits(a, want["rec_ids"]), k
        assert G.same_bits(b, want["rec_pts"]), k


def test_batch_counts_per_pair(ctx):
    """A batch's summaries carry each pair's own candidate-pair, test and
    escalation counts: equal to the pair dispatched alone."""
    names = [k for k in sorted(CASES) if k.startswith("crack")] + ["two_spheres", "bm014", "bunny_plane"]
    pairs = [(CASES[k]["src"], CASES[k]["cut"]) for k in names]
    rng = np.random.default_rng(meshgen.SEED_BASE + 77)
    pairs += [meshgen.crack_pair(rng, target_tris=t) for t in (2000, 30000, 120000)]
    out = ctx.dispatch_batch(pairs, fetch=False)
    for (s, c), (summ, _, _) in zip(pairs, out):
        r = ctx.dispatch(s, c, fetch=False)
        assert (summ["num_pairs"], summ["num_tests"], summ["escalations"]) == \
            (r.num_pairs, r.num_tests, tuple(r.escalations))
        assert summ["num_records"] == r.num_records


@pytest.mark.parametrize("kind", ["cross_mesh", "wrapping", "far"])
def test_index_outside_its_mesh(ctx, kind):
    """Each mesh's indices are checked against its own vertex count, as the
    reference's input conversion does (preproc.cpp:390-460): a source index
    naming a cut vertex, a cut index that wraps when offset by the source
    vertex count and an index past every vertex give MCGPU_INVALID_INPUT, as
    the oracle does; in a batch only that pair's status changes and the other
    pairs keep their records."""
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
    assert ctx.dispatch(src, cut).status == L.INVALID_INPUT
    names = ["crack1", "two_spheres"]
    pairs = [(CASES["crack1"]["src"], CASES["crack1"]["cut"]), (src, cut),
             (CASES["two_spheres"]["src"], CASES["two_spheres"]["cut"])]
    out = ctx.dispatch_batch(pairs)
    assert out[1][0]["status"] == L.INVALID_INPUT
    for k, (summ, ids, pts) in zip(names, [out[0], out[2]]):
        assert summ["status"] == int(CASES[k]["status"]), k
        a, b = canonical_records(ids, pts)
        assert G.same_bits(a, CASES[k]["rec_ids"]), k
        assert G.same_bits(b, CASES[k]["rec_pts"]), k
    # the context is unaffected afterwards
    r = ctx.dispatch(c["src"], c["cut"])
    assert r.status == 0 and r.num_records == 169


def _packed_records(ids, pts, off, i):
    a, b = int(off[i]), int(off[i + 1])
    return canonical_records(ids[a:b], pts[a:b])


@pytest.mark.parametrize("device", [False, True])
def test_packed_equals_golden(ctx, device):
    import torch
    from mcut_gb300 import pack_pairs
    names = [k for k in sorted(CASES) if k.startswith("crack")] + ["two_spheres", "bm014", "bm052"]
    names = [k for k in names if CASES[k]["src"]["fs"] is None and CASES[k]["cut"]["fs"] is None
             and not CASES[k]["float_input"]]
    packed = pack_pairs([(CASES[k]["src"], CASES[k]["cut"]) for k in names])
    if device:
        packed = dict(packed, v=torch.from_numpy(packed["v"]).cuda(), f=torch.from_numpy(packed["f"]).cuda())
    sums, ids, pts, off = ctx.dispatch_packed(packed, device=device)
    assert len(off) == len(names) + 1
    for i, k in enumerate(names):
        want = CASES[k]
        assert sums[i].status == int(want["status"]), k
        assert G.same_bits(sums[i].cut_eps, want["cut_eps"]), k
        a, b = _packed_records(ids, pts, off, i)
        assert G.same_bits(a, want["rec_ids"]), k
        assert G.same_bits(b, want["rec_pts"]), k


def test_packed_fracture_batch_vs_oracle(ctx):
    """A 48-pair slice of the fracture batch (uneven icosphere / crack-grid
    pairs) in one packed pass, every pair against the oracle."""
    from mcut_gb300 import pack_pairs
    pairs = meshgen.batch_pairs(48, seed=meshgen.SEED_BASE + 40)
    sums, ids, pts, off = ctx.dispatch_packed(pack_pairs(pairs))
    total = 0
    for i, (s, c) in enumerate(pairs):
        want = oracle.front_end(s, c, impl="port", threads=16)
        assert sums[i].status == want["status"], i
        if want["status"] in (2, 3):
            continue
        w_ids, w_pts = canonical_records(want["rec_ids"], want["rec_pts"])
        a, b = _packed_records(ids, pts, off, i)
        assert G.same_bits(a, w_ids), i
        assert G.same_bits(b, w_pts), i
        total += len(a)
    assert total > 0


@pytest.mark.parametrize("name", ["two_spheres", "crack1", "bm014"])
def test_face_boxes_and_vertices_match_oracle(ctx, name):
    """The face boxes (cut boxes enlarged by eps) and ps coordinates the
    dispatch used, bit for bit."""
    c = CASES[name]
    ctx.dispatch(c["src"], c["cut"], fetch=False)
    want = oracle.front_end(c["src"], c["cut"], impl="port", threads=4)
    assert G.same_bits(ctx.face_boxes(), want["face_boxes"].reshape(-1, 6))
    v = ctx.vertices()
    assert G.same_bits(v, np.concatenate([want["src_xyz"].reshape(-1, 3), want["cut_xyz"].reshape(-1, 3)]))


def _cone(k, apex_z=0.6, base_z=-0.6, r=1.0):
    """Closed cone: k triangles around the apex and k around the base centre,
    both vertices of valence k."""
    ang = np.linspace(0.0, 2.0 * np.pi, k, endpoint=False) + 0.1234
    ring = np.stack([r * np.cos(ang), r * np.sin(ang), np.full(k, base_z)], 1)
    v = np.concatenate([ring, [[0.0, 0.0, apex_z], [0.0, 0.0, base_z]]])
    f = []
    for i in range(k):
        j = (i + 1) % k
        f += [i, j, k, j, i, k + 1]
    return dict(v=np.ascontiguousarray(v), f=np.asarray(f, np.uint32), fs=None)


@pytest.mark.parametrize("k", [40, 200])
def test_high_valence_vertex_against_oracle(ctx, k):
    """The apex has more incident faces than the fixed incidence slots (16):
    the call reruns with CSR incidence, the next (fused) call keeps it, and a
    context that always uses CSR lists agrees."""
    import os
    from mcut_gb300 import Context
    s = _cone(k)
    c = meshgen.grid(24, 1.5, lambda X, Y: 0.05 + 0.03 * X + 0.02 * Y)
    want = oracle.front_end(s, c, impl="port", threads=4)
    assert int(want["status"]) == 0 and len(want["rec_ids"]) > 0
    for _ in range(2):
        r = ctx.dispatch(s, c, keep_tests=True, keep_pairs=True)
        check_against(r, want, meshgen.num_faces(s))
    os.environ["MCGPU_INC_SLOTS"] = "0"
    try:
        csr = Context(0)
    finally:
        del os.environ["MCGPU_INC_SLOTS"]
    try:
        check_against(csr.dispatch(s, c, keep_tests=True, keep_pairs=True), want, meshgen.num_faces(s))
    finally:
        csr.close()
