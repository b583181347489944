"""The device's halfedge mesh and input checks equal the oracle's.

mcgpu_halfedge_mesh builds, on the device, the halfedge mesh MCUT builds
from a caller's arrays (client_input_arrays_to_hmesh, hmesh_t::add_face /
add_edge) with check_input_mesh's and mesh_is_closed's outcomes. The oracle
(oracle/hmesh_oracle.c, pinned against the reference's own hmesh_t in
tests/test_hmesh_oracle.py) runs MCUT's face-by-face loop. Status, failing
face, edge and component counts, closedness and every array (halfedge
targets, faces, next, prev, corner halfedges, per-vertex halfedge lists)
must be equal: on every fixture mesh and polygon soup, seeded random
families, seeded corruptions of each rejected kind, device-resident inputs
(with face sizes on the device), and the full-size workload meshes.
"""
import zlib

import numpy as np
import pytest

import fuzz_cases as F
import golden_cases as G
import oracle
from mcut_gb300 import meshgen
from test_hmesh_oracle import _corruptions, _faces, soup

pytestmark = pytest.mark.gpu

CASES = G.all_cases()
ARRAYS = ["he_target", "he_face", "he_next", "he_prev", "corner_he", "v_off", "v_he"]


@pytest.fixture(scope="module")
def ctx():
    from mcut_gb300 import Context
    c = Context(0)
    yield c
    c.close()


def _same(got, want):
    for k in ("status", "bad_face", "n_edges", "n_components", "closed"):
        assert got[k] == want[k], (k, got[k], want[k])
    for k in ARRAYS:
        if k in want:
            assert np.array_equal(np.asarray(got[k], np.int64), np.asarray(want[k], np.int64)), k


def _check(ctx, f, fs, nv):
    want = oracle.hmesh(f, fs, nv, "port")
    got = ctx.halfedge_mesh(dict(f=np.asarray(f, np.uint32), fs=None if fs is None else np.asarray(fs, np.uint32),
                                 nv=nv))
    _same(got, want)
    return got


@pytest.mark.parametrize("name", sorted(CASES))
def test_fixture_meshes_and_soups(ctx, name):
    c = CASES[name]
    for m in (c["src"], c["cut"]):
        f, fs = _faces(m)
        _check(ctx, f, fs, len(m["v"]))
    _check(ctx, *soup(c["src"], c["cut"]))


def test_random_families(ctx):
    for s, c, _ in F.fracture(0, 10) + F.lattice(0, 10) + F.quads(0.05, 5):
        for m in (s, c):
            f, fs = _faces(m)
            _check(ctx, f, fs, len(m["v"]))
        _check(ctx, *soup(s, c))


@pytest.mark.parametrize("name", ["two_spheres", "bm014", "bm029", "quad_pent", "crack1", "bunny_plane"])
def test_corrupted_inputs(ctx, name):
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    kinds = set()
    for m in (CASES[name]["src"], CASES[name]["cut"]):
        for _ in range(3):
            for kind, f, fs, nv in _corruptions(rng, m):
                kinds.add((kind, _check(ctx, f, fs, nv)["status"]))
    assert ("repeated", oracle.HM_NON_MANIFOLD) in kinds and ("two_components", oracle.HM_COMPONENTS) in kinds


def test_device_inputs(ctx):
    """Device-resident indices, and face sizes scanned on the device."""
    torch = pytest.importorskip("torch")
    for name in ("two_spheres", "bunny_plane", "quad_pent"):
        c = CASES[name]
        for m in (c["src"], c["cut"]):
            f, fs = _faces(m)
            want = oracle.hmesh(f, fs, len(m["v"]), "port")
            df = torch.from_numpy(np.asarray(f, np.uint32).view(np.int32)).cuda()
            dfs = None if fs is None else torch.from_numpy(np.asarray(fs, np.uint32).view(np.int32)).cuda()
            _same(ctx.halfedge_mesh(dict(f=df, fs=dfs, nv=len(m["v"])), device=True), want)


def test_full_size_workload_meshes(ctx):
    """The headline pair's meshes (327,680 and 2,093,058 triangles), the
    precision-stress cube (3,145,728) and their soup."""
    s, c = meshgen.sphere_heightfield(16.0)
    for m in (s, c):
        r = _check(ctx, *_faces(m), len(m["v"]))
        assert r["status"] == oracle.HM_OK
    assert _check(ctx, *_faces(s), len(s["v"]))["closed"] and not _check(ctx, *_faces(c), len(c["v"]))["closed"]
    cube, _ = meshgen.cube_coplanar(16.0)
    _check(ctx, *_faces(cube), len(cube["v"]))
    _check(ctx, *soup(s, c))
