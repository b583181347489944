"""Fragment parity through MCUT's own host stages.

The reference is rebuilt with its front-end seam opened (oracle/make_seam.py):
dispatch()'s narrow-phase block (kernel.cpp:2415-3206) takes the records and
the maps built from them from a hook, and everything after it -- cut-path
edges, polygon clipping, connected components, mcGetConnectedComponents --
is the reference's own code. Each case compares the connected components of
that dispatch (result code; per CC its type, vertex count and face count, as
a multiset) with the unmodified mcDispatch's, recorded in the fixtures
(mc_result, mc_ccs).

Hand-overs:
  * the oracle's, computed for every front-end pass of the dispatch (the
    harness's live mode), floating-polygon re-entries included;
  * the GPU library's, recorded on a GB300 for every pass
    (tests/golden/seam_gpu.npz, made by tests/golden/make_seam_gpu.py from the
    passes in tests/golden/seam_passes.npz) and replayed pass by pass after a
    check that the reference's soup holds the coordinates the GPU used.

Numbering: the records are delivered in a canonical order (the tested edge's
first face corner, then the tested face); MCUT numbers its intersection
vertices in its edge map's iteration order instead (an std::unordered_map,
split into parallel_for blocks). MCUT's host stages are numbering-sensitive
on a few inputs: a fragment's vertex count changes with the numbering while
its faces do not (ORDER_SENSITIVE below; test_numbering_changes_mcut_output
shows it with the reference's own code). With the hand-over renumbered as the
reference numbers it, every case matches exactly; in the canonical numbering
every other case does.

Skipped where the seam harness is neither built nor buildable (no reference
checkout: set MCUT_REF_ROOT).
"""
import os

import numpy as np
import pytest

import golden_cases as G
import oracle

pytestmark = pytest.mark.skipif(not oracle.seam_available(),
                                reason="seam harness not built and MCUT_REF_ROOT unset")

CASES = G.all_cases()
HERE = os.path.dirname(os.path.abspath(__file__))
WITH_CCS = sorted(k for k, c in CASES.items() if "mc_ccs" in c and int(c["mc_result"]) != -9999)
# cases where MCUT's own host stages give a different fragment vertex count
# under a different numbering of the same intersection vertices
ORDER_SENSITIVE = {"bm011", "bm015"}
MAPS = ["edge_off", "cp_pairs", "cp_off", "cp_vtx", "face_keys", "face_off", "face_vtx", "border"]


def _ccs(a):
    return sorted(map(tuple, np.asarray(a).reshape(-1, 3).tolist()))


def _user_meshes(c):
    src, cut = c["src"], c["cut"]
    if int(c["float_input"]):
        src = dict(src, v=src["v"].astype(np.float32))
        cut = dict(cut, v=cut["v"].astype(np.float32))
    flags = oracle.MC_DISPATCH_VERTEX_ARRAY_FLOAT if int(c["float_input"]) else oracle.MC_DISPATCH_VERTEX_ARRAY_DOUBLE
    return src, cut, flags


def _check(r, c):
    assert r["error"] == 0, r["msg"]
    assert r["result"] == int(c["mc_result"])
    if r["result"] == 0:
        assert _ccs(r["ccs"]) == _ccs(c["mc_ccs"])


@pytest.mark.parametrize("name", WITH_CCS)
def test_oracle_hand_over_reference_numbering(name):
    c = CASES[name]
    src, cut, flags = _user_meshes(c)
    _check(oracle.seam_dispatch(src, cut, flags=flags, reference_numbering=True), c)


@pytest.mark.parametrize("name", [k for k in WITH_CCS if k not in ORDER_SENSITIVE])
def test_oracle_hand_over_canonical_numbering(name):
    c = CASES[name]
    src, cut, flags = _user_meshes(c)
    _check(oracle.seam_dispatch(src, cut, flags=flags), c)


@pytest.mark.parametrize("name", sorted(ORDER_SENSITIVE))
def test_numbering_changes_mcut_output(name):
    """The same records, numbered canonically: MCUT's host stages keep every
    CC's type and face count but change one fragment's vertex count."""
    c = CASES[name]
    src, cut, flags = _user_meshes(c)
    r = oracle.seam_dispatch(src, cut, flags=flags)
    assert r["error"] == 0 and r["result"] == 0
    got, want = _ccs(r["ccs"]), _ccs(c["mc_ccs"])
    assert got != want
    assert sorted((t, f) for t, _, f in got) == sorted((t, f) for t, _, f in want)


def _gpu_passes(z, name):
    """The GPU's hand-over of every pass of pass set `name`."""
    n = int(PASSES[name + "/passes"])
    out = []
    for k in range(n):
        pre = f"{name}/p{k}/"
        h = {m: z[pre + m] for m in MAPS} if pre + "edge_off" in z.files else None
        if h is not None:
            h["rec_ids"], h["rec_pts"] = z[pre + "rec_ids"], z[pre + "rec_pts"]
        out.append(dict(hand_over=h, coord_hash=int(z[pre + "hash"]), status=int(z[pre + "status"]),
                        gp_violation=int(z[pre + "status"]) == 1))
    return out


GPU_FIXTURE = os.path.join(HERE, "golden", "seam_gpu.npz")
PASSES_FIXTURE = os.path.join(HERE, "golden", "seam_passes.npz")


@pytest.fixture(scope="module")
def gpu_z():
    if not os.path.exists(GPU_FIXTURE):
        pytest.skip("no GPU hand-over fixture (tests/golden/make_seam_gpu.py)")
    return np.load(GPU_FIXTURE)


PASSES = np.load(PASSES_FIXTURE)


def _replayable(name):
    return name + "/passes" in PASSES.files and int(PASSES[name + "/passes"]) > 0


@pytest.mark.parametrize("numbering", ["reference", "canonical"])
@pytest.mark.parametrize("name", [k for k in WITH_CCS if _replayable(k)])
def test_gpu_hand_over(gpu_z, name, numbering):
    c = CASES[name]
    if numbering == "canonical" and name in ORDER_SENSITIVE:
        pytest.skip("MCUT's output depends on the numbering here (test_numbering_changes_mcut_output)")
    canonical_set = name + "/c"
    passes = _gpu_passes(gpu_z, canonical_set if numbering == "canonical" and canonical_set + "/passes"
                         in PASSES.files else name)
    assert passes, name
    for p in passes:
        assert p["status"] in (0, 1), (name, p["status"])
    src, cut, flags = _user_meshes(c)
    r = oracle.seam_dispatch(src, cut, passes=passes, flags=flags, reference_numbering=numbering == "reference")
    assert r["calls"] == len(passes)
    _check(r, c)


def test_gpu_fixture_covers_every_pass(gpu_z):
    """The GPU ran every recorded pass on the coordinates the reference's soup holds."""
    for name in sorted(k[: -len("/passes")] for k in PASSES.files if k.endswith("/passes")):
        for k in range(int(PASSES[name + "/passes"])):
            assert int(gpu_z[f"{name}/p{k}/hash"]) == int(PASSES[f"{name}/p{k}/hash"]), (name, k)


@pytest.mark.parametrize("name", [k for k in WITH_CCS if int(CASES[k]["status"]) == 0])
def test_fixture_records_are_mcdispatch_records(name):
    """The unmodified reference's own narrow phase inside mcDispatch, read at
    the seam (observer): its records and point bits equal the fixture's,
    which the oracle and the device are compared with. Dispatches with a
    re-entry pass are left out (the observer sees the last pass)."""
    c = CASES[name]
    src, cut, flags = _user_meshes(c)
    o = oracle.observe_reference(src, cut, flags=flags)
    if o["calls"] != 1:
        pytest.skip("the dispatch ran more than one front-end pass")
    key = lambda ids, pts: sorted((tuple(sorted(r[:2])) + (r[2],), p.tobytes())  # noqa: E731
                                  for r, p in zip(np.asarray(ids).tolist(), np.asarray(pts, np.float64)))
    assert key(o["rec_ids"], o["rec_pts"]) == key(c["rec_ids"], c["rec_pts"])
