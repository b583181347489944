"""Record every front-end pass of the reference's mcDispatch on the fixture
cases, as its polygon soup arrives at the seam (kernel.cpp:2415): the inputs
the GPU library is then run on (tests/golden/make_seam_gpu.py) so that its
records can be replayed into the reference's host stages pass by pass.

Run where the reference checkout exists (builds the seam harness,
oracle/make_seam.py):

    python tests/golden/make_seam_passes.py --ref-root /path/to/mcut   (or MCUT_REF_ROOT=...)

-> tests/golden/seam_passes.npz, per case name (every fixture with the
reference's connected components, mc_ccs):
  <case>/passes                 number of front-end passes the dispatch ran
  <case>/pK/hash                FNV-1a of pass K's soup coordinates
  <case>/pK/eps                 the cut-box enlargement given to pass K
  <case>/pK/{src,cut}_{v,f,fs}  pass K's meshes (K >= 1 only: pass 0 is the
                                fixture's own meshes, recentred)
  <case>/c/...                  the same for the canonical numbering where its
                                passes differ (a re-entry soup depends on the
                                numbering of the pass before it)
A pass's meshes are the soup's source then cut vertices (recentred
coordinates) and each face in its mesh's own corner order (the soup holds cut
faces from their second corner; the harness turns them back). The passes are recorded with the
oracle computing each pass's hand-over (the harness's live mode), so every
re-entry (floating polygons) follows the reference's own control flow.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "seam_passes.npz")


def dispatch_flags(oracle, c):
    return oracle.MC_DISPATCH_VERTEX_ARRAY_FLOAT if int(c["float_input"]) else oracle.MC_DISPATCH_VERTEX_ARRAY_DOUBLE


def user_meshes(c):
    src, cut = c["src"], c["cut"]
    if int(c["float_input"]):
        src = dict(src, v=src["v"].astype(np.float32))
        cut = dict(cut, v=cut["v"].astype(np.float32))
    return src, cut


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=os.environ.get("MCUT_REF_ROOT"),
                    help="reference checkout (default: $MCUT_REF_ROOT)")
    args = ap.parse_args()
    if not args.ref_root:
        ap.error("name the reference checkout with --ref-root or MCUT_REF_ROOT")
    os.environ["MCUT_REF_ROOT"] = args.ref_root
    import importlib
    import oracle
    importlib.reload(oracle)
    import golden_cases as G
    from mcut_gb300 import recentre

    d = {}
    for name, c in sorted(G.all_cases().items()):
        if "mc_ccs" not in c or int(c["mc_result"]) == -9999:
            continue  # no reference result (the reference aborted on it)
        src, cut = user_meshes(c)
        r = oracle.seam_dispatch(src, cut, flags=dispatch_flags(oracle, c), reference_numbering=True,
                                 want_inputs=True)
        record(d, name, c, r["inputs"], oracle, recentre)
        # a re-entry pass's soup depends on the numbering of the pass before it:
        # the canonical numbering's passes are kept too where they differ
        rc = oracle.seam_dispatch(src, cut, flags=dispatch_flags(oracle, c), want_inputs=True)
        hashes = lambda inputs: [oracle.coordinate_hash(np.concatenate([i["src"]["v"], i["cut"]["v"]]))  # noqa: E731
                                 for i in inputs]
        if hashes(rc["inputs"]) != hashes(r["inputs"]):
            record(d, name + "/c", c, rc["inputs"], oracle, recentre)
        print(f"  {name}: {len(r['inputs'])} pass(es), result {r['result']}")
    np.savez_compressed(OUT, **d)
    print(OUT)


def record(d, name, c, inputs, oracle, recentre):
    d[name + "/passes"] = np.int32(len(inputs))
    for k, inp in enumerate(inputs):
        xyz = np.concatenate([inp["src"]["v"], inp["cut"]["v"]])
        d[f"{name}/p{k}/hash"] = np.uint64(oracle.coordinate_hash(xyz))
        d[f"{name}/p{k}/eps"] = np.float64(inp["cut_eps"])
        if k == 0:
            # pass 0 is the fixture's meshes, recentred as the library recentres them
            sx, cx, _ = recentre(c["src"], c["cut"], float_input=bool(int(c["float_input"])))
            assert oracle.coordinate_hash(np.concatenate([sx, cx])) == d[f"{name}/p0/hash"], name
            for side in ("src", "cut"):
                assert np.array_equal(inp[side]["f"], np.asarray(c[side]["f"], np.uint32)), name
            continue
        for side in ("src", "cut"):
            m = inp[side]
            d[f"{name}/p{k}/{side}_v"] = m["v"]
            d[f"{name}/p{k}/{side}_f"] = m["f"]
            d[f"{name}/p{k}/{side}_fs"] = m["fs"] if m["fs"] is not None else np.zeros(0, np.uint32)

if __name__ == "__main__":
    main()
