"""Record the connected components of the reference's mcDispatch on the
fixture cases as mcGetConnectedComponentData hands them to the caller
(frontend.cpp:2006-2832): the arrays the device's component wire format
(mcgpu_halfedge_mesh + queries 37-41) is held to.

Run where the reference checkout exists:

    python tests/golden/make_cc_wire.py --ref-root /path/to/mcut   (or MCUT_REF_ROOT=...)

-> tests/golden/cc_wire.npz, per case name (fixtures whose dispatch succeeds,
components of at most 1,500 faces):
  <case>/n                    number of components kept
  <case>/K/{type,vd,vf,face,fsize,adj,adjsize,edge}
                              component K's type, VERTEX_DOUBLE, VERTEX_FLOAT,
                              FACE, FACE_SIZE, FACE_ADJACENT_FACE,
                              FACE_ADJACENT_FACE_SIZE and EDGE arrays
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "tests")]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "cc_wire.npz")
MAX_FACES = 1500


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
    oracle.build(ref=True)
    import golden_cases as G

    d = {}
    for name, c in sorted(G.all_cases().items()):
        if "mc_ccs" not in c or int(c["mc_result"]) != 0:
            continue  # no components (the dispatch failed, or the reference aborted on it)
        src, cut = c["src"], c["cut"]
        flags = oracle.MC_DISPATCH_VERTEX_ARRAY_DOUBLE
        if int(c["float_input"]):
            src = dict(src, v=src["v"].astype(np.float32))
            cut = dict(cut, v=cut["v"].astype(np.float32))
            flags = oracle.MC_DISPATCH_VERTEX_ARRAY_FLOAT
        rc, ccs = oracle.cc_wire(src, cut, flags)
        assert rc == 0, (name, rc)
        kept = [w for w in ccs if len(w["fsize"]) <= MAX_FACES]
        d[f"{name}/n"] = np.int32(len(kept))
        for k, w in enumerate(kept):
            for key in ("vd", "vf", "face", "fsize", "adj", "adjsize", "edge"):
                d[f"{name}/{k}/{key}"] = w[key]
            d[f"{name}/{k}/type"] = np.int32(w["type"])
        print(f"  {name}: {len(kept)} of {len(ccs)} components")
    np.savez_compressed(OUT, **d)
    print(OUT, os.path.getsize(OUT))


if __name__ == "__main__":
    main()
