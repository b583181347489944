"""Run the GPU library on every front-end pass recorded in seam_passes.npz and
keep its records and hand-over maps (run on the GPU host):

    python tests/golden/make_seam_gpu.py [--out tests/golden/seam_gpu.npz]

Every pass set (a case, and "<case>/c" where the canonical numbering's
re-entry passes differ) is run. Pass 0 of a case is the fixture's own meshes in user coordinates
(mcgpu_dispatch with MCGPU_RECENTRE, as MCUT's caller hands them over); a
re-entry pass K >= 1 is the soup recorded there, in internal coordinates with
its recorded cut_eps. Per case and pass:
  <case>/pK/status    the front end's mcgpu_status
  <case>/pK/hash      FNV-1a of the coordinates the device used (MCGPU_DATA_VERTICES)
  <case>/pK/rec_ids   [R,5] q, r, tested face, f0, f1 (canonical order)
  <case>/pK/rec_pts   [R,3]
  <case>/pK/<map>     the hand-over maps (Context.hand_over)
tests/test_seam_fragments.py replays them into the reference's host stages.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path[:0] = [ROOT, os.path.join(ROOT, "tests")]
HERE = os.path.dirname(os.path.abspath(__file__))
MAPS = ["edge_off", "cp_pairs", "cp_off", "cp_vtx", "face_keys", "face_off", "face_vtx", "border"]


def fnv1a(xyz) -> int:
    """FNV-1a over the coordinates' bytes (the seam harness's check)."""
    h = 1469598103934665603
    for b in np.ascontiguousarray(xyz, dtype=np.float64).tobytes():
        h = ((h ^ b) * 1099511628211) & 0xFFFFFFFFFFFFFFFF
    return h


def pass_meshes(z, name, k):
    def mesh(side):
        fs = z[f"{name}/p{k}/{side}_fs"]
        return dict(v=z[f"{name}/p{k}/{side}_v"], f=z[f"{name}/p{k}/{side}_f"], fs=fs if fs.size else None)
    return mesh("src"), mesh("cut")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--out", default=os.path.join(HERE, "seam_gpu.npz"))
    args = ap.parse_args()
    import golden_cases as G
    from mcut_gb300 import Context
    cases = G.all_cases()
    z = np.load(os.path.join(HERE, "seam_passes.npz"))
    # pass sets: "<case>" (the reference's numbering) and "<case>/c" (canonical)
    names = sorted(k[: -len("/passes")] for k in z.files if k.endswith("/passes"))
    ctx = Context(0)
    d = {}
    for name in names:
        c = cases[name.split("/")[0]]
        for k in range(int(z[name + "/passes"])):
            if k == 0:
                r = ctx.dispatch(c["src"], c["cut"], float_input=bool(int(c["float_input"])))
            else:
                s, t = pass_meshes(z, name, k)
                r = ctx.dispatch(s, t, cut_eps=float(z[f"{name}/p{k}/eps"]), recentre=False)
            pre = f"{name}/p{k}/"
            d[pre + "status"] = np.int32(r.status)
            d[pre + "hash"] = np.uint64(fnv1a(ctx.vertices()))
            d[pre + "rec_ids"] = r.record_ids
            d[pre + "rec_pts"] = r.record_points
            if r.status in (0, 1):
                h = ctx.hand_over()
                for m in MAPS:
                    d[pre + m] = h[m]
        print(f"  {name}: {int(z[name + '/passes'])} pass(es)")
    ctx.close()
    np.savez_compressed(args.out, **d)
    print(args.out)


if __name__ == "__main__":
    main()
