"""Regenerate the golden fixtures from the UNMODIFIED reference.

Run where the reference checkout exists (it compiles the reference sources in
place into oracle/_ref via oracle/Makefile):

    python tests/golden/make_golden.py --ref-root /path/to/mcut   (or MCUT_REF_ROOT=...)

Every fixture stores the inputs (so hosts without the reference can replay
them) and the reference's own outputs:
  * front end, from oracle/ref_harness.cpp driving build_oibvh,
    intersectOIBVHs and the reference's predicate / plane / point-in-polygon
    functions: status, candidate pairs, every culled (edge, face) test with
    both orient3d signs + type + point-in-polygon char, records + points;
  * full public-API dispatch (mcDispatch / mcGetConnectedComponents): result
    code, per-CC (type, vertex count, face count), intersection-point count.

Fixture files:
  benchmarks.npz   the 64 mesh pairs of the reference's benchmark test
                   (tests/meshes/benchmarks/{src,cut}-meshNNN.off)
  named.npz        bunny vs bunnyCuttingPlanePartial (tests/meshes)
  synthetic.npz    the synthetic workloads at reduced size (and C1 in full)
  configs.npz      hand-built edge cases: touching edges, vertex on face,
                   zero-area face, disjoint boxes, coplanar faces, float input
  predicates.npz   orient3d signs / orient2d values on random and
                   near-degenerate inputs (::orient3d, ::orient2d)
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from mcut_gb300 import meshgen  # noqa: E402

OUT = os.path.dirname(os.path.abspath(__file__))
FE_KEYS = ["pairs", "tests", "test_info", "rec_ids", "rec_pts"]


def _put_mesh(d, pre, m):
    d[pre + "v"] = m["v"]
    d[pre + "f"] = m["f"]
    d[pre + "fs"] = m["fs"] if m["fs"] is not None else np.zeros(0, np.uint32)


def safe_dispatch(oracle, src, cut, flags):
    """Full reference dispatch in a forked child: the reference aborts the
    process on some inputs (a failed internal assertion), which must not end
    the fixture run. An abort is recorded as result code -9999."""
    import pickle
    rfd, wfd = os.pipe()
    pid = os.fork()
    if pid == 0:
        os.close(rfd)
        try:
            devnull = os.open(os.devnull, os.O_WRONLY)
            os.dup2(devnull, 1)
            os.dup2(devnull, 2)
            r = oracle.dispatch(src, cut, flags=flags)
            os.write(wfd, pickle.dumps(r))
        finally:
            os._exit(0)
    os.close(wfd)
    chunks = []
    while True:
        b = os.read(rfd, 1 << 20)
        if not b:
            break
        chunks.append(b)
    os.close(rfd)
    os.waitpid(pid, 0)
    if not chunks:
        return dict(result=-9999, ccs=np.zeros((0, 3), np.int32), n_ivtx=-1)
    return pickle.loads(b"".join(chunks))


def record_case(d, name, src, cut, oracle, float_input=False, dispatch=True):
    _put_mesh(d, name + "/src_", src)
    _put_mesh(d, name + "/cut_", cut)
    fe = oracle.front_end(src, cut, impl="ref", float_input=float_input)
    d[name + "/status"] = np.int32(fe["status"])
    d[name + "/bad_face"] = np.int32(fe["bad_face"])
    d[name + "/cut_eps"] = np.float64(fe["cut_eps"])
    d[name + "/float_input"] = np.int32(int(float_input))
    for k in FE_KEYS:
        d[name + "/" + k] = fe[k]
    if dispatch:
        flags = oracle.MC_DISPATCH_VERTEX_ARRAY_FLOAT if float_input else oracle.MC_DISPATCH_VERTEX_ARRAY_DOUBLE
        srcd, cutd = src, cut
        if float_input:
            srcd = dict(src, v=src["v"].astype(np.float32))
            cutd = dict(cut, v=cut["v"].astype(np.float32))
        r = safe_dispatch(oracle, srcd, cutd, flags)
        d[name + "/mc_result"] = np.int32(r["result"])
        d[name + "/mc_ccs"] = r["ccs"]
        d[name + "/mc_ivtx"] = np.int64(r["n_ivtx"])
    print(f"  {name}: status={fe['status']} pairs={len(fe['pairs'])} tests={len(fe['tests'])} "
          f"records={len(fe['rec_ids'])}" + (f" mc={d[name + '/mc_result']} ccs={len(d[name + '/mc_ccs'])}"
                                             if dispatch else ""))


def tri(v, f=None):
    v = np.asarray(v, dtype=np.float64).reshape(-1, 3)
    f = np.arange(v.shape[0], dtype=np.uint32) if f is None else np.asarray(f, dtype=np.uint32)
    return dict(v=v, f=f.ravel(), fs=None)


def poly(v, f, fs):
    return dict(v=np.asarray(v, np.float64).reshape(-1, 3), f=np.asarray(f, np.uint32),
                fs=np.asarray(fs, np.uint32))


def edge_cases():
    """Configurations chosen to exercise each branch of the narrow phase."""
    base = tri([[0, 0, 0], [4, 0, 0], [0, 4, 0]])
    cases = {}
    # clean crossing of two triangles
    cases["cross"] = (base, tri([[1, 1, -1], [1, 1, 2], [2, -1, 0.5]]))
    # an edge of the cut triangle lies across an edge of the source triangle
    cases["edge_on_edge"] = (base, tri([[-1, 2, -2], [5, 2, 2], [-1, 2, 2]]))
    # a cut vertex lies inside the source face
    cases["vertex_on_face"] = (base, tri([[1, 1, 0], [3, 1, -2], [1, 3, -2]]))
    # a cut vertex coincides with a source vertex
    cases["vertex_on_vertex"] = (base, tri([[0, 0, 0], [1, -1, 3], [-1, 1, 3]]))
    # the cut triangle lies in the source plane
    cases["coplanar"] = (base, tri([[1, 1, 0], [3, 0.5, 0], [0.5, 3, 0]]))
    # disjoint bounding boxes: no candidate pair at all
    cases["disjoint"] = (base, tri([[10, 10, 10], [11, 10, 10], [10, 11, 10]]))
    # a zero-area source face next to a valid one
    cases["zero_area"] = (tri([[-1, -1, 0], [1, -1, 0], [1, 1, 0], [-1, -1, 0]], [0, 1, 2, 0, 2, 3]),
                          tri([[-1, 0, 1], [2, 0, 1], [2, 0, -1], [-1, 0, 1.5]], [0, 1, 2, 0, 2, 3]))
    # a fine triangle below the |n|^2 >= 1e-9 threshold (0.5e-5 legs)
    cases["tiny_face"] = (tri([[0, 0, 0], [3e-5, 0, 0], [0, 3e-5, 0]]),
                          tri([[1e-5, 1e-5, -1], [1e-5, 1e-5, 1], [2e-5, -1e-5, 0.5]]))
    # a quad and a pentagon (non-triangle faces take the triplet path)
    cases["quad_pent"] = (poly([[0, 0, 0], [4, 0, 0], [4, 4, 0], [0, 4, 0]], [0, 1, 2, 3], [4]),
                          poly([[1, 1, -1], [3, 1.5, -1], [3.2, 2.5, 1], [2, 3.5, 2], [0.8, 2.6, 1]],
                               [0, 1, 2, 3, 4], [5]))
    return cases


def predicate_cases(rng, n=6000):
    """Random and near-degenerate orient3d / orient2d inputs."""
    pts3 = []
    for _ in range(n // 2):
        pts3.append(rng.uniform(-1, 1, size=(4, 3)))
    for _ in range(n // 2):
        # d nearly on the plane of a, b, c
        a, b, c = rng.uniform(-1, 1, size=(3, 3))
        u, w = rng.uniform(-2, 2, size=2)
        d = a + u * (b - a) + w * (c - a)
        d = d + rng.normal(size=3) * 10.0 ** rng.integers(-18, -10)
        if rng.random() < 0.3:
            d = a + u * (b - a) + w * (c - a)
        pts3.append(np.stack([a, b, c, d]))
    for _ in range(n // 4):
        # exactly coplanar on a dyadic lattice (orient3d == 0)
        a, b, c = rng.integers(-16, 17, size=(3, 3)) / 8.0
        i, j = rng.integers(-3, 4, size=2)
        pts3.append(np.stack([a, b, c, a + i * (b - a) + j * (c - a)]))
    pts2 = []
    for _ in range(n // 4):
        a, b = rng.integers(-16, 17, size=(2, 2)) / 8.0
        pts2.append(np.stack([a, b, a + rng.integers(-3, 4) * (b - a)]))
    for _ in range(n // 2):
        pts2.append(rng.uniform(-1, 1, size=(3, 2)))
    for _ in range(n // 2):
        a, b = rng.uniform(-1, 1, size=(2, 2))
        t = rng.uniform(-2, 2)
        c = a + t * (b - a) + rng.normal(size=2) * 10.0 ** rng.integers(-18, -10)
        pts2.append(np.stack([a, b, c]))
    return np.array(pts3), np.array(pts2)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref-root", default=os.environ.get("MCUT_REF_ROOT"),
                    help="reference checkout (default: $MCUT_REF_ROOT)")
    args = ap.parse_args()
    if not args.ref_root:
        ap.error("name the reference checkout with --ref-root or MCUT_REF_ROOT")
    import oracle  # noqa: E402
    oracle.build(ref=True, ref_root=args.ref_root)

    bench_dir = os.path.join(args.ref_root, "tests", "meshes", "benchmarks")
    d = {}
    print("benchmarks")
    for i in range(64):
        s = meshgen.read_off(os.path.join(bench_dir, f"src-mesh{i:03d}.off"))
        c = meshgen.read_off(os.path.join(bench_dir, f"cut-mesh{i:03d}.off"))
        record_case(d, f"bm{i:03d}", s, c, oracle)
    np.savez_compressed(os.path.join(OUT, "benchmarks.npz"), **d)

    d = {}
    print("named")
    mesh_dir = os.path.join(args.ref_root, "tests", "meshes")
    record_case(d, "bunny_plane", meshgen.read_off(os.path.join(mesh_dir, "bunny.off")),
                meshgen.read_off(os.path.join(mesh_dir, "bunnyCuttingPlanePartial.off")), oracle)
    np.savez_compressed(os.path.join(OUT, "named.npz"), **d)

    d = {}
    print("synthetic")
    record_case(d, "two_spheres", *meshgen.two_spheres(), oracle)
    record_case(d, "two_spheres_x16", *meshgen.two_spheres(16.0), oracle)
    record_case(d, "sphere_hf_small", *meshgen.sphere_heightfield(1.0, level=4, n=96), oracle)
    record_case(d, "sphere_hf_small_x16", *meshgen.sphere_heightfield(16.0, level=4, n=96), oracle)
    record_case(d, "cube_coplanar_small_x16", *meshgen.cube_coplanar(16.0, m=24, n=12), oracle, dispatch=False)
    rng = np.random.default_rng(meshgen.SEED_BASE + 4)
    for k in range(6):
        record_case(d, f"crack{k}", *meshgen.crack_pair(rng), oracle)
    np.savez_compressed(os.path.join(OUT, "synthetic.npz"), **d)

    d = {}
    print("configs")
    for name, (s, c) in edge_cases().items():
        record_case(d, name, s, c, oracle)
    s, c = edge_cases()["cross"]
    record_case(d, "cross_float", s, c, oracle, float_input=True)
    np.savez_compressed(os.path.join(OUT, "configs.npz"), **d)

    print("predicates")
    rng = np.random.default_rng(meshgen.SEED_BASE + 99)
    p3, p2 = predicate_cases(rng)
    o3 = np.array([oracle.ref_orient3d(*p) for p in p3])
    o2 = np.array([oracle.ref_orient2d(*p) for p in p2])
    np.savez_compressed(os.path.join(OUT, "predicates.npz"), p3=p3, o3=o3, p2=p2, o2=o2)
    print("done")


if __name__ == "__main__":
    main()
