#!/usr/bin/env python
"""Throughput of the MCUT intersection front end on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Workload (one step = one front-end dispatch of one mesh pair): the single
large pair, x16-scaled so the reference accepts its faces -- a level-7
icosphere with radial noise N(0, 0.01) (327,680 triangles) against a
1024 x 1024 height field of 8 random sinusoids (2,093,058 triangles),
all coordinates multiplied by 16 (exact in fp64). Synthetic, seeded.

Metric: cut pairs/s (completed front-end dispatches per second: trees
built, traversal, narrow phase, records + status delivered).
  value : inputs resident in HBM (the reference's internal, recentred
          coordinates and face indices), L2 flushed before every step,
          each step timed with CUDA events.
  e2e   : the same dispatch through the C ABI with host buffers: the
          host->device upload of coordinates + indices and the
          device->host read of the records inside the timed region.
The reference arm (--impl reference) times the CPU restatement of the
reference's front end (oracle/, the same algorithm: OIBVH build, serial
breadth-first traversal, edge-face narrow phase) on the host cores.

With torchrun (N > 1) every rank runs its own replica of the workload on
its GPU (the front end has no cross-GPU exchange): value is the sum of the
ranks' throughputs over the max-over-ranks time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = ("sphere_heightfield_x16: level-7 noisy icosphere (327,680 tris) vs 1024x1024 height field "
            "(2,093,058 tris), coordinates x16")
METRIC = "cut pairs/s"
UNIT = "pairs/s"

# algorithmic bytes per unit of work, per stage
BYTES = {
    "bounds": ("face", 116),       # read idx 12 + positions ~12 (twice: mesh boxes, face boxes), write
                                   # fp64 box 48 + fp32 box 24 + key 4 + id 4
    "sort": ("face", 52),          # 3 passes x (8 read + 8 write) + histogram
    "hierarchy": ("node", 184),    # node write 64 + the leaf cluster's 4 face ids and fp32 boxes 112 + keys 8
    "traverse": ("pair-of-trees", None),
    "adjacency": ("face", 40),     # incidence count + fill over indices, planes of candidates
    "narrow": ("test", 152),       # edge 2x24 + face 3x24 + plane 32 (+40 per record)
}


# the kernels each stage's CUDA events bracket (k_src_packets and the incidence
# kernels run on the second stream inside the hierarchy and adjacency stages)
STAGE_KERNELS = {
    "upload": ["k_prep"],  # batches only: one pair's indices are made global by k_face_bounds
    "bounds": ["k_init_dispatch", "k_vertex_bounds", "k_mesh_frames", "k_face_bounds"],
    "sort": ["k_upsweep", "k_digit_scan", "k_downsweep"],
    "hierarchy": ["k_clusters", "k_build", "k_src_packets"],
    "traverse": ["k_top_cut", "k_traverse_wave"],
    "adjacency": ["k_plane_slots", "k_planes", "k_triplets", "k_mark_vertices", "k_vf_slots", "k_vf_count",
                  "k_vf_fill"],
    "narrow": ["k_pair_tests", "k_narrow_signs", "k_finish_planes", "k_narrow_hits", "k_rank_records",
               "k_scatter_records"],
}


def ncu_figures(stage):
    """The stage's DRAM traffic and its kernels' ncu pipe / SIMT figures from
    profiles/traffic.json (one capture of the workload; see that file's
    sources): (traffic bytes, {figure: {kernel: value}}), or (None, {})."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            tj = json.load(fh)
    except (OSError, ValueError):
        return None, {}
    figs = {}
    for key in ("fp64_pipe_active_pct", "fp32_pipe_active_pct", "threads_per_warp_instruction", "l2_hit_pct"):
        sel = {k: v for k, v in tj.get(key, {}).items() if k.split("<")[0] in STAGE_KERNELS[stage]}
        if sel:
            figs[key] = sel
    return tj.get(stage), figs


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.p = None
        self.path = os.path.join(tempfile.gettempdir(), f"mcgpu_clocks_{os.getpid()}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.fh = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}",
                                       "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.fh,
                                      stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            try:
                self.p.wait(timeout=5)
            except Exception:
                self.p.kill()
            self.fh.close()

    def summary(self):
        if not self.p:
            return None
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        try:
            for line in open(self.path):
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    mx.append(float(f[2]))
                except ValueError:
                    continue
                for k, v in zip(names, f[5:9]):
                    if v.lower() == "active":
                        reasons.add(k)
        except Exception:
            return None
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def make_workload(name="c2"):
    """C2x16 (the headline pair) or C3x16 (the coplanar lattice cube)."""
    from mcut_gb300 import meshgen
    return meshgen.cube_coplanar(16.0) if name == "c3" else meshgen.sphere_heightfield(16.0)


def dist_init(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if args.impl == "gb300" else "gloo")
    return world, rank, local


def reduce_max(x, world):
    """Max over ranks (NCCL on the GPU arm, gloo on CPU)."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def cpu_port_run(src, cut, steps, warmup, threads):
    """The oracle (CPU restatement of the reference front end), timed."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    oracle.build()
    for _ in range(warmup):
        oracle.front_end(src, cut, impl="port", threads=threads)
    ts = []
    for _ in range(steps):
        t0 = time.perf_counter()
        oracle.front_end(src, cut, impl="port", threads=threads)
        ts.append(time.perf_counter() - t0)
    return ts


def bench_config(world):
    """The config dict both arms print (arm-specific notes go under "arm")."""
    return {"workload": WORKLOAD, "l2": "flushed (256 MB write) before every GPU step",
            "parallelism": f"replicas x{world}"}


def run_reference(args, world, rank):
    if rank != 0:
        return
    src, cut = make_workload()
    threads = os.cpu_count() or 1
    steps = max(1, args.steps)
    ts = cpu_port_run(src, cut, steps, args.warmup, threads)
    v = steps / sum(ts)
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * sum(ts) / steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(world),
        "arm": {"path": "CPU restatement of the reference front end (oracle/)"},
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{steps} full front-end dispatches of the workload"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_single(workload="c2"):
    """Two dispatches of the workload from device-resident inputs: the launches
    of the second one are what a profiler capture should select (-s skips the
    first dispatch's launches)."""
    import ctypes as C
    import torch
    from mcut_gb300 import Context, recentre
    from mcut_gb300 import _lib as L
    src, cut = make_workload(workload)
    sx, cx, eps = recentre(src, cut)
    ctx = Context(0)
    lib = L.load()
    d = [torch.from_numpy(a).cuda() for a in (sx, cx, src["f"].astype(np.int32), cut["f"].astype(np.int32))]
    ms = L.Mesh(d[0].data_ptr(), d[2].data_ptr(), None, sx.shape[0], src["f"].shape[0] // 3)
    mc = L.Mesh(d[1].data_ptr(), d[3].data_ptr(), None, cx.shape[0], cut["f"].shape[0] // 3)
    sm = L.Summary()
    for _ in range(2):
        L.check(lib.mcgpu_dispatch(ctx._h, L.DEVICE_POINTERS, C.byref(ms), C.byref(mc), eps, C.byref(sm)), "dispatch")
    torch.cuda.synchronize()
    print(json.dumps({"single": True, "status": L.STATUS_NAMES[sm.status], "records": int(sm.num_records),
                      "kernel_launches_per_dispatch": int(sm.kernel_launches)}))


def run_single_host():
    """Two dispatches of the workload through the e2e call (the caller's host
    arrays in internal coordinates, read by the bounds kernels over the host
    link, records read back): the second one's launches are what a profiler
    capture should select."""
    from mcut_gb300 import Context, recentre
    src, cut = make_workload()
    sx, cx, eps = recentre(src, cut)
    ctx = Context(0)
    si, ci = dict(v=sx, f=src["f"], fs=None), dict(v=cx, f=cut["f"], fs=None)
    for _ in range(2):
        r = ctx.dispatch(si, ci, cut_eps=eps, recentre=False)
    print(json.dumps({"single_host": True, "status": r.status_name, "records": int(r.num_records),
                      "kernel_launches_per_dispatch": int(r.kernel_launches)}))


BATCH_WORKLOAD = ("fracture batch: 4096 independent pairs, icosphere level U{2..5} r U(0.5,1.5) noise N(0,0.005) "
                  "vs n x n crack grid n U{8..128}, random rotation, offset U(-0.3,0.3), z noise N(0,0.02)")


def run_batch(ctx, lib, steps, world):
    """The batched path against the plain per-dispatch path on the same
    4096 fracture pairs, inputs resident in HBM (internal coordinates)."""
    import ctypes as C
    import torch
    from mcut_gb300 import meshgen, pack_pairs
    from mcut_gb300 import _lib as L

    pairs = meshgen.batch_pairs(4096)
    pk = pack_pairs(pairs)
    n = len(pairs)
    dv = torch.from_numpy(pk["v"]).cuda()
    df = torch.from_numpy(pk["f"]).cuda()
    dpk = dict(pk, v=dv, f=df)
    nfaces = int(pk["counts"][:, 1].sum() + pk["counts"][:, 3].sum())

    # the autotuner picks leaf size / traversal / packet size on a 256-pair sample
    spk = pack_pairs(pairs[:256])
    spk = dict(spk, v=torch.from_numpy(spk["v"]).cuda(), f=torch.from_numpy(spk["f"]).cuda())
    tuning, tune_ms = ctx.autotune(spk, device=True, repeats=2)
    del spk

    # batched: one packed pass over all pairs
    launches = 0
    for _ in range(2):
        sums, _, _, _ = ctx.dispatch_packed(dpk, device=True, fetch=False)
    torch.cuda.synchronize()
    barrier(world)
    st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    bt = []
    for _ in range(steps):
        torch.cuda.synchronize()
        st.record()
        sums, _, _, _ = ctx.dispatch_packed(dpk, device=True, fetch=False)
        en.record()
        torch.cuda.synchronize()
        bt.append(st.elapsed_time(en))
        launches += sums[0].kernel_launches
    barrier(world)
    b_ms = reduce_max(sum(bt), world) / steps
    status = {}
    nrec = 0
    for i in range(n):
        k = L.STATUS_NAMES[sums[i].status]
        status[k] = status.get(k, 0) + 1
        nrec += int(sums[i].num_records)

    # end to end: packed host arrays -> records + offsets back on the host
    # (3 warm-up calls: the layout's stage-by-stage call, its first one-graph
    # call, which grows the buffers, and the graph capture)
    et = []
    for _ in range(3 + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        _, ids, pts, off = ctx.dispatch_packed(pk, device=False, fetch=True)
        et.append(time.perf_counter() - t0)
    e_s = reduce_max(sum(et[3:]), world) / steps

    # plain: one mcgpu_dispatch per pair on the same device-resident arrays
    cnt = pk["counts"].astype(np.int64)
    vb = np.concatenate([[0], np.cumsum(cnt[:, 0] + cnt[:, 2])])
    fb = np.concatenate([[0], np.cumsum(3 * (cnt[:, 1] + cnt[:, 3]))])
    meshes = []
    for i in range(n):
        ms = L.Mesh(dv.data_ptr() + 24 * int(vb[i]), df.data_ptr() + 4 * int(fb[i]), None,
                    int(cnt[i, 0]), int(cnt[i, 1]))
        mc = L.Mesh(dv.data_ptr() + 24 * int(vb[i] + cnt[i, 0]), df.data_ptr() + 4 * int(fb[i] + 3 * cnt[i, 1]),
                    None, int(cnt[i, 2]), int(cnt[i, 3]))
        meshes.append((ms, mc, float(pk["eps"][i])))
    sm = L.Summary()
    for ms, mc, e in meshes[:32]:
        L.check(lib.mcgpu_dispatch(ctx._h, L.DEVICE_POINTERS, C.byref(ms), C.byref(mc), e, C.byref(sm)), "dispatch")
    torch.cuda.synchronize()
    barrier(world)
    lat = []
    plain_rec = 0
    t_all = time.perf_counter()
    for ms, mc, e in meshes:
        st.record()
        L.check(lib.mcgpu_dispatch(ctx._h, L.DEVICE_POINTERS, C.byref(ms), C.byref(mc), e, C.byref(sm)), "dispatch")
        en.record()
        en.synchronize()
        lat.append(st.elapsed_time(en))
        plain_rec += int(sm.num_records)
    t_all = time.perf_counter() - t_all
    barrier(world)
    p_s = reduce_max(t_all, world)
    return {
        "workload": BATCH_WORKLOAD, "pairs": n, "faces": nfaces, "status": status, "records": nrec,
        "records_plain": plain_rec,
        "batched": {"value": world * n / (b_ms / 1e3), "unit": UNIT, "ms_per_batch": b_ms,
                    "kernel_launches_per_batch": launches // steps},
        "batched_e2e": {"value": world * n / e_s, "unit": UNIT, "ms_per_batch": 1e3 * e_s,
                        "h2d_bytes_per_step": int(pk["v"].nbytes + pk["f"].nbytes),
                        "d2h_bytes_per_step": int(ids.nbytes + pts.nbytes + off.nbytes)},
        "plain": {"value": world * n / p_s, "unit": UNIT,
                  "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99))}},
        "batched_over_plain": (n / (b_ms / 1e3)) / (n / p_s),
        "autotuned": {"tuning": tuning, "sample_pairs": 256, "sample_ms": tune_ms},
    }


def run_configs(ctx, lib, world, cpu=True):
    """C1 (the reference's CPU-runnable case: two level-3 icospheres) through
    the C ABI from host arrays in user coordinates, as mcDispatch receives
    them, against the CPU restatement; and C3x16 (lattice cube vs a grid
    coincident with its top face, z nudged by U(-1e-12, 1e-12)): the
    escalation rates of the orient3d filters."""
    import torch
    from mcut_gb300 import meshgen
    out = {}
    s, c = meshgen.two_spheres()
    for _ in range(5):
        r = ctx.dispatch(s, c)
    n = 200
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(n):
        r = ctx.dispatch(s, c)
    g = n / (time.perf_counter() - t0)
    c1 = {"workload": "C1: level-3 icosphere r=1 vs level-3 icosphere r=0.8 at (0.5, 0.3, 0.1), fp64",
          "gpu_e2e": {"value": world * g, "unit": UNIT, "records": int(r.num_records), "status": r.status_name}}
    if cpu:
        for th in (1, os.cpu_count() or 1):
            ts = cpu_port_run(s, c, 20, 2, th)
            c1[f"cpu_port_{th}_threads"] = {"value": len(ts) / sum(ts), "unit": UNIT}
    out["c1"] = c1
    s, c = meshgen.cube_coplanar(16.0)
    from mcut_gb300 import _lib as L
    from mcut_gb300 import recentre
    import ctypes as C
    sx, cx, eps = recentre(s, c)
    d = [torch.from_numpy(a).cuda() for a in (sx, cx, s["f"].astype(np.int32), c["f"].astype(np.int32))]
    ms = L.Mesh(d[0].data_ptr(), d[2].data_ptr(), None, sx.shape[0], s["f"].shape[0] // 3)
    mc = L.Mesh(d[1].data_ptr(), d[3].data_ptr(), None, cx.shape[0], c["f"].shape[0] // 3)
    sm = L.Summary()
    for _ in range(3):
        L.check(lib.mcgpu_dispatch(ctx._h, L.DEVICE_POINTERS, C.byref(ms), C.byref(mc), eps, C.byref(sm)), "dispatch")
    st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t = []
    for _ in range(5):
        torch.cuda.synchronize()
        st.record()
        L.check(lib.mcgpu_dispatch(ctx._h, L.DEVICE_POINTERS, C.byref(ms), C.byref(mc), eps, C.byref(sm)), "dispatch")
        en.record()
        torch.cuda.synchronize()
        t.append(st.elapsed_time(en))
    # end to end from user coordinates (recentred as mcDispatch does), records
    # read back, after 3 warm-up calls of this layout
    for _ in range(3):
        ctx.dispatch(s, c)
    te = []
    for _ in range(3):
        t0 = time.perf_counter()
        r = ctx.dispatch(s, c)
        te.append(1e3 * (time.perf_counter() - t0))
    esc = [int(x) for x in r.escalations]
    tot = max(1, sum(esc))
    out["c3"] = {"workload": "C3x16: 512^2-per-face lattice cube (3,145,728 tris) vs 256x256 grid on its top face "
                             "plane, z + U(-1e-12, 1e-12), x16",
                 "status": r.status_name, "pairs": int(r.num_pairs), "tests": int(r.num_tests),
                 "records": int(r.num_records), "ms_per_dispatch": float(np.median(t)),
                 "ms_per_dispatch_e2e": float(np.median(te)),
                 "escalations": {"fp32_filter": esc[0], "fp64_filter": esc[1], "adaptive_or_exact": esc[2],
                                 "rates": [e / tot for e in esc]}}
    out["hmesh"] = run_hmesh(ctx, cpu)
    out["cutpath"] = run_cutpath(ctx, cpu)
    return out


def run_hmesh(ctx, cpu=True):
    """The halfedge mesh and input checks of the headline pair's two meshes
    (client_input_arrays_to_hmesh + check_input_mesh + mesh_is_closed) on the
    device, from device-resident indices, wall time per call (the call reads
    its counts back); beside it the CPU restatement of MCUT's face-by-face
    loop (oracle/hmesh_oracle.c, one thread) on the same meshes."""
    import torch
    from mcut_gb300 import meshgen
    s, c = meshgen.sphere_heightfield(16.0)
    res = {"workload": "halfedge mesh + input checks of the C2x16 meshes (327,680 and 2,093,058 tris)"}
    for name, m in (("source", s), ("cut", c)):
        f = torch.from_numpy(np.ascontiguousarray(m["f"], np.uint32).view(np.int32)).cuda()
        mesh = dict(f=f, fs=None, nv=len(m["v"]))
        for _ in range(3):
            r = ctx.halfedge_mesh(mesh, device=True, fetch=False)
        ts = []
        for _ in range(10):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = ctx.halfedge_mesh(mesh, device=True, fetch=False)
            ts.append(1e3 * (time.perf_counter() - t0))
        row = {"faces": int(len(m["f"]) // 3), "edges": int(r["n_edges"]), "status": int(r["status"]),
               "closed": bool(r["closed"]), "gpu_ms": float(np.median(ts)), "kernel_launches": int(r["kernel_launches"])}
        if cpu:
            sys.path.insert(0, os.path.join(ROOT, "oracle"))
            import oracle
            t0 = time.perf_counter()
            oracle.hmesh(m["f"], None, len(m["v"]), "port")
            row["cpu_port_1_thread_ms"] = 1e3 * (time.perf_counter() - t0)
        res[name] = row
    # a connected component's wire arrays (mcGetConnectedComponentData: faces,
    # face adjacency and counts, edges, float vertices), the cut mesh taken as
    # one component, from device arrays to host arrays
    f = torch.from_numpy(np.ascontiguousarray(c["f"], np.uint32).view(np.int32)).cuda()
    v = torch.from_numpy(np.ascontiguousarray(c["v"], np.float64)).cuda()
    for _ in range(2):
        w = ctx.cc_wire(dict(v=v, f=f, fs=None), device=True)
    ts = []
    for _ in range(5):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        w = ctx.cc_wire(dict(v=v, f=f, fs=None), device=True)
        ts.append(1e3 * (time.perf_counter() - t0))
    row = {"faces": int(len(c["f"]) // 3), "adjacent_faces": int(len(w["adj"])), "gpu_ms": float(np.median(ts))}
    if cpu:
        t0 = time.perf_counter()
        h = oracle.hmesh(c["f"], None, len(c["v"]), "port")
        oracle.cc_wire_of_hmesh(h, np.full(len(c["f"]) // 3, 3, np.uint32), c["v"])
        row["cpu_port_1_thread_ms"] = 1e3 * (time.perf_counter() - t0)
    res["cc_wire"] = row
    return res


def run_cutpath(ctx, cpu=True):
    """The cut-path edges of the headline dispatch (kernel.cpp:3332-3632) on
    the device: wall time of the first cut-path query after a dispatch whose
    hand-over is already built (the build, its count readback and one small
    query); beside it the CPU restatement (oracle/cutpath_oracle.c, one
    thread) on the same hand-over."""
    import ctypes as C
    import torch
    from mcut_gb300 import meshgen, recentre
    from mcut_gb300 import _lib as L
    s, c = meshgen.sphere_heightfield(16.0)
    sx, cx, eps = recentre(s, c)
    d = [torch.from_numpy(a).cuda() for a in (sx, cx, s["f"].astype(np.int32), c["f"].astype(np.int32))]
    ms = L.Mesh(d[0].data_ptr(), d[2].data_ptr(), None, sx.shape[0], s["f"].shape[0] // 3)
    mc = L.Mesh(d[1].data_ptr(), d[3].data_ptr(), None, cx.shape[0], c["f"].shape[0] // 3)
    lib, sm, nb = L.load(), L.Summary(), C.c_uint64(0)
    st = np.zeros(2, np.uint32)
    ts = []
    for rep in range(13):
        L.check(lib.mcgpu_dispatch(ctx._h, L.DEVICE_POINTERS, C.byref(ms), C.byref(mc), eps, C.byref(sm)), "dispatch")
        L.check(lib.mcgpu_get_data(ctx._h, L.DATA_CUTPATH_PAIRS, 0, None, C.byref(nb)), "hand-over")
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        L.check(lib.mcgpu_get_data(ctx._h, L.DATA_CUTPATH_STATUS, 8, st.ctypes.data, C.byref(nb)), "cut path")
        if rep >= 3:
            ts.append(1e3 * (time.perf_counter() - t0))
    cp = ctx.cut_path()
    row = {"workload": "cut-path edges of the C2x16 dispatch (10,974 intersection vertices)",
           "edges": int(len(cp["edges"])), "faces": int(len(cp["face_keys"])), "status": int(cp["status"]),
           "gpu_ms": float(np.median(ts))}
    if cpu:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import oracle
        hand = ctx.hand_over()
        hand["rec_ids"] = ctx._get(L.DATA_RECORD_IDS, np.uint32, 5)
        hand["rec_pts"] = ctx._get(L.DATA_RECORD_POINTS, np.float64, 3)
        xyz = ctx.vertices()
        soup = oracle.soup_faces(s, c)
        t0 = time.perf_counter()
        oracle.cutpath_of(s, c, xyz, hand, soup)
        row["cpu_port_1_thread_ms"] = 1e3 * (time.perf_counter() - t0)
    return row


SERVED_WORKLOAD = ("served: open-loop Poisson arrivals; each request one fracture pair with total triangles "
                   "log-uniform in [1e3, 1e6]; 30% name one of 64 device-resident cut meshes; HBM budget 150 GiB")


def make_served(n_pool=256, n_resident=64, n_req=1200):
    from mcut_gb300 import meshgen
    rng = np.random.default_rng(meshgen.SEED_BASE + 5)
    logu = lambda k: np.exp(rng.uniform(np.log(1e3), np.log(1e6), k))  # noqa: E731
    pool = [meshgen.crack_pair(rng, target_tris=int(t)) for t in logu(n_pool)]
    resident = [meshgen.crack_pair(rng, target_tris=int(t))[1] for t in logu(n_resident)]
    trace = []
    for _ in range(n_req):
        i = int(rng.integers(n_pool))
        trace.append((i, int(rng.integers(n_resident)) if rng.random() < 0.3 else None))
    return pool, resident, trace


def run_served(ctx, world):
    """Plain per-dispatch path vs the request server on the same request
    trace: closed loop (all queued) for throughput, then Poisson arrivals at
    fractions of that rate for p50/p99 latency (submission -> records on the
    host)."""
    import threading
    from mcut_gb300 import Server

    pool, resident, trace = make_served()
    srv = Server(0, hbm_budget_bytes=150 << 30)
    cids = [srv.add_cut(c) for c in resident]

    def pair_of(i, r):
        return pool[i][0], (resident[r] if r is not None else pool[i][1])

    # plain: one mcgpu_dispatch per request from host arrays (recentred as
    # mcDispatch does), records read back
    n_plain = 300
    for i, r in trace[:n_plain]:  # one untimed pass over the same requests
        ctx.dispatch(*pair_of(i, r))
    lat_p = []
    t0 = time.perf_counter()
    for i, r in trace[:n_plain]:
        a = time.perf_counter()
        ctx.dispatch(*pair_of(i, r))
        lat_p.append(1e3 * (time.perf_counter() - a))
    plain = n_plain / (time.perf_counter() - t0)

    def submit(i, r):
        s_, c_ = pool[i][0], pool[i][1]
        return srv.submit(s_, cut_id=cids[r]) if r is not None else srv.submit(s_, c_)

    def closed(n):
        t0 = time.perf_counter()
        ts = [submit(i, r) for i, r in trace[:n]]
        lat = []
        for t in ts:
            lat.append(srv.wait(t)[1])
            srv.release(t)
        return n / (time.perf_counter() - t0), lat

    # warm-up: one untimed pass over the whole trace (the worker pools grow to
    # the batches' sizes, the host pages are first touched over the link),
    # then the median of three timed passes (all three reported)
    closed(len(trace))
    runs = sorted((closed(len(trace)) for _ in range(3)), key=lambda x: x[0])
    sat, lat_c = runs[1]

    def open_loop(rate, n):
        rng = np.random.default_rng(7)
        gaps = rng.exponential(1.0 / rate, n)
        ts, lat = [], []
        done = threading.Event()

        def waiter():
            k = 0
            while k < n:
                while k >= len(ts):
                    time.sleep(0.0002)
                lat.append(srv.wait(ts[k])[1])
                srv.release(ts[k])
                k += 1
            done.set()

        th = threading.Thread(target=waiter)
        th.start()
        t0 = time.perf_counter()
        nxt = t0
        for k in range(n):
            nxt += gaps[k]
            while time.perf_counter() < nxt:
                time.sleep(min(0.0005, max(0.0, nxt - time.perf_counter())))
            i, r = trace[k % len(trace)]
            ts.append(submit(i, r))
        done.wait()
        th.join()
        el = time.perf_counter() - t0
        return {"rate_per_s": rate, "requests": n, "throughput": n / el,
                "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}

    sweep = []
    for frac in (0.25, 0.5, 0.8):
        rate = frac * sat
        sweep.append(open_loop(rate, int(min(len(trace), max(200, rate * 1.5)))))
    st = srv.stats()
    srv.close()
    return {
        "workload": SERVED_WORKLOAD, "requests": len(trace), "resident_cut_meshes": len(resident),
        "plain": {"value": world * plain, "unit": UNIT, "requests": n_plain,
                  "latency_ms": {"p50": float(np.percentile(lat_p, 50)), "p99": float(np.percentile(lat_p, 99))}},
        "served_saturated": {"value": world * sat, "unit": UNIT, "passes": [world * x[0] for x in runs],
                             "latency_ms": {"p50": float(np.percentile(lat_c, 50)),
                                            "p99": float(np.percentile(lat_c, 99))}},
        "served_over_plain": sat / plain,
        "open_loop": sweep,
        "server": {"workers": 3, "batches": st["batches"], "peak_inflight_bytes": st["peak_inflight_bytes"],
                   "resident_bytes": st["resident_bytes"]},
    }


def run_gpu(args, world, rank, local):
    import torch
    import ctypes as C
    from mcut_gb300 import Context, recentre
    from mcut_gb300 import _lib as L
    from mcut_gb300.frontend import _as_mesh

    torch.cuda.set_device(local)
    src, cut = make_workload()
    sx, cx, eps = recentre(src, cut)
    fs_, fc_ = src["f"], cut["f"]
    ctx = Context(local)
    lib = L.load()

    # device-resident inputs: the reference's internal coordinates + indices
    d_sx = torch.from_numpy(sx).cuda()
    d_cx = torch.from_numpy(cx).cuda()
    d_fs = torch.from_numpy(fs_.astype(np.int32)).cuda()
    d_fc = torch.from_numpy(fc_.astype(np.int32)).cuda()
    ms = L.Mesh(d_sx.data_ptr(), d_fs.data_ptr(), None, sx.shape[0], fs_.shape[0] // 3)
    mc = L.Mesh(d_cx.data_ptr(), d_fc.data_ptr(), None, cx.shape[0], fc_.shape[0] // 3)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # > 129 MB L2
    sm = L.Summary()

    def step_dev(flags=L.DEVICE_POINTERS):
        L.check(lib.mcgpu_dispatch(ctx._h, flags, C.byref(ms), C.byref(mc), eps, C.byref(sm)), "dispatch")

    # stage times: CUDA events on the context stream around each stage's
    # launches (direct launches; the timed loop below replays launch graphs)
    stage_acc = {k: 0.0 for k in L.STAGES}
    n_prof = max(3, min(args.steps, 10))
    for _ in range(2):
        step_dev(L.DEVICE_POINTERS | L.PROFILE)
    for _ in range(n_prof):
        flush.zero_()
        torch.cuda.synchronize()
        step_dev(L.DEVICE_POINTERS | L.PROFILE)
        for k, v in zip(L.STAGES, sm.stage_ms):
            stage_acc[k] += v / n_prof

    for _ in range(max(args.warmup, 3)):
        step_dev()
    torch.cuda.synchronize()
    barrier(world)
    times, launches = [], 0
    st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        for _ in range(args.steps):
            flush.zero_()
            torch.cuda.synchronize()
            st.record()
            step_dev()
            en.record()
            torch.cuda.synchronize()
            times.append(st.elapsed_time(en))
            launches += sm.kernel_launches
    barrier(world)
    tot_ms = reduce_max(sum(times), world)
    value = world * args.steps / (tot_ms / 1e3)
    summ = {"status": L.STATUS_NAMES[sm.status], "pairs": int(sm.num_pairs), "tests": int(sm.num_tests),
            "records": int(sm.num_records), "escalations": list(map(int, sm.escalations))}

    # end to end through the C ABI with host buffers (internal coordinates as
    # the reference's hmesh holds them)
    hs, _k1 = _as_mesh(dict(v=sx, f=fs_, fs=None))
    hc, _k2 = _as_mesh(dict(v=cx, f=fc_, fs=None))
    rid = np.empty(max(1, sm.num_records) * 5, np.uint32)
    rpt = np.empty(max(1, sm.num_records) * 3, np.float64)
    nb = C.c_uint64(0)

    def step_e2e():
        L.check(lib.mcgpu_dispatch(ctx._h, 0, C.byref(hs), C.byref(hc), eps, C.byref(sm)), "dispatch")
        L.check(lib.mcgpu_get_data(ctx._h, L.DATA_RECORD_IDS, rid.nbytes, rid.ctypes.data, C.byref(nb)), "ids")
        L.check(lib.mcgpu_get_data(ctx._h, L.DATA_RECORD_POINTS, rpt.nbytes, rpt.ctypes.data, C.byref(nb)), "pts")

    for _ in range(2):
        step_e2e()
    barrier(world)
    e2e_t = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        step_e2e()
        e2e_t.append(time.perf_counter() - t0)
    e2e_tot = reduce_max(sum(e2e_t), world)
    batch = None if args.no_batch else run_batch(ctx, lib, 3, world)
    served = None if args.no_batch else run_served(ctx, world)
    configs = None if args.no_batch else run_configs(ctx, lib, world, cpu=not args.no_cpu_baseline)
    e2e_value = world * args.steps / e2e_tot
    h2d = sx.nbytes + cx.nbytes + fs_.nbytes + fc_.nbytes
    d2h = int(sm.num_records) * (20 + 24)

    if rank != 0:
        return
    # roofline of the dominant stage
    hbm, src_peak = peaks()
    per = dict(stage_acc)
    comp = {k: per[k] for k in ("bounds", "sort", "hierarchy", "traverse", "adjacency", "narrow")}
    dom = max(comp, key=comp.get)
    Fs, Fc = fs_.shape[0] // 3, fc_.shape[0] // 3
    if dom == "traverse":
        algo = 48 * (2 * Fs + 2 * Fc) + 8 * summ["pairs"]
        units = f"48 B x (2Fs + 2Fc) + 8 B x {summ['pairs']} pairs"
    elif dom == "narrow":
        algo = 152 * summ["tests"] + 40 * summ["records"]
        units = f"152 B x {summ['tests']} tests + 40 B x {summ['records']} records"
    elif dom == "hierarchy":
        algo = 184 * (Fc // 4)
        units = f"184 B x {Fc // 4} leaf clusters of 4 faces"
    else:
        algo = BYTES[dom][1] * (Fs + Fc)
        units = f"{BYTES[dom][1]} B x {Fs + Fc} faces"
    achieved = algo / (per[dom] / 1e3) / 1e9
    # DRAM traffic and, per kernel of the stage, pipe activity, lanes per warp
    # instruction and L2 hits (ncu)
    traffic, figs = ncu_figures(dom)
    # the fp64-bound kernels against the device's fp64 rate, measured here:
    # a kernel's fp64 operations per second = its fp64 pipe's active share
    # (ncu, traffic.json) x that rate
    g = C.c_double(0.0)
    fp64 = None
    if lib.mcgpu_measure_fp64_rate(local, C.byref(g)) == L.OK and g.value > 0:
        pct = figs.get("fp64_pipe_active_pct", {})
        fp64 = {"peak_gops": g.value, "peak_source": "measured (mcgpu_measure_fp64_rate: separately rounded "
                                                     "fp64 multiply + add chains on every SM, CUDA events)",
                "achieved_gops": {k: g.value * v / 100.0 for k, v in pct.items()},
                "frac": {k: v / 100.0 for k, v in pct.items()}}
    cpu = None
    if not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        ts = cpu_port_run(src, cut, 3, 1, threads)
        cpu = {"value": 1.0 / statistics.median(ts), "unit": UNIT, "cores": threads, "kind": "port",
               "sample": "median of 3 full front-end dispatches of the workload after 1 warm-up "
                         "(oracle/, CPU restatement)"}
    ms_step = tot_ms / args.steps
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(world),
        "arm": {"path": "plain GPU per-dispatch path"},
        "latency_ms": {"p50": float(np.percentile(times, 50)), "p99": float(np.percentile(times, 99))},
        "roofline": {"bound": "hbm", "kernel": dom, "stage_kernels": STAGE_KERNELS[dom], "achieved": achieved,
                     "peak": hbm, "unit": "GB/s",
                     "frac": achieved / hbm, "traffic": traffic, **figs,
                     "algorithmic_bytes": algo,
                     "algorithmic_bytes_rule": units, "peak_source": f"{src_peak} (MEASURED_PEAKS.json hbm_gbs)",
                     "fp64": fp64},
        "stage_ms": {k: round(v, 4) for k, v in per.items()},
        "front_end": summ,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": d2h,
                "ms_per_step": 1e3 * e2e_tot / args.steps},
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
        "batch": batch,
        "served": served,
        "configs": configs,
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched (4096 pairs) and served (request stream) measurements")
    ap.add_argument("--single", action="store_true",
                    help="one warm-up dispatch + one dispatch of the workload, nothing else (for ncu captures)")
    ap.add_argument("--workload", default="c2", choices=["c2", "c3"],
                    help="the pair --single dispatches (C2x16 or C3x16)")
    ap.add_argument("--single-host", action="store_true",
                    help="the same through the e2e call: host arrays in internal coordinates (for ncu captures)")
    args = ap.parse_args()
    world, rank, local = dist_init(args)
    if args.single:
        run_single(args.workload)
    elif args.single_host:
        run_single_host()
    elif args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gpu(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
