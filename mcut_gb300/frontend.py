"""Host-side mirror of the reference's front-end seam, over the C ABI.

    ctx = Context()
    r = ctx.dispatch(src, cut)               # build_oibvh x2 + intersectOIBVHs +
                                             # kernel.cpp:1781-3206, on the GPU
    r.status, r.records, r.points

A mesh is a dict(v=[V,3] float64, f=flat uint32 indices, fs=uint32 sizes or
None for triangles), as mcut_gb300.meshgen makes them. Identifiers follow the
reference's polygon soup (see include/mcut_gb300.h).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib as L


def _as_mesh(m, float_input=False):
    v = np.ascontiguousarray(m["v"], dtype=np.float32 if float_input else np.float64)
    f = np.ascontiguousarray(m["f"], dtype=np.uint32)
    fs = None if m.get("fs") is None else np.ascontiguousarray(m["fs"], dtype=np.uint32)
    nf = int(fs.shape[0]) if fs is not None else int(f.shape[0] // 3)
    cm = L.Mesh(v.ctypes.data, f.ctypes.data, None if fs is None else fs.ctypes.data, v.shape[0], nf)
    return cm, (v, f, fs)


@dataclass
class FrontEndResult:
    status: int
    status_name: str
    bad_face: int
    cut_eps: float
    num_pairs: int
    num_tests: int
    num_records: int
    escalations: tuple
    stage_ms: dict
    kernel_launches: int
    perturbations: int = 0                           # general-position enforcement attempts applied
    perturbation: tuple = (0.0, 0.0, 0.0)            # the last perturbation (recentred units)
    record_ids: np.ndarray = field(default=None)     # [R,5] q, r, face, f0, f1
    record_points: np.ndarray = field(default=None)  # [R,3]
    pairs: np.ndarray = field(default=None)          # [P,2]
    tests: np.ndarray = field(default=None)          # [T,3]
    test_info: np.ndarray = field(default=None)      # [T,4] int8


class Context:
    """One GPU context (stream + device memory pool), like an MCUT context."""

    def __init__(self, device: int = 0):
        self._lib = L.load()
        self._h = C.c_void_p()
        L.check(self._lib.mcgpu_context_create(C.byref(self._h), int(device)), "mcgpu_context_create")

    def close(self):
        if self._h:
            self._lib.mcgpu_context_release(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _get(self, query, dtype, cols):
        n = C.c_uint64(0)
        L.check(self._lib.mcgpu_get_data(self._h, query, 0, None, C.byref(n)), "mcgpu_get_data(size)")
        out = np.empty(n.value // np.dtype(dtype).itemsize, dtype=dtype)
        if n.value:
            L.check(self._lib.mcgpu_get_data(self._h, query, n.value, out.ctypes.data, C.byref(n)),
                    "mcgpu_get_data")
        return out.reshape(-1, cols)

    def dispatch(self, src, cut, cut_eps: float | None = None, recentre: bool = True, float_input: bool = False,
                 keep_tests: bool = False, keep_pairs: bool = False, profile: bool = False,
                 fetch: bool = True, enforce_general_position: bool | str = False) -> FrontEndResult:
        """One front-end dispatch. enforce_general_position: True perturbs the
        cut mesh on a general-position violation (MC_DISPATCH_ENFORCE_GENERAL_
        POSITION), "absolute" with the context's constant as the absolute scale."""
        flags = (L.RECENTRE if recentre else 0) | (L.VERTEX_ARRAY_FLOAT if float_input else 0) \
            | (L.KEEP_TESTS if keep_tests else 0) | (L.KEEP_PAIRS if keep_pairs else 0) \
            | (L.PROFILE if profile else 0)
        if enforce_general_position == "absolute":
            flags |= L.ENFORCE_GENERAL_POSITION_ABSOLUTE
        elif enforce_general_position:
            flags |= L.ENFORCE_GENERAL_POSITION
        ms, ks = _as_mesh(src, float_input)
        mc, kc = _as_mesh(cut, float_input)
        sm = L.Summary()
        rc = self._lib.mcgpu_dispatch(self._h, flags, C.byref(ms), C.byref(mc),
                                      float(cut_eps if cut_eps is not None else 0.0), C.byref(sm))
        L.check(rc, "mcgpu_dispatch")
        del ks, kc
        r = FrontEndResult(
            status=sm.status, status_name=L.STATUS_NAMES[sm.status], bad_face=sm.bad_face, cut_eps=sm.cut_eps,
            num_pairs=sm.num_pairs, num_tests=sm.num_tests, num_records=sm.num_records,
            escalations=tuple(sm.escalations), stage_ms=dict(zip(L.STAGES, list(sm.stage_ms))),
            kernel_launches=sm.kernel_launches, perturbations=sm.perturbations,
            perturbation=tuple(sm.perturbation))
        if fetch:
            r.record_ids = self._get(L.DATA_RECORD_IDS, np.uint32, 5)
            r.record_points = self._get(L.DATA_RECORD_POINTS, np.float64, 3)
            if keep_pairs:
                r.pairs = self._get(L.DATA_PAIRS, np.uint32, 2)
            if keep_tests:
                r.tests = self._get(L.DATA_TESTS, np.uint32, 3)
                r.test_info = self._get(L.DATA_TEST_INFO, np.int8, 4)
        return r

    def hand_over(self) -> dict:
        """The record hand-over of the last (single) dispatch: what dispatch()'s
        host stages read from the narrow phase (kernel.cpp:2599-2655), built on
        the device. Keys as oracle.seam: edge_off, cp_pairs [K,2], cp_off,
        cp_vtx, face_keys, face_off, face_vtx, border (m0 vertex ids), plus
        partial_cut."""
        g = lambda q, cols=1: self._get(q, np.uint32, cols)  # noqa: E731
        d = dict(edge_off=g(L.DATA_EDGE_RECORD_OFFSETS).reshape(-1), cp_pairs=g(L.DATA_CUTPATH_PAIRS, 2),
                 cp_off=g(L.DATA_CUTPATH_OFFSETS).reshape(-1), cp_vtx=g(L.DATA_CUTPATH_VERTICES).reshape(-1),
                 face_keys=g(L.DATA_FACE_KEYS).reshape(-1), face_off=g(L.DATA_FACE_OFFSETS).reshape(-1),
                 face_vtx=g(L.DATA_FACE_VERTICES).reshape(-1), border=g(L.DATA_BORDER_VERTICES).reshape(-1))
        d["partial_cut"] = bool(g(L.DATA_PARTIAL_CUT).reshape(-1)[0])
        return d

    def cut_path(self) -> dict:
        """The cut path of the last (single) dispatch: the edges MCUT's m0 gets
        from the hand-over (kernel.cpp:3332-3632), built on the device. Keys as
        oracle.cutpath: status, bad_key, edges [E,2] (first, second vertex;
        halfedge 2e runs first -> second), face_keys, face_off, face_edges,
        ivtx_off, ivtx_he."""
        g = lambda q, cols=1: self._get(q, np.uint32, cols)  # noqa: E731
        st = g(L.DATA_CUTPATH_STATUS).reshape(-1)
        return dict(status=int(st[0]), bad_key=int(st[1]) if st[0] else 0, edges=g(L.DATA_CUTPATH_EDGES, 2),
                    face_keys=g(L.DATA_CUTPATH_FACE_KEYS).reshape(-1),
                    face_off=g(L.DATA_CUTPATH_FACE_OFFSETS).reshape(-1),
                    face_edges=g(L.DATA_CUTPATH_FACE_EDGES).reshape(-1),
                    ivtx_off=g(L.DATA_CUTPATH_VERTEX_OFFSETS).reshape(-1),
                    ivtx_he=g(L.DATA_CUTPATH_VERTEX_HALFEDGES).reshape(-1))

    def floating_polygons(self) -> dict:
        """The floating polygons of the last (single) dispatch (kernel.cpp:
        4078-4200), from its cut path on the device: faces, off, vtx (m0 ids
        around each polygon from its smallest), normals [P,3], mc."""
        g = lambda q, dt=np.uint32, cols=1: self._get(q, dt, cols)  # noqa: E731
        return dict(faces=g(L.DATA_FLOATING_FACES).reshape(-1), off=g(L.DATA_FLOATING_OFFSETS).reshape(-1),
                    vtx=g(L.DATA_FLOATING_VERTICES).reshape(-1), normals=g(L.DATA_FLOATING_NORMALS, np.float64, 3),
                    mc=g(L.DATA_FLOATING_NORMAL_COMPONENTS, np.int32).reshape(-1))

    def halfedge_mesh(self, mesh, device: bool = False, fetch: bool = True) -> dict:
        """MCUT's halfedge mesh of one mesh and its input checks on the device
        (mcgpu_halfedge_mesh). mesh: dict(f=indices, fs=sizes or None,
        v or nv=vertex count); with ``device`` f (and fs) are torch CUDA
        tensors. -> dict(status, bad_face, n_edges, n_components, closed,
        kernel_launches[, he_target, he_face, he_next, he_prev, corner_he,
        v_off, v_he])."""
        ptr = (lambda a: a.data_ptr()) if device else (lambda a: a.ctypes.data)
        f = mesh["f"] if device else np.ascontiguousarray(mesh["f"], dtype=np.uint32)
        fs = mesh.get("fs")
        if fs is not None and not device:
            fs = np.ascontiguousarray(fs, dtype=np.uint32)
        nv = int(mesh["nv"]) if "nv" in mesh else int(len(mesh["v"]))
        nf = int(fs.shape[0]) if fs is not None else int(f.shape[0] // 3)
        cm = L.Mesh(None, ptr(f) if nf else None, None if fs is None else ptr(fs), nv, nf)
        rep = L.HmeshReport()
        L.check(self._lib.mcgpu_halfedge_mesh(self._h, L.DEVICE_POINTERS if device else 0, C.byref(cm),
                                              C.byref(rep)), "mcgpu_halfedge_mesh")
        out = dict(status=rep.status, bad_face=rep.bad_face, n_edges=rep.num_edges,
                   n_components=rep.num_components, closed=bool(rep.closed), kernel_launches=rep.kernel_launches)
        if fetch and rep.status in (L.HMESH_OK, L.HMESH_TOO_SMALL, L.HMESH_COMPONENTS):
            g = lambda q, dt: self._get(q, dt, 1).reshape(-1)  # noqa: E731
            out.update(he_target=g(L.DATA_HE_TARGET, np.uint32), he_face=g(L.DATA_HE_FACE, np.int32),
                       he_next=g(L.DATA_HE_NEXT, np.int32), he_prev=g(L.DATA_HE_PREV, np.int32),
                       corner_he=g(L.DATA_CORNER_HE, np.uint32), v_off=g(L.DATA_VERTEX_HE_OFFSETS, np.uint32),
                       v_he=g(L.DATA_VERTEX_HE, np.uint32))
        return out

    def cc_wire(self, cc, device: bool = False) -> dict:
        """A connected component's arrays as mcGetConnectedComponentData
        serialises them (frontend.cpp:2006-2832), computed on the device from
        the component's halfedge mesh. cc: dict(v=double vertices [V,3],
        f=indices in the component's corner order, fs=sizes or None). ->
        dict(status, face, adjsize, adj, edge, vf)."""
        ptr = (lambda a: a.data_ptr()) if device else (lambda a: a.ctypes.data)
        v = cc["v"] if device else np.ascontiguousarray(cc["v"], dtype=np.float64)
        f = cc["f"] if device else np.ascontiguousarray(cc["f"], dtype=np.uint32)
        fs = cc.get("fs")
        if fs is not None and not device:
            fs = np.ascontiguousarray(fs, dtype=np.uint32)
        nv = int(v.shape[0])
        nf = int(fs.shape[0]) if fs is not None else int(f.shape[0] // 3)
        cm = L.Mesh(ptr(v), ptr(f) if nf else None, None if fs is None else ptr(fs), nv, nf)
        rep = L.HmeshReport()
        L.check(self._lib.mcgpu_halfedge_mesh(self._h, L.DEVICE_POINTERS if device else 0, C.byref(cm),
                                              C.byref(rep)), "mcgpu_halfedge_mesh")
        out = dict(status=rep.status)
        if rep.status in (L.HMESH_OK, L.HMESH_TOO_SMALL, L.HMESH_COMPONENTS):
            g = lambda q, dt: self._get(q, dt, 1).reshape(-1)  # noqa: E731
            out.update(face=g(L.DATA_CC_FACE, np.uint32), adjsize=g(L.DATA_CC_FACE_ADJACENT_FACE_SIZE, np.uint32),
                       adj=g(L.DATA_CC_FACE_ADJACENT_FACE, np.uint32), edge=g(L.DATA_CC_EDGE, np.uint32),
                       vf=g(L.DATA_CC_VERTEX_FLOAT, np.float32).reshape(-1, 3))
        return out

    def memory(self) -> dict:
        """Device bytes the context's pool holds and its cap (0: none)."""
        held, cap = C.c_uint64(0), C.c_uint64(0)
        L.check(self._lib.mcgpu_context_get_memory(self._h, C.byref(held), C.byref(cap)), "mcgpu_context_get_memory")
        return {"device_bytes": held.value, "limit_bytes": cap.value}

    def set_memory_limit(self, limit_bytes: int = 0):
        L.check(self._lib.mcgpu_context_set_memory_limit(self._h, int(limit_bytes)), "mcgpu_context_set_memory_limit")

    def trim(self):
        L.check(self._lib.mcgpu_context_trim(self._h), "mcgpu_context_trim")

    def set_general_position(self, constant: float = 1e-4, attempts: int = 4):
        """Enforcement constant and attempts (mcBindState MC_CONTEXT_GENERAL_POSITION_ENFORCEMENT_*)."""
        L.check(self._lib.mcgpu_context_set_general_position(self._h, float(constant), int(attempts)),
                "mcgpu_context_set_general_position")

    def general_position(self):
        c, a = C.c_double(), C.c_uint32()
        L.check(self._lib.mcgpu_context_get_general_position(self._h, C.byref(c), C.byref(a)),
                "mcgpu_context_get_general_position")
        return c.value, a.value

    def set_tuning(self, leaf_size=4, traversal=0, packet_faces=32, stack_depth=64, split_round=2):
        t = L.Tuning(leaf_size, traversal, packet_faces, stack_depth, split_round)
        L.check(self._lib.mcgpu_context_set_tuning(self._h, C.byref(t)), "mcgpu_context_set_tuning")

    def tuning(self) -> dict:
        t = L.Tuning()
        L.check(self._lib.mcgpu_context_get_tuning(self._h, C.byref(t)), "mcgpu_context_get_tuning")
        return {k: int(getattr(t, k)) for k, _ in L.Tuning._fields_}

    def autotune(self, packed, device: bool = False, repeats: int = 3):
        """Pick the fastest tuning for batches like ``packed`` (kept on this
        context). Returns (tuning dict, mean ms per batch)."""
        ptr = (lambda a: a.data_ptr()) if device else (lambda a: a.ctypes.data)
        b = L.Batch(int(packed["counts"].shape[0]), ptr(packed["v"]), ptr(packed["f"]), None,
                    packed["counts"].ctypes.data, packed["eps"].ctypes.data)
        t = L.Tuning()
        ms = C.c_float(0)
        L.check(self._lib.mcgpu_autotune(self._h, L.DEVICE_POINTERS if device else 0, C.byref(b), repeats,
                                         C.byref(t), C.byref(ms)), "mcgpu_autotune")
        return {k: int(getattr(t, k)) for k, _ in L.Tuning._fields_}, ms.value

    def vertices(self):
        return self._get(L.DATA_VERTICES, np.float64, 3)

    def face_boxes(self):
        return self._get(L.DATA_FACE_BOXES, np.float64, 6)

    def dispatch_batch(self, pairs, recentre: bool = True, cut_eps=None, fetch: bool = True):
        """Many independent (src, cut) pairs in one pass. Returns per-pair
        (summary dict, record ids, record points)."""
        n = len(pairs)
        ms = (L.Mesh * n)()
        mc = (L.Mesh * n)()
        keep = []
        for i, (s, c) in enumerate(pairs):
            a, ka = _as_mesh(s)
            b, kb = _as_mesh(c)
            ms[i], mc[i] = a, b
            keep += [ka, kb]
        sums = (L.Summary * n)()
        eps = None
        if cut_eps is not None:
            eps = (C.c_double * n)(*[float(e) for e in cut_eps])
        flags = L.RECENTRE if recentre else 0
        L.check(self._lib.mcgpu_dispatch_batch(self._h, flags, n, ms, mc, eps, sums), "mcgpu_dispatch_batch")
        del keep
        out = []
        for i in range(n):
            s = sums[i]
            ids = pts = None
            if fetch:
                ids = self._batch_get(i, L.DATA_RECORD_IDS, np.uint32, 5)
                pts = self._batch_get(i, L.DATA_RECORD_POINTS, np.float64, 3)
            out.append((dict(status=s.status, bad_face=s.bad_face, cut_eps=s.cut_eps, num_records=s.num_records,
                             num_pairs=s.num_pairs, num_tests=s.num_tests, escalations=tuple(s.escalations)),
                        ids, pts))
        return out

    def dispatch_packed(self, packed, recentre: bool = False, device: bool = False, fetch: bool = True,
                        profile: bool = False):
        """One pass over a packed batch (see ``pack_pairs``). With ``device``
        ``packed["v"]`` and ``packed["f"]`` are torch CUDA tensors (counts and
        eps stay numpy). Returns (summaries
        [n] structure array, record ids [R,5], points [R,3], offsets [n+1])."""
        n = int(packed["counts"].shape[0])
        ptr = (lambda a: a.data_ptr()) if device else (lambda a: a.ctypes.data)
        eps = packed.get("eps")
        b = L.Batch(n, ptr(packed["v"]), ptr(packed["f"]), None,
                    packed["counts"].ctypes.data,
                    None if (eps is None or recentre) else eps.ctypes.data)
        sums = (L.Summary * n)()
        flags = (L.RECENTRE if recentre else 0) | (L.DEVICE_POINTERS if device else 0) | (L.PROFILE if profile else 0)
        L.check(self._lib.mcgpu_dispatch_packed(self._h, flags, C.byref(b), sums), "mcgpu_dispatch_packed")
        if not fetch:
            return sums, None, None, None
        ids = self._get(L.DATA_RECORD_IDS, np.uint32, 5)
        pts = self._get(L.DATA_RECORD_POINTS, np.float64, 3)
        off = self._get(L.DATA_RECORD_OFFSETS, np.uint64, 1).reshape(-1)
        return sums, ids, pts, off

    def _batch_get(self, pair, query, dtype, cols):
        n = C.c_uint64(0)
        L.check(self._lib.mcgpu_get_batch_data(self._h, pair, query, 0, None, C.byref(n)), "get_batch_data")
        out = np.empty(n.value // np.dtype(dtype).itemsize, dtype=dtype)
        if n.value:
            L.check(self._lib.mcgpu_get_batch_data(self._h, pair, query, n.value, out.ctypes.data, C.byref(n)),
                    "get_batch_data")
        return out.reshape(-1, cols)


class Server:
    """Continuous-batching request server on one GPU (mcgpu_server_*).

        srv = Server(device=0)
        cid = srv.add_cut(cut)                   # resident cut mesh
        t = srv.submit(src, cut)                 # or srv.submit(src, cut_id=cid)
        summary, latency_ms = srv.wait(t)
        ids, pts = srv.records(t); srv.release(t)

    Meshes are user coordinates (double); the server recentres them as
    mcDispatch does. The numpy arrays of a request are kept alive here until
    it is released.
    """

    def __init__(self, device: int = 0, workers: int = 0, max_batch_pairs: int = 0, max_batch_faces: int = 0,
                 hbm_budget_bytes: int = 0, linger_us: int = 0):
        self._lib = L.load()
        self._h = C.c_void_p()
        cfg = L.ServerConfig(device, workers, max_batch_pairs, max_batch_faces, hbm_budget_bytes, linger_us, 0)
        L.check(self._lib.mcgpu_server_create(C.byref(self._h), C.byref(cfg)), "mcgpu_server_create")
        self._keep = {}

    def close(self):
        if self._h:
            self._lib.mcgpu_server_release(self._h)
            self._h = C.c_void_p()
            self._keep.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def add_cut(self, cut) -> int:
        m, keep = _as_mesh(cut)
        cid = C.c_uint32(0)
        L.check(self._lib.mcgpu_server_add_cut_mesh(self._h, C.byref(m), C.byref(cid)), "mcgpu_server_add_cut_mesh")
        return cid.value

    def submit(self, src, cut=None, cut_id: int | None = None) -> int:
        ms, ks = _as_mesh(src)
        keep = [ms, ks]
        pc = None
        if cut is not None:
            mc, kc = _as_mesh(cut)
            keep += [mc, kc]
            pc = C.byref(mc)
        t = C.c_uint64(0)
        L.check(self._lib.mcgpu_server_submit(self._h, C.byref(ms), pc, L.NO_CUT if cut_id is None else int(cut_id),
                                              C.byref(t)), "mcgpu_server_submit")
        self._keep[t.value] = keep
        return t.value

    def wait(self, ticket: int, timeout_ms: int = -1):
        sm = L.Summary()
        lat = C.c_double(0)
        L.check(self._lib.mcgpu_server_wait(self._h, ticket, timeout_ms, C.byref(sm), C.byref(lat)),
                "mcgpu_server_wait")
        return sm, lat.value

    def records(self, ticket: int):
        out = []
        for q, dt, cols in ((L.DATA_RECORD_IDS, np.uint32, 5), (L.DATA_RECORD_POINTS, np.float64, 3)):
            n = C.c_uint64(0)
            L.check(self._lib.mcgpu_server_get_data(self._h, ticket, q, 0, None, C.byref(n)), "get_data")
            a = np.empty(n.value // np.dtype(dt).itemsize, dt)
            if n.value:
                L.check(self._lib.mcgpu_server_get_data(self._h, ticket, q, n.value, a.ctypes.data, C.byref(n)),
                        "get_data")
            out.append(a.reshape(-1, cols))
        return out[0], out[1]

    def release(self, ticket: int):
        L.check(self._lib.mcgpu_server_release_request(self._h, ticket), "mcgpu_server_release_request")
        self._keep.pop(ticket, None)

    def cancel(self, ticket: int) -> int:
        """Takes a queued request out of the queue; returns the status code
        (OK, or NOT_READY when a batch already holds it)."""
        return self._lib.mcgpu_server_cancel(self._h, ticket)

    def stats(self) -> dict:
        st = L.ServerStats()
        L.check(self._lib.mcgpu_server_get_stats(self._h, C.byref(st)), "mcgpu_server_get_stats")
        return {k: int(getattr(st, k)) for k, _ in L.ServerStats._fields_}


def pack_pairs(pairs, recentre_coords: bool = True):
    """Pack (src, cut) triangle-mesh pairs end to end (the mcgpu_batch
    layout). With ``recentre_coords`` the coordinates are the reference's
    internal ones and ``eps`` the per-pair cut-box enlargement."""
    vs, fs, counts, eps = [], [], [], []
    for s, c in pairs:
        assert s.get("fs") is None and c.get("fs") is None, "packed batches here hold triangles"
        if recentre_coords:
            sx, cx, e = recentre(s, c)
        else:
            sx, cx, e = s["v"], c["v"], 0.0
        vs += [np.asarray(sx, np.float64).reshape(-1, 3), np.asarray(cx, np.float64).reshape(-1, 3)]
        fs += [np.asarray(s["f"], np.uint32), np.asarray(c["f"], np.uint32)]
        counts.append((sx.shape[0], s["f"].shape[0] // 3, cx.shape[0], c["f"].shape[0] // 3))
        eps.append(e)
    return dict(v=np.ascontiguousarray(np.concatenate(vs)), f=np.ascontiguousarray(np.concatenate(fs)),
                counts=np.ascontiguousarray(np.array(counts, np.uint32)), eps=np.array(eps, np.float64))


def recentre(src, cut, float_input: bool = False):
    """The reference's recentring (host): -> (src_xyz, cut_xyz, cut_eps)."""
    lib = L.load()
    ms, ks = _as_mesh(src, float_input)
    mc, kc = _as_mesh(cut, float_input)
    so = np.empty((ms.num_vertices, 3), np.float64)
    co = np.empty((mc.num_vertices, 3), np.float64)
    eps = C.c_double(0)
    L.check(lib.mcgpu_recentre(L.VERTEX_ARRAY_FLOAT if float_input else 0, C.byref(ms), C.byref(mc),
                               so.ctypes.data, co.ctypes.data, C.byref(eps)), "mcgpu_recentre")
    del ks, kc
    return so, co, eps.value
