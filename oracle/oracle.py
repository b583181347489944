"""ctypes front for the CPU oracles (test infrastructure only).

    front_end(src, cut, impl="port")  -> dict   plain-C restatement (liboracle.so)
    front_end(src, cut, impl="ref")   -> dict   the unmodified reference (_ref/libref_harness.so)
    dispatch(src, cut, flags)         -> dict   full reference mcDispatch (CC counts)

Only tests, the package's smoke check and the CPU-baseline leg of bench.py
import this module. The product path never does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libref_harness.so")

FE_OK, FE_GP_VIOLATION, FE_DEGENERATE_SRC_FACE, FE_DEGENERATE_CUT_FACE, FE_INVALID_INPUT = range(5)
MC_DISPATCH_VERTEX_ARRAY_FLOAT = 1 << 0
MC_DISPATCH_VERTEX_ARRAY_DOUBLE = 1 << 1
MC_DISPATCH_ENFORCE_GENERAL_POSITION = 1 << 15


class FeResult(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("bad_face", C.c_int32), ("cut_eps", C.c_double),
        ("n_pairs", C.c_int64), ("pairs", C.POINTER(C.c_uint32)),
        ("n_tests", C.c_int64), ("tests", C.POINTER(C.c_uint32)), ("test_info", C.POINTER(C.c_int8)),
        ("n_records", C.c_int64), ("rec_ids", C.POINTER(C.c_uint32)), ("rec_pts", C.POINTER(C.c_double)),
        ("face_boxes", C.POINTER(C.c_double)), ("src_xyz", C.POINTER(C.c_double)),
        ("cut_xyz", C.POINTER(C.c_double)),
    ]


_libs = {}


# The reference checkout the harness is compiled from: named by MCUT_REF_ROOT
# (no default). Once built, oracle/_ref/ serves without the checkout.
REF_ROOT = os.environ.get("MCUT_REF_ROOT") or None


def ref_checkout() -> bool:
    """True when MCUT_REF_ROOT names a reference checkout."""
    return bool(REF_ROOT) and os.path.isdir(os.path.join(REF_ROOT, "source"))


def ref_available() -> bool:
    """True when the reference harness is built or can be built here."""
    return os.path.exists(REF_LIB) or ref_checkout()


def build(ref: bool = False, ref_root: str | None = None) -> None:
    """Compile liboracle.so (and, with ref=True, the reference harness) via the Makefile.
    The harness needs the reference checkout (ref_root, else MCUT_REF_ROOT);
    without one an already built harness is kept as it is."""
    ref_root = ref_root or REF_ROOT
    if ref and not ref_root:
        if os.path.exists(REF_LIB):
            return
        raise RuntimeError("the reference harness needs MCUT_REF_ROOT (a reference checkout)")
    cmd = ["make", "-s", "-C", HERE] + (["ref"] if ref else ["liboracle.so"])
    if ref:
        cmd.append(f"REF_ROOT={ref_root}")
    subprocess.run(cmd, check=True)


def _lib(impl: str):
    if impl in _libs:
        return _libs[impl]
    path = PORT_LIB if impl == "port" else REF_LIB
    if not os.path.exists(path):
        build(ref=(impl == "ref"))
    lib = C.CDLL(path)
    fn = lib.oracle_front_end2 if impl == "port" else lib.ref_front_end2
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                   C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                   C.c_int, C.c_int, C.c_double, C.c_int, C.c_void_p, C.POINTER(FeResult)]
    fr = lib.oracle_free if impl == "port" else lib.ref_free
    fr.argtypes = [C.POINTER(FeResult)]
    if impl == "ref":
        for nm, k in (("ref_orient3d", 4), ("ref_orient2d", 3)):
            getattr(lib, nm).restype = C.c_double
            getattr(lib, nm).argtypes = [C.c_void_p] * k
        lib.ref_dispatch.restype = C.c_int
        lib.ref_dispatch.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                     C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                     C.c_uint32, C.c_int, C.c_char_p, C.c_void_p, C.c_int,
                                     C.POINTER(C.c_int), C.POINTER(C.c_long)]
    _libs[impl] = (lib, fn, fr)
    return _libs[impl]


def _mesh_args(m, float_input=False):
    v = np.ascontiguousarray(m["v"], dtype=np.float32 if float_input else np.float64)
    f = np.ascontiguousarray(m["f"], dtype=np.uint32)
    fs = None if m.get("fs") is None else np.ascontiguousarray(m["fs"], dtype=np.uint32)
    nf = int(fs.shape[0]) if fs is not None else int(f.shape[0] // 3)
    keep = (v, f, fs)
    return keep, [v.ctypes.data, f.ctypes.data, None if fs is None else fs.ctypes.data, v.shape[0], nf]


def _arr(ptr, n, dtype):
    if n == 0 or not ptr:  # an array the producer did not fill (e.g. after invalid input)
        return np.zeros(0, dtype=dtype)
    return np.ctypeslib.as_array(ptr, shape=(n,)).astype(dtype, copy=True)


def front_end(src, cut, impl: str = "port", threads: int = 0, float_input: bool = False,
              gp_constant: float = 1e-4, gp_absolute: bool = False, perturbation=None):
    """Run one front-end dispatch; canonical-ordered numpy outputs.

    gp_constant / gp_absolute set the cut-box enlargement (the reference's
    general-position constant times the cut box diagonal, or the constant
    alone); `perturbation` (3 doubles) runs the narrow phase of one
    general-position enforcement attempt: the cut vertices plus the
    perturbation against the unperturbed pairs and face boxes."""
    lib, fn, fr = _lib(impl)
    ks, sa = _mesh_args(src, float_input)
    kc, ca = _mesh_args(cut, float_input)
    res = FeResult()
    pert = None if perturbation is None else np.ascontiguousarray(perturbation, dtype=np.float64)
    rc = fn(*sa, *ca, int(bool(float_input)), int(threads), float(gp_constant), int(bool(gp_absolute)),
            None if pert is None else pert.ctypes.data, C.byref(res))
    if rc != 0:
        raise RuntimeError(f"oracle front_end failed rc={rc}")
    nsf, ncf = sa[4], ca[4]
    out = dict(
        status=int(res.status), bad_face=int(res.bad_face), cut_eps=float(res.cut_eps),
        pairs=_arr(res.pairs, 2 * res.n_pairs, np.uint32).reshape(-1, 2),
        tests=_arr(res.tests, 3 * res.n_tests, np.uint32).reshape(-1, 3),
        test_info=_arr(res.test_info, 4 * res.n_tests, np.int8).reshape(-1, 4),
        rec_ids=_arr(res.rec_ids, 3 * res.n_records, np.uint32).reshape(-1, 3),
        rec_pts=_arr(res.rec_pts, 3 * res.n_records, np.float64).reshape(-1, 3),
        face_boxes=_arr(res.face_boxes, 6 * (nsf + ncf), np.float64).reshape(-1, 6),
        src_xyz=_arr(res.src_xyz, 3 * sa[3], np.float64).reshape(-1, 3),
        cut_xyz=_arr(res.cut_xyz, 3 * ca[3], np.float64).reshape(-1, 3),
    )
    fr(C.byref(res))
    del ks, kc
    return out


class FeSeam(C.Structure):
    _fields_ = [("n_records", C.c_int64), ("rec_ids", C.POINTER(C.c_uint32)), ("rec_pts", C.POINTER(C.c_double)),
                ("n_edges", C.c_uint32), ("edge_off", C.POINTER(C.c_uint32)),
                ("n_cutpath", C.c_uint32), ("cp_pairs", C.POINTER(C.c_uint32)), ("cp_off", C.POINTER(C.c_uint32)),
                ("cp_vtx", C.POINTER(C.c_uint32)),
                ("n_faces", C.c_uint32), ("face_keys", C.POINTER(C.c_uint32)), ("face_off", C.POINTER(C.c_uint32)),
                ("face_vtx", C.POINTER(C.c_uint32)),
                ("n_border", C.c_uint32), ("border", C.POINTER(C.c_uint32))]


SEAM_KEYS = ["rec_ids", "rec_pts", "edge_off", "cp_pairs", "cp_off", "cp_vtx", "face_keys", "face_off", "face_vtx",
             "border"]


def seam(src, cut, rec_ids, rec_pts):
    """The record hand-over of one pass (kernel.cpp:2599-2655, oracle_seam):
    records in canonical order with their edges' faces, and the derived maps
    dispatch()'s host stages read, as flat arrays (see mcut_oracle.h)."""
    lib, _, _ = _lib("port")
    if not hasattr(lib, "_seam_ready"):
        lib.oracle_seam.restype = C.c_int
        lib.oracle_seam.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p,
                                    C.c_uint32, C.c_uint32, C.c_void_p, C.c_void_p, C.c_int64, C.POINTER(FeSeam)]
        lib.oracle_seam_free.argtypes = [C.POINTER(FeSeam)]
        lib._seam_ready = True
    ks, sa = _mesh_args(src)
    kc, ca = _mesh_args(cut)
    r3 = np.ascontiguousarray(np.asarray(rec_ids, dtype=np.uint32)[:, :3])
    p3 = np.ascontiguousarray(rec_pts, dtype=np.float64)
    out = FeSeam()
    rc = lib.oracle_seam(sa[1], sa[2], sa[3], sa[4], ca[1], ca[2], ca[3], ca[4], r3.ctypes.data, p3.ctypes.data,
                         len(r3), C.byref(out))
    if rc != 0:
        raise RuntimeError("oracle_seam: a record's edge is not in the meshes")
    nr = int(out.n_records)
    d = dict(
        rec_ids=_arr(out.rec_ids, 5 * nr, np.uint32).reshape(-1, 5),
        rec_pts=_arr(out.rec_pts, 3 * nr, np.float64).reshape(-1, 3),
        edge_off=_arr(out.edge_off, out.n_edges + 1, np.uint32),
        cp_pairs=_arr(out.cp_pairs, 2 * out.n_cutpath, np.uint32).reshape(-1, 2),
        cp_off=_arr(out.cp_off, out.n_cutpath + 1, np.uint32),
        face_keys=_arr(out.face_keys, out.n_faces, np.uint32),
        face_off=_arr(out.face_off, out.n_faces + 1, np.uint32),
        border=_arr(out.border, out.n_border, np.uint32),
    )
    d["cp_vtx"] = _arr(out.cp_vtx, int(d["cp_off"][-1]), np.uint32)
    d["face_vtx"] = _arr(out.face_vtx, int(d["face_off"][-1]), np.uint32)
    lib.oracle_seam_free(C.byref(out))
    del ks, kc
    return d


SEAM_LIB = os.path.join(HERE, "_ref", "libseam_harness.so")


def seam_available() -> bool:
    """True when the seam harness (the reference with its front-end seam
    opened, make_seam.py) is built or can be built here."""
    return os.path.exists(SEAM_LIB) or ref_checkout()


def _seam_lib():
    if "seam" in _libs:
        return _libs["seam"]
    if not os.path.exists(SEAM_LIB) or ref_checkout():
        if not ref_checkout() and not os.path.exists(SEAM_LIB):
            raise RuntimeError("the seam harness needs MCUT_REF_ROOT (a reference checkout)")
        if ref_checkout():
            subprocess.run(["make", "-s", "-C", HERE, "seam", f"REF_ROOT={REF_ROOT}"], check=True)
    _lib("port")
    lib = C.CDLL(SEAM_LIB)
    lib.seam_dispatch.restype = C.c_int
    lib.seam_dispatch.argtypes = [C.c_int, C.c_int, C.c_int, C.POINTER(FeSeam), C.c_void_p, C.c_void_p,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                  C.c_uint32, C.c_int, C.c_char_p, C.c_void_p, C.c_void_p, C.c_int,
                                  C.POINTER(C.c_int), C.POINTER(C.c_int), C.POINTER(C.c_int), C.c_char_p, C.c_int]
    lib.seam_observe_reference.restype = C.c_int
    lib.seam_observe_reference.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                           C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                           C.c_uint32, C.c_int, C.c_char_p, C.c_void_p, C.c_void_p, C.c_int64,
                                           C.POINTER(C.c_int64), C.POINTER(C.c_int)]
    lib.seam_pass_input.restype = C.c_int
    lib.seam_pass_input.argtypes = [C.c_int, C.c_void_p, C.POINTER(C.c_double)] + [C.c_void_p] * 5
    lib.seam_coordinate_hash.restype = C.c_uint64
    lib.seam_coordinate_hash.argtypes = [C.c_void_p, C.c_uint64]
    _libs["seam"] = lib
    return lib


def coordinate_hash(xyz) -> int:
    """FNV-1a of ps coordinates (source then cut vertices), as a replay checks them."""
    a = np.ascontiguousarray(xyz, dtype=np.float64).reshape(-1)
    return int(_seam_lib().seam_coordinate_hash(a.ctypes.data, a.size))


def observe_reference(src, cut, flags: int = MC_DISPATCH_VERTEX_ARRAY_DOUBLE, helpers: int = 0,
                      cap: int = 1 << 22):
    """The unmodified reference's mcDispatch, observed at the seam: the records
    of its last front-end pass in its own numbering. -> dict(result, rec_ids
    [n,3] (q, r, tested face), rec_pts [n,3], calls)."""
    import tempfile
    lib = _seam_lib()
    fin = bool(flags & MC_DISPATCH_VERTEX_ARRAY_FLOAT)
    ks, sa = _mesh_args(src, fin)
    kc, ca = _mesh_args(cut, fin)
    rec = np.zeros((cap, 3), np.uint32)
    pts = np.zeros((cap, 3), np.float64)
    n, calls = C.c_int64(0), C.c_int(0)
    with tempfile.TemporaryDirectory() as wd:
        res = lib.seam_observe_reference(*sa, *ca, int(flags), int(helpers), wd.encode(), rec.ctypes.data,
                                         pts.ctypes.data, cap, C.byref(n), C.byref(calls))
    del ks, kc
    m = min(n.value, cap)
    return dict(result=int(res), rec_ids=rec[:m].copy(), rec_pts=pts[:m].copy(), calls=calls.value)


def _fe_seam(h, keep):
    """An FeSeam view of a hand-over dict (oracle.seam's keys); None: empty."""
    if h is None:
        return FeSeam()
    def u32(a):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.uint32).reshape(-1))
        keep.append(a)
        return a.ctypes.data_as(C.POINTER(C.c_uint32))
    pts = np.ascontiguousarray(np.asarray(h["rec_pts"], dtype=np.float64).reshape(-1))
    keep.append(pts)
    return FeSeam(n_records=len(h["rec_ids"]), rec_ids=u32(h["rec_ids"]),
                  rec_pts=pts.ctypes.data_as(C.POINTER(C.c_double)),
                  n_edges=len(h["edge_off"]) - 1, edge_off=u32(h["edge_off"]),
                  n_cutpath=len(h["cp_off"]) - 1, cp_pairs=u32(h["cp_pairs"]), cp_off=u32(h["cp_off"]),
                  cp_vtx=u32(h["cp_vtx"]),
                  n_faces=len(h["face_off"]) - 1, face_keys=u32(h["face_keys"]), face_off=u32(h["face_off"]),
                  face_vtx=u32(h["face_vtx"]),
                  n_border=len(h["border"]), border=u32(h["border"]))


def seam_dispatch(src, cut, passes=None, flags: int = MC_DISPATCH_VERTEX_ARRAY_DOUBLE, helpers: int = 0,
                  max_cc: int = 4096, reference_numbering: bool = False, want_inputs: bool = False):
    """mcDispatch of the reference with its front end replaced at the seam
    (kernel.cpp:2415-3206) and its host stages unchanged.

    passes=None: the oracle computes every front-end pass (live). Otherwise a
    list, one entry per front-end pass in order, of dict(hand_over=<dict as
    oracle.seam or the GPU's records + Context.hand_over>, coord_hash=<int,
    0 unchecked>, gp_violation=<bool>) replayed in turn.
    reference_numbering renumbers each hand-over's intersection vertices in
    the order the reference's own narrow phase gives them (its edge map's
    iteration order, in parallel_for blocks); otherwise the hand-over's
    canonical order is kept.
    -> dict(result, ccs [n,3] (type, vertices, faces), used_vertices [n]
    (vertices the CC's faces reference), calls, error, msg[, inputs: each
    pass's soup as the hook saw it])."""
    import tempfile
    lib = _seam_lib()
    fin = bool(flags & MC_DISPATCH_VERTEX_ARRAY_FLOAT)
    ks, sa = _mesh_args(src, fin)
    kc, ca = _mesh_args(cut, fin)
    keep = []
    n_rep = 0 if passes is None else len(passes)
    arr = hashes = stats = None
    if n_rep:
        arr = (FeSeam * n_rep)(*[_fe_seam(p["hand_over"], keep) for p in passes])
        hashes = np.array([int(p.get("coord_hash", 0)) for p in passes], np.uint64)
        stats = np.array([int(bool(p.get("gp_violation", False))) for p in passes], np.int32)
    cc = np.zeros((max_cc, 3), np.int32)
    used = np.zeros(max_cc, np.int32)
    n_cc, calls, err = C.c_int(0), C.c_int(0), C.c_int(0)
    msg = C.create_string_buffer(256)
    with tempfile.TemporaryDirectory() as wd:
        res = lib.seam_dispatch(0 if passes is None else 1, int(bool(reference_numbering)), n_rep, arr,
                                None if hashes is None else hashes.ctypes.data,
                                None if stats is None else stats.ctypes.data,
                                *sa, *ca, int(flags), int(helpers), wd.encode(), cc.ctypes.data, used.ctypes.data,
                                max_cc, C.byref(n_cc), C.byref(calls), C.byref(err), msg, 256)
    del ks, kc, keep
    n = min(n_cc.value, max_cc)
    out = dict(result=int(res), ccs=cc[:n].copy(), used_vertices=used[:n].copy(), calls=calls.value,
               error=err.value, msg=msg.value.decode())
    if want_inputs:
        out["inputs"] = [_pass_input(lib, k) for k in range(calls.value)]
    return out


def _pass_input(lib, k):
    cnt = np.zeros(6, np.uint32)
    eps = C.c_double(0.0)
    lib.seam_pass_input(k, cnt.ctypes.data, C.byref(eps), None, None, None, None, None)
    vs, vc, fs, fc, ns, nc = (int(x) for x in cnt)
    x = np.zeros((vs + vc, 3), np.float64)
    si, ss = np.zeros(ns, np.uint32), np.zeros(fs, np.uint32)
    ci, cs = np.zeros(nc, np.uint32), np.zeros(fc, np.uint32)
    lib.seam_pass_input(k, cnt.ctypes.data, C.byref(eps), x.ctypes.data, si.ctypes.data, ss.ctypes.data,
                        ci.ctypes.data, cs.ctypes.data)
    tri = lambda sz: None if np.all(sz == 3) else sz  # noqa: E731
    return dict(src=dict(v=x[:vs].copy(), f=si, fs=tri(ss)), cut=dict(v=x[vs:].copy(), f=ci, fs=tri(cs)),
                cut_eps=float(eps.value))


def front_end_internal(src, cut, cut_eps: float, threads: int = 0):
    """One front-end pass of the oracle over internal (recentred) double
    coordinates with the given cut-box enlargement (oracle_front_end_internal).
    Same outputs as front_end."""
    lib, _, fr = _lib("port")
    if not hasattr(lib, "_internal_ready"):
        lib.oracle_front_end_internal.restype = C.c_int
        lib.oracle_front_end_internal.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                                  C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                                  C.c_double, C.c_int, C.POINTER(FeResult)]
        lib._internal_ready = True
    ks, sa = _mesh_args(src)
    kc, ca = _mesh_args(cut)
    res = FeResult()
    if lib.oracle_front_end_internal(*sa, *ca, float(cut_eps), int(threads), C.byref(res)) != 0:
        raise RuntimeError("oracle front_end_internal failed")
    out = dict(
        status=int(res.status), bad_face=int(res.bad_face), cut_eps=float(res.cut_eps),
        pairs=_arr(res.pairs, 2 * res.n_pairs, np.uint32).reshape(-1, 2),
        tests=_arr(res.tests, 3 * res.n_tests, np.uint32).reshape(-1, 3),
        test_info=_arr(res.test_info, 4 * res.n_tests, np.int8).reshape(-1, 4),
        rec_ids=_arr(res.rec_ids, 3 * res.n_records, np.uint32).reshape(-1, 3),
        rec_pts=_arr(res.rec_pts, 3 * res.n_records, np.float64).reshape(-1, 3),
    )
    fr(C.byref(res))
    del ks, kc
    return out


def _pts(*ps):
    return [np.ascontiguousarray(p, dtype=np.float64) for p in ps]


def ref_orient3d(a, b, c, d) -> float:
    lib, _, _ = _lib("ref")
    k = _pts(a, b, c, d)
    return lib.ref_orient3d(*[x.ctypes.data for x in k])


def ref_orient2d(a, b, c) -> float:
    lib, _, _ = _lib("ref")
    k = _pts(a, b, c)
    return lib.ref_orient2d(*[x.ctypes.data for x in k])


def port_orient3d_sign(a, b, c, d) -> int:
    lib, _, _ = _lib("port")
    lib.oracle_orient3d_sign.argtypes = [C.c_void_p] * 4
    k = _pts(a, b, c, d)
    return lib.oracle_orient3d_sign(*[x.ctypes.data for x in k])


def port_orient2d(a, b, c) -> float:
    lib, _, _ = _lib("port")
    lib.oracle_orient2d.restype = C.c_double
    lib.oracle_orient2d.argtypes = [C.c_void_p] * 3
    k = _pts(a, b, c)
    return lib.oracle_orient2d(*[x.ctypes.data for x in k])


def dispatch(src, cut, flags: int = MC_DISPATCH_VERTEX_ARRAY_DOUBLE, helpers: int = 0, max_cc: int = 4096):
    """Full reference mcDispatch. Returns status, CCs as (type, nverts, nfaces), and
    the intersection-point count of the last kernel invocation."""
    lib, _, _ = _lib("ref")
    fin = bool(flags & MC_DISPATCH_VERTEX_ARRAY_FLOAT)
    ks, sa = _mesh_args(src, fin)
    kc, ca = _mesh_args(cut, fin)
    info = np.zeros((max_cc, 3), dtype=np.int32)
    ncc = C.c_int(0)
    niv = C.c_long(-1)
    with tempfile.TemporaryDirectory() as td:
        rc = lib.ref_dispatch(*sa, *ca, int(flags), int(helpers), td.encode(), info.ctypes.data, max_cc,
                              C.byref(ncc), C.byref(niv))
    del ks, kc
    return dict(result=rc, ccs=info[:ncc.value].copy(), n_ivtx=int(niv.value))


class CcWire(C.Structure):
    _fields_ = [("type", C.c_int32), ("nv", C.c_uint32), ("nf", C.c_uint32), ("nidx", C.c_uint32),
                ("nadj", C.c_uint32), ("ne", C.c_uint32), ("vd", C.POINTER(C.c_double)),
                ("vf", C.POINTER(C.c_float)), ("face", C.POINTER(C.c_uint32)), ("fsize", C.POINTER(C.c_uint32)),
                ("adj", C.POINTER(C.c_uint32)), ("adjsize", C.POINTER(C.c_uint32)), ("edge", C.POINTER(C.c_uint32))]


def cc_wire(src, cut, flags: int = MC_DISPATCH_VERTEX_ARRAY_DOUBLE):
    """Full reference mcDispatch, then every connected component's arrays as
    mcGetConnectedComponentData returns them (frontend.cpp:2006-2832):
    (result, [dict(type, vd, vf, face, fsize, adj, adjsize, edge)])."""
    lib, _, _ = _lib("ref")
    lib.ref_cc_wire.restype = C.c_int
    lib.ref_cc_wire.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32,
                                C.c_uint32, C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.POINTER(CcWire))]
    lib.ref_cc_wire_free.argtypes = [C.POINTER(CcWire), C.c_int]
    fin = bool(flags & MC_DISPATCH_VERTEX_ARRAY_FLOAT)
    ks, sa = _mesh_args(src, fin)
    kc, ca = _mesh_args(cut, fin)
    n = C.c_int(0)
    w = C.POINTER(CcWire)()
    with tempfile.TemporaryDirectory() as td:
        rc = lib.ref_cc_wire(*sa, *ca, int(flags), td.encode(), C.byref(n), C.byref(w))
    del ks, kc
    out = []
    for i in range(n.value):
        c = w[i]
        out.append(dict(type=int(c.type), vd=_arr(c.vd, 3 * c.nv, np.float64).reshape(-1, 3),
                        vf=_arr(c.vf, 3 * c.nv, np.float32).reshape(-1, 3), face=_arr(c.face, c.nidx, np.uint32),
                        fsize=_arr(c.fsize, c.nf, np.uint32), adj=_arr(c.adj, c.nadj, np.uint32),
                        adjsize=_arr(c.adjsize, c.nf, np.uint32), edge=_arr(c.edge, 2 * c.ne, np.uint32)))
    if n.value:
        lib.ref_cc_wire_free(w, n.value)
    return rc, out


def cc_corners(face, fsize):
    """A component's faces in its halfedge mesh's corner order: the serialised
    face lists are the targets of each face's halfedges (get_vertices_around_face,
    hmesh.cpp:705-733), so corner i of the mesh is serialised entry i - 1."""
    off = np.concatenate([[0], np.cumsum(fsize.astype(np.int64))])
    out = np.empty_like(face)
    for i in range(len(fsize)):
        a, b = off[i], off[i + 1]
        out[a:b] = np.roll(face[a:b], 1)
    return out


def cc_wire_of_hmesh(h, fsize, vd):
    """Restatement of the wire arrays from a halfedge mesh (oracle.hmesh's dict
    over a component's faces in corner order): vertices around each face (the
    targets of its corner halfedges), the faces across each of its halfedges
    that have one (get_faces_around_face, hmesh.cpp:796-818) with their counts,
    each edge's vertex(e, 0) / vertex(e, 1) (the targets of halfedges 2e and
    2e + 1, hmesh.cpp:234-256), and the float vertices (static_cast<float>)."""
    ch = h["corner_he"].astype(np.int64)
    face = h["he_target"][ch]
    across = h["he_face"][ch ^ 1]
    off = np.concatenate([[0], np.cumsum(fsize.astype(np.int64))])
    fid = np.repeat(np.arange(len(fsize)), fsize.astype(np.int64))
    keep = across >= 0
    adj = across[keep].astype(np.uint32)
    adjsize = np.bincount(fid[keep], minlength=len(fsize)).astype(np.uint32)
    edge = h["he_target"].astype(np.uint32)  # 2e then 2e + 1: vertex(e, 0), vertex(e, 1)
    return dict(face=face.astype(np.uint32), adj=adj, adjsize=adjsize, edge=edge,
                vf=np.asarray(vd, dtype=np.float64).astype(np.float32))


HM_OK, HM_FACE_SIZE, HM_INDEX_RANGE, HM_DUPLICATE_INDEX, HM_NON_MANIFOLD, HM_TOO_SMALL, HM_COMPONENTS = range(7)


class HmResult(C.Structure):
    _fields_ = [
        ("status", C.c_int32), ("bad_face", C.c_int32), ("n_edges", C.c_uint32), ("n_components", C.c_uint32),
        ("closed", C.c_int32), ("he_target", C.POINTER(C.c_uint32)), ("he_face", C.POINTER(C.c_int32)),
        ("he_next", C.POINTER(C.c_int32)), ("he_prev", C.POINTER(C.c_int32)),
        ("corner_he", C.POINTER(C.c_uint32)), ("v_off", C.POINTER(C.c_uint32)), ("v_he", C.POINTER(C.c_uint32)),
    ]


def hmesh(f, fs, nv: int, impl: str = "port"):
    """One mesh's halfedge mesh and input checks (the connectivity MCUT builds
    from the caller's arrays): status, failing face, edges, and per halfedge
    its target / face / next / prev, per face corner its halfedge, per vertex
    the halfedges ending there (CSR), the connected-component count and
    whether every halfedge has a face."""
    lib, _, _ = _lib(impl)
    fn = lib.oracle_hmesh if impl == "port" else lib.ref_hmesh
    fr = lib.oracle_hmesh_free if impl == "port" else lib.ref_hmesh_free
    fn.restype = C.c_int
    fn.argtypes = [C.c_void_p, C.c_void_p, C.c_uint32, C.c_uint32, C.POINTER(HmResult)]
    fr.argtypes = [C.POINTER(HmResult)]
    f = np.ascontiguousarray(f, dtype=np.uint32)
    fs = None if fs is None else np.ascontiguousarray(fs, dtype=np.uint32)
    nf = int(len(fs)) if fs is not None else int(len(f) // 3)
    res = HmResult()
    rc = fn(f.ctypes.data if len(f) else None, None if fs is None else fs.ctypes.data, int(nv), nf, C.byref(res))
    if rc != 0:
        raise RuntimeError(f"{impl} hmesh failed rc={rc}")
    out = dict(status=int(res.status), bad_face=int(res.bad_face), n_edges=int(res.n_edges),
               n_components=int(res.n_components), closed=bool(res.closed))
    if res.status in (HM_OK, HM_TOO_SMALL, HM_COMPONENTS):
        nh = 2 * res.n_edges
        out.update(
            he_target=_arr(res.he_target, nh, np.uint32), he_face=_arr(res.he_face, nh, np.int32),
            he_next=_arr(res.he_next, nh, np.int32), he_prev=_arr(res.he_prev, nh, np.int32),
            corner_he=_arr(res.corner_he, len(f), np.uint32), v_off=_arr(res.v_off, nv + 1, np.uint32),
            v_he=_arr(res.v_he, nh, np.uint32))
    fr(C.byref(res))
    return out


class CpResult(C.Structure):
    _fields_ = [("status", C.c_int32), ("bad_key", C.c_uint32), ("n_edges", C.c_uint32),
                ("edge_src", C.POINTER(C.c_uint32)), ("edge_tgt", C.POINTER(C.c_uint32)),
                ("n_faces", C.c_uint32), ("face_keys", C.POINTER(C.c_uint32)), ("face_off", C.POINTER(C.c_uint32)),
                ("face_edges", C.POINTER(C.c_uint32)),
                ("n_ivtx", C.c_uint32), ("ivtx_off", C.POINTER(C.c_uint32)), ("ivtx_he", C.POINTER(C.c_uint32))]


def soup_faces(src, cut):
    """The polygon soup's faces with their corners in the soup's order: a
    source face starts at its second corner (the targets of its halfedges),
    a cut face at its third (cs.get_vertices_around_face of the soup's
    edge-created face); cut vertex ids offset by the source vertex count.
    -> (offsets, indices) as the ps numbers faces (source, then cut)."""
    offs, idxs, base = [np.zeros(1, np.int64)], [], 0
    vs = len(src["v"])
    for m, rot, vo in ((src, 1, 0), (cut, 2, vs)):
        f = np.asarray(m["f"], dtype=np.int64) + vo
        if m.get("fs") is None:  # triangles: one roll of every row
            idxs.append(np.roll(f.reshape(-1, 3), -rot, axis=1).reshape(-1))
            offs.append(base + 3 * np.arange(1, len(f) // 3 + 1, dtype=np.int64))
            base += len(f)
            continue
        fs = np.asarray(m["fs"], dtype=np.int64)
        o = np.concatenate([[0], np.cumsum(fs)])
        for k in range(len(fs)):
            face = f[o[k]:o[k + 1]]
            r = rot % len(face)
            idxs.append(np.concatenate([face[r:], face[:r]]))
        offs.append(base + o[1:])
        base += int(o[-1])
    return np.concatenate(offs).astype(np.uint32), np.concatenate(idxs).astype(np.uint32)


def cutpath(nv, x, soup_off, soup_idx, registry, ivtx_xyz, cp_pairs, cp_off, cp_vtx):
    """MCUT's cut-path edge creation from a record hand-over (kernel.cpp:
    3332-3632, oracle_cutpath). registry: per intersection vertex (m0 id nv +
    i) its tested face and the tested edge's two faces (UINT32_MAX: none).
    -> dict(status, bad_key, edges [E,2] (src, tgt; halfedge 2e runs src ->
    tgt), face_keys, face_off, face_edges, ivtx_off, ivtx_he)."""
    lib, _, _ = _lib("port")
    if not hasattr(lib, "_cutpath_ready"):
        lib.oracle_cutpath.restype = C.c_int
        lib.oracle_cutpath.argtypes = [C.c_uint32, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_uint32,
                                       C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p,
                                       C.POINTER(CpResult)]
        lib.oracle_cutpath_free.argtypes = [C.POINTER(CpResult)]
        lib._cutpath_ready = True
    keep = []

    def arr(a, dt):
        a = np.ascontiguousarray(np.asarray(a, dtype=dt).reshape(-1))
        keep.append(a)
        return a.ctypes.data if a.size else None
    reg = np.asarray(registry, np.uint32).reshape(-1, 3)
    nf = len(soup_off) - 1
    res = CpResult()
    rc = lib.oracle_cutpath(int(nv), arr(x, np.float64), nf, arr(soup_off, np.uint32), arr(soup_idx, np.uint32),
                            len(reg), arr(reg, np.uint32), arr(ivtx_xyz, np.float64),
                            len(cp_off) - 1, arr(cp_pairs, np.uint32), arr(cp_off, np.uint32),
                            arr(cp_vtx, np.uint32), C.byref(res))
    if rc != 0:
        raise RuntimeError("oracle_cutpath failed")
    ne = int(res.n_edges)
    out = dict(status=int(res.status), bad_key=int(res.bad_key),
               edges=np.stack([_arr(res.edge_src, ne, np.uint32), _arr(res.edge_tgt, ne, np.uint32)], 1),
               face_keys=_arr(res.face_keys, res.n_faces, np.uint32),
               face_off=_arr(res.face_off, res.n_faces + 1, np.uint32),
               ivtx_off=_arr(res.ivtx_off, res.n_ivtx + 1, np.uint32))
    out["face_edges"] = _arr(res.face_edges, int(out["face_off"][-1]) if res.n_faces else 0, np.uint32)
    out["ivtx_he"] = _arr(res.ivtx_he, int(out["ivtx_off"][-1]) if res.n_ivtx else 0, np.uint32)
    lib.oracle_cutpath_free(C.byref(res))
    return out


def cutpath_of(src, cut, xyz, hand, soup=None):
    """The cut path of a pass from its internal coordinates (source then cut
    vertices) and its record hand-over (oracle.seam's keys); soup: the
    (offsets, indices) of soup_faces when already made."""
    off, idx = soup if soup is not None else soup_faces(src, cut)
    rid = np.asarray(hand["rec_ids"], np.uint32).reshape(-1, 5)
    return cutpath(len(xyz), xyz, off, idx, rid[:, 2:5], hand["rec_pts"], hand["cp_pairs"], hand["cp_off"],
                   hand["cp_vtx"])


def observe_cutpath(src, cut, flags: int = MC_DISPATCH_VERTEX_ARRAY_DOUBLE, helpers: int = 0):
    """The unmodified reference's mcDispatch with its cut-path edge creation
    (kernel.cpp:3332-3632) observed, once per front-end pass: its inputs in
    the form cutpath() takes them and its outputs (edges in creation order,
    ps_iface_to_m0_edge_list by face, ivtx_to_incoming_hlist per intersection
    vertex). -> (mcDispatch result, [dict(inputs..., want=dict(edges,
    face_keys, face_off, face_edges, ivtx_off, ivtx_he), bad)])."""
    lib = _seam_lib()
    if not hasattr(lib, "_cutpath_obs"):
        lib.seam_cutpath_count.restype = C.c_int
        lib.seam_cutpath_observation.restype = C.c_int
        lib.seam_cutpath_observation.argtypes = [C.c_int, C.c_void_p] + [C.c_void_p] * 14
        lib._cutpath_obs = True
    res = observe_reference(src, cut, flags=flags, helpers=helpers)
    obs = []
    for k in range(lib.seam_cutpath_count()):
        sz = np.zeros(16, np.uint64)
        lib.seam_cutpath_observation(k, sz.ctypes.data, *([None] * 14))
        n = [int(v) for v in sz]
        x, ix = np.zeros(n[1]), np.zeros(n[5])
        u = [np.zeros(n[i], np.uint32) for i in (2, 3, 4, 6, 7, 8, 9, 10, 11, 12, 13, 14)]
        lib.seam_cutpath_observation(k, sz.ctypes.data, x.ctypes.data, ix.ctypes.data, *[a.ctypes.data for a in u])
        soup_off, soup_idx, reg, key_pairs, key_off, key_vtx, edges, face_keys, face_off, face_edges, ivtx_off, \
            ivtx_he = u
        obs.append(dict(nv=n[0], x=x.reshape(-1, 3), soup_off=soup_off, soup_idx=soup_idx, reg=reg.reshape(-1, 3),
                        ivtx_xyz=ix.reshape(-1, 3), cp_pairs=key_pairs.reshape(-1, 2), cp_off=key_off,
                        cp_vtx=key_vtx, bad=n[15],
                        want=dict(edges=edges.reshape(-1, 2), face_keys=face_keys, face_off=face_off,
                                  face_edges=face_edges, ivtx_off=ivtx_off, ivtx_he=ivtx_he)))
    return res["result"], obs


class FpResult(C.Structure):
    _fields_ = [("n_polygons", C.c_uint32), ("faces", C.POINTER(C.c_uint32)), ("off", C.POINTER(C.c_uint32)),
                ("vtx", C.POINTER(C.c_uint32)), ("normals", C.POINTER(C.c_double)), ("mc", C.POINTER(C.c_int32))]


def floating(nv, registry, edges, x=None, soup=None):
    """MCUT's floating-polygon detection (kernel.cpp:4078-4200,
    oracle_floating) from the cut path: -> dict(faces, off, vtx, normals, mc)
    with each polygon's m0 vertex ids in cycle order from its smallest; with
    the ps coordinates x and the soup's (offsets, indices) each face's unit
    normal and largest component."""
    lib, _, _ = _lib("port")
    if not hasattr(lib, "_floating_ready"):
        lib.oracle_floating.restype = C.c_int
        lib.oracle_floating.argtypes = [C.c_uint32, C.c_void_p, C.c_void_p, C.c_void_p, C.c_uint32, C.c_void_p,
                                        C.c_uint32, C.c_void_p, C.POINTER(FpResult)]
        lib.oracle_floating_free.argtypes = [C.POINTER(FpResult)]
        lib._floating_ready = True
    reg = np.ascontiguousarray(np.asarray(registry, np.uint32).reshape(-1, 3))
    e = np.ascontiguousarray(np.asarray(edges, np.uint32).reshape(-1, 2))
    keep = []
    if x is not None:
        keep = [np.ascontiguousarray(x, np.float64).reshape(-1), np.ascontiguousarray(soup[0], np.uint32),
                np.ascontiguousarray(soup[1], np.uint32)]
    res = FpResult()
    lib.oracle_floating(int(nv), *([k.ctypes.data for k in keep] if keep else [None, None, None]), len(reg),
                        reg.ctypes.data if reg.size else None, len(e), e.ctypes.data if e.size else None,
                        C.byref(res))
    n = int(res.n_polygons)
    out = dict(faces=_arr(res.faces, n, np.uint32), off=_arr(res.off, n + 1, np.uint32),
               normals=_arr(res.normals, 3 * n, np.float64).reshape(-1, 3), mc=_arr(res.mc, n, np.int32))
    out["vtx"] = _arr(res.vtx, int(out["off"][-1]) if n else 0, np.uint32)
    lib.oracle_floating_free(C.byref(res))
    return out


def observe_floating(src, cut, flags: int = MC_DISPATCH_VERTEX_ARRAY_DOUBLE, helpers: int = 0):
    """The unmodified reference's mcDispatch with its cut path and its
    floating-polygon detection observed, per front-end pass that reached the
    detection: (result, cut-path observations, [dict(faces, off, mc, normals
    [P,3], xyz [V,3])]). A pass's floating observation follows its cut-path
    observation."""
    result, cps = observe_cutpath(src, cut, flags=flags, helpers=helpers)
    lib = _seam_lib()
    if not hasattr(lib, "_floating_obs"):
        lib.seam_floating_count.restype = C.c_int
        lib.seam_floating_observation.restype = C.c_int
        lib.seam_floating_observation.argtypes = [C.c_int, C.c_void_p] + [C.c_void_p] * 5
        lib._floating_obs = True
    obs = []
    for k in range(lib.seam_floating_count()):
        sz = np.zeros(2, np.uint64)
        lib.seam_floating_observation(k, sz.ctypes.data, None, None, None, None, None)
        p, v = int(sz[0]), int(sz[1])
        faces, off, mc = np.zeros(p, np.uint32), np.zeros(p + 1, np.uint32), np.zeros(p, np.uint32)
        normals, xyz = np.zeros((p, 3)), np.zeros((v, 3))
        lib.seam_floating_observation(k, sz.ctypes.data, faces.ctypes.data, off.ctypes.data, mc.ctypes.data,
                                      normals.ctypes.data, xyz.ctypes.data)
        obs.append(dict(faces=faces, off=off, mc=mc, normals=normals, xyz=xyz))
    return result, cps, obs
