"""ctypes binding of libmcut_gb300.so (the C ABI declared in include/mcut_gb300.h).

The library is the product: there is no CPU fallback. Loading fails loudly
when it has not been built.
"""
from __future__ import annotations

import ctypes as C
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libmcut_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "mcut_gb300.h")

OK, GP_VIOLATION, DEGENERATE_SRC_FACE, DEGENERATE_CUT_FACE, INVALID_INPUT, CUDA_ERROR, OUT_OF_MEMORY, \
    INVALID_VALUE, TOO_LARGE, NOT_READY, CANCELLED = range(11)
STATUS_NAMES = ["OK", "GP_VIOLATION", "DEGENERATE_SRC_FACE", "DEGENERATE_CUT_FACE", "INVALID_INPUT",
                "CUDA_ERROR", "OUT_OF_MEMORY", "INVALID_VALUE", "TOO_LARGE", "NOT_READY", "CANCELLED"]
NO_CUT = 0xFFFFFFFF

VERTEX_ARRAY_FLOAT = 1 << 0
RECENTRE = 1 << 1
KEEP_TESTS = 1 << 2
KEEP_PAIRS = 1 << 3
PROFILE = 1 << 4
DEVICE_POINTERS = 1 << 5
ENFORCE_GENERAL_POSITION = 1 << 6
ENFORCE_GENERAL_POSITION_ABSOLUTE = 1 << 7

DATA_RECORD_IDS, DATA_RECORD_POINTS, DATA_PAIRS, DATA_TESTS, DATA_TEST_INFO, DATA_VERTICES, DATA_FACE_BOXES, \
    DATA_RECORD_OFFSETS = range(1, 9)
# the record hand-over of a single dispatch (the maps dispatch()'s host stages read)
DATA_EDGE_RECORD_OFFSETS, DATA_CUTPATH_PAIRS, DATA_CUTPATH_OFFSETS, DATA_CUTPATH_VERTICES, DATA_FACE_KEYS, \
    DATA_FACE_OFFSETS, DATA_FACE_VERTICES, DATA_BORDER_VERTICES, DATA_PARTIAL_CUT = range(9, 18)

# the halfedge mesh of the last mcgpu_halfedge_mesh call
DATA_HE_TARGET, DATA_HE_FACE, DATA_HE_NEXT, DATA_HE_PREV, DATA_CORNER_HE, DATA_VERTEX_HE_OFFSETS, \
    DATA_VERTEX_HE = range(18, 25)
# the cut path of a single dispatch (m0's edges from the hand-over)
DATA_CUTPATH_STATUS, DATA_CUTPATH_EDGES, DATA_CUTPATH_FACE_KEYS, DATA_CUTPATH_FACE_OFFSETS, \
    DATA_CUTPATH_FACE_EDGES, DATA_CUTPATH_VERTEX_OFFSETS, DATA_CUTPATH_VERTEX_HALFEDGES = range(25, 32)
# its floating polygons
DATA_FLOATING_FACES, DATA_FLOATING_OFFSETS, DATA_FLOATING_VERTICES, DATA_FLOATING_NORMALS, \
    DATA_FLOATING_NORMAL_COMPONENTS = range(32, 37)
# a connected component's arrays as MCUT serialises them, from the last halfedge mesh
DATA_CC_FACE, DATA_CC_FACE_ADJACENT_FACE_SIZE, DATA_CC_FACE_ADJACENT_FACE, DATA_CC_EDGE, \
    DATA_CC_VERTEX_FLOAT = range(37, 42)
# mcgpu_hmesh_status (the oracle's HM_* values)
HMESH_OK, HMESH_FACE_SIZE, HMESH_INDEX_RANGE, HMESH_DUPLICATE_INDEX, HMESH_NON_MANIFOLD, HMESH_TOO_SMALL, \
    HMESH_COMPONENTS = range(7)

STAGES = ["upload", "bounds", "sort", "hierarchy", "traverse", "adjacency", "narrow", "download"]


class Mesh(C.Structure):
    _fields_ = [("vertices", C.c_void_p), ("face_indices", C.c_void_p), ("face_sizes", C.c_void_p),
                ("num_vertices", C.c_uint32), ("num_faces", C.c_uint32)]


class Batch(C.Structure):
    _fields_ = [("num_pairs", C.c_uint32), ("vertices", C.c_void_p), ("face_indices", C.c_void_p),
                ("face_sizes", C.c_void_p), ("mesh_counts", C.c_void_p), ("cut_eps", C.c_void_p)]


class Summary(C.Structure):
    _fields_ = [("status", C.c_int32), ("bad_face", C.c_int32), ("cut_eps", C.c_double),
                ("num_pairs", C.c_uint64), ("num_tests", C.c_uint64), ("num_records", C.c_uint64),
                ("escalations", C.c_uint64 * 3), ("stage_ms", C.c_float * 8),
                ("kernel_launches", C.c_uint32), ("perturbations", C.c_uint32),
                ("perturbation", C.c_double * 3)]


class Tuning(C.Structure):
    _fields_ = [("leaf_size", C.c_uint32), ("traversal", C.c_uint32), ("packet_faces", C.c_uint32),
                ("stack_depth", C.c_uint32), ("split_round", C.c_uint32)]


class ServerConfig(C.Structure):
    _fields_ = [("device", C.c_int), ("workers", C.c_uint32), ("max_batch_pairs", C.c_uint32),
                ("max_batch_faces", C.c_uint64), ("hbm_budget_bytes", C.c_uint64), ("linger_us", C.c_uint32),
                ("reserved", C.c_uint32)]


class ServerStats(C.Structure):
    _fields_ = [(k, C.c_uint64) for k in ("submitted", "completed", "batches", "pending", "inflight_bytes",
                                          "peak_inflight_bytes", "resident_bytes", "resident_meshes",
                                          "pool_bytes", "peak_reserved_bytes", "pool_trims", "cancelled")]


class HmeshReport(C.Structure):
    _fields_ = [("status", C.c_int32), ("bad_face", C.c_int32), ("num_edges", C.c_uint32),
                ("num_components", C.c_uint32), ("closed", C.c_int32), ("kernel_launches", C.c_uint32)]


class LibraryNotBuilt(RuntimeError):
    pass


_lib = None


def exported_names_in_header(path: str = HEADER):
    """Every function the C header declares."""
    txt = open(path).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(mcgpu_\w+)\s*\(", txt, re.M)))


def load():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise LibraryNotBuilt(f"{LIB_PATH} is missing: run `python -m mcut_gb300.build` (needs nvcc)")
    lib = C.CDLL(LIB_PATH)
    ctx = C.c_void_p
    lib.mcgpu_context_create.argtypes = [C.POINTER(ctx), C.c_int]
    lib.mcgpu_context_release.argtypes = [ctx]
    lib.mcgpu_dispatch.argtypes = [ctx, C.c_uint32, C.POINTER(Mesh), C.POINTER(Mesh), C.c_double,
                                   C.POINTER(Summary)]
    lib.mcgpu_dispatch_batch.argtypes = [ctx, C.c_uint32, C.c_uint32, C.POINTER(Mesh), C.POINTER(Mesh),
                                         C.POINTER(C.c_double), C.POINTER(Summary)]
    lib.mcgpu_dispatch_packed.argtypes = [ctx, C.c_uint32, C.POINTER(Batch), C.POINTER(Summary)]
    lib.mcgpu_get_data.argtypes = [ctx, C.c_uint32, C.c_uint64, C.c_void_p, C.POINTER(C.c_uint64)]
    lib.mcgpu_get_batch_data.argtypes = [ctx, C.c_uint32, C.c_uint32, C.c_uint64, C.c_void_p,
                                         C.POINTER(C.c_uint64)]
    lib.mcgpu_recentre.argtypes = [C.c_uint32, C.POINTER(Mesh), C.POINTER(Mesh), C.c_void_p, C.c_void_p,
                                   C.POINTER(C.c_double)]
    lib.mcgpu_dispatch_noalloc.argtypes = [C.c_void_p, C.POINTER(Mesh), C.POINTER(Mesh), C.c_double, C.c_void_p,
                                           C.c_void_p, C.c_uint64, C.POINTER(Summary)]
    lib.mcgpu_context_set_tuning.argtypes = [ctx, C.POINTER(Tuning)]
    lib.mcgpu_context_get_tuning.argtypes = [ctx, C.POINTER(Tuning)]
    lib.mcgpu_context_set_general_position.argtypes = [ctx, C.c_double, C.c_uint32]
    lib.mcgpu_context_get_general_position.argtypes = [ctx, C.POINTER(C.c_double), C.POINTER(C.c_uint32)]
    lib.mcgpu_autotune.argtypes = [ctx, C.c_uint32, C.POINTER(Batch), C.c_uint32, C.POINTER(Tuning),
                                   C.POINTER(C.c_float)]
    lib.mcgpu_context_get_memory.argtypes = [ctx, C.POINTER(C.c_uint64), C.POINTER(C.c_uint64)]
    lib.mcgpu_context_set_memory_limit.argtypes = [ctx, C.c_uint64]
    lib.mcgpu_context_trim.argtypes = [ctx]
    lib.mcgpu_measure_fp64_rate.argtypes = [C.c_int, C.POINTER(C.c_double)]
    srv = C.c_void_p
    lib.mcgpu_server_create.argtypes = [C.POINTER(srv), C.POINTER(ServerConfig)]
    lib.mcgpu_server_release.argtypes = [srv]
    lib.mcgpu_server_add_cut_mesh.argtypes = [srv, C.POINTER(Mesh), C.POINTER(C.c_uint32)]
    lib.mcgpu_server_submit.argtypes = [srv, C.POINTER(Mesh), C.POINTER(Mesh), C.c_uint32, C.POINTER(C.c_uint64)]
    lib.mcgpu_server_wait.argtypes = [srv, C.c_uint64, C.c_int, C.POINTER(Summary), C.POINTER(C.c_double)]
    lib.mcgpu_server_get_data.argtypes = [srv, C.c_uint64, C.c_uint32, C.c_uint64, C.c_void_p, C.POINTER(C.c_uint64)]
    lib.mcgpu_server_release_request.argtypes = [srv, C.c_uint64]
    lib.mcgpu_server_cancel.argtypes = [srv, C.c_uint64]
    lib.mcgpu_server_get_stats.argtypes = [srv, C.POINTER(ServerStats)]
    lib.mcgpu_last_error.restype = C.c_char_p
    for name in exported_names_in_header():
        if name not in ("mcgpu_last_error",):
            getattr(lib, name).restype = C.c_int
    _lib = lib
    return lib


def last_error() -> str:
    return load().mcgpu_last_error().decode()


def check(rc: int, what: str):
    if rc != OK:
        raise RuntimeError(f"{what} failed: {STATUS_NAMES[rc] if 0 <= rc < len(STATUS_NAMES) else rc}: "
                           f"{last_error()}")
