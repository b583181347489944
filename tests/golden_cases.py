"""Loader for the committed golden fixtures (tests/golden/*.npz)."""
from __future__ import annotations

import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FE_KEYS = ["pairs", "tests", "test_info", "rec_ids", "rec_pts"]


def _mesh(z, pre):
    fs = z[pre + "fs"]
    return dict(v=z[pre + "v"], f=z[pre + "f"], fs=fs if fs.size else None)


def load(fname):
    """-> {case name: dict(src, cut, status, bad_face, cut_eps, float_input, pairs, ...)}"""
    z = np.load(os.path.join(GOLDEN, fname))
    names = sorted({k.split("/")[0] for k in z.files})
    out = {}
    for n in names:
        c = dict(src=_mesh(z, n + "/src_"), cut=_mesh(z, n + "/cut_"))
        for k in ["status", "bad_face", "cut_eps", "float_input"] + FE_KEYS:
            c[k] = z[n + "/" + k]
        for k in ["mc_result", "mc_ccs", "mc_ivtx"]:
            if n + "/" + k in z.files:
                c[k] = z[n + "/" + k]
        out[n] = c
    return out


def all_cases():
    out = {}
    for f in ("benchmarks.npz", "named.npz", "synthetic.npz", "configs.npz"):
        out.update(load(f))
    return out


def same_bits(a, b):
    a, b = np.asarray(a), np.asarray(b)
    if a.shape != b.shape:
        return False
    if a.dtype.kind == "f":
        return bool(np.array_equal(a.view(np.uint64 if a.itemsize == 8 else np.uint32),
                                   b.astype(a.dtype).view(np.uint64 if a.itemsize == 8 else np.uint32)))
    return bool(np.array_equal(a, b))


def perturbation_cube():
    """The cube of the reference's general-position test
    (tests/source/perturbationState.cpp:47-68): float vertices, six quads;
    cut by itself every face is coplanar with a face of the other mesh."""
    v = np.array([-1, -1, 1, 1, -1, 1, 1, -1, -1, -1, -1, -1,
                  -1, 1, 1, 1, 1, 1, 1, 1, -1, -1, 1, -1], np.float32).reshape(-1, 3)
    f = np.array([3, 2, 1, 0, 4, 5, 6, 7, 0, 1, 5, 4, 1, 2, 6, 5, 2, 3, 7, 6, 3, 0, 4, 7], np.uint32)
    return dict(v=v, f=f, fs=np.full(6, 4, np.uint32))
