"""The C ABI library builds, loads and exports what include/mcut_gb300.h declares.

CPU-only: no compute call touches a GPU here. mcgpu_recentre is host code
and is checked bit-for-bit against the oracle's restatement of the
reference's recentring.
"""
import ctypes as C
import os
import subprocess

import numpy as np
import pytest

import golden_cases as G
import oracle
from mcut_gb300 import _lib as L
from mcut_gb300 import meshgen
from mcut_gb300.frontend import recentre


@pytest.fixture(scope="module", autouse=True)
def _built():
    if not os.path.exists(L.LIB_PATH):
        from mcut_gb300 import build
        build.build()
    oracle.build()


def test_every_declared_symbol_is_exported():
    declared = L.exported_names_in_header()
    assert len(declared) >= 8
    out = subprocess.run(["nm", "-D", "--defined-only", L.LIB_PATH], capture_output=True, text=True, check=True)
    exported = {line.split()[-1] for line in out.stdout.splitlines() if " T " in line}
    missing = [d for d in declared if d not in exported]
    assert not missing, missing


def test_library_loads_and_binds():
    lib = L.load()
    for name in L.exported_names_in_header():
        assert hasattr(lib, name)


def test_header_is_plain_c():
    import re
    txt = re.sub(r"/\*.*?\*/", "", open(L.HEADER).read(), flags=re.S)
    txt = re.sub(r"//[^\n]*", "", txt)
    assert "torch" not in txt and "at::" not in txt and "std::" not in txt and "class " not in txt


@pytest.mark.parametrize("case", ["two_spheres", "crack0", "sphere_hf_small_x16"])
def test_host_recentre_matches_oracle(case):
    c = G.load("synthetic.npz")[case]
    s, k, eps = recentre(c["src"], c["cut"])
    o = oracle.front_end(c["src"], c["cut"], impl="port")
    assert G.same_bits(s, o["src_xyz"]) and G.same_bits(k, o["cut_xyz"])
    assert G.same_bits(eps, c["cut_eps"])


def test_host_recentre_float_input_matches_oracle():
    c = G.load("configs.npz")["cross_float"]
    s, k, eps = recentre(c["src"], c["cut"], float_input=True)
    o = oracle.front_end(c["src"], c["cut"], impl="port", float_input=True)
    assert G.same_bits(s, o["src_xyz"]) and G.same_bits(k, o["cut_xyz"])
    assert G.same_bits(eps, c["cut_eps"])


def test_null_arguments_are_errors_not_crashes():
    lib = L.load()
    eps = C.c_double(0)
    assert lib.mcgpu_recentre(0, None, None, None, None, C.byref(eps)) == L.INVALID_VALUE
    assert "null" in L.last_error()
    assert lib.mcgpu_context_create(None, 0) == L.INVALID_VALUE
    assert lib.mcgpu_context_set_general_position(None, 1e-4, 4) == L.INVALID_VALUE
    assert lib.mcgpu_context_get_general_position(None, None, None) == L.INVALID_VALUE
    assert lib.mcgpu_get_data(None, L.DATA_RECORD_IDS, 0, None, None) == L.INVALID_VALUE
    b = L.Batch(0, None, None, None, None, None)
    assert lib.mcgpu_dispatch_packed(None, 0, C.byref(b), None) == L.INVALID_VALUE


def test_pack_pairs_layout():
    """The packed batch is the internal layout: per pair source then cut
    vertices (recentred), source then cut local indices, counts per mesh."""
    from mcut_gb300 import pack_pairs
    pairs = meshgen.batch_pairs(5, seed=meshgen.SEED_BASE + 41)
    pk = pack_pairs(pairs)
    v0 = f0 = 0
    for i, (s, c) in enumerate(pairs):
        sx, cx, eps = recentre(s, c)
        nsv, nsf, ncv, ncf = (int(x) for x in pk["counts"][i])
        assert (nsv, ncv) == (s["v"].shape[0], c["v"].shape[0])
        assert (nsf, ncf) == (meshgen.num_faces(s), meshgen.num_faces(c))
        assert G.same_bits(pk["v"][v0:v0 + nsv], sx) and G.same_bits(pk["v"][v0 + nsv:v0 + nsv + ncv], cx)
        assert np.array_equal(pk["f"][f0:f0 + 3 * nsf], s["f"])
        assert np.array_equal(pk["f"][f0 + 3 * nsf:f0 + 3 * (nsf + ncf)], c["f"])
        assert G.same_bits(pk["eps"][i], eps)
        v0 += nsv + ncv
        f0 += 3 * (nsf + ncf)
    assert v0 == pk["v"].shape[0] and f0 == pk["f"].shape[0]
