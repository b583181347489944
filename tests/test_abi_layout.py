"""The ctypes mirrors of the C structs have the C compiler's layout.

A small C program compiled against include/mcut_gb300.h (and the oracle's
header) prints sizeof / offsetof of every field; each ctypes Structure the
Python host and the tests pass across the boundary must agree field for
field. This also compiles the public header as plain C99.
"""
import ctypes as C
import os
import re
import shutil
import subprocess

import pytest

from mcut_gb300 import _lib as L
import oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
BUILD = os.path.join(ROOT, "tests", "_build")

STRUCTS = [
    ("mcgpu_mesh", L.Mesh), ("mcgpu_batch", L.Batch), ("mcgpu_summary", L.Summary),
    ("mcgpu_tuning", L.Tuning), ("mcgpu_server_config", L.ServerConfig), ("mcgpu_server_stats", L.ServerStats),
    ("mcgpu_hmesh_report", L.HmeshReport),
    ("fe_result", oracle.FeResult), ("hm_result", oracle.HmResult),
]


def _header_constants():
    with open(L.HEADER) as fh:
        return sorted(set(re.findall(r"\bMCGPU_[A-Z0-9_]+\b", fh.read())))


def _oracle_constants():
    with open(os.path.join(ROOT, "oracle", "mcut_oracle.h")) as fh:
        return sorted(set(re.findall(r"\b(?:FE|HM)_[A-Z0-9_]+\b", fh.read())))


def _c_layout():
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "mcut_gb300.h"', '#include "mcut_oracle.h"',
             "int main(void) {"]
    for name in _header_constants() + _oracle_constants():
        lines.append(f'  printf("{name} %llu\\n", (unsigned long long)({name}));')
    for cname, cls in STRUCTS:
        lines.append(f'  printf("{cname} %zu\\n", sizeof({cname}));')
        for field, _ in cls._fields_:
            lines.append(f'  printf("{cname}.{field} %zu %zu\\n", offsetof({cname}, {field}), '
                         f'sizeof((({cname}*)0)->{field}));')
    lines += ["  return 0;", "}"]
    os.makedirs(BUILD, exist_ok=True)
    src, exe = os.path.join(BUILD, "layout.c"), os.path.join(BUILD, "layout")
    with open(src, "w") as fh:
        fh.write("\n".join(lines) + "\n")
    subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                    "-I", os.path.join(ROOT, "oracle"), "-o", exe, src], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    lay = {}
    for ln in out.splitlines():
        name, *nums = ln.split()
        lay[name] = tuple(int(x) for x in nums)
    return lay


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_ctypes_structs_match_the_c_layout():
    lay = _c_layout()
    for cname, cls in STRUCTS:
        assert lay[cname] == (C.sizeof(cls),), cname
        for field, _ in cls._fields_:
            d = getattr(cls, field)
            assert lay[f"{cname}.{field}"] == (d.offset, d.size), (cname, field)


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_python_constants_match_the_header():
    """Every status, flag, data query and stage the header names has the same
    value in the Python host."""
    lay = _c_layout()
    checked = 0
    for name in _header_constants():
        short = name[len("MCGPU_"):]
        if short.startswith("STAGE_"):
            want = L.STAGES.index(short[len("STAGE_"):].lower())
        else:
            want = getattr(L, short)
        assert lay[name] == (want,), name
        checked += 1
    assert checked == len(_header_constants()) >= 30


@pytest.mark.skipif(shutil.which("gcc") is None, reason="no C compiler")
def test_oracle_constants_match_its_header():
    lay = _c_layout()
    names = _oracle_constants()
    for name in names:
        assert lay[name] == (getattr(oracle, name),), name
    assert len(names) >= 12
