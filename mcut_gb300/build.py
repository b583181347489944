"""Build the GB300 front-end library in-tree (no cmake, no torch extension).

    python -m mcut_gb300.build      ->  mcut_gb300/libmcut_gb300.so

Each .cu compiles to an object in parallel, for sm_103a only, with
--fmad=false (every multiply and add rounds separately, as the reference's
fp64 arithmetic does) and -lineinfo for ncu source attribution.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libmcut_gb300.so")
OBJ = os.path.join(HERE, "_build")
SOURCES = ["fe_sort.cu", "fe_kernels.cu", "fe_derived.cu", "fe_cutpath.cu", "fe_hmesh.cu", "fe_api.cu", "fe_noalloc.cu", "fe_server.cu"]
NVCC = os.environ.get("NVCC", "nvcc")
# --fmad=false keeps device a*b+c as two roundings; -ffp-contract=off does the
# same for the host code (aarch64 g++ would otherwise fuse them, which changes
# the recentred coordinates the reference computes).
FLAGS = ["-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-lineinfo", "--fmad=false", "-std=c++17",
         "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I", CSRC]


def _compile(src: str) -> str:
    obj = os.path.join(OBJ, src.replace(".cu", ".o"))
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))] + \
        [os.path.join(ROOT, "include", "mcut_gb300.h")]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    subprocess.run([NVCC, *FLAGS, "-c", path, "-o", obj], check=True)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    srcs = [s for s in SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_compile, srcs))
    if not os.path.exists(OUT) or any(os.path.getmtime(o) > os.path.getmtime(OUT) for o in objs):
        subprocess.run([NVCC, "-shared", "-gencode", "arch=compute_103a,code=sm_103a", *objs, "-o", OUT,
                        "-lcudart"], check=True)
    if verbose:
        print(OUT)
    return OUT


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
