"""mcut_gb300: GB300-native intersection front end for the MCUT mesh-cutting library.

The CUDA library (libmcut_gb300.so, C ABI in include/mcut_gb300.h) is the
product; this package is its Python host side: ctypes bindings
(``_lib``), the front-end mirror of the reference seam (``frontend``),
seeded synthetic workloads (``meshgen``) and the in-tree build (``build``).
"""
from .frontend import Context, FrontEndResult, Server, pack_pairs, recentre  # noqa: F401
