"""Copy the reference sources and open the seam between the front end and the
host stages (TEST INFRASTRUCTURE ONLY).

    python oracle/make_seam.py REF_ROOT OUT_DIR

OUT_DIR (git-ignored, under oracle/_ref/) receives REF_ROOT's source/ and
include/ trees unchanged except for source/kernel.cpp, where dispatch()'s
narrow-phase block (the records and the maps built from them,
kernel.cpp:2415-3206) runs only when no seam hook is installed; with a hook
(oracle/seam_hook.h) the hook supplies the same outputs and dispatch()
continues with its own host stages (cut-path edges, clipping, connected
components) exactly as the reference wrote them. After the cut-path edges
are made (kernel.cpp:3332-3632) an observer, when installed, sees them with
their maps, and another sees the floating polygons detected
(kernel.cpp:4078-4200). The edit is anchored on source text, not line numbers, and fails
loudly if an anchor is missing.
"""
from __future__ import annotations

import os
import shutil
import sys

HOOK_DECL = """
// ---- seam hook (inserted by oracle/make_seam.py) ----
#include "seam_hook.h"
mcut_seam_front_end_fn g_mcut_seam_front_end = nullptr;
extern "C" void mcut_seam_install(mcut_seam_front_end_fn fn) { g_mcut_seam_front_end = fn; }
mcut_seam_observer_fn g_mcut_seam_observer = nullptr;
extern "C" void mcut_seam_observe(mcut_seam_observer_fn fn) { g_mcut_seam_observer = fn; }
mcut_seam_cutpath_fn g_mcut_seam_cutpath_observer = nullptr;
extern "C" void mcut_seam_observe_cutpath(mcut_seam_cutpath_fn fn) { g_mcut_seam_cutpath_observer = fn; }
mcut_seam_floating_fn g_mcut_seam_floating_observer = nullptr;
extern "C" void mcut_seam_observe_floating(mcut_seam_floating_fn fn) { g_mcut_seam_floating_observer = fn; }
// ---- end seam hook ----

"""

HOOK_CALL = """
    // ---- seam hook (inserted by oracle/make_seam.py) ----
    if (g_mcut_seam_front_end != nullptr) {
        int seam_status = 0;
        const bool seam_ok = g_mcut_seam_front_end(ps, sm_vtx_cnt, sm_face_count, m0,
            m0_ivtx_to_intersection_registry_entry, cm_border_reentrant_ivtx_list, ps_intersecting_edges,
            cutpath_edge_creation_info, ps_iface_to_ivtx_list, partial_cut_detected, seam_status,
            ps_edge_face_intersection_pairs, (int)input.scheduler->get_num_threads());
        if (!seam_ok) {
            output.status = status_t::INVALID_MESH_INTERSECTION;
            return;
        }
        if (seam_status != 0) {
            output.status = status_t::GENERAL_POSITION_VIOLATION;
            return;
        }
    } else {
    // ---- end seam hook ----
"""

HOOK_CLOSE = """
        // ---- seam observer (inserted by oracle/make_seam.py): the reference's own records, in its order
        if (g_mcut_seam_observer != nullptr)
            g_mcut_seam_observer(ps, m0, m0_ivtx_to_intersection_registry_entry);
    } // ---- seam hook: end of the reference's own narrow phase ----
"""

HOOK_CUTPATH = """    // ---- seam cut-path observer (inserted by oracle/make_seam.py): the cut-path edges and their maps
    if (g_mcut_seam_cutpath_observer != nullptr)
        g_mcut_seam_cutpath_observer(ps, m0, m0_ivtx_to_intersection_registry_entry, cutpath_edge_creation_info,
            m0_cutpath_edges, ps_iface_to_m0_edge_list, ivtx_to_incoming_hlist);
"""

HOOK_FLOATING = """    // ---- seam floating-polygon observer (inserted by oracle/make_seam.py)
    if (g_mcut_seam_floating_observer != nullptr)
        g_mcut_seam_floating_observer(output.detected_floating_polygons);
"""

ANCHOR_DISPATCH = "\nvoid dispatch(output_t& output, const input_t& input)\n"
ANCHOR_PUSH = '    TIMESTACK_PUSH("Calculate intersection points (edge-to-face)");\n'
ANCHOR_END = "#endif\n\n    // Create edges from the new intersection points\n"
ANCHOR_CUTPATH = "    // NOTE: at this stage we have all vertices and edges which are needed to clip\n"
ANCHOR_FLOATING = "    if (!output.detected_floating_polygons.empty()) {\n"


def patch_kernel(text: str) -> str:
    for a in (ANCHOR_DISPATCH, ANCHOR_PUSH, ANCHOR_END, ANCHOR_CUTPATH, ANCHOR_FLOATING):
        if text.count(a) != 1:
            raise SystemExit(f"make_seam: anchor not found exactly once: {a.strip()[:60]!r}")
    text = text.replace(ANCHOR_DISPATCH, "\n" + HOOK_DECL + ANCHOR_DISPATCH.lstrip("\n"))
    text = text.replace(ANCHOR_PUSH, ANCHOR_PUSH + HOOK_CALL)
    text = text.replace(ANCHOR_END, "#endif\n" + HOOK_CLOSE + "\n    // Create edges from the new intersection points\n")
    text = text.replace(ANCHOR_CUTPATH, HOOK_CUTPATH + ANCHOR_CUTPATH)
    text = text.replace(ANCHOR_FLOATING, HOOK_FLOATING + ANCHOR_FLOATING)
    return text


def main():
    if len(sys.argv) != 3:
        raise SystemExit(__doc__)
    ref, out = sys.argv[1], sys.argv[2]
    if not os.path.isdir(os.path.join(ref, "source")):
        raise SystemExit(f"make_seam: {ref} is not a reference checkout")
    for sub in ("source", "include"):
        dst = os.path.join(out, sub)
        if os.path.isdir(dst):
            shutil.rmtree(dst)
        shutil.copytree(os.path.join(ref, sub), dst)
        for root, _, files in os.walk(dst):  # the checkout may be read-only
            for f in files:
                os.chmod(os.path.join(root, f), 0o644)
    k = os.path.join(out, "source", "kernel.cpp")
    with open(k) as fh:
        text = fh.read()
    with open(k, "w") as fh:
        fh.write(patch_kernel(text))


if __name__ == "__main__":
    main()
