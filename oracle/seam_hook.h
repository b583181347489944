// The seam between MCUT's intersection front end and its host stages, as a
// hook (TEST INFRASTRUCTURE ONLY; the product library never includes it).
//
// oracle/make_seam.py copies the reference sources and inserts, in
// dispatch() (kernel.cpp), a call to the hook installed here in place of the
// narrow-phase block (kernel.cpp:2415-3206). The hook hands dispatch() what
// that block produces and everything after it reads (kernel.cpp:2377-2413):
// the intersection vertices appended to m0, their registry entries (tested
// edge, tested face), ps_intersecting_edges, cutpath_edge_creation_info,
// ps_iface_to_ivtx_list, cm_border_reentrant_ivtx_list,
// partial_cut_detected, and the status (0 success, 1 general-position
// violation). Returning false stops the dispatch (a hand-over the harness
// could not apply). It also sees the reference's edge -> tested faces map
// (kernel.cpp:1779-2177, still computed in the copy) and the context's helper
// thread count: the reference numbers its intersection vertices in that map's
// iteration order, split into parallel_for blocks (tpool.h:420-472).
#pragma once
#include <map>
#include <unordered_map>
#include <utility>
#include <vector>

#include "mcut/internal/hmesh.h"
#include "mcut/internal/kernel.h"
#include "mcut/internal/utils.h"

typedef bool (*mcut_seam_front_end_fn)(const hmesh_t& ps, int sm_vtx_cnt, int sm_face_count, hmesh_t& m0,
    std::vector<std::pair<ed_t, fd_t>>& registry, std::vector<vd_t>& cm_border_reentrant_ivtx_list,
    std::unordered_map<ed_t, std::vector<vd_t>>& ps_intersecting_edges,
    std::map<pair<fd_t>, std::vector<vd_t>>& cutpath_edge_creation_info,
    std::unordered_map<fd_t, std::vector<vd_t>>& ps_iface_to_ivtx_list, bool& partial_cut_detected, int& status,
    const std::unordered_map<ed_t, std::vector<fd_t>>& ps_edge_face_intersection_pairs, int helper_threads);

// set by the harness; null runs the reference's own narrow phase
extern mcut_seam_front_end_fn g_mcut_seam_front_end;
extern "C" void mcut_seam_install(mcut_seam_front_end_fn fn);

// Observer of the reference's own narrow phase (no hook installed): called
// after it with the polygon soup, m0 (the intersection vertices appended) and
// the registry in the reference's numbering.
typedef void (*mcut_seam_observer_fn)(const hmesh_t& ps, const hmesh_t& m0,
    const std::vector<std::pair<ed_t, fd_t>>& registry);
extern mcut_seam_observer_fn g_mcut_seam_observer;
extern "C" void mcut_seam_observe(mcut_seam_observer_fn fn);

// Observer of the cut-path edge creation (kernel.cpp:3332-3632): called after
// it with its inputs (the soup, m0's intersection vertices and their
// registry, cutpath_edge_creation_info) and outputs (m0_cutpath_edges, in
// creation order, ps_iface_to_m0_edge_list, ivtx_to_incoming_hlist).
typedef void (*mcut_seam_cutpath_fn)(const hmesh_t& ps, const hmesh_t& m0,
    const std::vector<std::pair<ed_t, fd_t>>& registry,
    const std::map<pair<fd_t>, std::vector<vd_t>>& cutpath_edge_creation_info,
    const std::vector<ed_t>& m0_cutpath_edges, const std::unordered_map<fd_t, std::vector<ed_t>>& ps_iface_to_m0_edge_list,
    const std::unordered_map<vd_t, std::vector<hd_t>>& ivtx_to_incoming_hlist);
extern mcut_seam_cutpath_fn g_mcut_seam_cutpath_observer;
extern "C" void mcut_seam_observe_cutpath(mcut_seam_cutpath_fn fn);

// Observer of the floating-polygon detection (kernel.cpp:4078-4200): the
// detected polygons per ps face, before dispatch() stops on them.
typedef void (*mcut_seam_floating_fn)(const std::map<fd_t, std::vector<floating_polygon_info_t>>& polygons);
extern mcut_seam_floating_fn g_mcut_seam_floating_observer;
extern "C" void mcut_seam_observe_floating(mcut_seam_floating_fn fn);
