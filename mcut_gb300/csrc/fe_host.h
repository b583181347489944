// Host-side pieces shared by the dispatch entry points and the request server.
#pragma once
#include <cstdint>
#include <string>

#include "mcut_gb300.h"

namespace mcgpu {

// records `msg` as this thread's mcgpu_last_error() and returns `code`
int set_error(int code, const std::string& msg);

// bounds and centroid of one mesh's user coordinates, summed in vertex order
// (calculate_vertex_parameters, preproc.cpp:2124-2290)
struct MeshStats {
    double mn[3], mx[3], com[3];
};
void mesh_stats(const void* v, bool fin, uint32_t n, MeshStats& st);
void pair_frame(const MeshStats& S, const MeshStats& Cm, double* com, double* t);
void apply_frame(bool fin, const mcgpu_mesh& m, const double* com, const double* t, double* out);
// cut_eps: |translated cut box diagonal|, or 1 (absolute), times the
// general-position constant (preproc.cpp:2518, 2664-2676)
double frame_eps(const MeshStats& Cm, const double* t, double constant = 1e-4, bool absolute = false);

// A cut mesh kept on the device: double user coordinates and triangle
// indices, with its host-side stats (so a pair's frame needs only the source).
struct ResidentCut {
    const double* X;
    const uint32_t* idx;
    uint32_t nv, nf;
    MeshStats st;
    // its own tree over the user coordinates (tree_ncl == 0: none; the pair's
    // cut faces then join the batch's tree)
    const void* tree_nodes;
    const uint32_t* tree_leaf_face;
    const uint32_t* tree_cl_start;
    const uint8_t* tree_cl_n;
    uint32_t tree_ncl;
};

// mcgpu_dispatch_batch over host meshes with MCGPU_RECENTRE, where a non-null
// resident[p] stands in for cuts[p] (cuts[p] is then ignored).
int dispatch_with_resident(mcgpu_context c, uint32_t flags, uint32_t n, const mcgpu_mesh* srcs,
    const mcgpu_mesh* cuts, const ResidentCut* const* resident, mcgpu_summary* out);

} // namespace mcgpu
