// MCUT's cut-path edge creation on the device (fe_cutpath.cu): the edges of
// the cut path from one dispatch's record hand-over.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace mcgpu {

// slots of CutpathOut::counts
enum {
    kCpEdges = 0,       // edges made
    kCpFaces = 1,       // faces with an edge list
    kCpFaceEntries = 2, // their entries
    kCpHalfedges = 3,   // incoming halfedge entries (2 per edge)
    kCpBadKey = 4,      // the first key with fewer than two vertices, 0xFFFFFFFF if none
    kCpCounts = 8
};

// The dispatch's polygon soup and hand-over, as the cut-path stage reads them.
struct CutpathInput {
    const double* X;         // ps vertex coordinates (vertices from xsplit on in Xc)
    const double* Xc;
    uint32_t xsplit;
    const uint32_t* fidx;    // global face-vertex ids, input corner order
    const uint32_t* foff;    // null: triangles
    uint32_t nv, nf, fs;     // ps vertices, faces, source faces (a cut face's soup corners start at its third)
    const uint32_t* rec_ids; // R records (q, r, tested face, f0, f1): intersection vertex nv + i
    const double* rec_pts;   // R points
    uint32_t nrec;
    const uint32_t* cp_pairs;  // K keys (source face, cut face), ascending
    const uint32_t* cp_off;    // K + 1
    const uint32_t* cp_vtx;    // their vertices, each list ascending
    uint32_t n_keys, n_entries;
};

// Scratch for C = n_entries - n_keys candidate edges (cutpath_scratch_bytes).
struct CutpathScratch {
    uint32_t* cand;           // [4C]: first vertex, second vertex, key, kind (0 two vertices, 1 sorted run)
    uint32_t* inside;         // [2C]: a sorted run's two faces holding the midpoint
    uint32_t* sorted;         // [n_entries] each long key's vertices along their line
    double* proj;             // [n_entries]
    unsigned long long* pk[2]; // [C] pair keys (double-buffered)
    uint32_t* pv[2];
    uint32_t* made;           // [C + 1] 1 for the candidates that make an edge, then edge ids (exclusive scan)
    unsigned long long* fk[2]; // [5C] (face, edge) entries
    uint32_t* fv[2];
    unsigned long long* hk[2]; // [2C] (vertex, halfedge) entries
    uint32_t* hv[2];
    uint32_t* flags;          // [5C + 1]
    uint32_t* sort_temp;
    uint32_t* scan_temp;
};

// Outputs (capacities for C candidates and R records): edges 2C, face_keys
// 5C, face_off 5C + 1, face_edges 5C, ivtx_off R + 1, ivtx_he 2C.
struct CutpathOut {
    uint32_t* edges;
    uint32_t* face_keys;
    uint32_t* face_off;
    uint32_t* face_edges;
    uint32_t* ivtx_off;
    uint32_t* ivtx_he;
    uint32_t* counts; // [kCpCounts]
};

// Floating polygons (kernel.cpp:4078-4200) from the cut path: a circular
// cut path (every vertex on two of its edges, none on a soup border edge)
// whose vertices all pierce the same face. Scratch and outputs for R
// intersection vertices.
enum { kFpPolygons = 0, kFpVertices = 1, kFpError = 2, kFpCounts = 4 };
struct FloatingScratch {
    uint32_t* parent;          // [R]
    uint32_t* flags;           // [R]
    uint32_t* size;            // [R]
    unsigned long long* k[2];  // [R] (face, root) keys
    uint32_t* v[2];            // [R]
    uint32_t* sort_temp;
    uint32_t* scan_temp;
};
struct FloatingOut {
    uint32_t* faces;   // [R] each polygon's ps face (polygons by face, then smallest vertex)
    uint32_t* off;     // [R + 1]
    uint32_t* vtx;     // [R] m0 ids, each polygon from its smallest, first towards its lowest edge's other end
    double* normals;   // [3R] the face's unit normal (compute_polygon_plane_coefficients)
    int32_t* mc;       // [R] its largest component
    uint32_t* counts;  // [kFpCounts]
};
size_t floating_sort_temp_bytes(uint32_t nrec);
size_t floating_scan_temp_bytes(uint32_t nrec);
void launch_floating(const CutpathInput& in, const CutpathOut& cp, FloatingScratch& w, FloatingOut& o,
    cudaStream_t s);

size_t cutpath_sort_temp_bytes(uint32_t n_candidates);
size_t cutpath_scan_temp_bytes(uint32_t n_candidates);

void launch_cutpath(const CutpathInput& in, CutpathScratch& w, CutpathOut& o, cudaStream_t s);

} // namespace mcgpu
