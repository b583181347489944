// The halfedge mesh of one input mesh and its input checks on the device
// (fe_hmesh.cu).
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mcgpu {

// status codes, in the priority a face's checks have (a face's own errors
// before a non-manifold corner); the values are mcgpu_hmesh_status's
enum {
    HM_CODE_FACE_SIZE = 1,
    HM_CODE_INDEX_RANGE = 2,
    HM_CODE_DUPLICATE_INDEX = 3,
    HM_CODE_NON_MANIFOLD = 4
};

// slots of HmeshScratch::counts
enum { kHmEdges = 0, kHmBorder = 1, kHmComponents = 2, kHmCounts = 4 };

struct HmeshInput {
    const uint32_t* idx;  // [nidx] face-vertex indices
    const uint32_t* foff; // [nf+1] face offsets; null: triangles
    uint32_t nv, nf;
    uint64_t nidx;
};

// open-addressing table of undirected edges: key (min << 32 | max) + 1
// (0 = empty), the lowest slot meeting the edge, the lowest per direction
struct HmeshTable {
    unsigned long long* key;  // [mask+1], zeroed
    uint32_t* first;          // [mask+1], all ones
    uint32_t* dir_first;      // [2 (mask+1)], all ones
    unsigned long long mask;  // buckets - 1 (a power of two minus one, buckets >= 2 nidx)
};

struct HmeshScratch {
    uint32_t* slot_face;          // [nidx] (polygons only)
    uint32_t* slot_bucket;        // [nidx]
    uint32_t* eid;                // [nidx] creating-slot flags, then edge ids
    uint32_t* vcur;               // [nv], zeroed
    uint32_t* parent;             // [nv]
    uint32_t* scan_temp;          // scan_temp_bytes(max(nidx, nv + 1))
    unsigned long long* err;      // [1] lowest (face << 3 | code), all ones = none
    uint32_t* counts;             // [kHmCounts], zeroed
};

// the halfedge arrays (as hmesh_t holds them): halfedge 2e runs the way the
// corner that created edge e runs, 2e + 1 the other way
struct HmeshOut {
    uint32_t* he_target;  // [2E]
    int32_t* he_face;     // [2E], -1 (memset) = border
    int32_t* he_next;     // [2E], -1 = unlinked
    int32_t* he_prev;     // [2E]
    uint32_t* corner_he;  // [nidx]
    uint32_t* v_off;      // [nv+1], zeroed: counts, then offsets
    uint32_t* v_he;       // [2E]
};

// phase 1: face checks, edge table, creating-slot flags, edge ids and count
// (counts[kHmEdges]); the error word tells whether phase 2 may run
void launch_hmesh_edges(const HmeshInput& in, HmeshTable& t, HmeshScratch& w, cudaStream_t s);
// phase 2 (no error): halfedges, links, per-vertex lists, border flag,
// connected components (counts[kHmBorder], counts[kHmComponents])
void launch_hmesh_build(const HmeshInput& in, const HmeshTable& t, HmeshScratch& w, HmeshOut& o, uint32_t ne,
    cudaStream_t s);

// A connected component's arrays as mcGetConnectedComponentData serialises
// them (frontend.cpp:2006-2832) from its halfedge mesh: vertices around each
// face (the targets of its halfedges, hmesh.cpp:705-733), the faces across
// its halfedges (get_faces_around_face, hmesh.cpp:796-818) with their
// counts. Edges are he_target itself (vertex(e, 0) / vertex(e, 1) are the
// targets of halfedges 2e / 2e + 1, hmesh.cpp:234-256).
struct CcWireOut {
    uint32_t* face;    // [nidx]
    uint32_t* pos;     // [nidx + 1] exclusive scan of "a face across this corner's halfedge"
    uint32_t* adj;     // [pos[nidx]]
    uint32_t* adj_n;   // [nf]
};
size_t cc_wire_scan_bytes(uint64_t nidx);
// returns the adjacency count through *total (a readback)
void launch_cc_wire(const HmeshOut& o, const uint32_t* foff, uint32_t nf, uint64_t nidx, CcWireOut& w,
    uint32_t* scan_temp, uint32_t* total, cudaStream_t s);
// static_cast<float> of n doubles (IEEE round to nearest)
void launch_to_float(const double* x, uint64_t n, float* out, cudaStream_t s);

} // namespace mcgpu
