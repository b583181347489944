// The record hand-over on the device (fe_derived.cu): the derived maps of one
// dispatch's records that dispatch()'s host stages read.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

namespace mcgpu {

// slots of DerivedOut::counts
enum {
    kDerivedEdges = 0,          // intersected edges (runs of records)
    kDerivedCutpath = 1,        // (source face, cut face) keys
    kDerivedCutpathEntries = 2, // their vertices
    kDerivedFaces = 3,          // faces with an intersection vertex
    kDerivedFaceEntries = 4,    // their vertices
    kDerivedBorder = 5,         // records on cut-mesh border edges
    kDerivedCounts = 8
};

// scratch for R records: ck/cv 2R entries each (double-buffered), fk/fv 3R,
// flags 7R + 1, sort and scan temporaries as the functions below size them
struct DerivedScratch {
    unsigned long long* ck[2];
    uint32_t* cv[2];
    uint32_t* fk[2];
    uint32_t* fv[2];
    uint32_t* flags;
    uint32_t* sort_temp;
    uint32_t* scan_temp;
};

// outputs for R records (capacities): edge_off R + 1, border R, cp_pairs 4R,
// cp_off 2R + 1, face_keys 3R, face_off 3R + 1; cp_vtx / face_vtx are set to
// the sorted vertex columns inside DerivedScratch
struct DerivedOut {
    uint32_t* edge_off;
    uint32_t* border;
    uint32_t* cp_pairs;
    uint32_t* cp_off;
    uint32_t* face_keys;
    uint32_t* face_off;
    uint32_t* counts; // [kDerivedCounts]
    const uint32_t* cp_vtx;
    const uint32_t* face_vtx;
};

size_t derived_sort_temp_bytes(uint32_t nrec);
size_t derived_scan_temp_bytes(uint32_t nrec);

// rec_ids: nrec records (q, r, tested face, f0, f1) of one pair in canonical
// order, ps ids; vs source vertices, nv = Vs + Vc, fs source faces, nf = Fs + Fc
void launch_derived(const uint32_t* rec_ids, uint32_t nrec, uint32_t vs, uint32_t nv, uint32_t fs, uint32_t nf,
    DerivedScratch& w, DerivedOut& o, cudaStream_t s);

} // namespace mcgpu
