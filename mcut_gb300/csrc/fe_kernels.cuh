// Kernel interface of the GB300 intersection front end (host-callable launchers).
//
// Layout in HBM (one dispatch or one batch of independent pairs; a single
// dispatch is a batch of one):
//   X          double[nv][3]      ps vertex coordinates, pair after pair; within a
//                                 pair the source vertices then the cut vertices
//                                 (a single dispatch from device arrays reads the
//                                 caller's two arrays in place: X and Xc)
//   foff       uint32[nf+1]       CSR offsets of ps faces into fidx
//   fidx       uint32[foff[nf]]   global vertex ids (cut-mesh ids already offset)
//   face_pair  uint32[nf]         pair id | kCutBit for cut-mesh faces
//   fbox       double[nf][6]      exact fp64 face boxes (cut boxes enlarged by eps)
//   tree       Node[ncl-1]        LBVH over leaf clusters of `leaf_size` consecutive
//                                 cut faces (Morton order, never across pairs),
//                                 key = pair << 23 | Morton
//   pairs      uint64[P]          (source face << 32 | cut face), global ids
//   tests      Test[T]            culled edge-face tests
//   records    Record[R]          intersection records, sorted by (edge, face)
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace mcgpu {

constexpr uint32_t kCutBit = 0x80000000u;
constexpr int32_t kNoBad = 0x7F7F7F7F; // pair_bad when no face is degenerate (memset 0x7F)
constexpr int32_t kNoRoot = (int32_t)0x80000000; // pair_root of a pair without an internal tree node
// Morton code width: 23 (8, 8 and 7 bits per axis), which with the mesh bit
// keeps one pair's keys within three 8-bit radix passes, or 30 (10 per axis,
// four passes; the tree over 2 M faces is no better for the extra bits)
#ifndef MCGPU_MORTON_BITS
#define MCGPU_MORTON_BITS 23
#endif
constexpr int kMortonBits = MCGPU_MORTON_BITS;
static_assert(kMortonBits == 30 || kMortonBits == 23, "Morton width");

struct __align__(16) Node {
    float4 b0;            // left  lo.x lo.y lo.z hi.x
    float4 b1;            // left  hi.y hi.z | right lo.x lo.y
    float4 b2;            // right lo.z hi.x hi.y hi.z
    int32_t child[2];     // >= 0: internal node; < 0: ~(sorted leaf position)
    uint32_t prange[2];   // pair-id range of each child: lo | hi << 16
};

// A pair whose cut mesh is resident with its own tree (ncl > 0): the tree
// was built once over the mesh's user coordinates (fp32 boxes rounded
// outward, leaves of consecutive Morton-sorted faces), and the pair's source
// faces walk it with their boxes mapped back from the pair's frame; its cut
// faces take no part in the batch's sort and tree. ncl == 0: not resident.
struct __align__(16) ResPair {
    const Node* nodes;          // [ncl - 1]
    const uint32_t* leaf_face;  // [nf] the mesh's faces (local ids) in leaf order
    const uint32_t* cl_start;   // [ncl] first position of each leaf in leaf_face
    const uint8_t* cl_n;        // [ncl]
    uint32_t ncl, pad;
    double mag[3];              // per axis: the largest |coordinate| of the mesh
    double pad2;
};

struct Test {
    uint32_t q, r;    // oriented edge (global vertex ids)
    uint32_t g;       // tested face (global)
    uint32_t f0, f1;  // faces of the edge (f0: lowest, owns the orientation), f1 may be kNone
    uint32_t slot;    // halfedge slot of q->r in f0: the edge's first face corner
};

struct Problem {
    uint32_t n_pairs;
    uint32_t nv, nf;
    uint32_t ns, nc;            // total source / cut faces
    const double* X;
    const double* Xc;           // with xsplit: vertices >= xsplit live here (index - xsplit)
    uint32_t xsplit;            // 0xFFFFFFFF: every vertex in X
    const uint32_t* foff;
    const uint32_t* fidx;
    const uint32_t* face_pair;  // null for one pair: cut faces are those from face_split on
    // one pair: entries from fidx_split on are raw cut indices in fidx_cut,
    // global id = raw + cut_vbase (null: fidx holds global ids)
    const uint32_t* fidx_cut;
    uint32_t fidx_split, cut_vbase, face_split;
    // per pair tables [n_pairs (+1)]
    const uint32_t* pair_fbase; // first ps face of the pair
    const uint32_t* pair_fs;    // source faces of the pair
    const uint32_t* pair_vbase; // first ps vertex of the pair
    const uint32_t* pair_vs;    // source vertices of the pair
    const uint32_t* pair_sbase; // first position of the pair in the source-face list
    const uint32_t* pair_cbase; // first position of the pair in the cut-face list
    const double* pair_eps;     // cut-box enlargement
    const uint32_t* pair_clbase;// first leaf cluster of the pair
    const float4* X32;          // fp32 copies of the vertices (orient3d's first filter); null: not used
    int all_triangles;          // foff[f] == 3f
    uint32_t leaf_size;         // cut faces per tree leaf (consecutive in Morton order, one pair)
    uint32_t ncl;               // total leaf clusters
    // pairs with a resident cut tree (null: none): their cut faces are not in
    // the cut-face list, the batch tree or pair_clbase's clusters
    const ResPair* res_pairs;   // [n_pairs]
    const double* pair_frames;  // [n_pairs][6] com xyz, t xyz (x' = (x - com) + t), for res_pairs
};

struct Work {
    double* fbox;                     // [nf*6]
    float* fbox32;                    // [nf*6] the same boxes rounded outward to fp32
    unsigned long long* mesh_box;     // [n_pairs*2*6] ordered-uint64 min/max
    uint32_t* fidx_out;               // one pair: the bounds kernel writes the global ps indices here
    uint32_t* face_pair_out;          // ... and the face -> pair table (null for a batch: k_prep made them)
    float4* x32;                      // [nv] the bounds kernel writes each vertex's fp32 copy here (null: none)
    // one pair from the caller's host arrays (the device reads pageable
    // memory): the vertex bounds kernel reads the vertices there, source then
    // cut (hx_src null: from P.X), and writes the device copy hx_out
    const double* hx_src;
    const double* hx_cut;
    double* hx_out;
    // user coordinates (MCGPU_RECENTRE): the raw vertices gathered to the
    // device (float or double, the internal layout) and each pair's frame
    // (com xyz, t xyz); the vertex bounds kernel writes x' = (x - com) + t to
    // hx_out (x_raw null: not used)
    const void* x_raw;
    int raw_float;
    const double* frames;
    uint32_t* fidx_fix;               // a batch: the global table the bounds kernel reads, where it replaces an
                                      // index outside its mesh (null for one pair: fidx_out gets the fix)
    void* mesh_frame;                 // [n_pairs*2*2] float4: fp32 box low corner, 1023 / extent
    // sort buffers (keys u32 for one pair, u64 for batches); the cut keys and
    // values follow the source ones in the same arrays (ckeys[b] = skeys[b] + ns)
    void* skeys[2];                   // source-face keys
    uint32_t* svals[2];
    void* ckeys[2];                   // cut-face keys
    uint32_t* cvals[2];
    uint32_t* sort_temp;
    void* cl_key;                     // [ncl] key of each leaf cluster's first face
    uint32_t* cl_start;               // [ncl] first sorted position of the cluster
    uint8_t* cl_n;                    // [ncl] faces in the cluster
    long long* leaf_key_box;          // unused (kept null)
    void* top;                        // [64] top cut of the cut tree (WaveTop, 32 B each)
    void* split;                      // [split_cap] slow packets' remaining walks (144 B each)
    uint64_t split_cap;
    Node* nodes;                      // [ncl-1]
    uint32_t* split_far;              // [ncl-1] per split position: far leaf of the first child to arrive
    void* split_box;                  // [2(ncl-1)] per split position and side: that child's box (32 B)
    unsigned long long* pairs;        // [pair_cap]
    uint32_t* counters;               // [16]: 0 pairs, 1 tests, 2 records, 3 cand faces, 4 poly faces,
                                      //        5..7 escalations, 8 traversal work cursor, 9 packets, 10 narrow hits,
                                      //        11 queued projections, 12 incidence slot overflow,
                                      //        13 top-cut entries, 14 split entries, 15 second-launch work cursor
    uint2* packets;                   // [ns] query packets: sorted source positions [x, y]
    uint8_t* cand;                    // [nf]
    uint32_t* plane_slot;             // [nf]
    void* planes;                     // FacePlane[cap]
    uint32_t* proj_flag;              // [plane_cap] projection queued
    uint32_t* proj_list;              // [plane_cap] triangles whose plane is finished (face ids)
    uint32_t* poly_list;              // [nf] faces with > 3 vertices among candidates
    uint8_t* vneed;                   // [nv]
    uint32_t* voff;                   // [nv+1]
    uint32_t* vcur;                   // [nv]
    uint32_t* vface;                  // [incidence cap]
    uint32_t* scan_temp;
    Test* tests;                      // [test_cap]
    int8_t* test_info;                // [test_cap*4]
    unsigned long long* rec_key[2];   // [test_cap]
    uint32_t* rec_val[2];
    double* rec_pt_raw;               // [test_cap*3]
    uint32_t* rec_ids;                // [test_cap*5] final, sorted
    double* rec_pts;                  // [test_cap*3] final, sorted
    uint32_t* pair_status;            // [n_pairs] ST_* bits
    int32_t* pair_bad;                // [n_pairs] lowest degenerate ps face (local), INT_MAX if none
    uint32_t* pair_nrec;              // [n_pairs+1] first sorted record of each pair (+ total)
    int32_t* pair_root;               // [n_pairs] a batch's node whose subtree holds exactly the pair's leaf
                                      //   clusters (kNoRoot: none, the pair has one cluster or none); null: one pair
    uint32_t* pair_cnt;               // [n_pairs*5] a batch's per-pair counts: candidate pairs, tests,
                                      //   escalations (fp32 / fp64 / exact); null: one pair (counters only)
    double* tri_scratch;              // polygon triplet scratch (24-byte entries)
    uint64_t tri_scratch_cap;         // entries
    uint64_t tri_stride;              // entries per polygon (largest C(n,3)); 0: no polygons
    uint64_t pair_cap, test_cap, inc_cap, plane_cap;
    uint32_t inc_slots;               // 0: CSR incidence (voff offsets, vface lists); K: K slots per vertex, voff counts
    // tuning (results do not depend on it)
    uint32_t traversal;               // 0 warp/packet breadth-first, 1 warp/packet depth-first, 2 thread/face
    uint32_t packet_faces;            // source faces per query packet (1..32)
    uint32_t stack_depth;             // per-thread stack of traversal 2 (64 or 512)
    uint32_t split_round;             // traversal 0: rounds before a slow packet is split (0: never)
};

// stage launchers (all asynchronous on `s`)
// Pin: the input view the bounds kernel reads the indices through (for one
// pair the raw source / cut indices); P: the global view of later stages
void launch_bounds_morton(const Problem& P, const Problem& Pin, Work& W, bool wide_keys, int key_bits, cudaStream_t s);
int launch_sort(const Problem& P, Work& W, bool wide_keys, int key_bits, cudaStream_t s, int& cut_buf);
void launch_hierarchy(const Problem& P, Work& W, bool wide_keys, int cut_buf, cudaStream_t s);
void launch_packets(const Problem& P, Work& W, int src_buf, cudaStream_t s);
void launch_traverse(const Problem& P, Work& W, int src_buf, int cut_buf, bool deep, cudaStream_t s);
void launch_adjacency_planes(const Problem& P, Work& W, cudaStream_t s); // planes + incidence on one stream
void launch_planes(const Problem& P, Work& W, cudaStream_t s);           // candidate-face planes (+ triplets)
void launch_incidence(const Problem& P, Work& W, cudaStream_t s);        // vertex -> face incidence
void launch_tests(const Problem& P, Work& W, cudaStream_t s);
void launch_narrow(const Problem& P, Work& W, bool keep_tests, cudaStream_t s);
int launch_records(const Problem& P, Work& W, uint32_t n_records, cudaStream_t s);

// A resident cut mesh's own tree over its user coordinates (fp64 X [nv][3],
// triangles idx [nf][3]); mn / mx: its vertex bounds. Scratch and outputs as
// resident_tree_sizes gives them; an index past nv reads vertex 0 (a pair
// naming the mesh reports MCGPU_INVALID_INPUT from its own index check).
struct ResTreeSizes { uint64_t ncl, nodes_bytes, leaf_bytes, start_bytes, n_bytes, scratch_bytes; };
ResTreeSizes resident_tree_sizes(uint32_t nf, uint32_t leaf_size);
struct ResTreeOut { Node* nodes; uint32_t* leaf_face; uint32_t* cl_start; uint8_t* cl_n; };
void build_resident_tree(const double* X, const uint32_t* idx, uint32_t nv, uint32_t nf, const double* mn,
    const double* mx, uint32_t leaf_size, void* scratch, const ResTreeOut& out, cudaStream_t s);
// clears `mask` in every pair's status bits
void launch_clear_status(uint32_t* pair_status, uint32_t n_pairs, uint32_t mask, cudaStream_t s);
// record ordering from the device's record count (at most cap = kRankSortMax
// records; above cap nothing is written); returns the sorted-key buffer
int launch_records_dev(const Problem& P, Work& W, uint32_t cap, cudaStream_t s);
constexpr uint32_t kRankSortMax = 24576; // records ordered by one rank launch

} // namespace mcgpu
