/*
 * mcut_gb300 — GB300-native intersection front end for MCUT, C ABI.
 *
 * This library replaces the data-parallel front end of one MCUT dispatch:
 *
 *   reference seam                                   replaced by
 *   -----------------------------------------------  ---------------------------
 *   build_oibvh(src) / build_oibvh(cut, eps)          mcgpu_dispatch (stage 1: face
 *     source/preproc.cpp:2456, 2685                     boxes, Morton codes, radix
 *     source/bvh.cpp:219-636                            sort, LBVH + refit)
 *   intersectOIBVHs(...)                              mcgpu_dispatch (stage 2:
 *     source/preproc.cpp:2839, bvh.cpp:638-783          tree traversal -> face pairs)
 *   dispatch() front section                          mcgpu_dispatch (stage 3: edge /
 *     source/kernel.cpp:1781-3206                       face expansion, culling,
 *                                                       planes, orient3d narrow
 *                                                       phase, records + points)
 *
 * Everything downstream of the records (cut-path tracing, polygon clipping,
 * connected components; kernel.cpp:3332 onwards) stays in the host C++ that
 * calls this library. Plain pointers and sizes only; no C++ or torch types.
 *
 * Identifiers are the reference's polygon-soup ("ps") ids of one dispatch
 * (kernel.cpp:1593-1732): vertices [0,Vs) source then [Vs,Vs+Vc) cut mesh,
 * faces [0,Fs) source then [Fs,Fs+Fc) cut mesh. An edge is reported as
 * (q, r): source and target of its primary halfedge, i.e. its direction in
 * the lowest-numbered face containing it (hmesh.cpp:405-651), with f0 that
 * face and f1 the other face or 0xFFFFFFFF on a border.
 *
 * Threading: a context owns one CUDA stream and its device memory; calls on
 * one context must be serialised by the caller (MCUT runs one API thread per
 * context, frontend.h:548-580). Different contexts may run concurrently.
 * Errors never abort the process: every entry point returns an mcgpu_status.
 */
#ifndef MCUT_GB300_H
#define MCUT_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mcgpu_context_t* mcgpu_context;

/* Results of a front-end dispatch. GP_VIOLATION / DEGENERATE_* are valid
 * outcomes of the algorithm (the reference reports them as status_t values,
 * kernel.h:52-92, and mcDispatch turns them into MC_INVALID_OPERATION);
 * the others are failures of the call. */
typedef enum mcgpu_status {
    MCGPU_OK = 0,
    MCGPU_GP_VIOLATION = 1,        /* touching / on-edge / on-vertex configuration */
    MCGPU_DEGENERATE_SRC_FACE = 2, /* a candidate source face has |Newell n|^2 < 1e-9 */
    MCGPU_DEGENERATE_CUT_FACE = 3,
    MCGPU_INVALID_INPUT = 4,       /* a face with fewer than 3 vertices or an index out of range;
                                      MCUT's other input checks run before the seam */
    MCGPU_CUDA_ERROR = 5,
    MCGPU_OUT_OF_MEMORY = 6,
    MCGPU_INVALID_VALUE = 7,       /* bad argument (null pointer, unknown query, ...) */
    MCGPU_TOO_LARGE = 8,           /* exceeds a fixed capacity of the entry point */
    MCGPU_NOT_READY = 9,           /* a served request has not completed yet */
    MCGPU_CANCELLED = 10           /* a served request was cancelled before it ran */
} mcgpu_status;

/* dispatch flags */
#define MCGPU_VERTEX_ARRAY_FLOAT (1u << 0) /* vertices are float[3*V] (MC_DISPATCH_VERTEX_ARRAY_FLOAT) */
#define MCGPU_RECENTRE (1u << 1)           /* vertices are user coordinates: apply preproc's
                                              recentring (preproc.cpp:2124-2290, 147-181) and
                                              derive cut_eps = |cut box diagonal| * the context's
                                              general-position constant (default 1e-4) */
#define MCGPU_KEEP_TESTS (1u << 2)         /* keep every culled edge-face test and its predicates */
#define MCGPU_KEEP_PAIRS (1u << 3)         /* keep the candidate face pairs */
#define MCGPU_PROFILE (1u << 4)            /* time the stages with CUDA events */
#define MCGPU_DEVICE_POINTERS (1u << 5)    /* mesh arrays are device pointers (recentred, double); a
                                              single pair's and a packed batch's coordinates are read
                                              in place, so keep them alive while results are read */
#define MCGPU_ENFORCE_GENERAL_POSITION (1u << 6)
/* mcgpu_dispatch only: on a general-position violation, perturb the cut mesh
   by uniform(-1, 1) * cut_eps per axis (the reference's mt19937 sequence, one
   per context) and run the narrow phase again against the unperturbed pairs
   and face boxes, up to the context's attempts; still violated after the
   last attempt, the status stays MCGPU_GP_VIOLATION (the reference throws
   "max perturbation iterations reached"). MC_DISPATCH_ENFORCE_GENERAL_POSITION,
   preproc.cpp:2590-2699, 2933-2945. */
#define MCGPU_ENFORCE_GENERAL_POSITION_ABSOLUTE (1u << 7)
/* the same, with MCGPU_RECENTRE's cut_eps = the context's constant alone
   instead of constant * |cut box diagonal| (MC_DISPATCH_ENFORCE_GENERAL_POSITION_ABSOLUTE) */

typedef struct mcgpu_mesh {
    const void* vertices;         /* double[3*num_vertices], float with MCGPU_VERTEX_ARRAY_FLOAT */
    const uint32_t* face_indices; /* concatenated face-vertex indices */
    const uint32_t* face_sizes;   /* NULL: all faces are triangles (preproc.cpp:206) */
    uint32_t num_vertices;
    uint32_t num_faces;
} mcgpu_mesh;

/* stage_ms[] slots filled with MCGPU_PROFILE */
enum {
    MCGPU_STAGE_UPLOAD = 0,   /* host->device copies */
    MCGPU_STAGE_BOUNDS = 1,   /* face boxes, mesh boxes, Morton codes */
    MCGPU_STAGE_SORT = 2,     /* radix sorts */
    MCGPU_STAGE_HIERARCHY = 3,/* LBVH hierarchy + refit */
    MCGPU_STAGE_TRAVERSE = 4, /* tree traversal -> candidate pairs */
    MCGPU_STAGE_ADJACENCY = 5,/* vertex->face incidence + face planes */
    MCGPU_STAGE_NARROW = 6,   /* edge-face expansion, culling, narrow phase, records */
    MCGPU_STAGE_DOWNLOAD = 7  /* device->host copies */
};

typedef struct mcgpu_summary {
    int32_t status;           /* mcgpu_status of the front end */
    int32_t bad_face;         /* lowest degenerate candidate ps face, or -1 */
    double cut_eps;           /* cut-mesh face-box enlargement used */
    uint64_t num_pairs;       /* candidate (source face, cut face) pairs */
    uint64_t num_tests;       /* culled edge-face tests */
    uint64_t num_records;     /* intersection records (type '1', point inside) */
    uint64_t escalations[3];  /* orient3d signs decided by: fp32 filter, fp64 filter, the later
                                 stages (adaptive B/C, then the exact expansion)
                                 (in a batch, these four counts are the pair's own) */
    float stage_ms[8];        /* per-stage device time of the call (MCGPU_PROFILE; a batch's
                                 summaries all carry the batch's times) */
    uint32_t kernel_launches; /* CUDA kernels this call launched (whole batch) */
    uint32_t perturbations;   /* general-position enforcement: cut-mesh perturbations applied */
    double perturbation[3];   /* the last perturbation applied (recentred units), else 0
                                 (MC_CONNECTED_COMPONENT_DATA_DISPATCH_PERTURBATION_VECTOR) */
} mcgpu_summary;

/* mcgpu_get_data queries */
typedef enum mcgpu_data {
    MCGPU_DATA_RECORD_IDS = 1,    /* uint32[5*R]: q, r, tested face, f0, f1, ordered by the edge's first
                                     face corner in the source-then-cut face arrays, then face */
    MCGPU_DATA_RECORD_POINTS = 2, /* double[3*R]: intersection points (recentred coordinates) */
    MCGPU_DATA_PAIRS = 3,         /* uint32[2*P]: (source face, cut face); MCGPU_KEEP_PAIRS */
    MCGPU_DATA_TESTS = 4,         /* uint32[3*T]: q, r, face; MCGPU_KEEP_TESTS */
    MCGPU_DATA_TEST_INFO = 5,     /* int8[4*T]: sign(orient3d q), sign(orient3d r), type char, pip char */
    MCGPU_DATA_VERTICES = 6,      /* double[3*(Vs+Vc)]: the ps coordinates used */
    MCGPU_DATA_FACE_BOXES = 7,    /* double[6*(Fs+Fc)]: min xyz, max xyz (cut boxes enlarged) */
    MCGPU_DATA_RECORD_OFFSETS = 8, /* uint64[n_pairs+1]: first record of each pair of the last
                                     dispatch (records of a batch are grouped by pair), then R */
    /* The record hand-over of a single dispatch: the maps dispatch()'s host
     * stages read (kernel.cpp:2599-2655, merged at 2673-2714), built on the
     * device from the records at the first such query. Record i is MCUT's
     * intersection vertex Vs + Vc + i of m0 (the "m0 ids" below); keys
     * ascend and each key's vertices ascend. */
    MCGPU_DATA_EDGE_RECORD_OFFSETS = 9,  /* uint32[E+1]: records [o[e], o[e+1]) share the e-th intersected
                                            ps edge, their (q, r) (ps_intersecting_edges) */
    MCGPU_DATA_CUTPATH_PAIRS = 10,       /* uint32[2*K]: (source face, cut face) of every face pair an
                                            intersection vertex lies on (cutpath_edge_creation_info keys) */
    MCGPU_DATA_CUTPATH_OFFSETS = 11,     /* uint32[K+1]: pair k's vertices are [o[k], o[k+1]) of ... */
    MCGPU_DATA_CUTPATH_VERTICES = 12,    /* uint32[o[K]]: m0 ids */
    MCGPU_DATA_FACE_KEYS = 13,           /* uint32[M]: ps faces an intersection vertex lies on: the tested
                                            face and the edge's faces (ps_iface_to_ivtx_list keys) */
    MCGPU_DATA_FACE_OFFSETS = 14,        /* uint32[M+1] */
    MCGPU_DATA_FACE_VERTICES = 15,       /* uint32[o[M]]: m0 ids */
    MCGPU_DATA_BORDER_VERTICES = 16,     /* uint32[B]: m0 ids of records on cut-mesh border edges
                                            (cm_border_reentrant_ivtx_list) */
    MCGPU_DATA_PARTIAL_CUT = 17,         /* uint32[1]: 1 if B > 0 (partial_cut_detected), else 0 */
    /* The halfedge mesh of the last mcgpu_halfedge_mesh call (E edges, halfedge 2e runs the way the
     * face corner that created edge e runs, 2e + 1 the other way; hmesh.cpp:406-651) */
    MCGPU_DATA_HE_TARGET = 18,           /* uint32[2E]: vertex each halfedge ends at */
    MCGPU_DATA_HE_FACE = 19,             /* int32[2E]: its face, -1 on a border */
    MCGPU_DATA_HE_NEXT = 20,             /* int32[2E]: next halfedge around its face, -1 on a border */
    MCGPU_DATA_HE_PREV = 21,             /* int32[2E] */
    MCGPU_DATA_CORNER_HE = 22,           /* uint32[corners]: the halfedge of face corner i (v_i -> v_i+1) */
    MCGPU_DATA_VERTEX_HE_OFFSETS = 23,   /* uint32[V+1]: vertex v's halfedges are [o[v], o[v+1]) of ... */
    MCGPU_DATA_VERTEX_HE = 24,           /* uint32[2E]: the halfedges ending at each vertex, in creation order */
    /* The cut path of a single dispatch (kernel.cpp:3332-3632): the edges MCUT's m0 gets from the
     * hand-over's cutpath_edge_creation_info, built on the device at the first such query. Edge e is
     * m0's e-th edge; its halfedge 2e runs from its first vertex to its second, 2e + 1 back. */
    MCGPU_DATA_CUTPATH_STATUS = 25,      /* uint32[2]: 0, or 1 when a key holds fewer than two intersection
                                            vertices (MCUT stops the dispatch there: the arrays below are
                                            then not used); that key's index, else 0xFFFFFFFF */
    MCGPU_DATA_CUTPATH_EDGES = 26,       /* uint32[2E]: m0 ids of each edge's first and second vertex
                                            (m0_cutpath_edges in creation order) */
    MCGPU_DATA_CUTPATH_FACE_KEYS = 27,   /* uint32[F]: ps faces with cut-path edges, ascending
                                            (ps_iface_to_m0_edge_list keys) */
    MCGPU_DATA_CUTPATH_FACE_OFFSETS = 28, /* uint32[F+1] */
    MCGPU_DATA_CUTPATH_FACE_EDGES = 29,  /* uint32[o[F]]: each face's edges in the order MCUT appends them */
    MCGPU_DATA_CUTPATH_VERTEX_OFFSETS = 30, /* uint32[R+1]: per intersection vertex (record order) ... */
    MCGPU_DATA_CUTPATH_VERTEX_HALFEDGES = 31, /* uint32[2E]: ... the halfedges entering it in creation order
                                            (ivtx_to_incoming_hlist) */
    /* Floating polygons of a single dispatch (kernel.cpp:4078-4200), from its cut path: a circular cut
     * path (every vertex on two of its edges, none on a border edge of the soup) whose vertices all
     * pierce the same face. MCUT stops the dispatch on them (DETECTED_FLOATING_POLYGON), partitions
     * each such face and runs the front end again. P polygons, by face, then smallest vertex. */
    MCGPU_DATA_FLOATING_FACES = 32,      /* uint32[P]: the ps face holding each polygon */
    MCGPU_DATA_FLOATING_OFFSETS = 33,    /* uint32[P+1] */
    MCGPU_DATA_FLOATING_VERTICES = 34,   /* uint32[o[P]]: m0 ids around each polygon, from its smallest */
    MCGPU_DATA_FLOATING_NORMALS = 35,    /* double[3P]: the face's unit normal (floating_polygon_info_t) */
    MCGPU_DATA_FLOATING_NORMAL_COMPONENTS = 36, /* int32[P]: its largest component */
    /* A connected component's arrays as mcGetConnectedComponentData hands them to the caller
     * (frontend.cpp:2006-2832), from the halfedge mesh of the last mcgpu_halfedge_mesh call over
     * the component's faces in its corner order (F faces, E edges, V vertices) */
    MCGPU_DATA_CC_FACE = 37,             /* uint32[corners]: vertices around each face, the targets of
                                            its halfedges (MC_CONNECTED_COMPONENT_DATA_FACE) */
    MCGPU_DATA_CC_FACE_ADJACENT_FACE_SIZE = 38, /* uint32[F]: faces across each face's halfedges */
    MCGPU_DATA_CC_FACE_ADJACENT_FACE = 39, /* uint32[sum]: those faces, face by face, halfedge order */
    MCGPU_DATA_CC_EDGE = 40,             /* uint32[2E]: vertex(e, 0), vertex(e, 1) of each edge */
    MCGPU_DATA_CC_VERTEX_FLOAT = 41      /* float[3V]: the call's double vertices rounded to float
                                            (needs the vertices at the mcgpu_halfedge_mesh call) */
} mcgpu_data;

/* Context with its own stream and device memory pool on `device`.
 * Replaces: nothing in the reference (mcCreateContext, mcut.cpp:62-86, makes
 * the host context; the caller creates one of these beside it). */
int mcgpu_context_create(mcgpu_context* ctx, int device);
int mcgpu_context_release(mcgpu_context ctx);

/* One front-end dispatch: source mesh `src` against cut mesh `cut`.
 * Replaces build_oibvh x2 + intersectOIBVHs (preproc.cpp:2456, 2685, 2839;
 * bvh.cpp:219-783) and kernel.cpp:1781-3206 of dispatch().
 * Vertices are the reference's internal (recentred) coordinates unless
 * MCGPU_RECENTRE is given; cut_eps is the cut-mesh box enlargement
 * (preproc.cpp:2667-2693), ignored with MCGPU_RECENTRE. Host arrays are read
 * before the call returns. Results stay in the context until the next
 * dispatch on it. Returns MCGPU_OK when the call ran; the front end's own
 * outcome is out->status. */
int mcgpu_dispatch(mcgpu_context ctx, uint32_t flags, const mcgpu_mesh* src, const mcgpu_mesh* cut, double cut_eps,
    mcgpu_summary* out);

/* Copy a result array of the last dispatch. Two-call pattern as
 * mcGetConnectedComponentData (mcut.cpp:806): mem == NULL && bytes == 0
 * returns the size in *bytes_out. */
int mcgpu_get_data(mcgpu_context ctx, uint32_t query, uint64_t bytes, void* mem, uint64_t* bytes_out);

/* Many independent pairs in one pass (one launch per stage over all pairs).
 * Replaces n_pairs sequential mcDispatch front ends. Per-pair results are
 * summaries[i] and mcgpu_get_batch_data(ctx, i, ...). cut_eps may be NULL
 * with MCGPU_RECENTRE. */
int mcgpu_dispatch_batch(mcgpu_context ctx, uint32_t flags, uint32_t n_pairs, const mcgpu_mesh* srcs,
    const mcgpu_mesh* cuts, const double* cut_eps, mcgpu_summary* summaries);
int mcgpu_get_batch_data(mcgpu_context ctx, uint32_t pair, uint32_t query, uint64_t bytes, void* mem,
    uint64_t* bytes_out);

/* A batch of pairs packed end to end (the layout the library uses
 * internally, so the upload is one copy per array). For pair i, in order:
 * its source vertices then its cut vertices in `vertices`, and its source
 * face indices then its cut face indices in `face_indices`, each mesh's
 * indices LOCAL to that mesh (0-based), as mcDispatch takes them
 * (mcut.h:1003-1040). mesh_counts[4*i .. 4*i+3] = source vertices, source
 * faces, cut vertices, cut faces. face_sizes (NULL: triangles) follows the
 * same order. cut_eps[i] as in mcgpu_dispatch (may be NULL with
 * MCGPU_RECENTRE). With MCGPU_DEVICE_POINTERS the three arrays are device
 * pointers and `vertices` is read in place (keep it alive while results of
 * the dispatch are read). */
typedef struct mcgpu_batch {
    uint32_t num_pairs;
    const void* vertices;
    const uint32_t* face_indices;
    const uint32_t* face_sizes;
    const uint32_t* mesh_counts;
    const double* cut_eps;
} mcgpu_batch;

/* mcgpu_dispatch_batch over a packed batch. Replaces num_pairs sequential
 * mcDispatch front ends (the fracture use case: many independent uneven
 * pairs). Summaries as mcgpu_dispatch_batch; records of every pair with
 * mcgpu_get_data (grouped by pair, MCGPU_DATA_RECORD_OFFSETS) or per pair
 * with mcgpu_get_batch_data. */
int mcgpu_dispatch_packed(mcgpu_context ctx, uint32_t flags, const mcgpu_batch* batch, mcgpu_summary* summaries);

/* Launch tuning of a context. No setting changes any result (the pair set,
 * tests and records are independent of the tree's shape and of the
 * traversal order), only the speed. */
typedef struct mcgpu_tuning {
    uint32_t leaf_size;    /* cut faces per tree leaf, 1..16 (default 4) */
    uint32_t traversal;    /* 0: one warp per source packet, breadth-first (default);
                              1: one warp per source packet, depth-first;
                              2: one thread per source face */
    uint32_t packet_faces; /* source faces per packet = queries per warp, 1..32 (default 32) */
    uint32_t stack_depth;  /* per-thread stack of traversal 2: 64 (default) or 512 */
    uint32_t split_round;  /* traversal 0: walk rounds after which a packet with work left is split
                              across warps (a second launch); 0 never splits (default 2) */
} mcgpu_tuning;

int mcgpu_context_set_tuning(mcgpu_context ctx, const mcgpu_tuning* tuning);
int mcgpu_context_get_tuning(mcgpu_context ctx, mcgpu_tuning* tuning);

/* General-position enforcement of a context: the constant (> 0) scales
 * MCGPU_RECENTRE's cut_eps and the perturbations, attempts (>= 1) bounds the
 * perturbations of one dispatch; defaults 1e-4 and 4 (frontend.h:596-597).
 * Replaces mcBindState / mcGetInfo with MC_CONTEXT_GENERAL_POSITION_
 * ENFORCEMENT_CONSTANT / _ATTEMPTS (frontend.cpp:390-410, 335-350). */
int mcgpu_context_set_general_position(mcgpu_context ctx, double constant, uint32_t attempts);
int mcgpu_context_get_general_position(mcgpu_context ctx, double* constant, uint32_t* attempts);

/* Autotuner: runs `sample` (a packed batch, as mcgpu_dispatch_packed with
 * `flags`) under each candidate tuning -- leaf size {2, 4, 8} x {warp per
 * packet of 16 or 32 faces breadth-first, warp per packet depth-first,
 * thread per face with stack 64 or 512} -- `repeats` times each after one
 * warm-up, plus packet splitting on / off for the breadth-first walk;
 * keeps the fastest on ctx and returns it with its mean time.
 * No counterpart in the reference. */
int mcgpu_autotune(mcgpu_context ctx, uint32_t flags, const mcgpu_batch* sample, uint32_t repeats,
    mcgpu_tuning* best, float* best_ms);

/* The reference's recentring on the host (calculate_vertex_parameters +
 * client_input_arrays_to_hmesh, preproc.cpp:2124-2290, 147-181): writes the
 * internal coordinates of both meshes and the default cut-box enlargement
 * (|translated cut box diagonal| * 1e-4, preproc.cpp:2518, 2667-2676). */
int mcgpu_recentre(uint32_t flags, const mcgpu_mesh* src, const mcgpu_mesh* cut, double* src_out, double* cut_out,
    double* cut_eps_out);

/* Front-end dispatch that allocates no GPU or pinned memory. No counterpart
 * in the reference (MCUT allocates freely on the host). It is for callers
 * that may not call cudaMalloc when they need the records: a plugin that must
 * stay inside its host application's own device-memory arena, a process whose
 * device memory another framework's caching allocator already holds, a frame
 * loop that cannot wait on the driver's allocator. All scratch sits in one
 * file-scope __device__ array of about 12 MB that every GPU loading this
 * library keeps until exit. The call reads counters back into host variables
 * between its stages, so it waits for `stream` three or four times and
 * returns when its GPU work is done; it cannot be recorded into a CUDA
 * graph, and on a stream that is being captured it returns
 * MCGPU_INVALID_VALUE before any GPU call (the capture stays valid).
 * Limits: triangles only; at most 16384 vertices and 16384 faces over both
 * meshes, 32768 candidate pairs, 65536 edge-face tests -- anything larger
 * returns MCGPU_TOO_LARGE. Every call shares that array and it keeps the
 * previous call's contents (each call clears what it needs): calls whose GPU
 * work overlaps race, so serialise them. The first call on a device looks up
 * the array's address; make it before any stream capture begins.
 * src/cut: DEVICE pointers to internal (recentred) double coordinates and
 * uint32 triangle indices (face_sizes NULL). record_ids (uint32[5*capacity])
 * and record_points (double[3*capacity]) are device buffers filled as
 * MCGPU_DATA_RECORD_IDS / _POINTS of mcgpu_dispatch. stream: a cudaStream_t,
 * or NULL for the default stream. Returns MCGPU_OK when it ran; the front
 * end's outcome is out->status. */
int mcgpu_dispatch_noalloc(void* stream, const mcgpu_mesh* src, const mcgpu_mesh* cut, double cut_eps,
    uint32_t* record_ids, double* record_points, uint64_t record_capacity, mcgpu_summary* out);

/* Outcome of mcgpu_halfedge_mesh, in the order MCUT checks a mesh. */
typedef enum mcgpu_hmesh_status {
    MCGPU_HMESH_OK = 0,
    MCGPU_HMESH_FACE_SIZE = 1,       /* a face with fewer than 3 vertices */
    MCGPU_HMESH_INDEX_RANGE = 2,     /* an index >= the mesh's vertex count */
    MCGPU_HMESH_DUPLICATE_INDEX = 3, /* a vertex twice in one face */
    MCGPU_HMESH_NON_MANIFOLD = 4,    /* a directed halfedge in two faces */
    MCGPU_HMESH_TOO_SMALL = 5,       /* fewer than 3 vertices or no face */
    MCGPU_HMESH_COMPONENTS = 6       /* the vertex graph is not one connected component */
} mcgpu_hmesh_status;

typedef struct mcgpu_hmesh_report {
    int32_t status;           /* mcgpu_hmesh_status */
    int32_t bad_face;         /* the face a conversion error (codes 1-4) stopped at, else -1 */
    uint32_t num_edges;       /* set once the conversion succeeded (codes 0, 5, 6) */
    uint32_t num_components;  /* connected components of the vertex graph (codes 0, 6) */
    int32_t closed;           /* every halfedge has a face (mesh_is_closed); set with num_edges */
    uint32_t kernel_launches; /* CUDA kernels this call launched */
} mcgpu_hmesh_report;

/* MCUT's halfedge mesh of one input mesh and its input checks, on the
 * device. Replaces client_input_arrays_to_hmesh (preproc.cpp:57-468, face by
 * face through hmesh_t::add_face / add_edge, hmesh.cpp:406-651),
 * check_input_mesh (preproc.cpp:505-579) and mesh_is_closed
 * (preproc.cpp:1957-1994): the same status and failing face as that
 * face-by-face loop, the same edge and halfedge numbering, next / prev links
 * and per-vertex halfedge lists. The connectivity reads the indices and face
 * sizes only; double vertices, when given (float input is not), are rounded
 * to float for MCGPU_DATA_CC_VERTEX_FLOAT. With MCGPU_DEVICE_POINTERS the
 * arrays are device arrays. The results stay in the context until its next
 * mcgpu_halfedge_mesh call (mcgpu_get_data queries 18-24; 37-41, a
 * connected component's arrays as MCUT serialises them, when the mesh is a
 * component given in its corner order). Returns MCGPU_OK when it ran; the
 * mesh's outcome is out->status. */
int mcgpu_halfedge_mesh(mcgpu_context ctx, uint32_t flags, const mcgpu_mesh* mesh, mcgpu_hmesh_report* out);

/* ---- Request server: continuous batching on one GPU ------------------------
 * Replaces MCUT's per-context task queue for the front end (mcEnqueueDispatch,
 * mcut.cpp:459-552; frontend.h:548-580) when many independent dispatches
 * arrive over time. `workers` threads each own a context (stream + device
 * pool); a free worker takes the queued requests that fit its batch limits
 * and the HBM admission budget, runs them as one batched dispatch, and
 * completes them. Requests arriving meanwhile join the next batch, and the
 * workers' batches overlap on the device. Meshes are user coordinates
 * (double) and are recentred as mcDispatch does; like mcEnqueueDispatch,
 * the caller's arrays must stay valid until the request completes
 * (frontend.cpp:690-711). Cut meshes added with mcgpu_server_add_cut_mesh
 * stay resident on the device with their own tree (built once there, over
 * the user coordinates): a request naming one uploads only its source mesh,
 * and its source faces walk that tree instead of the cut faces joining the
 * batch's sort and tree. Device memory: the resident meshes (coordinates,
 * indices and tree; the build's scratch while it runs) plus what every worker
 * may hold -- its pool while idle, its batch's cap while it runs one --
 * stay within hbm_budget_bytes. A batch's cap is its requests' estimated
 * bytes with slack; its context cannot grow past it
 * (mcgpu_context_set_memory_limit). Idle workers' pools are freed when a
 * batch does not fit beside them; a batch that meets its cap runs again
 * with all the free budget, then in halves, and a request that still does
 * not fit completes with MCGPU_TOO_LARGE (as does one whose estimate alone
 * exceeds the budget, at submission). */
typedef struct mcgpu_server_t* mcgpu_server;

typedef struct mcgpu_server_config {
    int device;
    uint32_t workers;          /* batches in flight at once; 0 -> 3 */
    uint32_t max_batch_pairs;  /* requests per batch; 0 -> 512 */
    uint64_t max_batch_faces;  /* faces per batch (a larger request runs alone); 0 -> 16 Mi */
    uint64_t hbm_budget_bytes; /* 0 -> 150 GiB */
    uint32_t linger_us;        /* while other batches run, a short queue waits up to this long for
                                  more requests; 0 -> 400, > 1e6 -> never wait */
    uint32_t reserved;
} mcgpu_server_config;

typedef struct mcgpu_server_stats {
    uint64_t submitted, completed, batches, pending;
    uint64_t inflight_bytes, peak_inflight_bytes; /* estimated bytes of the requests in batches */
    uint64_t resident_bytes, resident_meshes;
    uint64_t pool_bytes;          /* device bytes the workers' pools hold now */
    uint64_t peak_reserved_bytes; /* peak of resident bytes + every worker's allowance: the bound
                                     on the device memory the server held */
    uint64_t pool_trims;          /* pools freed to make room */
    uint64_t cancelled;           /* requests cancelled before they ran */
} mcgpu_server_stats;

int mcgpu_server_create(mcgpu_server* server, const mcgpu_server_config* config);
/* Completes every queued request, then frees the server. */
int mcgpu_server_release(mcgpu_server server);
/* Keep a triangle cut mesh (double user coordinates) on the device. */
int mcgpu_server_add_cut_mesh(mcgpu_server server, const mcgpu_mesh* cut, uint32_t* cut_id);
/* Queue one request: `cut`, or NULL and a resident `cut_id`. */
int mcgpu_server_submit(mcgpu_server server, const mcgpu_mesh* src, const mcgpu_mesh* cut, uint32_t cut_id,
    uint64_t* ticket);
/* Take a queued request out of the queue before a batch takes it: it
 * completes with MCGPU_CANCELLED (MCGPU_NOT_READY: it is in a running batch;
 * MCGPU_INVALID_VALUE: it has completed). Its ticket stays until released. */
int mcgpu_server_cancel(mcgpu_server server, uint64_t ticket);
/* Wait for a request (timeout_ms < 0: no limit; MCGPU_NOT_READY on timeout).
 * latency_ms: submission to records on the host. */
int mcgpu_server_wait(mcgpu_server server, uint64_t ticket, int timeout_ms, mcgpu_summary* out,
    double* latency_ms);
/* MCGPU_DATA_RECORD_IDS / _POINTS of a completed request (two-call size pattern). */
int mcgpu_server_get_data(mcgpu_server server, uint64_t ticket, uint32_t query, uint64_t bytes, void* mem,
    uint64_t* bytes_out);
int mcgpu_server_release_request(mcgpu_server server, uint64_t ticket);
int mcgpu_server_get_stats(mcgpu_server server, mcgpu_server_stats* out);

/* ---- Device memory of a context ------------------------------------------
 * A context keeps its device buffers between calls (a grow-only pool).
 * mcgpu_context_get_memory: the bytes the pool holds now and its cap.
 * mcgpu_context_set_memory_limit: a call that would grow the pool past
 * limit_bytes fails with MCGPU_OUT_OF_MEMORY before that buffer is freed
 * (0: no cap). mcgpu_context_trim: waits for the context's streams, then
 * frees the whole pool and the captured launch graphs; the record, pair,
 * hand-over and halfedge-mesh queries of earlier calls are gone. */
int mcgpu_context_get_memory(mcgpu_context ctx, uint64_t* device_bytes, uint64_t* limit_bytes);
int mcgpu_context_set_memory_limit(mcgpu_context ctx, uint64_t limit_bytes);
int mcgpu_context_trim(mcgpu_context ctx);

/* The device's fp64 arithmetic rate in G operations/s: independent chains of
 * separately rounded multiplies and adds (the form the library's fp64 code
 * takes), timed with CUDA events over a fixed loop on every SM. The
 * denominator of the fp64-bound kernels' roofline. */
int mcgpu_measure_fp64_rate(int device, double* gops);

/* Human-readable description of the last failure on this thread. */
const char* mcgpu_last_error(void);

#ifdef __cplusplus
}
#endif
#endif /* MCUT_GB300_H */
