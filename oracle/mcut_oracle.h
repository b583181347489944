/*
 * CPU oracle for the MCUT intersection front end (test infrastructure only).
 *
 * Two implementations fill the same result record:
 *   - mcut_oracle.c      : a plain-C restatement of the reference algorithm
 *                          (builds anywhere, including the aarch64 GPU host);
 *   - ref_harness.cpp    : drives the unmodified reference sources compiled
 *                          into _ref/libmcut_ref.so (only where the reference
 *                          checkout exists).
 * The product library never links, loads or calls either of them.
 *
 * Identifiers follow the reference's polygon soup ("ps", kernel.cpp:1593-1732):
 *   ps vertex ids : source vertices [0, Vs), cut-mesh vertices [Vs, Vs+Vc)
 *   ps face ids   : source faces [0, Fs),    cut-mesh faces   [Fs, Fs+Fc)
 *   an edge       : (q, r) = source/target vertex of its primary halfedge,
 *                   i.e. the orientation it has in the lowest-numbered face
 *                   that contains it (hmesh.cpp:405-651, add_edge/add_face).
 */
#ifndef MCUT_ORACLE_H
#define MCUT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (kernel.h:52-92 mapped to the front end) */
enum {
    FE_OK = 0,
    FE_GP_VIOLATION = 1,       /* a touching / on-edge / on-vertex configuration */
    FE_DEGENERATE_SRC_FACE = 2,/* candidate source face with |Newell n|^2 < 1e-9 */
    FE_DEGENERATE_CUT_FACE = 3,
    FE_INVALID_INPUT = 4
};

/* One dispatch of the front end. All arrays are malloc'd by the producer and
 * released with the producer's free function. Tests/records are in canonical
 * order: ascending (q, r, face). */
typedef struct fe_result {
    int32_t status;
    int32_t bad_face;          /* ps face id of a degenerate face, else -1 */
    double cut_eps;            /* cut-mesh face-box enlargement */
    int64_t n_pairs;
    uint32_t *pairs;           /* 2*n_pairs: (source face, cut face), ascending */
    int64_t n_tests;
    uint32_t *tests;           /* 3*n_tests: (q, r, face) of each culled edge-face test */
    int8_t *test_info;         /* 4*n_tests: sign(orient3d q), sign(orient3d r), type char, pip char */
    int64_t n_records;
    uint32_t *rec_ids;         /* 3*n_records: (q, r, face) */
    double *rec_pts;           /* 3*n_records */
    double *face_boxes;        /* 6*(Fs+Fc): min xyz, max xyz (cut boxes enlarged) */
    double *src_xyz;           /* 3*Vs recentred coordinates */
    double *cut_xyz;           /* 3*Vc recentred coordinates */
} fe_result;

/* One front-end pass over internal (recentred) double coordinates with a
 * given cut-box enlargement (no recentring): what the front end computes
 * inside dispatch(). */
int oracle_front_end_internal(const double *xs, const uint32_t *sf, const uint32_t *sfs, uint32_t nsv, uint32_t nsf,
    const double *xc, const uint32_t *cf, const uint32_t *cfs, uint32_t ncv, uint32_t ncf, double eps, int threads,
    fe_result *out);
void oracle_free(fe_result *r);

/* The record hand-over of one front-end pass (kernel.cpp:2599-2655 and the
 * merge at kernel.cpp:2673-2714): what dispatch()'s host stages read from the
 * narrow phase. Every record becomes an intersection vertex of m0 with id
 * Vs + Vc + its position in the record order, which here is canonical: by
 * the tested edge's first face corner in the source-then-cut face arrays (the
 * edge's creation order in MCUT's halfedge mesh), then the tested face. The
 * reference numbers them in its threads' merge order instead.
 * Maps (vertex lists ascending, keys ascending as the reference's std::map
 * keeps them):
 *   edges     ps_intersecting_edges: records [edge_off[e], edge_off[e+1]) share
 *             the e-th intersected edge (their q, r)
 *   cutpath   cutpath_edge_creation_info: key (source face, cut face) of the
 *             tested face and each face of the tested edge
 *   faces     ps_iface_to_ivtx_list: the tested face and the edge's faces
 *   border    cm_border_reentrant_ivtx_list: records whose edge is a cut-mesh
 *             border edge; n_border > 0 is partial_cut_detected */
typedef struct fe_seam {
    int64_t n_records;
    uint32_t *rec_ids;         /* 5*R: q, r, tested face, f0 (the edge's first face), f1 (other or ~0u) */
    double *rec_pts;           /* 3*R */
    uint32_t n_edges;
    uint32_t *edge_off;        /* [n_edges+1] */
    uint32_t n_cutpath;
    uint32_t *cp_pairs;        /* [2*n_cutpath] */
    uint32_t *cp_off;          /* [n_cutpath+1] */
    uint32_t *cp_vtx;          /* [cp_off[n_cutpath]] m0 ids */
    uint32_t n_faces;
    uint32_t *face_keys;       /* [n_faces] */
    uint32_t *face_off;        /* [n_faces+1] */
    uint32_t *face_vtx;        /* [face_off[n_faces]] m0 ids */
    uint32_t n_border;
    uint32_t *border;          /* [n_border] m0 ids */
} fe_seam;

/* From a pass's records (rec3: q, r, face per record, any order; pts) and the
 * two meshes' faces. Returns 0, or -1 if a record's edge is not in the meshes. */
int oracle_seam(const uint32_t *sf, const uint32_t *sfs, uint32_t nsv, uint32_t nsf, const uint32_t *cf,
    const uint32_t *cfs, uint32_t ncv, uint32_t ncf, const uint32_t *rec3, const double *pts, int64_t nr,
    fe_seam *out);
void oracle_seam_free(fe_seam *s);

/* Input-mesh conversion and checks (hmesh_oracle.c; ref_hmesh in the
 * harness): the halfedge mesh MCUT builds from one mesh's arrays and the
 * outcome of its input checks. */
enum {
    HM_OK = 0,
    HM_FACE_SIZE = 1,       /* a face with fewer than 3 vertices */
    HM_INDEX_RANGE = 2,     /* a vertex index >= the vertex count */
    HM_DUPLICATE_INDEX = 3, /* a vertex twice in one face */
    HM_NON_MANIFOLD = 4,    /* a directed halfedge in two faces */
    HM_TOO_SMALL = 5,       /* fewer than 3 vertices or no face */
    HM_COMPONENTS = 6       /* the vertex graph is not one connected component */
};

typedef struct hm_result {
    int32_t status;
    int32_t bad_face;       /* the face a conversion error stopped at, else -1 */
    uint32_t n_edges;       /* this and the arrays: set once the conversion succeeded */
    uint32_t n_components;
    int32_t closed;         /* every halfedge has a face (mesh_is_closed, preproc.cpp:1957-1994) */
    uint32_t *he_target;    /* [2*n_edges] */
    int32_t *he_face;       /* [2*n_edges], -1 = no face */
    int32_t *he_next;       /* [2*n_edges], -1 = unlinked */
    int32_t *he_prev;       /* [2*n_edges] */
    uint32_t *corner_he;    /* one per face corner: the halfedge v_i -> v_i+1 */
    uint32_t *v_off;        /* [nv+1] */
    uint32_t *v_he;         /* the halfedges ending at each vertex, creation order */
} hm_result;

int oracle_hmesh(const uint32_t *f, const uint32_t *fs, uint32_t nv, uint32_t nf, hm_result *out);
void oracle_hmesh_free(hm_result *r);

/* MCUT's cut-path edge creation from the record hand-over (kernel.cpp:
 * 3332-3632; cutpath_oracle.c). Inputs: the ps vertex count nv and
 * coordinates x; the ps faces with their corners in the polygon soup's order
 * (soup_off / soup_idx, ps vertex ids); per intersection vertex (m0 id nv + i)
 * its registry (tested face, the tested edge's two faces, UINT32_MAX for
 * none) and coordinates; cutpath_edge_creation_info in key order (key_pairs:
 * source face, cut face; key_off / key_vtx: its vertices in list order). */
typedef struct cp_result {
    int32_t status;         /* 0; 1: a key with fewer than two vertices (dispatch stops) */
    uint32_t bad_key;       /* that key */
    uint32_t n_edges;       /* m0_cutpath_edges: edge e runs edge_src[e] -> edge_tgt[e] (halfedge 2e) */
    uint32_t *edge_src, *edge_tgt;
    uint32_t n_faces;       /* ps_iface_to_m0_edge_list: faces ascending, each edge list in append order */
    uint32_t *face_keys, *face_off, *face_edges;
    uint32_t n_ivtx;        /* ivtx_to_incoming_hlist, per intersection vertex in creation order */
    uint32_t *ivtx_off, *ivtx_he;
} cp_result;

int oracle_cutpath(uint32_t nv, const double *x, uint32_t nf, const uint32_t *soup_off, const uint32_t *soup_idx,
    uint32_t n_ivtx, const uint32_t *reg, const double *ivtx_xyz, uint32_t n_keys, const uint32_t *key_pairs,
    const uint32_t *key_off, const uint32_t *key_vtx, cp_result *out);
void oracle_cutpath_free(cp_result *r);

/* MCUT's floating-polygon detection (kernel.cpp:4078-4200) from the cut
 * path: per intersection vertex (m0 id nv + i) its registry as above and the
 * cut-path edges (first, second vertex). Polygons: their ps face ascending,
 * each polygon's m0 vertex ids in cycle order from its smallest. */
typedef struct fp_result {
    uint32_t n_polygons;
    uint32_t *faces;       /* [n_polygons] */
    uint32_t *off;         /* [n_polygons + 1] */
    uint32_t *vtx;
    double *normals;       /* [3 n_polygons]: the face's unit normal (x given) */
    int32_t *mc;           /* [n_polygons]: its largest component, -1 without x */
} fp_result;
int oracle_floating(uint32_t nv, const double *x, const uint32_t *soup_off, const uint32_t *soup_idx, uint32_t n_ivtx,
    const uint32_t *reg, uint32_t n_edges, const uint32_t *edges, fp_result *out);
void oracle_floating_free(fp_result *r);

#ifdef __cplusplus
}
#endif
#endif
