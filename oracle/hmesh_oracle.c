/*
 * Plain-C restatement of MCUT's input-mesh conversion and input checks:
 * the halfedge mesh that client_input_arrays_to_hmesh builds from the
 * caller's arrays (preproc.cpp:57-468; the single-threaded branch,
 * preproc.cpp:390-460, whose face-by-face order is the deterministic one)
 * through hmesh_t::add_face / add_edge (hmesh.cpp:406-651), and the mesh
 * checks of check_input_mesh (preproc.cpp:505-579): at least 3 vertices, at
 * least one face, exactly one connected component of the vertex graph
 * (find_connected_components, kernel.cpp:235-364; a vertex no face uses is a
 * component of its own), and whether the mesh is closed (mesh_is_closed,
 * preproc.cpp:1957-1994).
 *
 * TEST INFRASTRUCTURE ONLY: the oracle for the device edge table and validity
 * pass; the product library never links it. tests/test_hmesh_oracle.py pins
 * every array against the reference's own hmesh_t (oracle/ref_harness.cpp).
 *
 * Numbering, as add_edge creates it: an undirected edge gets the next id the
 * first time a face corner (v_i -> v_i+1, faces in order, corners in order)
 * meets it; its halfedge 2e runs in that first direction and 2e+1 the other
 * way. A corner reuses an existing edge's halfedge in its own direction, and
 * fails (non-manifold) if that halfedge already has a face. Next / prev link
 * the halfedges of each face in corner order; border halfedges stay unlinked.
 * Each vertex lists the halfedges that end at it, in creation order.
 */
#include "mcut_oracle.h"

#include <stdlib.h>
#include <string.h>

typedef struct {
    uint64_t *key; /* (min << 32 | max) + 1, 0 = empty */
    uint32_t *val;
    uint64_t cap;
} edge_map;

static uint64_t mix64(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

/* the edge id of {a, b}, or insert `next` and return it */
static uint32_t edge_find_or_add(edge_map *m, uint32_t a, uint32_t b, uint32_t next, int *added)
{
    const uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
    const uint64_t k = (((uint64_t)lo << 32) | hi) + 1;
    uint64_t i = mix64(k) & (m->cap - 1);
    for (;;) {
        if (m->key[i] == k) { *added = 0; return m->val[i]; }
        if (m->key[i] == 0) {
            m->key[i] = k;
            m->val[i] = next;
            *added = 1;
            return next;
        }
        i = (i + 1) & (m->cap - 1);
    }
}

static uint32_t uf_find(uint32_t *p, uint32_t x)
{
    while (p[x] != x) {
        p[x] = p[p[x]];
        x = p[x];
    }
    return x;
}

int oracle_hmesh(const uint32_t *f, const uint32_t *fs, uint32_t nv, uint32_t nf, hm_result *out)
{
    memset(out, 0, sizeof *out);
    out->bad_face = -1;
    uint64_t nidx = 0;
    for (uint32_t i = 0; i < nf; ++i) nidx += fs ? fs[i] : 3;
    uint64_t cap = 16;
    while (cap < 2 * nidx + 16) cap <<= 1;
    edge_map m = { (uint64_t *)calloc(cap, 8), (uint32_t *)malloc(4 * cap), cap };
    /* at most one edge per corner */
    const uint64_t hmax = 2 * (nidx ? nidx : 1);
    out->he_target = (uint32_t *)malloc(4 * hmax);
    out->he_face = (int32_t *)malloc(4 * hmax);
    out->he_next = (int32_t *)malloc(4 * hmax);
    out->he_prev = (int32_t *)malloc(4 * hmax);
    out->corner_he = (uint32_t *)malloc(4 * (nidx ? nidx : 1));
    out->v_off = (uint32_t *)calloc((size_t)nv + 1, 4);
    out->v_he = (uint32_t *)malloc(4 * hmax);
    uint32_t ne = 0;
    uint64_t o = 0;
    int st = HM_OK;
    /* client_input_arrays_to_hmesh, face by face (preproc.cpp:390-460) */
    for (uint32_t i = 0; i < nf && st == HM_OK; ++i) {
        const uint32_t n = fs ? fs[i] : 3;
        if (n < 3) { st = HM_FACE_SIZE; out->bad_face = (int32_t)i; break; }
        for (uint32_t j = 0; j < n && st == HM_OK; ++j) {
            const uint32_t v = f[o + j];
            if (v >= nv) { st = HM_INDEX_RANGE; out->bad_face = (int32_t)i; break; }
            for (uint32_t k = 0; k < j; ++k)
                if (f[o + k] == v) { st = HM_DUPLICATE_INDEX; out->bad_face = (int32_t)i; break; }
        }
        if (st != HM_OK) break;
        /* add_face (hmesh.cpp:523-651) */
        for (uint32_t j = 0; j < n; ++j) {
            const uint32_t v0 = f[o + j], v1 = f[o + (j + 1) % n];
            int added = 0;
            const uint32_t e = edge_find_or_add(&m, v0, v1, ne, &added);
            if (added) {
                /* add_edge (hmesh.cpp:406-521): h0 = 2e ends at v1, h1 = 2e+1 at v0 */
                out->he_target[2 * e] = v1;
                out->he_target[2 * e + 1] = v0;
                out->he_face[2 * e] = out->he_face[2 * e + 1] = -1;
                out->he_next[2 * e] = out->he_next[2 * e + 1] = -1;
                out->he_prev[2 * e] = out->he_prev[2 * e + 1] = -1;
                ++ne;
            }
            const uint32_t h = out->he_target[2 * e] == v1 ? 2 * e : 2 * e + 1;
            if (out->he_face[h] >= 0) { st = HM_NON_MANIFOLD; out->bad_face = (int32_t)i; break; }
            out->he_face[h] = (int32_t)i;
            out->corner_he[o + j] = h;
        }
        if (st != HM_OK) break;
        for (uint32_t j = 0; j < n; ++j) {
            const uint32_t h = out->corner_he[o + j], nh = out->corner_he[o + (j + 1) % n];
            out->he_next[h] = (int32_t)nh;
            out->he_prev[nh] = (int32_t)h;
        }
        o += n;
    }
    free(m.key);
    free(m.val);
    out->status = st;
    if (st != HM_OK) return 0; /* only the status and the failing face are defined */
    out->n_edges = ne;
    /* each vertex's halfedges (those ending at it) in creation order: edge e
     * appends 2e+1 to its first source and 2e to its first target */
    for (uint32_t h = 0; h < 2 * ne; ++h) out->v_off[out->he_target[h] + 1]++;
    for (uint32_t v = 0; v < nv; ++v) out->v_off[v + 1] += out->v_off[v];
    {
        uint32_t *cur = (uint32_t *)malloc(4 * ((size_t)nv + 1));
        memcpy(cur, out->v_off, 4 * (size_t)nv);
        for (uint32_t e = 0; e < ne; ++e) {
            const uint32_t h1 = 2 * e + 1, h0 = 2 * e;
            out->v_he[cur[out->he_target[h1]]++] = h1;
            out->v_he[cur[out->he_target[h0]]++] = h0;
        }
        free(cur);
    }
    /* mesh_is_closed (preproc.cpp:1957-1994): no halfedge without a face */
    out->closed = 1;
    for (uint32_t h = 0; h < 2 * ne; ++h)
        if (out->he_face[h] < 0) { out->closed = 0; break; }
    /* check_input_mesh (preproc.cpp:505-579) */
    if (nv < 3 || nf < 1) { out->status = HM_TOO_SMALL; return 0; }
    uint32_t *p = (uint32_t *)malloc(4 * (size_t)nv);
    for (uint32_t v = 0; v < nv; ++v) p[v] = v;
    for (uint32_t e = 0; e < ne; ++e) {
        const uint32_t a = uf_find(p, out->he_target[2 * e]), b = uf_find(p, out->he_target[2 * e + 1]);
        if (a != b) p[a < b ? b : a] = a < b ? a : b;
    }
    uint32_t nc = 0;
    for (uint32_t v = 0; v < nv; ++v) nc += uf_find(p, v) == v;
    free(p);
    out->n_components = nc;
    if (nc != 1) out->status = HM_COMPONENTS;
    return 0;
}

void oracle_hmesh_free(hm_result *r)
{
    free(r->he_target); free(r->he_face); free(r->he_next); free(r->he_prev);
    free(r->corner_he); free(r->v_off); free(r->v_he);
    memset(r, 0, sizeof *r);
}
