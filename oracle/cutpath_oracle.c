/*
 * CPU oracle for MCUT's cut-path edge creation (TEST INFRASTRUCTURE ONLY; the
 * product library never links it).
 *
 * dispatch() turns the intersection vertices into the edges of the cut path
 * (kernel.cpp:3332-3632): for each (source face, cut face) key of
 * cutpath_edge_creation_info, in the std::map's key order,
 *   - fewer than two vertices: the dispatch stops (INVALID_MESH_INTERSECTION,
 *     or GENERAL_POSITION_VIOLATION when enforcement is on; kernel.cpp:3416-3431);
 *   - two vertices a, b (in the list's order): the edge a -> b unless an edge
 *     joins them already; it goes to both faces' edge lists and to those of the
 *     faces across the two faces' edges that lie in both vertices' registries
 *     (update_neighouring_ps_iface_m0_edge_list, kernel.cpp:1420-1495);
 *   - more: the vertices sorted along their line (linear_projection_sort,
 *     kernel.cpp:1500-1541: projections onto normalize(first - second) from
 *     the first, ordered by libstdc++'s std::sort), and each consecutive pair
 *     joined -- unless an edge joins them already -- when the midpoint lies
 *     inside ('i') exactly two of the non-virtual faces both registries share;
 *     the edge goes to those faces' lists.
 * Edge e is m0's e-th edge (m0 holds no edge before this stage): halfedge 2e
 * runs from its first vertex to its second and is an incoming halfedge of the
 * second, 2e + 1 of the first (ivtx_to_incoming_hlist).
 *
 * A vertex's registry is {tested face, the faces of its tested edge}
 * (ps_get_ivtx_registry_entry_faces, kernel.cpp:1407-1415); a border edge's
 * missing face is UINT32_MAX (a virtual face).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "mcut_oracle.h"

/* ---- the narrow phase's plane and point-in-polygon (same arithmetic as
 * mcut_oracle.c: compute_polygon_plane_coefficients math.cpp:130-239,
 * calculate_projection_matrix math.cpp:710-793, compute_point_in_polygon_test
 * math.cpp:643-703, 851-902) ---- */
static double cp_dot3(const double *a, const double *b)
{
    double o = 0.0;
    o = o + a[0] * b[0];
    o = o + a[1] * b[1];
    o = o + a[2] * b[2];
    return o;
}

typedef struct { double n[3]; int mc; double P[2][3]; } cp_plane;

static void cp_projection(const double *nrm, int mc, double P[2][3])
{
    double len = sqrt(cp_dot3(nrm, nrm));
    double a[3] = { nrm[0] / len, nrm[1] / len, nrm[2] / len };
    double b[3] = { 0.0, 0.0, 0.0 };
    int s = (0.0 < nrm[mc]) - (nrm[mc] < 0.0);
    b[mc] = 1.0 * (double)s;
    double I[3][3] = { { 1.0, 0.0, 0.0 }, { 0.0, -1.0, 0.0 }, { 0.0, 0.0, 1.0 } };
    double R[3][3];
    memcpy(R, I, sizeof R);
    if (a[0] != b[0] || a[1] != b[1] || a[2] != b[2]) {
        double apb[3] = { a[0] + b[0], a[1] + b[1], a[2] + b[2] };
        double adb = cp_dot3(a, b);
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) R[i][j] = (((apb[i] * apb[j]) / adb) * 2.0) - I[i][j];
    }
    double K[2][3] = { { 0 } };
    if (mc == 0) { K[0][1] = 1.0; K[1][2] = 1.0; }
    else if (mc == 1) { K[0][0] = 1.0; K[1][2] = 1.0; }
    else { K[0][0] = 1.0; K[1][1] = 1.0; }
    for (int i = 0; i < 2; ++i)
        for (int j = 0; j < 3; ++j) {
            double acc = 0.0;
            for (int k = 0; k < 3; ++k) acc = acc + K[i][k] * R[k][j];
            P[i][j] = acc;
        }
}

/* 0: a plane; 1: degenerate (the narrow phase rejected such faces already) */
static int cp_face_plane(const double *x, const uint32_t *fv, int n, cp_plane *pl)
{
    double nx = 0.0, ny = 0.0, nz = 0.0;
    for (int i = 0; i < n; ++i) {
        const double *c = x + 3 * (size_t)fv[i], *d = x + 3 * (size_t)fv[(i + 1) % n];
        nx = nx + (c[1] - d[1]) * (c[2] + d[2]);
        ny = ny + (c[2] - d[2]) * (c[0] + d[0]);
        nz = nz + (c[0] - d[0]) * (c[1] + d[1]);
    }
    double nn[3] = { nx, ny, nz };
    double sq = cp_dot3(nn, nn);
    if (isnan(nx) || isnan(ny) || isnan(nz) || sq < 1e-9 || sq == 0.0) return 1;
    double len = sqrt(sq);
    pl->n[0] = nx / len; pl->n[1] = ny / len; pl->n[2] = nz / len;
    double big = 0.0;
    pl->mc = 0;
    for (int i = 0; i < 3; ++i) {
        double t = fabs(pl->n[i]);
        if (t > big) { big = t; pl->mc = i; }
    }
    cp_projection(pl->n, pl->mc, pl->P);
    return 0;
}

static void cp_project(const double P[2][3], const double *v, double *out)
{
    double r0 = 0.0, r1 = 0.0;
    for (int c = 0; c < 3; ++c) {
        r0 = r0 + P[0][c] * v[c];
        r1 = r1 + P[1][c] * v[c];
    }
    out[0] = r0;
    out[1] = r1;
}

static char cp_pip(const double *p, const double *x, const uint32_t *fv, int n, const cp_plane *pl)
{
    double q[2];
    cp_project(pl->P, p, q);
    double (*poly)[2] = (double (*)[2])malloc(sizeof(double) * 2 * (size_t)n);
    for (int i = 0; i < n; ++i) cp_project(pl->P, x + 3 * (size_t)fv[i], poly[i]);
    int rc = 0, lc = 0;
    char res = 0;
    for (int i = 0; i < n && !res; ++i) {
        double xi = poly[i][0] - q[0], yi = poly[i][1] - q[1];
        if (xi == 0.0 && yi == 0.0) { res = 'v'; break; }
        int il = (i + n - 1) % n;
        double xl = poly[il][0] - q[0], yl = poly[il][1] - q[1];
        int rs = (yi > 0.0) != (yl > 0.0);
        int ls = (yi < 0.0) != (yl < 0.0);
        if (rs || ls) {
            double t = (xi * yl - xl * yi) / (yl - yi);
            if (rs && t > 0.0) rc++;
            if (ls && t < 0.0) lc++;
        }
    }
    free(poly);
    if (res) return res;
    if ((rc % 2) != (lc % 2)) return 'e';
    return (rc % 2) == 1 ? 'i' : 'o';
}

/* ---- libstdc++'s std::sort of (vertex, projection) by projection: the same
 * introsort + final insertion sort schedule (bits/stl_algo.h
 * __introsort_loop, __final_insertion_sort), so that equal projections keep
 * the reference's order ---- */
typedef struct { uint32_t v; double p; } proj_t;
static int pj_less(const proj_t *a, const proj_t *b) { return a->p < b->p; }
static void pj_swap(proj_t *a, proj_t *b) { proj_t t = *a; *a = *b; *b = t; }
static void pj_ins(proj_t *f, long n)
{
    for (long i = 1; i < n; ++i) {
        proj_t v = f[i];
        if (pj_less(&v, &f[0])) {
            memmove(f + 1, f, sizeof(proj_t) * (size_t)i);
            f[0] = v;
        } else {
            long j = i;
            while (pj_less(&v, &f[j - 1])) { f[j] = f[j - 1]; --j; }
            f[j] = v;
        }
    }
}
static void pj_unguarded_ins(proj_t *f, long from, long n)
{
    for (long i = from; i < n; ++i) {
        proj_t v = f[i];
        long j = i;
        while (pj_less(&v, &f[j - 1])) { f[j] = f[j - 1]; --j; }
        f[j] = v;
    }
}
static void pj_median(proj_t *res, proj_t *a, proj_t *b, proj_t *c)
{
    if (pj_less(a, b)) {
        if (pj_less(b, c)) pj_swap(res, b);
        else if (pj_less(a, c)) pj_swap(res, c);
        else pj_swap(res, a);
    } else if (pj_less(a, c)) pj_swap(res, a);
    else if (pj_less(b, c)) pj_swap(res, c);
    else pj_swap(res, b);
}
static void pj_sift(proj_t *f, long hole, long len, proj_t v)
{
    long top = hole, child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (pj_less(&f[child], &f[child - 1])) child--;
        f[hole] = f[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        f[hole] = f[child - 1];
        hole = child - 1;
    }
    long parent = (hole - 1) / 2;
    while (hole > top && pj_less(&f[parent], &v)) {
        f[hole] = f[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    f[hole] = v;
}
static void pj_heap(proj_t *f, long n)
{
    if (n < 2) return;
    for (long parent = (n - 2) / 2;; --parent) {
        pj_sift(f, parent, n, f[parent]);
        if (parent == 0) break;
    }
    for (long last = n - 1; last > 0; --last) {
        proj_t v = f[last];
        f[last] = f[0];
        pj_sift(f, 0, last, v);
    }
}
static void pj_introsort(proj_t *f, long n, int depth)
{
    while (n > 16) {
        if (depth == 0) { pj_heap(f, n); return; }
        --depth;
        long mid = n / 2;
        pj_median(&f[0], &f[1], &f[mid], &f[n - 1]);
        long lo = 1, hi = n;
        for (;;) {
            while (pj_less(&f[lo], &f[0])) ++lo;
            --hi;
            while (pj_less(&f[0], &f[hi])) --hi;
            if (!(lo < hi)) break;
            pj_swap(&f[lo], &f[hi]);
            ++lo;
        }
        pj_introsort(f + lo, n - lo, depth);
        n = lo;
    }
}
static void pj_sort(proj_t *f, long n)
{
    if (n < 2) return;
    int lg = 63 - __builtin_clzll((unsigned long long)n);
    pj_introsort(f, n, 2 * lg);
    if (n > 16) {
        pj_ins(f, 16);
        pj_unguarded_ins(f, 16, n);
    } else {
        pj_ins(f, n);
    }
}

/* ---- small containers ---- */
typedef struct { uint64_t *key; uint32_t *val; uint64_t mask; } cp_hash;
static uint64_t cp_mix(uint64_t x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}
static void cp_hash_init(cp_hash *h, uint64_t n)
{
    uint64_t cap = 16;
    while (cap < 2 * n + 2) cap <<= 1;
    h->key = (uint64_t *)malloc(sizeof(uint64_t) * cap);
    h->val = (uint32_t *)malloc(sizeof(uint32_t) * cap);
    memset(h->key, 0xff, sizeof(uint64_t) * cap);
    h->mask = cap - 1;
}
/* the slot of key (empty: key[s] == UINT64_MAX) */
static uint64_t cp_hash_find(const cp_hash *h, uint64_t key)
{
    uint64_t s = cp_mix(key) & h->mask;
    while (h->key[s] != UINT64_MAX && h->key[s] != key) s = (s + 1) & h->mask;
    return s;
}

typedef struct { uint32_t key, val, seq; } triple_t;
typedef struct { triple_t *a; uint64_t n, cap; } tvec;
static void tv_push(tvec *v, uint32_t key, uint32_t val)
{
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 64;
        v->a = (triple_t *)realloc(v->a, sizeof(triple_t) * v->cap);
    }
    v->a[v->n].key = key;
    v->a[v->n].val = val;
    v->a[v->n].seq = (uint32_t)v->n;
    v->n++;
}
static int triple_cmp(const void *x, const void *y)
{
    const triple_t *a = (const triple_t *)x, *b = (const triple_t *)y;
    if (a->key != b->key) return a->key < b->key ? -1 : 1;
    return a->seq < b->seq ? -1 : (a->seq > b->seq);
}

/* registry faces of m0 vertex v (an intersection vertex) */
static void registry(const uint32_t *reg, uint32_t nv, uint32_t v, uint32_t r[3])
{
    const uint32_t *e = reg + 3 * (size_t)(v - nv);
    r[0] = e[0];
    r[1] = e[1];
    r[2] = e[2];
}
static int in3(const uint32_t r[3], uint32_t f) { return f != UINT32_MAX && (r[0] == f || r[1] == f || r[2] == f); }

int oracle_cutpath(uint32_t nv, const double *x, uint32_t nf, const uint32_t *soup_off, const uint32_t *soup_idx,
    uint32_t n_ivtx, const uint32_t *reg, const double *ivtx_xyz, uint32_t n_keys, const uint32_t *key_pairs,
    const uint32_t *key_off, const uint32_t *key_vtx, cp_result *out)
{
    memset(out, 0, sizeof *out);
    /* directed ps edge -> face, for the faces across a face's edges */
    cp_hash dir;
    cp_hash_init(&dir, soup_off[nf]);
    for (uint32_t f = 0; f < nf; ++f) {
        const uint32_t o = soup_off[f], n = soup_off[f + 1] - o;
        for (uint32_t k = 0; k < n; ++k) {
            const uint64_t key = ((uint64_t)soup_idx[o + k] << 32) | soup_idx[o + (k + 1) % n];
            const uint64_t s = cp_hash_find(&dir, key);
            if (dir.key[s] == UINT64_MAX) { dir.key[s] = key; dir.val[s] = f; }
        }
    }
    /* the coordinates of m0's vertices: ps vertices, then the intersection vertices */
    #define M0X(v) ((v) < nv ? x + 3 * (size_t)(v) : ivtx_xyz + 3 * (size_t)((v) - nv))
    cp_hash made; /* edges made so far, by their unordered vertex pair */
    uint64_t npairs = 0;
    for (uint32_t k = 0; k < n_keys; ++k) npairs += key_off[k + 1] - key_off[k];
    cp_hash_init(&made, npairs + 1);
    uint32_t *esrc = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(npairs + 1));
    uint32_t *etgt = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(npairs + 1));
    uint32_t ne = 0;
    tvec flist = { 0 }, hlist = { 0 };
    cp_plane *planes = (cp_plane *)calloc(nf ? nf : 1, sizeof(cp_plane));
    uint8_t *have_plane = (uint8_t *)calloc(nf ? nf : 1, 1);

    for (uint32_t k = 0; k < n_keys && out->status == 0; ++k) {
        const uint32_t sm_face = key_pairs[2 * k], cm_face = key_pairs[2 * k + 1];
        const uint32_t *L = key_vtx + key_off[k];
        const uint32_t m = key_off[k + 1] - key_off[k];
        if (m < 2) {
            out->status = 1;
            out->bad_key = k;
            break;
        }
        uint32_t *seq = (uint32_t *)malloc(sizeof(uint32_t) * m);
        int check_pip = 0;
        if (m == 2) {
            seq[0] = L[0];
            seq[1] = L[1];
        } else {
            /* linear_projection_sort (kernel.cpp:1500-1541) */
            const double *o = M0X(L[0]), *d = M0X(L[1]);
            double v[3] = { o[0] - d[0], o[1] - d[1], o[2] - d[2] };
            const double len = sqrt(cp_dot3(v, v));
            const double dir3[3] = { v[0] / len, v[1] / len, v[2] / len };
            proj_t *pj = (proj_t *)malloc(sizeof(proj_t) * m);
            for (uint32_t i = 0; i < m; ++i) {
                const double *p = M0X(L[i]);
                const double w[3] = { o[0] - p[0], o[1] - p[1], o[2] - p[2] };
                pj[i].v = L[i];
                pj[i].p = cp_dot3(w, dir3);
            }
            pj_sort(pj, m);
            for (uint32_t i = 0; i < m; ++i) seq[i] = pj[i].v;
            free(pj);
            check_pip = 1;
        }
        for (uint32_t i = 1; i < m; ++i) {
            const uint32_t a = seq[i - 1], b = seq[i];
            const uint64_t ukey = ((uint64_t)(a < b ? a : b) << 32) | (a < b ? b : a);
            const uint64_t slot = cp_hash_find(&made, ukey);
            if (made.key[slot] != UINT64_MAX) continue; /* m0.halfedge(a, b, true) exists */
            uint32_t ra[3], rb[3];
            registry(reg, nv, a, ra);
            registry(reg, nv, b, rb);
            uint32_t inside[3];
            int n_inside = 0;
            if (check_pip) {
                /* the shared faces (non-virtual, in a's registry order) whose area holds the midpoint */
                const double *pa = M0X(a), *pb = M0X(b);
                const double mid[3] = { (pb[0] + pa[0]) * 0.5, (pb[1] + pa[1]) * 0.5, (pb[2] + pa[2]) * 0.5 };
                for (int j = 0; j < 3; ++j) {
                    const uint32_t f = ra[j];
                    if (f == UINT32_MAX || !in3(rb, f)) continue;
                    if (!have_plane[f]) {
                        cp_face_plane(x, soup_idx + soup_off[f], (int)(soup_off[f + 1] - soup_off[f]), &planes[f]);
                        have_plane[f] = 1;
                    }
                    if (cp_pip(mid, x, soup_idx + soup_off[f], (int)(soup_off[f + 1] - soup_off[f]), &planes[f]) == 'i')
                        inside[n_inside++] = f;
                }
                if (n_inside != 2) continue;
            }
            const uint32_t e = ne++;
            made.key[slot] = ukey;
            made.val[slot] = e;
            esrc[e] = a;
            etgt[e] = b;
            if (check_pip) {
                tv_push(&flist, inside[0], e);
                tv_push(&flist, inside[1], e);
            } else {
                tv_push(&flist, sm_face, e);
                tv_push(&flist, cm_face, e);
                /* the faces across sm_face's and cm_face's edges in both registries */
                const uint32_t two[2] = { sm_face, cm_face };
                for (int s = 0; s < 2; ++s) {
                    const uint32_t f = two[s], o = soup_off[f], n = soup_off[f + 1] - o;
                    for (uint32_t c = 0; c < n; ++c) {
                        const uint64_t rk = ((uint64_t)soup_idx[o + (c + 1) % n] << 32) | soup_idx[o + c];
                        const uint64_t ds = cp_hash_find(&dir, rk);
                        if (dir.key[ds] == UINT64_MAX) continue;
                        const uint32_t g = dir.val[ds];
                        if (!in3(ra, g) || !in3(rb, g)) continue;
                        /* once per face (the list is checked for the edge) */
                        int dup = 0;
                        for (uint64_t q = flist.n; q-- > 0 && flist.a[q].val == e;)
                            if (flist.a[q].key == g) { dup = 1; break; }
                        if (!dup) tv_push(&flist, g, e);
                    }
                }
            }
            tv_push(&hlist, b - nv, 2 * e);     /* a -> b ends at b */
            tv_push(&hlist, a - nv, 2 * e + 1); /* its opposite at a */
        }
        free(seq);
    }
    #undef M0X
    out->n_edges = ne;
    out->edge_src = esrc;
    out->edge_tgt = etgt;
    /* per-face edge lists in append order */
    if (flist.n) qsort(flist.a, (size_t)flist.n, sizeof(triple_t), triple_cmp);
    uint32_t nfk = 0;
    for (uint64_t i = 0; i < flist.n; ++i) nfk += (i == 0 || flist.a[i].key != flist.a[i - 1].key);
    out->n_faces = nfk;
    out->face_keys = (uint32_t *)malloc(sizeof(uint32_t) * (nfk ? nfk : 1));
    out->face_off = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)nfk + 1));
    out->face_edges = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(flist.n ? flist.n : 1));
    uint32_t j = 0;
    for (uint64_t i = 0; i < flist.n; ++i) {
        if (i == 0 || flist.a[i].key != flist.a[i - 1].key) {
            out->face_keys[j] = flist.a[i].key;
            out->face_off[j++] = (uint32_t)i;
        }
        out->face_edges[i] = flist.a[i].val;
    }
    out->face_off[nfk] = (uint32_t)flist.n;
    /* per intersection vertex: its incoming halfedges in creation order */
    if (hlist.n) qsort(hlist.a, (size_t)hlist.n, sizeof(triple_t), triple_cmp);
    out->n_ivtx = n_ivtx;
    out->ivtx_off = (uint32_t *)calloc((size_t)n_ivtx + 1, sizeof(uint32_t));
    out->ivtx_he = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(hlist.n ? hlist.n : 1));
    for (uint64_t i = 0; i < hlist.n; ++i) {
        out->ivtx_off[hlist.a[i].key + 1]++;
        out->ivtx_he[i] = hlist.a[i].val;
    }
    for (uint32_t v = 0; v < n_ivtx; ++v) out->ivtx_off[v + 1] += out->ivtx_off[v];
    free(flist.a);
    free(hlist.a);
    free(planes);
    free(have_plane);
    free(dir.key); free(dir.val);
    free(made.key); free(made.val);
    return 0;
}

void oracle_cutpath_free(cp_result *r)
{
    free(r->edge_src); free(r->edge_tgt); free(r->face_keys); free(r->face_off); free(r->face_edges);
    free(r->ivtx_off); free(r->ivtx_he);
    memset(r, 0, sizeof *r);
}

/* ---- floating polygons (kernel.cpp:4078-4200) ----
 * The cut path's connected components (through its edges); a component is a
 * circular cut path when every vertex has two edges and none lies on a ps
 * border edge (m0_cutpath_terminal_vertices, kernel.cpp:3850-3870: a vertex
 * whose tested edge is a border edge); it is a floating polygon when every
 * vertex has the same tested face -- the polygon lies inside that face. Each
 * polygon is listed from its smallest vertex id, first towards the other end
 * of that vertex's lowest-numbered edge; polygons ordered by face, then by
 * their smallest vertex. */
static uint32_t fp_find(uint32_t *parent, uint32_t v)
{
    while (parent[v] != v) {
        parent[v] = parent[parent[v]];
        v = parent[v];
    }
    return v;
}

typedef struct { uint32_t face, root; } fp_key;
static int fp_cmp(const void *x, const void *y)
{
    const fp_key *a = (const fp_key *)x, *b = (const fp_key *)y;
    if (a->face != b->face) return a->face < b->face ? -1 : 1;
    return a->root < b->root ? -1 : (a->root > b->root);
}

int oracle_floating(uint32_t nv, const double *x, const uint32_t *soup_off, const uint32_t *soup_idx, uint32_t n_ivtx,
    const uint32_t *reg, uint32_t n_edges, const uint32_t *edges, fp_result *out)
{
    memset(out, 0, sizeof *out);
    uint32_t *parent = (uint32_t *)malloc(sizeof(uint32_t) * (n_ivtx ? n_ivtx : 1));
    uint32_t *deg = (uint32_t *)calloc(n_ivtx ? n_ivtx : 1, sizeof(uint32_t));
    uint8_t *bad = (uint8_t *)calloc(n_ivtx ? n_ivtx : 1, 1);
    /* incident edges per vertex, ascending (CSR) */
    uint32_t *eoff = (uint32_t *)calloc((size_t)n_ivtx + 1, sizeof(uint32_t));
    uint32_t *einc = (uint32_t *)malloc(sizeof(uint32_t) * (2 * (size_t)n_edges + 1));
    for (uint32_t v = 0; v < n_ivtx; ++v) parent[v] = v;
    for (uint32_t e = 0; e < n_edges; ++e)
        for (int s = 0; s < 2; ++s) eoff[edges[2 * e + s] - nv + 1]++;
    for (uint32_t v = 0; v < n_ivtx; ++v) eoff[v + 1] += eoff[v];
    uint32_t *fill = (uint32_t *)malloc(sizeof(uint32_t) * (n_ivtx ? n_ivtx : 1));
    memcpy(fill, eoff, sizeof(uint32_t) * n_ivtx);
    for (uint32_t e = 0; e < n_edges; ++e) {
        const uint32_t a = edges[2 * e] - nv, b = edges[2 * e + 1] - nv;
        einc[fill[a]++] = e;
        einc[fill[b]++] = e;
        deg[a]++;
        deg[b]++;
        uint32_t ra = fp_find(parent, a), rb = fp_find(parent, b);
        if (ra != rb) {
            if (ra < rb) parent[rb] = ra; else parent[ra] = rb;
        }
    }
    for (uint32_t v = 0; v < n_ivtx; ++v) {
        if (!deg[v]) continue;
        const uint32_t r = fp_find(parent, v);
        if (deg[v] != 2 || reg[3 * v + 2] == UINT32_MAX || reg[3 * v] != reg[3 * r]) bad[r] = 1;
    }
    fp_key *keys = (fp_key *)malloc(sizeof(fp_key) * (n_ivtx ? n_ivtx : 1));
    uint32_t np = 0;
    for (uint32_t v = 0; v < n_ivtx; ++v)
        if (deg[v] && fp_find(parent, v) == v && !bad[v]) keys[np++] = (fp_key) { reg[3 * v], v };
    qsort(keys, np, sizeof(fp_key), fp_cmp);
    out->n_polygons = np;
    out->faces = (uint32_t *)malloc(sizeof(uint32_t) * (np ? np : 1));
    out->off = (uint32_t *)malloc(sizeof(uint32_t) * ((size_t)np + 1));
    out->vtx = (uint32_t *)malloc(sizeof(uint32_t) * (n_ivtx ? n_ivtx : 1));
    out->normals = (double *)calloc(3 * (size_t)(np ? np : 1), sizeof(double));
    out->mc = (int32_t *)malloc(sizeof(int32_t) * (np ? np : 1));
    uint32_t nvtx = 0;
    for (uint32_t p = 0; p < np; ++p) {
        out->faces[p] = keys[p].face;
        /* the face's plane (ps_tested_face_to_plane_normal / _max_comp) */
        cp_plane pl;
        const uint32_t f = keys[p].face;
        if (x && cp_face_plane(x, soup_idx + soup_off[f], (int)(soup_off[f + 1] - soup_off[f]), &pl) == 0) {
            memcpy(out->normals + 3 * (size_t)p, pl.n, sizeof pl.n);
            out->mc[p] = pl.mc;
        } else {
            out->mc[p] = -1;
        }
        out->off[p] = nvtx;
        const uint32_t start = keys[p].root;
        uint32_t cur = start, prev_e = UINT32_MAX;
        do {
            out->vtx[nvtx++] = cur + nv;
            /* the incident edge other than the one arrived by (the lowest first) */
            uint32_t e = einc[eoff[cur]];
            if (e == prev_e) e = einc[eoff[cur] + 1];
            const uint32_t a = edges[2 * e] - nv, b = edges[2 * e + 1] - nv;
            prev_e = e;
            cur = a == cur ? b : a;
        } while (cur != start && nvtx < n_ivtx);
    }
    out->off[np] = nvtx;
    free(parent); free(deg); free(bad); free(eoff); free(einc); free(fill); free(keys);
    return 0;
}

void oracle_floating_free(fp_result *r)
{
    free(r->faces); free(r->off); free(r->vtx); free(r->normals); free(r->mc);
    memset(r, 0, sizeof *r);
}
