// MCUT's cut-path edge creation on the device (kernel.cpp:3332-3632), from
// one dispatch's record hand-over.
//
// For each (source face, cut face) key of cutpath_edge_creation_info, in key
// order, the reference makes edges between the key's intersection vertices:
//   two vertices a, b: the edge a -> b, unless an edge joins them already; it
//     joins both faces' edge lists and those of the faces across the two
//     faces' edges that lie in both vertices' registries
//     (update_neighouring_ps_iface_m0_edge_list, kernel.cpp:1420-1495);
//   more: the vertices ordered along their line (linear_projection_sort,
//     kernel.cpp:1500-1541, projections onto normalize(first - second)
//     ordered by libstdc++'s std::sort), and each consecutive pair joined --
//     unless an edge joins them already -- when its midpoint lies inside
//     ('i') exactly two of the non-virtual faces both registries share; the
//     edge joins those two faces' lists;
//   fewer: the dispatch stops (kCpBadKey).
// Edge e is m0's e-th edge (m0 has no edge before this stage), halfedge 2e
// runs first -> second vertex and enters the second, 2e + 1 enters the first
// (ivtx_to_incoming_hlist). A vertex's registry is {tested face, the tested
// edge's faces} (ps_get_ivtx_registry_entry_faces, kernel.cpp:1407-1415).
//
// On the device every key's candidate edges are made at once (a sorted run
// by one thread, the midpoint tests by one thread per candidate); the edge a
// pair of vertices gets is the first candidate in key order that passes its
// test -- which is what the reference's "unless an edge joins them already"
// leaves, since a failed test makes no edge -- found by one radix sort of the
// passing candidates by vertex pair; an exclusive scan over the kept
// candidates numbers the edges in creation order. The per-face lists and the
// per-vertex halfedge lists are (face, edge) and (vertex, halfedge) entries
// sorted into flat offset arrays: each list in creation order.
#include <cstdint>

#include "fe_common.cuh"
#include "fe_cutpath.cuh"
#include "fe_sort.cuh"

namespace mcgpu {

namespace {

constexpr int kCB = 256;

__device__ __forceinline__ void cp_vertex(const CutpathInput& in, uint32_t v, double* x)
{
    const double* p;
    if (v >= in.nv) p = in.rec_pts + 3 * (size_t)(v - in.nv);
    else if (v < in.xsplit) p = in.X + 3 * (size_t)v;
    else p = in.Xc + 3 * (size_t)(v - in.xsplit);
    x[0] = p[0];
    x[1] = p[1];
    x[2] = p[2];
}
__device__ __forceinline__ uint32_t cp_face_o(const CutpathInput& in, uint32_t f) { return in.foff ? in.foff[f] : 3 * f; }
__device__ __forceinline__ uint32_t cp_face_n(const CutpathInput& in, uint32_t f)
{
    return in.foff ? in.foff[f + 1] - in.foff[f] : 3u;
}
// corner k of face f in the polygon soup's order: a source face lists its
// input corners from the second, a cut face from the third (the soup's
// get_vertices_around_face, hmesh.cpp:722-733, kernel.cpp:1650-1700)
__device__ __forceinline__ uint32_t cp_corner(const CutpathInput& in, uint32_t f, uint32_t o, uint32_t n, uint32_t k)
{
    uint32_t j = k + (f < in.fs ? 1u : 2u);
    if (j >= n) j -= n;
    return in.fidx[o + j];
}

// face f's unit normal and largest component from its soup corners
// (compute_polygon_plane_coefficients, math.cpp:130-239); false: no plane
__device__ bool cp_plane(const CutpathInput& in, uint32_t f, double* nrm, int& mc)
{
    const uint32_t o = cp_face_o(in, f), n = cp_face_n(in, f);
    double nx = 0.0, ny = 0.0, nz = 0.0, c[3], d[3], first[3];
    cp_vertex(in, cp_corner(in, f, o, n, 0), first);
    c[0] = first[0]; c[1] = first[1]; c[2] = first[2];
    for (uint32_t k = 0; k < n; ++k) {
        if (k + 1 < n) cp_vertex(in, cp_corner(in, f, o, n, k + 1), d);
        else { d[0] = first[0]; d[1] = first[1]; d[2] = first[2]; }
        nx = nx + (c[1] - d[1]) * (c[2] + d[2]);
        ny = ny + (c[2] - d[2]) * (c[0] + d[0]);
        nz = nz + (c[0] - d[0]) * (c[1] + d[1]);
        c[0] = d[0]; c[1] = d[1]; c[2] = d[2];
    }
    const double nn[3] = { nx, ny, nz };
    const double sq = dot3(nn, nn);
    if (isnan(nx) || isnan(ny) || isnan(nz) || sq < 1e-9 || sq == 0.0) return false;
    const double len = sqrt(sq);
    nrm[0] = nx / len; nrm[1] = ny / len; nrm[2] = nz / len;
    mc = 0;
    double big = 0.0;
    for (int i = 0; i < 3; ++i) {
        const double t = fabs(nrm[i]);
        if (t > big) { big = t; mc = i; }
    }
    return true;
}

// compute_point_in_polygon_test (math.cpp:643-703, 851-902) against face f,
// with the face's plane from its soup corners (compute_polygon_plane_
// coefficients, math.cpp:130-239) and calculate_projection_matrix
__device__ char cp_pip(const CutpathInput& in, uint32_t f, const double* pt)
{
    const uint32_t o = cp_face_o(in, f), n = cp_face_n(in, f);
    double nx = 0.0, ny = 0.0, nz = 0.0, c[3], d[3], first[3];
    cp_vertex(in, cp_corner(in, f, o, n, 0), first);
    c[0] = first[0]; c[1] = first[1]; c[2] = first[2];
    for (uint32_t k = 0; k < n; ++k) {
        if (k + 1 < n) cp_vertex(in, cp_corner(in, f, o, n, k + 1), d);
        else { d[0] = first[0]; d[1] = first[1]; d[2] = first[2]; }
        nx = nx + (c[1] - d[1]) * (c[2] + d[2]);
        ny = ny + (c[2] - d[2]) * (c[0] + d[0]);
        nz = nz + (c[0] - d[0]) * (c[1] + d[1]);
        c[0] = d[0]; c[1] = d[1]; c[2] = d[2];
    }
    const double nn[3] = { nx, ny, nz };
    const double sq = dot3(nn, nn);
    if (isnan(nx) || isnan(ny) || isnan(nz) || sq < 1e-9 || sq == 0.0) return 'o'; // no plane (the narrow phase stopped on such faces)
    const double len = sqrt(sq);
    const double nrm[3] = { nx / len, ny / len, nz / len };
    int mc = 0;
    double big = 0.0;
    for (int i = 0; i < 3; ++i) {
        const double t = fabs(nrm[i]);
        if (t > big) { big = t; mc = i; }
    }
    double Pm[6], q[2], prv[2];
    projection_matrix(nrm, mc, Pm);
    project2(Pm, pt, q);
    {
        double v[3];
        cp_vertex(in, cp_corner(in, f, o, n, n - 1), v);
        project2(Pm, v, prv);
    }
    int rc = 0, lc = 0;
    for (uint32_t i = 0; i < n; ++i) {
        double v[3], p2[2];
        cp_vertex(in, cp_corner(in, f, o, n, i), v);
        project2(Pm, v, p2);
        const double xi = p2[0] - q[0], yi = p2[1] - q[1];
        if (xi == 0.0 && yi == 0.0) return 'v';
        const double xl = prv[0] - q[0], yl = prv[1] - q[1];
        const bool rs = (yi > 0.0) != (yl > 0.0);
        const bool ls = (yi < 0.0) != (yl < 0.0);
        if (rs || ls) {
            const double x = (xi * yl - xl * yi) / (yl - yi);
            if (rs && x > 0.0) rc++;
            if (ls && x < 0.0) lc++;
        }
        prv[0] = p2[0]; prv[1] = p2[1];
    }
    if ((rc & 1) != (lc & 1)) return 'e';
    return (rc & 1) ? 'i' : 'o';
}

// face g holds an edge of face s reversed (the face across one of s's edges)
__device__ bool cp_across(const CutpathInput& in, uint32_t s, uint32_t g)
{
    const uint32_t os = cp_face_o(in, s), ns = cp_face_n(in, s), og = cp_face_o(in, g), ng = cp_face_n(in, g);
    for (uint32_t i = 0; i < ns; ++i) {
        const uint32_t u = in.fidx[os + i], v = in.fidx[os + (i + 1 == ns ? 0 : i + 1)];
        for (uint32_t j = 0; j < ng; ++j)
            if (in.fidx[og + j] == v && in.fidx[og + (j + 1 == ng ? 0 : j + 1)] == u) return true;
    }
    return false;
}

// libstdc++'s std::sort of (vertex, projection) pairs by projection, replayed
// (bits/stl_algo.h: __introsort_loop with a median-of-three pivot into the
// first slot and an unguarded partition, heap sort past 2 log2(n) levels,
// then __final_insertion_sort), on two parallel arrays
struct PjArr {
    uint32_t* v;
    double* p;
    __device__ bool less(long a, long b) const { return p[a] < p[b]; }
    __device__ void swap(long a, long b) const
    {
        const uint32_t tv = v[a]; v[a] = v[b]; v[b] = tv;
        const double tp = p[a]; p[a] = p[b]; p[b] = tp;
    }
};
__device__ void pj_insertion(const PjArr& f, long n)
{
    for (long i = 1; i < n; ++i) {
        const uint32_t vv = f.v[i];
        const double pv = f.p[i];
        if (pv < f.p[0]) {
            for (long j = i; j > 0; --j) { f.v[j] = f.v[j - 1]; f.p[j] = f.p[j - 1]; }
            f.v[0] = vv; f.p[0] = pv;
        } else {
            long j = i;
            while (pv < f.p[j - 1]) { f.v[j] = f.v[j - 1]; f.p[j] = f.p[j - 1]; --j; }
            f.v[j] = vv; f.p[j] = pv;
        }
    }
}
__device__ void pj_unguarded(const PjArr& f, long from, long n)
{
    for (long i = from; i < n; ++i) {
        const uint32_t vv = f.v[i];
        const double pv = f.p[i];
        long j = i;
        while (pv < f.p[j - 1]) { f.v[j] = f.v[j - 1]; f.p[j] = f.p[j - 1]; --j; }
        f.v[j] = vv; f.p[j] = pv;
    }
}
__device__ void pj_median(const PjArr& f, long res, long a, long b, long c)
{
    if (f.less(a, b)) {
        if (f.less(b, c)) f.swap(res, b);
        else if (f.less(a, c)) f.swap(res, c);
        else f.swap(res, a);
    } else if (f.less(a, c)) f.swap(res, a);
    else if (f.less(b, c)) f.swap(res, c);
    else f.swap(res, b);
}
__device__ void pj_sift(const PjArr& f, long hole, long len, uint32_t vv, double pv)
{
    long top = hole, child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (f.less(child, child - 1)) child--;
        f.v[hole] = f.v[child]; f.p[hole] = f.p[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        f.v[hole] = f.v[child - 1]; f.p[hole] = f.p[child - 1];
        hole = child - 1;
    }
    long parent = (hole - 1) / 2;
    while (hole > top && f.p[parent] < pv) {
        f.v[hole] = f.v[parent]; f.p[hole] = f.p[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    f.v[hole] = vv; f.p[hole] = pv;
}
__device__ void pj_heap(const PjArr& f, long n)
{
    if (n < 2) return;
    for (long parent = (n - 2) / 2;; --parent) {
        pj_sift(f, parent, n, f.v[parent], f.p[parent]);
        if (parent == 0) break;
    }
    for (long last = n - 1; last > 0; --last) {
        const uint32_t vv = f.v[last];
        const double pv = f.p[last];
        f.v[last] = f.v[0]; f.p[last] = f.p[0];
        pj_sift(f, 0, last, vv, pv);
    }
}
__device__ void pj_sort(PjArr f, long n)
{
    if (n < 2) return;
    // the introsort loop, with its recursion on the right part kept on a stack
    struct Range { long lo, n; int depth; };
    Range st[64];
    int sp = 0;
    st[sp++] = Range { 0, n, 2 * (63 - __clzll((long long)n)) };
    while (sp > 0) {
        Range r = st[--sp];
        PjArr g { f.v + r.lo, f.p + r.lo };
        long m = r.n;
        int depth = r.depth;
        while (m > 16) {
            if (depth == 0) { pj_heap(g, m); break; }
            --depth;
            pj_median(g, 0, 1, m / 2, m - 1);
            long lo = 1, hi = m;
            for (;;) {
                while (g.less(lo, 0)) ++lo;
                --hi;
                while (g.less(0, hi)) --hi;
                if (!(lo < hi)) break;
                g.swap(lo, hi);
                ++lo;
            }
            // the reference recurses into [lo, m) first, then loops on [0, lo);
            // both parts are disjoint, so the order they are sorted in is free
            if (sp < 64) st[sp++] = Range { r.lo + lo, m - lo, depth };
            else pj_heap(PjArr { g.v + lo, g.p + lo }, m - lo);
            m = lo;
        }
    }
    if (n > 16) {
        pj_insertion(f, 16);
        pj_unguarded(f, 16, n);
    } else {
        pj_insertion(f, n);
    }
}

__host__ __device__ __forceinline__ unsigned long long sentinel(int bits) { return bits >= 64 ? ~0ull : ((1ull << bits) - 1); }

// one thread per key: its candidate edges (a long key's vertices sorted along their line)
__global__ void __launch_bounds__(kCB) k_cp_candidates(CutpathInput in, CutpathScratch w, uint32_t* __restrict__ counts)
{
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < in.n_keys; k += gridDim.x * blockDim.x) {
        const uint32_t o = in.cp_off[k], m = in.cp_off[k + 1] - o, base = o - k;
        if (m < 2) {
            atomicMin(&counts[kCpBadKey], k);
            continue;
        }
        if (m == 2) {
            uint32_t* c = w.cand + 4 * (size_t)base;
            c[0] = in.cp_vtx[o];
            c[1] = in.cp_vtx[o + 1];
            c[2] = k;
            c[3] = 0;
            continue;
        }
        double org[3], dst[3], v[3], dir[3];
        cp_vertex(in, in.cp_vtx[o], org);
        cp_vertex(in, in.cp_vtx[o + 1], dst);
        for (int j = 0; j < 3; ++j) v[j] = org[j] - dst[j];
        const double len = sqrt(dot3(v, v));
        for (int j = 0; j < 3; ++j) dir[j] = v[j] / len;
        for (uint32_t i = 0; i < m; ++i) {
            double p[3], d[3];
            cp_vertex(in, in.cp_vtx[o + i], p);
            for (int j = 0; j < 3; ++j) d[j] = org[j] - p[j];
            w.sorted[o + i] = in.cp_vtx[o + i];
            w.proj[o + i] = dot3(d, dir);
        }
        pj_sort(PjArr { w.sorted + o, w.proj + o }, m);
        for (uint32_t i = 0; i + 1 < m; ++i) {
            uint32_t* c = w.cand + 4 * (size_t)(base + i);
            c[0] = w.sorted[o + i];
            c[1] = w.sorted[o + i + 1];
            c[2] = k;
            c[3] = 1;
        }
    }
}

// one thread per candidate: the midpoint test of a sorted run's pairs; the
// passing candidates keyed by their vertex pair
__global__ void __launch_bounds__(kCB) k_cp_filter(CutpathInput in, CutpathScratch w, uint32_t n_cand, int vbits)
{
    const unsigned long long none = sentinel(2 * vbits);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_cand; j += gridDim.x * blockDim.x) {
        const uint32_t* c = w.cand + 4 * (size_t)j;
        const uint32_t a = c[0], b = c[1];
        bool pass = true;
        if (c[3] == 1) {
            const uint32_t* ra = in.rec_ids + 5 * (size_t)(a - in.nv) + 2;
            const uint32_t* rb = in.rec_ids + 5 * (size_t)(b - in.nv) + 2;
            double pa[3], pb[3], mid[3];
            cp_vertex(in, a, pa);
            cp_vertex(in, b, pb);
            for (int t = 0; t < 3; ++t) mid[t] = (pb[t] + pa[t]) * 0.5;
            uint32_t hit[2] = { kNone, kNone }, nh = 0;
            for (int t = 0; t < 3; ++t) {
                const uint32_t f = ra[t];
                if (f == kNone || (rb[0] != f && rb[1] != f && rb[2] != f)) continue;
                if (cp_pip(in, f, mid) == 'i') {
                    if (nh < 2) hit[nh] = f;
                    ++nh;
                }
            }
            pass = nh == 2;
            w.inside[2 * (size_t)j] = hit[0];
            w.inside[2 * (size_t)j + 1] = hit[1];
        }
        const uint32_t lo = a < b ? a : b, hi = a < b ? b : a;
        w.pk[0][j] = pass ? (((unsigned long long)lo << vbits) | hi) : none;
        w.pv[0][j] = j;
    }
}

// the first passing candidate of each vertex pair (in candidate = key order) makes the edge
__global__ void __launch_bounds__(kCB) k_cp_first(const unsigned long long* __restrict__ pk,
    const uint32_t* __restrict__ pv, uint32_t n, int vbits, uint32_t* __restrict__ made)
{
    const unsigned long long none = sentinel(2 * vbits);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        made[pv[p]] = (pk[p] != none && (p == 0 || pk[p - 1] != pk[p])) ? 1u : 0u;
}

// the made edges, their face-list and halfedge entries
__global__ void __launch_bounds__(kCB) k_cp_emit(CutpathInput in, CutpathScratch w, uint32_t n_cand, int fbits,
    int ebits, int hbits, uint32_t* __restrict__ edges)
{
    const unsigned long long fnone = sentinel(fbits + ebits), hnone = sentinel(32 - __clz(in.nrec) + hbits);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n_cand; j += gridDim.x * blockDim.x) {
        unsigned long long* fk = w.fk[0] + 5 * (size_t)j;
        unsigned long long* hk = w.hk[0] + 2 * (size_t)j;
        for (int s = 0; s < 5; ++s) {
            fk[s] = fnone;
            w.fv[0][5 * (size_t)j + s] = 5 * j + s;
        }
        hk[0] = hk[1] = hnone;
        w.hv[0][2 * (size_t)j] = 2 * j;
        w.hv[0][2 * (size_t)j + 1] = 2 * j + 1;
        if (w.made[j + 1] == w.made[j]) continue; // no edge
        const uint32_t e = w.made[j];
        const uint32_t* c = w.cand + 4 * (size_t)j;
        const uint32_t a = c[0], b = c[1], k = c[2];
        edges[2 * (size_t)e] = a;
        edges[2 * (size_t)e + 1] = b;
        auto fkey = [&](uint32_t f) { return ((unsigned long long)f << ebits) | e; };
        if (c[3] == 1) {
            fk[0] = fkey(w.inside[2 * (size_t)j]);
            fk[1] = fkey(w.inside[2 * (size_t)j + 1]);
        } else {
            const uint32_t sm = in.cp_pairs[2 * (size_t)k], cm = in.cp_pairs[2 * (size_t)k + 1];
            fk[0] = fkey(sm);
            fk[1] = fkey(cm);
            const uint32_t* ra = in.rec_ids + 5 * (size_t)(a - in.nv) + 2;
            const uint32_t* rb = in.rec_ids + 5 * (size_t)(b - in.nv) + 2;
            int s = 2;
            for (int t = 0; t < 3; ++t) {
                const uint32_t f = ra[t];
                if (f == kNone || f == sm || f == cm || (rb[0] != f && rb[1] != f && rb[2] != f)) continue;
                if (cp_across(in, sm, f) || cp_across(in, cm, f)) fk[s++] = fkey(f);
            }
        }
        hk[0] = ((unsigned long long)(b - in.nv) << hbits) | (2ull * e);
        hk[1] = ((unsigned long long)(a - in.nv) << hbits) | (2ull * e + 1);
    }
}

// run heads of the sorted (face, edge) entries
__global__ void __launch_bounds__(kCB) k_cp_face_heads(const unsigned long long* __restrict__ fk, uint32_t n,
    int fbits, int ebits, uint32_t* __restrict__ flags)
{
    const unsigned long long none = sentinel(fbits + ebits);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        flags[p] = (fk[p] != none && (p == 0 || (fk[p - 1] >> ebits) != (fk[p] >> ebits))) ? 1u : 0u;
}

__global__ void __launch_bounds__(kCB) k_cp_face_out(const unsigned long long* __restrict__ fk, uint32_t n,
    int fbits, int ebits, const uint32_t* __restrict__ head_pos, CutpathOut o)
{
    const unsigned long long none = sentinel(fbits + ebits), emask = sentinel(ebits);
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) {
        if (fk[p] == none) continue;
        o.face_edges[p] = (uint32_t)(fk[p] & emask);
        const bool head = p == 0 || (fk[p - 1] >> ebits) != (fk[p] >> ebits);
        if (head) {
            o.face_keys[head_pos[p]] = (uint32_t)(fk[p] >> ebits);
            o.face_off[head_pos[p]] = p;
        }
        if (p + 1 == n || fk[p + 1] == none) { // the last entry
            o.face_off[head_pos[n]] = p + 1;
            o.counts[kCpFaces] = head_pos[n];
            o.counts[kCpFaceEntries] = p + 1;
        }
    }
}

// per intersection vertex: the first of its sorted (vertex, halfedge) entries
__global__ void __launch_bounds__(kCB) k_cp_ivtx_out(const unsigned long long* __restrict__ hk, uint32_t n,
    uint32_t nrec, int hbits, CutpathOut o)
{
    const unsigned long long none = sentinel(32 - __clz(nrec) + hbits), hmask = sentinel(hbits);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= nrec; i += gridDim.x * blockDim.x) {
        const unsigned long long key = (unsigned long long)i << hbits;
        uint32_t lo = 0, hi = n; // first entry >= key (the sentinel is above every vertex's)
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (hk[mid] < key) lo = mid + 1; else hi = mid;
        }
        o.ivtx_off[i] = lo;
        if (i == nrec) o.counts[kCpHalfedges] = lo;
    }
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
        if (hk[p] != none) o.ivtx_he[p] = (uint32_t)(hk[p] & hmask);
}

__global__ void k_cp_init(uint32_t* __restrict__ counts, uint32_t* __restrict__ face_off)
{
    if (threadIdx.x < kCpCounts) counts[threadIdx.x] = threadIdx.x == kCpBadKey ? 0xFFFFFFFFu : 0u;
    if (threadIdx.x == 0) face_off[0] = 0;
}

__global__ void k_cp_edges_count(const uint32_t* __restrict__ made, uint32_t n, uint32_t* __restrict__ counts)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) counts[kCpEdges] = made[n];
}

// ---- floating polygons ----
__global__ void __launch_bounds__(kCB) k_fp_init(uint32_t R, FloatingScratch w, unsigned long long none)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < R; v += gridDim.x * blockDim.x) {
        w.parent[v] = v;
        w.flags[v] = 0;
        w.size[v] = 0;
        w.k[0][v] = none;
        w.v[0][v] = v;
    }
}

// parents only ever point to smaller ids, so a find walks down to its root
__device__ __forceinline__ uint32_t fp_find(const uint32_t* parent, uint32_t x)
{
    for (;;) {
        const uint32_t p = *(volatile const uint32_t*)&parent[x];
        if (p == x) return x;
        x = p;
    }
}

// union of each cut-path edge's two vertices: a larger root is hooked under a
// smaller one by compare-and-swap; every failed exchange means another hook
// happened, so the retries are bounded; the cap only guards the loop
__global__ void __launch_bounds__(kCB) k_fp_union(const uint32_t* __restrict__ edges, const uint32_t* __restrict__ counts,
    uint32_t nv, uint32_t* parent, uint32_t* __restrict__ fcounts)
{
    const uint32_t ne = counts[kCpEdges];
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        uint32_t u = fp_find(parent, edges[2 * e] - nv), v = fp_find(parent, edges[2 * e + 1] - nv);
        for (uint32_t tries = 0;; ++tries) {
            if (u == v) break;
            if (tries > 1u << 24) { atomicExch(&fcounts[kFpError], 1u); break; }
            if (u < v) { const uint32_t t = u; u = v; v = t; }
            const uint32_t old = atomicCAS(&parent[u], u, v);
            if (old == u) break;
            u = fp_find(parent, old);
            v = fp_find(parent, v);
        }
    }
}

// every vertex's root; component sizes; a component is not a floating polygon
// when a vertex has other than two edges, lies on a border edge or pierces
// another face than its root
__global__ void __launch_bounds__(kCB) k_fp_flags(CutpathInput in, const uint32_t* __restrict__ ivtx_off,
    FloatingScratch w)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < in.nrec; v += gridDim.x * blockDim.x) {
        const uint32_t deg = ivtx_off[v + 1] - ivtx_off[v];
        if (deg == 0) continue;
        const uint32_t r = fp_find(w.parent, v);
        atomicAdd(&w.size[r], 1u);
        const uint32_t* rv = in.rec_ids + 5 * (size_t)v;
        const bool bad = deg != 2 || rv[4] == kNone || rv[2] != in.rec_ids[5 * (size_t)r + 2];
        if (bad) atomicOr(&w.flags[r], 1u);
    }
}

__global__ void __launch_bounds__(kCB) k_fp_roots(CutpathInput in, const uint32_t* __restrict__ ivtx_off,
    FloatingScratch w, int rbits, uint32_t* __restrict__ fcounts)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < in.nrec; v += gridDim.x * blockDim.x) {
        const bool root = ivtx_off[v + 1] > ivtx_off[v] && w.parent[v] == v && w.flags[v] == 0;
        if (root) {
            w.k[0][v] = ((unsigned long long)in.rec_ids[5 * (size_t)v + 2] << rbits) | v;
            atomicAdd(&fcounts[kFpPolygons], 1u);
        }
    }
}

__global__ void __launch_bounds__(kCB) k_fp_sizes(const unsigned long long* __restrict__ k,
    const uint32_t* __restrict__ roots, uint32_t R, unsigned long long none, const uint32_t* __restrict__ size,
    uint32_t* __restrict__ off)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < R; p += gridDim.x * blockDim.x)
        off[p] = k[p] != none ? size[roots[p]] : 0u;
}

// one thread per polygon: its face, normal, and its cycle from its root
__global__ void __launch_bounds__(kCB) k_fp_walk(CutpathInput in, CutpathOut cp, const unsigned long long* __restrict__ k,
    const uint32_t* __restrict__ roots, unsigned long long none, int rbits, FloatingOut o, const uint32_t* __restrict__ size)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < in.nrec; p += gridDim.x * blockDim.x) {
        if (k[p] == none) continue;
        const uint32_t root = roots[p], face = (uint32_t)(k[p] >> rbits), n = size[root], base = o.off[p];
        o.faces[p] = face;
        double nrm[3] = { 0.0, 0.0, 0.0 };
        int mc = -1;
        cp_plane(in, face, nrm, mc);
        o.normals[3 * (size_t)p] = nrm[0];
        o.normals[3 * (size_t)p + 1] = nrm[1];
        o.normals[3 * (size_t)p + 2] = nrm[2];
        o.mc[p] = mc;
        uint32_t cur = root, prev_e = kNone, i = 0;
        do {
            o.vtx[base + i++] = cur + in.nv;
            const uint32_t b = cp.ivtx_off[cur];
            const uint32_t e0 = cp.ivtx_he[b] >> 1, e1 = cp.ivtx_he[b + 1] >> 1;
            const uint32_t e = e0 == prev_e ? e1 : e0;
            prev_e = e;
            const uint32_t a = cp.edges[2 * (size_t)e] - in.nv, c = cp.edges[2 * (size_t)e + 1] - in.nv;
            cur = a == cur ? c : a;
        } while (cur != root && i < n);
    }
}

__global__ void k_fp_count_init(uint32_t* __restrict__ fcounts)
{
    if (threadIdx.x < kFpCounts) fcounts[threadIdx.x] = 0u;
}

__global__ void k_fp_vertices(const uint32_t* __restrict__ off, uint32_t R, uint32_t* __restrict__ fcounts)
{
    if (threadIdx.x == 0 && blockIdx.x == 0) fcounts[kFpVertices] = off[R];
}

int bits_for(uint64_t n) { return n ? 64 - __builtin_clzll(n) : 1; } // 2^bits > n

int grid(uint64_t n) { return (int)std::max<uint64_t>(1, std::min<uint64_t>((n + kCB - 1) / kCB, 152 * 8)); }

} // namespace

size_t floating_sort_temp_bytes(uint32_t nrec) { return radix_sort_temp_bytes(std::max<uint32_t>(nrec, 1)); }
size_t floating_scan_temp_bytes(uint32_t nrec) { return scan_temp_bytes(std::max<uint32_t>(nrec, 1)); }

void launch_floating(const CutpathInput& in, const CutpathOut& cp, FloatingScratch& w, FloatingOut& o,
    cudaStream_t s)
{
    const uint32_t R = in.nrec;
    g_launches++;
    k_fp_count_init<<<1, 32, 0, s>>>(o.counts);
    if (R == 0) {
        cudaMemsetAsync(o.off, 0, 4, s);
        return;
    }
    const int rbits = bits_for(R), fbits = bits_for(in.nf);
    const unsigned long long none = sentinel(rbits + fbits);
    g_launches += 4;
    k_fp_init<<<grid(R), kCB, 0, s>>>(R, w, none);
    k_fp_union<<<grid(R), kCB, 0, s>>>(cp.edges, cp.counts, in.nv, w.parent, o.counts);
    k_fp_flags<<<grid(R), kCB, 0, s>>>(in, cp.ivtx_off, w);
    k_fp_roots<<<grid(R), kCB, 0, s>>>(in, cp.ivtx_off, w, rbits, o.counts);
    const int b = radix_sort_pairs<unsigned long long>(w.k[0], w.v[0], w.k[1], w.v[1], R, 0, rbits + fbits,
        w.sort_temp, s);
    g_launches += 3;
    k_fp_sizes<<<grid(R), kCB, 0, s>>>(w.k[b], w.v[b], R, none, w.size, o.off);
    exclusive_scan(o.off, R, o.off + R, w.scan_temp, s);
    k_fp_walk<<<grid(R), kCB, 0, s>>>(in, cp, w.k[b], w.v[b], none, rbits, o, w.size);
    k_fp_vertices<<<1, 32, 0, s>>>(o.off, R, o.counts);
}

size_t cutpath_sort_temp_bytes(uint32_t n_candidates)
{
    return radix_sort_temp_bytes(5 * std::max<uint32_t>(n_candidates, 1));
}
size_t cutpath_scan_temp_bytes(uint32_t n_candidates) { return scan_temp_bytes(5 * std::max<uint32_t>(n_candidates, 1)); }

void launch_cutpath(const CutpathInput& in, CutpathScratch& w, CutpathOut& o, cudaStream_t s)
{
    const uint32_t C = in.n_entries - in.n_keys, R = in.nrec;
    g_launches++;
    k_cp_init<<<1, 32, 0, s>>>(o.counts, o.face_off);
    if (R == 0 || in.n_keys == 0) {
        cudaMemsetAsync(o.ivtx_off, 0, 4 * ((size_t)R + 1), s);
        return;
    }
    g_launches++;
    k_cp_candidates<<<grid(in.n_keys), kCB, 0, s>>>(in, w, o.counts);
    if (C == 0) {
        cudaMemsetAsync(o.ivtx_off, 0, 4 * ((size_t)R + 1), s);
        return;
    }
    const int vbits = bits_for((uint64_t)in.nv + R), fbits = bits_for(in.nf), ebits = bits_for(C),
              hbits = bits_for(2ull * C), rbits = bits_for(R);
    g_launches += 2;
    k_cp_filter<<<grid(C), kCB, 0, s>>>(in, w, C, vbits);
    const int pb = radix_sort_pairs<unsigned long long>(w.pk[0], w.pv[0], w.pk[1], w.pv[1], C, 0, 2 * vbits,
        w.sort_temp, s);
    k_cp_first<<<grid(C), kCB, 0, s>>>(w.pk[pb], w.pv[pb], C, vbits, w.made);
    exclusive_scan(w.made, C, w.made + C, w.scan_temp, s);
    g_launches += 2;
    k_cp_edges_count<<<1, 32, 0, s>>>(w.made, C, o.counts);
    k_cp_emit<<<grid(C), kCB, 0, s>>>(in, w, C, fbits, ebits, hbits, o.edges);
    const uint32_t nf5 = 5 * C, nh = 2 * C;
    const int fb = radix_sort_pairs<unsigned long long>(w.fk[0], w.fv[0], w.fk[1], w.fv[1], nf5, 0, fbits + ebits,
        w.sort_temp, s);
    const int hb = radix_sort_pairs<unsigned long long>(w.hk[0], w.hv[0], w.hk[1], w.hv[1], nh, 0, rbits + hbits,
        w.sort_temp, s);
    g_launches += 3;
    k_cp_face_heads<<<grid(nf5), kCB, 0, s>>>(w.fk[fb], nf5, fbits, ebits, w.flags);
    exclusive_scan(w.flags, nf5, w.flags + nf5, w.scan_temp, s);
    k_cp_face_out<<<grid(nf5), kCB, 0, s>>>(w.fk[fb], nf5, fbits, ebits, w.flags, o);
    k_cp_ivtx_out<<<grid(std::max<uint64_t>(nh, (uint64_t)R + 1)), kCB, 0, s>>>(w.hk[hb], nh, R, hbits, o);
}

} // namespace mcgpu
