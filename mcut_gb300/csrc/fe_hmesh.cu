// The halfedge mesh MCUT builds from a caller's arrays, and its input checks,
// on the device: client_input_arrays_to_hmesh (preproc.cpp:57-468, through
// hmesh_t::add_face / add_edge, hmesh.cpp:406-651), check_input_mesh
// (preproc.cpp:505-579) and mesh_is_closed (preproc.cpp:1957-1994).
//
// MCUT adds the faces one by one; every result here is the one that
// sequence gives, computed over all face corners at once:
//   * per-face errors (fewer than 3 corners, an index out of range, an index
//     an earlier corner of the face holds) come from one thread per face;
//   * each undirected edge {a, b} goes into an open-addressing table; the
//     table keeps the lowest corner slot that meets the edge (the corner that
//     creates it in face order) and, per direction, the lowest slot running
//     that way. A slot that is not the lowest of its direction repeats a
//     directed halfedge: its face is non-manifold. The lowest failing face
//     wins, a face's own errors before its non-manifold corner, as MCUT's
//     face-by-face loop reports them;
//   * edge ids are the ranks of the creating slots in slot order (one scan);
//     halfedge 2e runs the creating slot's way, 2e + 1 the other;
//   * next / prev follow the corner order of each face; each vertex lists the
//     halfedges ending at it in ascending id (creation) order;
//   * connected components of the vertex graph: lock-free union-find over
//     the edges (a larger root is hooked under a smaller one with
//     compare-and-swap, so every parent is smaller than its child and every
//     find ends); a vertex no face uses is a component of its own.
#include <cstdint>

#include "fe_hmesh.cuh"
#include "fe_sort.cuh"

namespace mcgpu {

namespace {

constexpr int kHBlock = 256;
constexpr unsigned long long kNoErr = ~0ull;

int hgrid(uint64_t n)
{
    const uint64_t g = (n + kHBlock - 1) / kHBlock;
    return (int)(g < 1 ? 1 : (g > 152 * 8 ? 152 * 8 : g));
}

__device__ __forceinline__ unsigned long long hmix(unsigned long long x)
{
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdULL;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ULL;
    x ^= x >> 33;
    return x;
}

// face of corner slot s, and the slot after s in its face
__device__ __forceinline__ uint32_t hm_face(const HmeshInput& in, const uint32_t* slot_face, uint64_t s)
{
    return in.foff ? slot_face[s] : (uint32_t)(s / 3);
}
__device__ __forceinline__ uint64_t hm_next(const HmeshInput& in, uint32_t f, uint64_t s)
{
    if (!in.foff) return (s % 3 == 2) ? s - 2 : s + 1;
    return s + 1 == in.foff[f + 1] ? in.foff[f] : s + 1;
}
__device__ __forceinline__ uint32_t hm_clamp(const HmeshInput& in, uint32_t v) { return v < in.nv ? v : in.nv; }

// per face: its own errors (preproc.cpp:390-460 checks each face before add_face)
__global__ void __launch_bounds__(kHBlock) k_hm_faces(HmeshInput in, uint32_t* __restrict__ slot_face,
    unsigned long long* __restrict__ err)
{
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < in.nf; f += gridDim.x * blockDim.x) {
        const uint64_t o = in.foff ? in.foff[f] : 3ull * f;
        const uint32_t n = in.foff ? in.foff[f + 1] - (uint32_t)o : 3u;
        if (in.foff)
            for (uint32_t j = 0; j < n; ++j) slot_face[o + j] = f;
        uint32_t code = 0;
        if (n < 3) code = HM_CODE_FACE_SIZE;
        for (uint32_t j = 0; j < n && code == 0; ++j) {
            const uint32_t v = in.idx[o + j];
            if (v >= in.nv) { code = HM_CODE_INDEX_RANGE; break; }
            for (uint32_t k = 0; k < j; ++k)
                if (in.idx[o + k] == v) { code = HM_CODE_DUPLICATE_INDEX; break; }
        }
        if (code) atomicMin(err, ((unsigned long long)f << 3) | code);
    }
}

// every corner slot's edge into the table: lowest slot per edge and per direction
__global__ void __launch_bounds__(kHBlock) k_hm_insert(HmeshInput in, const uint32_t* __restrict__ slot_face,
    HmeshTable t, uint32_t* __restrict__ slot_bucket, unsigned long long* __restrict__ err)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < in.nidx;
         s += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t f = hm_face(in, slot_face, s);
        const uint32_t a = hm_clamp(in, in.idx[s]), b = hm_clamp(in, in.idx[hm_next(in, f, s)]);
        const unsigned long long key = ((((unsigned long long)min(a, b)) << 32) | max(a, b)) + 1ull;
        unsigned long long i = hmix(key) & t.mask;
        // the table holds at least twice as many buckets as slots: a free bucket
        // is always reached; the bound only guards the loop
        uint64_t probes = 0;
        for (;; ++probes) {
            if (probes > t.mask) { atomicMin(err, kNoErr - 1); break; }
            const unsigned long long k = t.key[i];
            if (k == key) break;
            if (k == 0ull) {
                const unsigned long long old = atomicCAS(&t.key[i], 0ull, key);
                if (old == 0ull || old == key) break;
            }
            i = (i + 1) & t.mask;
        }
        if (probes > t.mask) continue;
        slot_bucket[s] = (uint32_t)i;
        atomicMin(&t.first[i], (uint32_t)s);
        atomicMin(&t.dir_first[2 * i + (a > b ? 1u : 0u)], (uint32_t)s);
    }
}

// creating slots (flags for the edge-id scan) and repeated directed halfedges
__global__ void __launch_bounds__(kHBlock) k_hm_flags(HmeshInput in, const uint32_t* __restrict__ slot_face,
    HmeshTable t, const uint32_t* __restrict__ slot_bucket, uint32_t* __restrict__ first_flag,
    unsigned long long* __restrict__ err)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < in.nidx;
         s += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t f = hm_face(in, slot_face, s);
        const uint32_t a = hm_clamp(in, in.idx[s]), b = hm_clamp(in, in.idx[hm_next(in, f, s)]);
        const uint32_t bk = slot_bucket[s];
        first_flag[s] = t.first[bk] == (uint32_t)s ? 1u : 0u;
        if (t.dir_first[2 * bk + (a > b ? 1u : 0u)] != (uint32_t)s)
            atomicMin(err, ((unsigned long long)f << 3) | HM_CODE_NON_MANIFOLD);
    }
}

// halfedge ids of the corners, their faces and the edges' targets
__global__ void __launch_bounds__(kHBlock) k_hm_halfedges(HmeshInput in, const uint32_t* __restrict__ slot_face,
    HmeshTable t, const uint32_t* __restrict__ slot_bucket, const uint32_t* __restrict__ eid, HmeshOut o)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < in.nidx;
         s += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t f = hm_face(in, slot_face, s);
        const uint32_t a = in.idx[s], b = in.idx[hm_next(in, f, s)];
        const uint32_t fs = t.first[slot_bucket[s]];
        const uint32_t e = eid[fs];
        const uint32_t ff = hm_face(in, slot_face, fs);
        const uint32_t fa = in.idx[fs], fb = in.idx[hm_next(in, ff, fs)];
        const uint32_t h = 2 * e + ((a > b) != (fa > fb) ? 1u : 0u);
        o.corner_he[s] = h;
        o.he_face[h] = (int32_t)f;
        if ((uint32_t)s == fs) {
            o.he_target[2 * e] = b;
            o.he_target[2 * e + 1] = a;
        }
    }
}

// next / prev around each face
__global__ void __launch_bounds__(kHBlock) k_hm_links(HmeshInput in, const uint32_t* __restrict__ slot_face, HmeshOut o)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < in.nidx;
         s += (uint64_t)gridDim.x * blockDim.x) {
        const uint32_t f = hm_face(in, slot_face, s);
        const uint32_t h = o.corner_he[s], nh = o.corner_he[hm_next(in, f, s)];
        o.he_next[h] = (int32_t)nh;
        o.he_prev[nh] = (int32_t)h;
    }
}

// halfedges ending at each vertex (counts), and whether some halfedge has no face
__global__ void __launch_bounds__(kHBlock) k_hm_count(uint32_t nhe, HmeshOut o, uint32_t* __restrict__ vcnt,
    uint32_t* __restrict__ border)
{
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < nhe; h += gridDim.x * blockDim.x) {
        atomicAdd(&vcnt[o.he_target[h]], 1u);
        if (o.he_face[h] < 0 && *(volatile uint32_t*)border == 0u) atomicOr(border, 1u);
    }
}

__global__ void __launch_bounds__(kHBlock) k_hm_fill(uint32_t nhe, HmeshOut o, uint32_t* __restrict__ vcur)
{
    for (uint32_t h = blockIdx.x * blockDim.x + threadIdx.x; h < nhe; h += gridDim.x * blockDim.x) {
        const uint32_t v = o.he_target[h];
        o.v_he[o.v_off[v] + atomicAdd(&vcur[v], 1u)] = h;
    }
}

// each vertex's list in ascending halfedge id (lists are short; insertion sort)
__global__ void __launch_bounds__(kHBlock) k_hm_order(uint32_t nv, HmeshOut o)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) {
        const uint32_t lo = o.v_off[v], hi = o.v_off[v + 1];
        for (uint32_t i = lo + 1; i < hi; ++i) {
            const uint32_t x = o.v_he[i];
            uint32_t j = i;
            while (j > lo && o.v_he[j - 1] > x) {
                o.v_he[j] = o.v_he[j - 1];
                --j;
            }
            o.v_he[j] = x;
        }
    }
}

__global__ void __launch_bounds__(kHBlock) k_hm_cc_init(uint32_t nv, uint32_t* __restrict__ parent)
{
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x) parent[v] = v;
}

// parents only ever point to smaller ids, so a find walks down to its root
__device__ __forceinline__ uint32_t cc_find(const uint32_t* parent, uint32_t x)
{
    for (;;) {
        const uint32_t p = *(volatile const uint32_t*)&parent[x];
        if (p == x) return x;
        x = p;
    }
}

__global__ void __launch_bounds__(kHBlock) k_hm_cc_union(uint32_t ne, const uint32_t* __restrict__ he_target,
    uint32_t* parent, unsigned long long* __restrict__ err)
{
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
        uint32_t u = cc_find(parent, he_target[2 * e]), v = cc_find(parent, he_target[2 * e + 1]);
        // each failed exchange means another thread hooked a root: the retries
        // are bounded by the hooks; the cap only guards the loop
        for (uint32_t tries = 0;; ++tries) {
            if (u == v) break;
            if (tries > 1u << 24) { atomicMin(err, kNoErr - 1); break; }
            if (u < v) { const uint32_t w = u; u = v; v = w; }
            const uint32_t old = atomicCAS(&parent[u], u, v);
            if (old == u) break;
            u = cc_find(parent, old);
            v = cc_find(parent, v);
        }
    }
}

__global__ void __launch_bounds__(kHBlock) k_hm_cc_count(uint32_t nv, const uint32_t* __restrict__ parent,
    uint32_t* __restrict__ ncomp)
{
    uint32_t c = 0;
    for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nv; v += gridDim.x * blockDim.x)
        c += parent[v] == v ? 1u : 0u;
    for (int off = 16; off; off >>= 1) c += __shfl_down_sync(0xFFFFFFFFu, c, off);
    if ((threadIdx.x & 31) == 0 && c) atomicAdd(ncomp, c);
}

} // namespace

void launch_hmesh_edges(const HmeshInput& in, HmeshTable& t, HmeshScratch& w, cudaStream_t s)
{
    g_launches += 3;
    k_hm_faces<<<hgrid(in.nf), kHBlock, 0, s>>>(in, w.slot_face, w.err);
    k_hm_insert<<<hgrid(in.nidx), kHBlock, 0, s>>>(in, w.slot_face, t, w.slot_bucket, w.err);
    k_hm_flags<<<hgrid(in.nidx), kHBlock, 0, s>>>(in, w.slot_face, t, w.slot_bucket, w.eid, w.err);
    // edge ids: exclusive scan of the creating-slot flags, the edge count after them
    exclusive_scan(w.eid, (uint32_t)in.nidx, w.counts + kHmEdges, w.scan_temp, s);
}

void launch_hmesh_build(const HmeshInput& in, const HmeshTable& t, HmeshScratch& w, HmeshOut& o, uint32_t ne,
    cudaStream_t s)
{
    const uint32_t nhe = 2 * ne;
    g_launches += 8;
    k_hm_halfedges<<<hgrid(in.nidx), kHBlock, 0, s>>>(in, w.slot_face, t, w.slot_bucket, w.eid, o);
    k_hm_links<<<hgrid(in.nidx), kHBlock, 0, s>>>(in, w.slot_face, o);
    k_hm_count<<<hgrid(nhe), kHBlock, 0, s>>>(nhe, o, o.v_off, w.counts + kHmBorder);
    exclusive_scan(o.v_off, in.nv + 1, nullptr, w.scan_temp, s);
    k_hm_fill<<<hgrid(nhe), kHBlock, 0, s>>>(nhe, o, w.vcur);
    k_hm_order<<<hgrid(in.nv), kHBlock, 0, s>>>(in.nv, o);
    k_hm_cc_init<<<hgrid(in.nv), kHBlock, 0, s>>>(in.nv, w.parent);
    k_hm_cc_union<<<hgrid(ne), kHBlock, 0, s>>>(ne, o.he_target, w.parent, w.err);
    k_hm_cc_count<<<hgrid(in.nv), kHBlock, 0, s>>>(in.nv, w.parent, w.counts + kHmComponents);
}

namespace {
__global__ void __launch_bounds__(kHBlock) k_cw_corners(uint64_t nidx, const uint32_t* __restrict__ corner_he,
    const uint32_t* __restrict__ he_target, const int32_t* __restrict__ he_face, uint32_t* __restrict__ face,
    uint32_t* __restrict__ flag)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s <= nidx; s += (uint64_t)gridDim.x * blockDim.x) {
        if (s == nidx) { flag[s] = 0u; continue; }
        const uint32_t h = corner_he[s];
        face[s] = he_target[h];
        flag[s] = he_face[h ^ 1u] >= 0 ? 1u : 0u;
    }
}

__global__ void __launch_bounds__(kHBlock) k_cw_adjacent(uint64_t nidx, const uint32_t* __restrict__ corner_he,
    const int32_t* __restrict__ he_face, const uint32_t* __restrict__ pos, uint32_t* __restrict__ adj)
{
    for (uint64_t s = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; s < nidx; s += (uint64_t)gridDim.x * blockDim.x) {
        const int32_t f = he_face[corner_he[s] ^ 1u];
        if (f >= 0) adj[pos[s]] = (uint32_t)f;
    }
}

__global__ void __launch_bounds__(kHBlock) k_cw_counts(uint32_t nf, const uint32_t* __restrict__ foff,
    const uint32_t* __restrict__ pos, uint32_t* __restrict__ adj_n)
{
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        const uint64_t a = foff ? foff[f] : 3ull * f, b = foff ? foff[f + 1] : 3ull * f + 3;
        adj_n[f] = pos[b] - pos[a];
    }
}

__global__ void __launch_bounds__(kHBlock) k_to_float(const double* __restrict__ x, uint64_t n, float* __restrict__ out)
{
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = __double2float_rn(x[i]);
}
} // namespace

size_t cc_wire_scan_bytes(uint64_t nidx) { return scan_temp_bytes((uint32_t)(nidx + 1)); }

void launch_cc_wire(const HmeshOut& o, const uint32_t* foff, uint32_t nf, uint64_t nidx, CcWireOut& w,
    uint32_t* scan_temp, uint32_t* total, cudaStream_t s)
{
    g_launches += 3;
    k_cw_corners<<<hgrid(nidx + 1), kHBlock, 0, s>>>(nidx, o.corner_he, o.he_target, o.he_face, w.face, w.pos);
    exclusive_scan(w.pos, (uint32_t)(nidx + 1), total, scan_temp, s);
    k_cw_adjacent<<<hgrid(nidx), kHBlock, 0, s>>>(nidx, o.corner_he, o.he_face, w.pos, w.adj);
    k_cw_counts<<<hgrid(nf), kHBlock, 0, s>>>(nf, foff, w.pos, w.adj_n);
}

void launch_to_float(const double* x, uint64_t n, float* out, cudaStream_t s)
{
    g_launches++;
    k_to_float<<<hgrid(n), kHBlock, 0, s>>>(x, n, out);
}

} // namespace mcgpu
