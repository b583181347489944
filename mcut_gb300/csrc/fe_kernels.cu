// Kernels of the GB300 intersection front end.
//
// Stage map (reference function -> kernel):
//   bvh.cpp:242-433  face boxes, mesh box, Morton codes   -> k_vertex_bounds, k_mesh_frames, k_face_bounds
//   bvh.cpp:437-442  std::sort by Morton code             -> radix_sort_pairs (fe_sort.cu)
//   bvh.cpp:444-635  implicit-tree build + refit          -> k_build (LBVH, built bottom-up with its boxes)
//   bvh.cpp:638-783  intersectOIBVHs                       -> k_traverse
//   kernel.cpp:1781-2177 edge->faces, edge boxes, culling -> k_pair_tests
//   kernel.cpp:2184-2356 tested-face planes               -> k_planes, k_triplets
//   kernel.cpp:2456-2658 narrow phase + records           -> k_narrow, k_gather_records
//
// The candidate-pair set does not depend on the tree's shape: internal boxes
// only prune, and every leaf-leaf test is the reference's exact closed fp64
// test. So the tree is a Karras LBVH with fp32 node boxes rounded outward,
// not the reference's implicit complete tree.

#include <climits>
#include <cstddef>
#include <cstdlib>
#include <cstring>

#include "fe_common.cuh"
#include "fe_kernels.cuh"
#include "fe_sort.cuh"

namespace mcgpu {

namespace {

constexpr int kBlock = 256;

// vertex v of the dispatch (two segments when the caller's arrays are read in place)
// ps face-vertex entry k as the bounds kernel reads it: a single pair's cut
// entries come from the caller's (or the uploaded) raw cut indices, offset
// by the source vertex count on the fly (fidx_cut != null); the bounds kernel
// writes the global table every later kernel reads directly
__device__ __forceinline__ uint32_t fidx_at(const Problem& P, uint64_t k)
{
    if (P.fidx_cut && k >= P.fidx_split) return P.fidx_cut[k - P.fidx_split] + P.cut_vbase;
    return P.fidx[k];
}
// pair id | kCutBit of ps face f (one pair without a table: cut faces from face_split on)
__device__ __forceinline__ uint32_t face_pair_of(const Problem& P, uint32_t f)
{
    if (!P.face_pair) return f >= P.face_split ? kCutBit : 0u;
    return P.face_pair[f];
}

__device__ __forceinline__ void load_v(const Problem& P, uint32_t v, double* x)
{
    if (v < P.xsplit) load_xyz(P.X, v, x);
    else load_xyz(P.Xc, v - P.xsplit, x);
}

__device__ __forceinline__ uint32_t face_n(const Problem& P, uint32_t f)
{
    return P.all_triangles ? 3u : (P.foff[f + 1] - P.foff[f]);
}
__device__ __forceinline__ uint32_t face_o(const Problem& P, uint32_t f)
{
    return P.all_triangles ? 3u * f : P.foff[f];
}

// warp-aggregated append: returns the slot for this thread's item
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want)
{
    const unsigned act = __activemask();
    const unsigned m = __ballot_sync(act, want);
    if (!want) return 0;
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(counter, (uint32_t)__popc(m));
    base = __shfl_sync(m, base, leader);
    return base + __popc(m & ((1u << lane) - 1u));
}

// Adds v[k] to cnt[5 p + f0 + k] for each distinct pair id p among the warp's
// lanes, one atomic per pair and value (lanes with p == kNone add nothing).
// All 32 lanes call it.
template <int K>
__device__ __forceinline__ void pair_add(uint32_t* cnt, uint32_t p, int f0, const uint32_t (&v)[K])
{
    const unsigned full = 0xFFFFFFFFu;
    const int lane = threadIdx.x & 31;
    unsigned todo = __ballot_sync(full, p != kNone);
    while (todo) {
        const int leader = __ffs(todo) - 1;
        const uint32_t lp = __shfl_sync(full, p, leader);
        const bool mine = p == lp;
        todo &= ~__ballot_sync(full, mine);
#pragma unroll
        for (int k = 0; k < K; ++k) {
            const uint32_t x = __reduce_add_sync(full, mine ? v[k] : 0u);
            if (lane == leader && x) atomicAdd(&cnt[(size_t)lp * 5 + f0 + k], x);
        }
    }
}

// ---------------------------------------------------------------------------
// face boxes + per-mesh boxes (bvh.cpp:242-368)
// ---------------------------------------------------------------------------
__device__ __forceinline__ void mesh_box_flush(unsigned long long* __restrict__ mesh_box, uint32_t key,
    const unsigned long long* lo, const unsigned long long* hi)
{
    unsigned long long* mb = mesh_box + (size_t)key * 6;
    for (int j = 0; j < 3; ++j) {
        atomicMin(&mb[j], lo[j]);
        atomicMax(&mb[3 + j], hi[j]);
    }
}

constexpr int kBoundsItems = 8; // vertices per thread per tile; a tile is kBlock * kBoundsItems consecutive vertices

__device__ __forceinline__ uint32_t expand_bits(uint32_t v)
{
    v = (v * 0x00010001u) & 0xFF0000FFu;
    v = (v * 0x00000101u) & 0x0F00F00Fu;
    v = (v * 0x00000011u) & 0xC30C30C3u;
    v = (v * 0x00000005u) & 0x49249249u;
    return v;
}

// Mesh boxes (the union of each mesh's vertices; they only steer the Morton
// codes, so a vertex no face uses may widen them harmlessly). Tiles are runs
// of consecutive vertices, almost always of one mesh: each thread folds in
// registers, the block folds in shared memory, one thread issues the
// atomics; a tile that straddles meshes falls back to per-thread atomics.
__global__ void __launch_bounds__(kBlock) k_vertex_bounds(Problem P, unsigned long long* __restrict__ mesh_box,
    float4* __restrict__ x32, const double* __restrict__ hx_src, const double* __restrict__ hx_cut,
    double* __restrict__ hx_out, const void* __restrict__ x_raw, int raw_float, const double* __restrict__ frames)
{
    __shared__ unsigned long long red[kBlock / 32][6];
    __shared__ uint32_t skey;
    const uint32_t tiles = (P.nv + kBlock * kBoundsItems - 1) / (kBlock * kBoundsItems);
    for (uint32_t tile = blockIdx.x; tile < tiles; tile += gridDim.x) {
        uint32_t key = kNone, p = 0;
        bool mixed = false;
        unsigned long long lo[3] = { ~0ull, ~0ull, ~0ull }, hi[3] = { 0ull, 0ull, 0ull };
        for (int it = 0; it < kBoundsItems; ++it) {
            const uint32_t v = tile * (kBlock * kBoundsItems) + it * kBlock + threadIdx.x;
            if (v >= P.nv) break;
            if (it == 0) { // the pair of the thread's first vertex, then a forward walk
                uint32_t l = 0, h = P.n_pairs;
                while (h - l > 1) {
                    const uint32_t mid = (l + h) >> 1;
                    if (P.pair_vbase[mid] <= v) l = mid; else h = mid;
                }
                p = l;
            }
            while (v >= P.pair_vbase[p + 1]) ++p;
            const uint32_t k = p * 2 + ((v - P.pair_vbase[p]) >= P.pair_vs[p] ? 1u : 0u);
            double x[3];
            if (hx_src) {
                // one pair from host arrays: read over the host link, kept on the device
                const uint32_t vs = P.pair_vs[0];
                const double* h = v < vs ? hx_src + 3 * (size_t)v : hx_cut + 3 * (size_t)(v - vs);
                x[0] = h[0];
                x[1] = h[1];
                x[2] = h[2];
                hx_out[3 * (size_t)v] = x[0];
                hx_out[3 * (size_t)v + 1] = x[1];
                hx_out[3 * (size_t)v + 2] = x[2];
            } else if (x_raw) {
                // user coordinates into the pair's frame, x' = (x - com) + t per
                // coordinate, in the input's precision (preproc.cpp:147-181)
                const double* fr = frames + 6 * (size_t)p;
                if (raw_float) {
                    const float* r = static_cast<const float*>(x_raw) + 3 * (size_t)v;
                    for (int j = 0; j < 3; ++j)
                        x[j] = (double)__fadd_rn(__fsub_rn(r[j], __double2float_rn(fr[j])), __double2float_rn(fr[3 + j]));
                } else {
                    const double* r = static_cast<const double*>(x_raw) + 3 * (size_t)v;
                    for (int j = 0; j < 3; ++j) x[j] = __dadd_rn(__dsub_rn(r[j], fr[j]), fr[3 + j]);
                }
                hx_out[3 * (size_t)v] = x[0];
                hx_out[3 * (size_t)v + 1] = x[1];
                hx_out[3 * (size_t)v + 2] = x[2];
            } else {
                load_v(P, v, x);
            }
            // the vertex's fp32 copy for orient3d's first filter
            if (x32) x32[v] = make_float4(f32_vertex_coord(x[0]), f32_vertex_coord(x[1]), f32_vertex_coord(x[2]), 0.0f);
            if (key != kNone && k != key) {
                mesh_box_flush(mesh_box, key, lo, hi);
                for (int j = 0; j < 3; ++j) { lo[j] = ~0ull; hi[j] = 0ull; }
                mixed = true;
            }
            key = k;
            for (int j = 0; j < 3; ++j) {
                lo[j] = min(lo[j], ord_of(x[j]));
                hi[j] = max(hi[j], ord_of(x[j]));
            }
        }
        if (threadIdx.x == 0) skey = key;
        __syncthreads();
        const uint32_t k0 = skey;
        const bool uniform = __syncthreads_and(!mixed && (key == k0 || key == kNone)) && k0 != kNone;
        if (uniform) {
            const unsigned full = 0xFFFFFFFFu;
            for (int off = 16; off; off >>= 1)
                for (int j = 0; j < 3; ++j) {
                    lo[j] = min(lo[j], __shfl_xor_sync(full, lo[j], off));
                    hi[j] = max(hi[j], __shfl_xor_sync(full, hi[j], off));
                }
            if ((threadIdx.x & 31) == 0)
                for (int j = 0; j < 3; ++j) { red[threadIdx.x >> 5][j] = lo[j]; red[threadIdx.x >> 5][3 + j] = hi[j]; }
            __syncthreads();
            if (threadIdx.x == 0) {
                for (int w = 1; w < kBlock / 32; ++w)
                    for (int j = 0; j < 3; ++j) {
                        lo[j] = min(lo[j], red[w][j]);
                        hi[j] = max(hi[j], red[w][3 + j]);
                    }
                mesh_box_flush(mesh_box, k0, lo, hi);
            }
        } else if (key != kNone) {
            mesh_box_flush(mesh_box, key, lo, hi);
        }
        __syncthreads();
    }
}

// Per mesh: the fp32 frame the Morton codes are quantised in -- the mesh
// box rounded outward, and 1023 / extent per axis (0 for a flat axis).
__global__ void k_mesh_frames(const unsigned long long* __restrict__ mesh_box, uint32_t nmesh,
    float4* __restrict__ frame)
{
    for (uint32_t m = blockIdx.x * blockDim.x + threadIdx.x; m < nmesh; m += gridDim.x * blockDim.x) {
        const unsigned long long* mb = mesh_box + (size_t)m * 6;
        float lo[3], sc[3];
        for (int j = 0; j < 3; ++j) {
            lo[j] = f32_rd(of_ord(mb[j]));
            const float ext = f32_ru(of_ord(mb[3 + j])) - lo[j];
            sc[j] = ext > 0.0f ? __fdiv_rn(1023.0f, ext) : 0.0f;
        }
        frame[2 * m] = make_float4(lo[0], lo[1], lo[2], 0.0f);
        frame[2 * m + 1] = make_float4(sc[0], sc[1], sc[2], 0.0f);
    }
}

// Morton code of a box centre already in frame units (0 .. 1023 across the
// mesh box): 8, 8 and 7 bits per axis (or 10 each with 30-bit codes)
__device__ __forceinline__ uint32_t morton_code(float c0, float c1, float c2)
{
    constexpr float top = kMortonBits == 30 ? 1023.0f : 255.0f, scale = kMortonBits == 30 ? 1.0f : 0.25f;
    const uint32_t m0 = expand_bits((uint32_t)fminf(fmaxf(c0 * scale, 0.0f), top));
    const uint32_t m1 = expand_bits((uint32_t)fminf(fmaxf(c1 * scale, 0.0f), top));
    const uint32_t m2 = expand_bits((uint32_t)fminf(fmaxf(c2 * scale, 0.0f), top));
    return kMortonBits == 30 ? m0 * 4 + m1 * 2 + m2 : (m0 * 4 + m1 * 2 + m2) >> 1;
}

// Face boxes (bvh.cpp:242-314, cut boxes enlarged as preproc.cpp:2693) and
// each face's Morton key (bvh.cpp:370-433). The code only orders leaves --
// any order gives the same pair set -- so it is formed in fp32 from the
// outward-rounded box: centre relative to the mesh frame, 8, 8 and 7 bits;
// the mesh bit above the key puts every source key before every cut key so
// one sort orders both meshes.
template <typename K>
__global__ void __launch_bounds__(kBlock) k_face_bounds(Problem P, double* __restrict__ fbox,
    float* __restrict__ fbox32, const float4* __restrict__ frame, K* __restrict__ skey, uint32_t* __restrict__ sval,
    K* __restrict__ ckey, uint32_t* __restrict__ cval, int mesh_bit, uint32_t* __restrict__ pair_status,
    uint8_t* __restrict__ cand, uint32_t* __restrict__ fidx_out, uint32_t* __restrict__ face_pair_out,
    uint32_t* fidx_fix)
{
    // triangles: the next face's indices are requested before this face's
    // work, so their latency (over the host link when the indices are the
    // caller's host arrays) overlaps it
    const uint32_t stride = gridDim.x * blockDim.x;
    uint32_t nidx[3] = { 0u, 0u, 0u };
    const uint32_t f0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (P.all_triangles && f0 < P.nf)
        for (int k = 0; k < 3; ++k) nidx[k] = fidx_at(P, 3ull * f0 + k);
    for (uint32_t f = f0; f < P.nf; f += stride) {
        uint32_t cidx[3] = { nidx[0], nidx[1], nidx[2] };
        if (P.all_triangles && f + stride < P.nf && f + stride > f)
            for (int k = 0; k < 3; ++k) nidx[k] = fidx_at(P, 3ull * (f + stride) + k);
        cand[f] = 0; // no candidate pair yet (the traversal sets it)
        const uint32_t fp = face_pair_of(P, f);
        if (face_pair_out) face_pair_out[f] = fp;
        const uint32_t p = fp & ~kCutBit;
        const bool is_cut = (fp & kCutBit) != 0;
        const uint32_t o = face_o(P, f), n = face_n(P, f);
        // an index must name a vertex of the face's own mesh (preproc.cpp:390-460
        // checks each mesh's indices against its own vertex count); a cut index
        // that wrapped when offset by the source count lands below this range
        const uint32_t vmid = P.pair_vbase[p] + P.pair_vs[p];
        const uint32_t vlo = is_cut ? vmid : P.pair_vbase[p], vhi = is_cut ? P.pair_vbase[p + 1] : vmid;
        // std::min / std::max folds from +-DBL_MAX in vertex order: each
        // running extreme is kept with its dkey(), so a step converts only
        // the new coordinate; a strict compare keeps the first of equal keys,
        // as the reference's fold does
        Box b;
        long long kmn[3], kmx[3];
        for (int j = 0; j < 3; ++j) {
            b.mn[j] = 1.7976931348623157e308;
            b.mx[j] = -1.7976931348623157e308;
            kmn[j] = dkey(b.mn[j]);
            kmx[j] = dkey(b.mx[j]);
        }
        bool bad = false;
        for (uint32_t k = 0; k < n; ++k) {
            uint32_t v = P.all_triangles ? cidx[k < 3 ? k : 0] : fidx_at(P, o + k);
            if (v < vlo || v >= vhi) {
                // the pair's outcome is MCGPU_INVALID_INPUT; every later kernel
                // reads the index table, so it gets the mesh's first vertex in place
                // of the bad index and no access leaves the vertex array
                bad = true;
                v = vlo;
                if (fidx_fix) fidx_fix[o + k] = v;
            }
            if (fidx_out) fidx_out[o + k] = v;
            double x[3];
            load_v(P, v, x);
            for (int j = 0; j < 3; ++j) {
                const long long kx = dkey(x[j]);
                if (kmx[j] < kx) { kmx[j] = kx; b.mx[j] = x[j]; }
                if (kx < kmn[j]) { kmn[j] = kx; b.mn[j] = x[j]; }
            }
        }
        if (bad) atomicOr(&pair_status[p], ST_INVALID);
        if (is_cut) {
            const double eps = P.pair_eps[p];
            if (eps > 0.0)
                for (int j = 0; j < 3; ++j) { b.mx[j] = b.mx[j] + eps; b.mn[j] = b.mn[j] - eps; }
        }
        double2* d = reinterpret_cast<double2*>(fbox + (size_t)f * 6);
        d[0] = make_double2(b.mn[0], b.mn[1]);
        d[1] = make_double2(b.mn[2], b.mx[0]);
        d[2] = make_double2(b.mx[1], b.mx[2]);
        float lo[3], hi[3];
        for (int j = 0; j < 3; ++j) { lo[j] = f32_rd(b.mn[j]); hi[j] = f32_ru(b.mx[j]); }
        float2* d32 = reinterpret_cast<float2*>(fbox32 + (size_t)f * 6);
        d32[0] = make_float2(lo[0], lo[1]);
        d32[1] = make_float2(lo[2], hi[0]);
        d32[2] = make_float2(hi[1], hi[2]);
        const uint32_t m = p * 2 + (is_cut ? 1u : 0u);
        const float4 fl = __ldg(&frame[2 * m]), fs = __ldg(&frame[2 * m + 1]);
        const float c0 = (0.5f * (lo[0] + hi[0]) - fl.x) * fs.x;
        const float c1 = (0.5f * (lo[1] + hi[1]) - fl.y) * fs.y;
        const float c2 = (0.5f * (lo[2] + hi[2]) - fl.z) * fs.z;
        const K key = ((K)p << kMortonBits) | (K)morton_code(c0, c1, c2) | ((K)(is_cut ? 1 : 0) << mesh_bit);
        const uint32_t local = f - P.pair_fbase[p];
        if (is_cut) {
            // a resident cut tree's faces stay out of the batch's sort and tree
            if (!P.res_pairs || P.res_pairs[p].ncl == 0) {
                const uint32_t pos = P.pair_cbase[p] + (local - P.pair_fs[p]);
                ckey[pos] = key;
                cval[pos] = f;
            }
        } else {
            const uint32_t pos = P.pair_sbase[p] + local;
            skey[pos] = key;
            sval[pos] = f;
        }
    }
}


// Morton code of the box centre in its mesh's box (morton3D, bvh.cpp:196-217),
// written to the source-face or cut-face key list.
// ---------------------------------------------------------------------------
// Karras (HPG 2012) hierarchy over the sorted cut-face keys; duplicate keys
// are ordered by position.
// ---------------------------------------------------------------------------
template <typename K>
__device__ __forceinline__ int delta(const K* __restrict__ key, int n, int i, int j)
{
    if (j < 0 || j >= n) return -1;
    const K a = key[i], b = key[j];
    if (a == b) return 8 * (int)sizeof(K) + __clz((unsigned)(i ^ j));
    if (sizeof(K) == 8) return __clzll((long long)((unsigned long long)a ^ (unsigned long long)b));
    return __clz((unsigned)((uint32_t)a ^ (uint32_t)b));
}

// Query packets: the source faces are Morton-sorted too, and every Karras
// subtree over them is a run of consecutive sorted faces split at a Morton
// cell boundary, hence spatially compact. A packet is a maximal subtree of at
// most 32 faces (its parent holds more); one warp walks the cut tree for it.
template <typename K>
__global__ void __launch_bounds__(kBlock) k_src_packets(const K* __restrict__ key, int n, uint2* __restrict__ packets,
    uint32_t* __restrict__ counters, int pmax)
{
    if (n <= pmax) {
        if (blockIdx.x == 0 && threadIdx.x == 0 && n > 0) {
            packets[0] = make_uint2(0u, (uint32_t)(n - 1));
            counters[9] = 1;
        }
        return;
    }
    for (int i0 = blockIdx.x * blockDim.x; i0 < n - 1; i0 += gridDim.x * blockDim.x) {
        const int i = i0 + threadIdx.x;
        bool emit0 = false, emit1 = false;
        int gamma = 0, lo = 0, hi = 0;
        if (i < n - 1) {
        const int d = (delta(key, n, i, i + 1) - delta(key, n, i, i - 1)) >= 0 ? 1 : -1;
        const int dmin = delta(key, n, i, i - d);
        int lmax = 2;
        while (delta(key, n, i, i + lmax * d) > dmin) lmax <<= 1;
        int l = 0;
        for (int t = lmax >> 1; t >= 1; t >>= 1)
            if (delta(key, n, i, i + (l + t) * d) > dmin) l += t;
        const int j = i + l * d;
        lo = min(i, j);
        hi = max(i, j);
        if (hi - lo + 1 > pmax) {
            const int dnode = delta(key, n, i, j);
            int s = 0;
            for (int t = (l + 1) >> 1;; t = (t + 1) >> 1) {
                if (delta(key, n, i, i + (s + t) * d) > dnode) s += t;
                if (t == 1) break;
            }
            gamma = i + s * d + min(d, 0);
            emit0 = gamma - lo + 1 <= pmax;
            emit1 = hi - gamma <= pmax;
        }
        }
        const uint32_t p0 = warp_append(&counters[9], emit0);
        if (emit0) packets[p0] = make_uint2((uint32_t)lo, (uint32_t)gamma);
        const uint32_t p1 = warp_append(&counters[9], emit1);
        if (emit1) packets[p1] = make_uint2((uint32_t)(gamma + 1), (uint32_t)hi);
    }
}

// a face's fp64 box as dkey() integers: (mn0,mn1) (mn2,mx0) (mx1,mx2)
__device__ __forceinline__ void load_key_box(const double* __restrict__ fbox, uint32_t f, longlong2& a, longlong2& b,
    longlong2& c)
{
    const Box x = load_box(fbox, f);
    a = make_longlong2(dkey(x.mn[0]), dkey(x.mn[1]));
    b = make_longlong2(dkey(x.mn[2]), dkey(x.mx[0]));
    c = make_longlong2(dkey(x.mx[1]), dkey(x.mx[2]));
}

// leaf clusters: `leaf_size` consecutive sorted cut faces of one pair
template <typename K>
__global__ void __launch_bounds__(kBlock) k_clusters(Problem P, const K* __restrict__ ckey, K* __restrict__ clkey,
    uint32_t* __restrict__ cl_start, uint8_t* __restrict__ cl_n, uint32_t* __restrict__ split_far)
{
    for (uint32_t c = blockIdx.x * blockDim.x + threadIdx.x; c < P.ncl; c += gridDim.x * blockDim.x) {
        if (c + 1 < P.ncl) split_far[c] = 0xFFFFFFFFu; // no child has reached split c yet (the tree build)
        uint32_t lo = 0, hi = P.n_pairs;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (P.pair_clbase[mid] <= c) lo = mid; else hi = mid;
        }
        const uint32_t start = P.pair_cbase[lo] + (c - P.pair_clbase[lo]) * P.leaf_size;
        const uint32_t end = min(start + P.leaf_size, P.pair_cbase[lo + 1]);
        clkey[c] = ckey[start];
        cl_start[c] = start;
        cl_n[c] = (uint8_t)(end - start);
    }
}

struct FBox { float lo[3], hi[3]; uint32_t plo, phi; };

// Bottom-up build of the binary radix tree over the sorted leaf clusters,
// boxes included (agglomerative LBVH, Apetrei, EG 2014). D(j), the boundary
// between sorted clusters j and j+1, is the XOR of their keys with the XOR of
// the positions below it (distinct keys, duplicates ordered by position, as
// the Karras construction orders them). The tree is the Cartesian tree of D:
// a node [l, r] is the left child of its parent when D(r) < D(l-1), and
// splits at its largest inner boundary. Every leaf thread climbs: at the
// parent's split position s the first child to arrive deposits its box and
// far end and stops; the second builds the parent. Nodes keep the Karras
// numbering (a left child is numbered by its right end, a right child by its
// left end, the root is 0), so the walk is unchanged.
//
// Block b owns clusters [W b, W (b+1)), W = kRefitWin. A split whose node lies
// inside the window -- D(s) is below some boundary on each side within the
// window, found by prefix and suffix maxima -- is exchanged through shared
// memory: the climb through a window touches no global memory. Splits whose
// node leaves the window use global acquire-release exchanges.
#ifndef MCGPU_REFIT_WIN
#define MCGPU_REFIT_WIN 128
#endif
constexpr int kRefitWin = MCGPU_REFIT_WIN;
constexpr uint32_t kNoFar = 0xFFFFFFFFu;

// D for 32-bit keys: key XOR above position XOR in one 64-bit word; for
// 64-bit keys the pair compared lexicographically
struct Dlt { unsigned long long x; uint32_t i; };
__device__ __forceinline__ bool dlt_less(const Dlt& a, const Dlt& b)
{
    return a.x < b.x || (a.x == b.x && a.i < b.i);
}
__device__ __forceinline__ bool dlt_less(unsigned long long a, unsigned long long b) { return a < b; }
__device__ __forceinline__ unsigned long long dlt_make(uint32_t a, uint32_t b, int j)
{
    return ((unsigned long long)(a ^ b) << 32) | (uint32_t)(j ^ (j + 1));
}
__device__ __forceinline__ Dlt dlt_make(unsigned long long a, unsigned long long b, int j)
{
    return Dlt { a ^ b, (uint32_t)(j ^ (j + 1)) };
}
template <typename T> __device__ __forceinline__ T dlt_top();
template <> __device__ __forceinline__ unsigned long long dlt_top<unsigned long long>() { return ~0ull; }
template <> __device__ __forceinline__ Dlt dlt_top<Dlt>() { return Dlt { ~0ull, ~0u }; }
template <typename T> __device__ __forceinline__ T dlt_bottom();
template <> __device__ __forceinline__ unsigned long long dlt_bottom<unsigned long long>() { return 0ull; }
template <> __device__ __forceinline__ Dlt dlt_bottom<Dlt>() { return Dlt { 0ull, 0u }; }
__device__ __forceinline__ unsigned long long dlt_shfl_up(unsigned long long d, int o)
{
    return __shfl_up_sync(0xFFFFFFFFu, d, o);
}
__device__ __forceinline__ unsigned long long dlt_shfl_down(unsigned long long d, int o)
{
    return __shfl_down_sync(0xFFFFFFFFu, d, o);
}
__device__ __forceinline__ Dlt dlt_shfl_up(const Dlt& d, int o)
{
    return Dlt { __shfl_up_sync(0xFFFFFFFFu, d.x, o), __shfl_up_sync(0xFFFFFFFFu, d.i, o) };
}
__device__ __forceinline__ Dlt dlt_shfl_down(const Dlt& d, int o)
{
    return Dlt { __shfl_down_sync(0xFFFFFFFFu, d.x, o), __shfl_down_sync(0xFFFFFFFFu, d.i, o) };
}
template <typename K>
using DltOf = decltype(dlt_make(K(), K(), 0));
// D(j); the mesh ends (j = -1, j = n-1) are above every boundary
template <typename K>
__device__ __forceinline__ DltOf<K> boundary_delta(const K* __restrict__ key, int n, int j)
{
    if (j < 0 || j >= n - 1) return dlt_top<DltOf<K>>();
    return dlt_make(__ldg(&key[j]), __ldg(&key[j + 1]), j);
}
__device__ __forceinline__ void store_fbox(FBox* p, const FBox& b)
{
    float4* q = reinterpret_cast<float4*>(p);
    q[0] = make_float4(b.lo[0], b.lo[1], b.lo[2], b.hi[0]);
    q[1] = make_float4(b.hi[1], b.hi[2], __uint_as_float(b.plo), __uint_as_float(b.phi));
}
__device__ __forceinline__ FBox load_fbox_cg(const FBox* p)
{
    const float4 a = __ldcg(reinterpret_cast<const float4*>(p)), c = __ldcg(reinterpret_cast<const float4*>(p) + 1);
    FBox b;
    b.lo[0] = a.x; b.lo[1] = a.y; b.lo[2] = a.z; b.hi[0] = a.w;
    b.hi[1] = c.x; b.hi[2] = c.y; b.plo = __float_as_uint(c.z); b.phi = __float_as_uint(c.w);
    return b;
}

template <typename K>
__global__ void __launch_bounds__(kRefitWin) k_build(Problem P, const K* __restrict__ key, int n,
    const float* __restrict__ fbox32, const uint32_t* __restrict__ leaf_face, const uint32_t* __restrict__ cl_start,
    const uint8_t* __restrict__ cl_n, Node* __restrict__ nodes, uint32_t* __restrict__ split_far,
    FBox* __restrict__ split_box, int32_t* __restrict__ pair_root)
{
    using D = DltOf<K>;
    constexpr int kW = kRefitWin / 32;
    __shared__ D sd[kRefitWin + 1];  // sd[t] = D(w0 - 1 + t)
    __shared__ D wagg[2][kW];
    __shared__ uint32_t sfar[kRefitWin];
    __shared__ uint8_t sinw[kRefitWin];
    __shared__ FBox sbox[kRefitWin][2];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int w0 = blockIdx.x * kRefitWin, w1 = min(n, w0 + kRefitWin) - 1;
    const int i = w0 + t;
    const bool valid = i <= w1;
    const D lowest = dlt_bottom<D>(); // below every boundary (a boundary's position XOR is >= 1)
    const D dm = valid ? boundary_delta(key, n, i) : lowest;
    sd[t + 1] = dm;
    if (t == 0) sd[0] = boundary_delta(key, n, w0 - 1);
    sfar[t] = kNoFar;
    // inclusive max-scans of D over the window, from the left and from the right
    D pre = dm, suf = dm;
    for (int o = 1; o < 32; o <<= 1) {
        const D a = dlt_shfl_up(pre, o), b = dlt_shfl_down(suf, o);
        if (lane >= o && dlt_less(pre, a)) pre = a;
        if (lane + o < 32 && dlt_less(suf, b)) suf = b;
    }
    if (lane == 31) wagg[0][warp] = pre;
    if (lane == 0) wagg[1][warp] = suf;
    D epre = dlt_shfl_up(pre, 1), esuf = dlt_shfl_down(suf, 1);
    __syncthreads();
    if (lane == 0) epre = sd[0];
    else if (dlt_less(epre, sd[0])) epre = sd[0];
    if (lane == 31) esuf = lowest;
    for (int w = 0; w < warp; ++w)
        if (dlt_less(epre, wagg[0][w])) epre = wagg[0][w];
    for (int w = warp + 1; w < kW; ++w)
        if (dlt_less(esuf, wagg[1][w])) esuf = wagg[1][w];
    // split i closes inside the window: a larger boundary on each side of it
    sinw[t] = (valid && i < w1 && dlt_less(dm, epre) && dlt_less(dm, esuf)) ? 1 : 0;
    __syncthreads();
    if (!valid) return;

    FBox fb;
    for (int j = 0; j < 3; ++j) { fb.lo[j] = 3.4e38f; fb.hi[j] = -3.4e38f; }
    {
        const uint32_t s0 = cl_start[i], cn = cl_n[i];
        const uint32_t f0 = __ldg(&leaf_face[s0]);
        fb.plo = fb.phi = face_pair_of(P, f0) & ~kCutBit;
        // four faces at a time, their loads in flight together
        for (uint32_t c0 = 0; c0 < cn; c0 += 4) {
            uint32_t lf[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) lf[u] = c0 + u < cn ? __ldg(&leaf_face[s0 + c0 + u]) : f0;
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const float2* b = reinterpret_cast<const float2*>(fbox32 + (size_t)lf[u] * 6);
                const float2 x = __ldg(b), y = __ldg(b + 1), z = __ldg(b + 2);
                fb.lo[0] = fminf(fb.lo[0], x.x); fb.lo[1] = fminf(fb.lo[1], x.y); fb.lo[2] = fminf(fb.lo[2], y.x);
                fb.hi[0] = fmaxf(fb.hi[0], y.y); fb.hi[1] = fmaxf(fb.hi[1], z.x); fb.hi[2] = fmaxf(fb.hi[2], z.y);
            }
        }
    }
    int l = i, r = i;
    D dl = sd[t], dr = sd[t + 1]; // D(l-1), D(r)
    for (;;) {
        const bool right = dlt_less(dr, dl); // the parent extends to the right: this node is its left child
        const int s = right ? r : l - 1;
        const int slot = right ? 0 : 1;
        const uint32_t far = (uint32_t)(right ? l : r);
        uint32_t prev;
        FBox o;
        const int ks = s - w0;
        if (ks >= 0 && ks < kRefitWin && sinw[ks]) {
            sbox[ks][slot] = fb;
            __threadfence_block();
            prev = atomicExch(&sfar[ks], far);
            __threadfence_block();
            if (prev == kNoFar) return;
            o = sbox[ks][slot ^ 1];
        } else {
            store_fbox(&split_box[2 * (size_t)s + slot], fb);
            // acq_rel exchange: releases this child's box, acquires the sibling's
            asm volatile("atom.exch.acq_rel.gpu.b32 %0, [%1], %2;" : "=r"(prev) : "l"(split_far + s), "r"(far) : "memory");
            if (prev == kNoFar) return;
            o = load_fbox_cg(&split_box[2 * (size_t)s + (slot ^ 1)]);
        }
        const int pl = right ? l : (int)prev, pr = right ? (int)prev : r;
        const D pdl = (pl >= w0 && pl <= w1 + 1) ? sd[pl - w0] : boundary_delta(key, n, pl - 1);
        const D pdr = (pr >= w0 - 1 && pr <= w1) ? sd[pr - w0 + 1] : boundary_delta(key, n, pr);
        const bool root = pl == 0 && pr == n - 1;
        const int pidx = root ? 0 : (dlt_less(pdr, pdl) ? pr : pl);
        const FBox& lb = right ? fb : o;
        const FBox& rb = right ? o : fb;
        Node* nd = &nodes[pidx];
        nd->b0 = make_float4(lb.lo[0], lb.lo[1], lb.lo[2], lb.hi[0]);
        nd->b1 = make_float4(lb.hi[1], lb.hi[2], rb.lo[0], rb.lo[1]);
        nd->b2 = make_float4(rb.lo[2], rb.hi[0], rb.hi[1], rb.hi[2]);
        *reinterpret_cast<int4*>(nd->child) = make_int4(pl == s ? ~s : s, s + 1 == pr ? ~(s + 1) : s + 1,
            (int)(lb.plo | (lb.phi << 16)), (int)(rb.plo | (rb.phi << 16)));
        for (int j = 0; j < 3; ++j) {
            fb.lo[j] = fminf(fb.lo[j], o.lo[j]);
            fb.hi[j] = fmaxf(fb.hi[j], o.hi[j]);
        }
        fb.plo = min(fb.plo, o.plo);
        fb.phi = max(fb.phi, o.phi);
        // the node that holds exactly one pair's clusters is that pair's root
        if (pair_root && fb.plo == fb.phi && (uint32_t)pl == P.pair_clbase[fb.plo]
            && (uint32_t)pr + 1u == P.pair_clbase[fb.plo + 1])
            pair_root[fb.plo] = pidx;
        if (root) return;
        l = pl;
        r = pr;
        dl = pdl;
        dr = pdr;
    }
}

// ---------------------------------------------------------------------------
// packet traversal: a warp takes 32 Morton-consecutive source faces, walks
// the tree ONCE with the union of their boxes (one shared-memory stack per
// warp, node loads broadcast, no divergence in the walk) and, at each leaf
// cluster the union reaches, every lane tests its own box exactly against
// the cluster's faces. Exact tests compare dkey() integers, bit-for-bit the
// reference's closed fp64 test (intersect_bounding_boxes, math.h:931-943).
// ---------------------------------------------------------------------------
constexpr int kPacketStack = 64;

__global__ void __launch_bounds__(kBlock) k_traverse_packet(Problem P, const double* __restrict__ fbox,
    const uint32_t* __restrict__ qface, const uint2* __restrict__ packets, const uint32_t* __restrict__ leaf_face,
    const uint32_t* __restrict__ cl_start, const uint8_t* __restrict__ cl_n, const long long* __restrict__ leaf_key_box,
    int nleaf, const Node* __restrict__ nodes, unsigned long long* __restrict__ pairs, uint64_t cap,
    uint32_t* __restrict__ counters, uint8_t* __restrict__ cand, uint32_t* __restrict__ pair_status)
{
    __shared__ int stack_all[kBlock / 32][kPacketStack];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    int* stack = stack_all[wib];
    const unsigned full = 0xFFFFFFFFu;
    const uint32_t npackets = counters[9];
    for (;;) {
        uint32_t pk = 0;
        if (lane == 0) pk = atomicAdd(&counters[8], 1u);
        pk = __shfl_sync(full, pk, 0);
        if (pk >= npackets) break;
        const uint2 range = packets[pk];
        const uint32_t t = range.x + lane;
        const bool active = t <= range.y;
        uint32_t s = 0, p = 0;
        long long qk[6];
        float ql[3], qh[3];
        if (active) {
            s = qface[t];
            p = P.face_pair[s] & ~kCutBit;
            const Box qb = load_box(fbox, s);
            for (int j = 0; j < 3; ++j) {
                qk[j] = dkey(qb.mn[j]);
                qk[3 + j] = dkey(qb.mx[j]);
                ql[j] = f32_rd(qb.mn[j]);
                qh[j] = f32_ru(qb.mx[j]);
            }
        } else {
            for (int j = 0; j < 3; ++j) { qk[j] = LLONG_MAX; qk[3 + j] = LLONG_MIN; ql[j] = 3.4e38f; qh[j] = -3.4e38f; }
            p = 0xFFFFu;
        }
        // packet box and pair range
        float ul[3] = { ql[0], ql[1], ql[2] }, uh[3] = { qh[0], qh[1], qh[2] };
        uint32_t pmin = active ? p : 0xFFFFu, pmax = active ? p : 0u;
        for (int off = 16; off; off >>= 1) {
            for (int j = 0; j < 3; ++j) {
                ul[j] = fminf(ul[j], __shfl_xor_sync(full, ul[j], off));
                uh[j] = fmaxf(uh[j], __shfl_xor_sync(full, uh[j], off));
            }
            pmin = min(pmin, __shfl_xor_sync(full, pmin, off));
            pmax = max(pmax, __shfl_xor_sync(full, pmax, off));
        }
        unsigned long long buf[8];
        int nb = 0;
        bool any = false;
        auto flush = [&]() {
            if (nb == 0) return;
            const uint32_t pos = atomicAdd(&counters[0], (uint32_t)nb);
            for (int k = 0; k < nb; ++k)
                if ((uint64_t)pos + k < cap) pairs[pos + k] = buf[k];
            nb = 0;
        };
        // each lane tests its own query against one leaf cluster (fp32 pre-test, then exact)
        auto leaf = [&](int li, float lx0, float ly0, float lz0, float hx0, float hy0, float hz0, uint32_t lp) {
            if (!active || lp != p) return;
            if (!(ql[0] <= hx0 && qh[0] >= lx0 && ql[1] <= hy0 && qh[1] >= ly0 && ql[2] <= hz0 && qh[2] >= lz0))
                return;
            const uint32_t s0 = __ldg(&cl_start[li]), cn = __ldg(&cl_n[li]);
            for (uint32_t u = 0; u < cn; ++u) {
                const uint32_t c2 = __ldg(&leaf_face[s0 + u]);
                longlong2 a, b, c;
                load_key_box(fbox, c2, a, b, c);
                // closed overlap: q.mn <= l.mx && q.mx >= l.mn on every axis
                if (qk[0] <= b.y && qk[3] >= a.x && qk[1] <= c.x && qk[4] >= a.y && qk[2] <= c.y && qk[5] >= b.x) {
                    buf[nb++] = ((unsigned long long)s << 32) | c2;
                    cand[c2] = 1;
                    any = true;
                    if (nb == 8) flush();
                }
            }
        };
        bool overflow = false;
        if (nleaf == 1) {
            // single cluster: its box is not stored in any node; test the faces directly
            leaf(0, -3.4e38f, -3.4e38f, -3.4e38f, 3.4e38f, 3.4e38f, 3.4e38f, active ? p : 0xFFFFu);
        } else {
            int sp = 0;
            if (lane == 0) stack[0] = 0;
            sp = 1;
            __syncwarp();
            while (sp > 0) {
                const int nd = stack[--sp];
                __syncwarp();
                const float4 a = __ldg(&nodes[nd].b0), b = __ldg(&nodes[nd].b1), c = __ldg(&nodes[nd].b2);
                const int2 ch = __ldg(reinterpret_cast<const int2*>(&nodes[nd].child[0]));
                const uint2 pr = __ldg(reinterpret_cast<const uint2*>(&nodes[nd].prange[0]));
                const bool hit0 = (pr.x & 0xFFFFu) <= pmax && pmin <= (pr.x >> 16) && ul[0] <= a.w && uh[0] >= a.x
                    && ul[1] <= b.x && uh[1] >= a.y && ul[2] <= b.y && uh[2] >= a.z;
                const bool hit1 = (pr.y & 0xFFFFu) <= pmax && pmin <= (pr.y >> 16) && ul[0] <= c.y && uh[0] >= b.z
                    && ul[1] <= c.z && uh[1] >= b.w && ul[2] <= c.w && uh[2] >= c.x;
                if (hit0) {
                    if (ch.x < 0) leaf(~ch.x, a.x, a.y, a.z, a.w, b.x, b.y, pr.x & 0xFFFFu);
                    else {
                        if (sp < kPacketStack) { if (lane == 0) stack[sp] = ch.x; ++sp; }
                        else overflow = true;
                    }
                }
                if (hit1) {
                    if (ch.y < 0) leaf(~ch.y, b.z, b.w, c.x, c.y, c.z, c.w, pr.y & 0xFFFFu);
                    else {
                        if (sp < kPacketStack) { if (lane == 0) stack[sp] = ch.y; ++sp; }
                        else overflow = true;
                    }
                }
                __syncwarp();
            }
        }
        flush();
        if (any) cand[s] = 1;
        if (overflow && lane == 0) atomicOr(&pair_status[pmin == 0xFFFFu ? 0 : pmin], ST_STACK);
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// Wave traversal: one warp per query packet, breadth-first over the cut tree.
// Each step the lanes take up to 32 frontier nodes at once (32 independent
// node loads in flight instead of one long chain of dependent loads), test
// both children against the packet's union box, and compact the surviving
// internal children into the next frontier (ballot + popc). Leaf clusters
// the union reaches are queued in shared memory; for each, every lane tests
// its own query box (fp32 pre-test, then the exact integer-key test). A
// frontier or queue overflow flags the pair for the per-thread deep re-run.
// ---------------------------------------------------------------------------
constexpr int kWaveFrontier = 256;
#ifndef MCGPU_WAVE_LEAVES
#define MCGPU_WAVE_LEAVES 64
#endif
#ifndef MCGPU_WAVE_OUT
#define MCGPU_WAVE_OUT 96
#endif
#ifndef MCGPU_TOP_DEPTH
#define MCGPU_TOP_DEPTH 6
#endif
constexpr int kWaveLeaves = MCGPU_WAVE_LEAVES;
constexpr int kWaveWarps = kBlock / 32;

struct WaveLeaf {
    float lo[3], hi[3];
    int id;
    uint32_t pr;
};

// The top of the cut tree is the same for every packet: the tree cut at
// depth kTopDepth (internal nodes at that depth, shallower leaves) is listed
// once per dispatch with each entry's box, and every packet's walk starts by
// testing that list -- kTopDepth fewer dependent levels per packet.
constexpr int kTopDepth = MCGPU_TOP_DEPTH;
constexpr int kTopMax = 1 << kTopDepth;
struct WaveTop {
    float lo[3], hi[3];
    int id;       // >= 0 internal node, < 0 ~leaf
    uint32_t pr;  // pair range lo | hi << 16
};
static_assert(sizeof(WaveTop) == 32, "the top-cut buffer holds 64 entries of 32 bytes");

// A slow packet's remaining walk, handed from the first traversal launch to
// the second: a group of its queries and up to 32 subtree roots to expand.
#ifndef MCGPU_SPLIT_STACK
#define MCGPU_SPLIT_STACK 8     // ... if more than this many nodes are still to expand
#endif
#ifndef MCGPU_SPLIT_GROUP
#define MCGPU_SPLIT_GROUP 2     // queries per split entry (1, 2, 4, 8, 16 or 32)
#endif
struct SplitEntry {
    uint32_t packet;
    uint32_t qmask;   // queries of the packet (lanes) this entry walks for
    uint32_t count;   // subtree roots in nodes[]
    uint32_t pad;
    int nodes[32];
};
static_assert(sizeof(SplitEntry) == 144, "split entries are 144 bytes");

__global__ void __launch_bounds__(32) k_top_cut(const Node* __restrict__ nodes, int nleaf, WaveTop* __restrict__ top,
    uint32_t* __restrict__ counters)
{
    __shared__ int cur[kTopMax], nxt[kTopMax];
    __shared__ int ncur, nnxt, ntop;
    const int lane = threadIdx.x;
    if (lane == 0) {
        cur[0] = 0;
        ncur = nleaf > 1 ? 1 : 0;
        ntop = 0;
    }
    __syncwarp();
    for (int depth = 1; depth <= kTopDepth && ncur > 0; ++depth) {
        if (lane == 0) nnxt = 0;
        __syncwarp();
        for (int i = lane; i < ncur; i += 32) {
            const Node nd = nodes[cur[i]];
            const float* b = reinterpret_cast<const float*>(&nd.b0);
            for (int k = 0; k < 2; ++k) {
                const int c = nd.child[k];
                if (c >= 0 && depth < kTopDepth) {
                    nxt[atomicAdd(&nnxt, 1)] = c;
                } else {
                    WaveTop e;
                    for (int j = 0; j < 3; ++j) { e.lo[j] = b[k * 6 + j]; e.hi[j] = b[k * 6 + 3 + j]; }
                    e.id = c;
                    e.pr = nd.prange[k];
                    top[atomicAdd(&ntop, 1)] = e;
                }
            }
        }
        __syncwarp();
        for (int i = lane; i < nnxt; i += 32) cur[i] = nxt[i];
        __syncwarp();
        if (lane == 0) ncur = nnxt;
        __syncwarp();
    }
    if (lane == 0) counters[13] = (uint32_t)ntop;
}

// Output goes through a per-warp staging buffer in shared memory and reaches
// the global pair list in blocks of up to kWaveOut pairs (one atomic each).
//
// Queued leaf clusters are tested lane-parallel: lane k takes queued leaf k
// and tests every query of the packet (kept in shared memory) against it, so
// a packet that reaches hundreds of leaves pays a few rounds of parallel
// loads instead of hundreds of dependent ones.
constexpr int kWaveOut = MCGPU_WAVE_OUT;

struct __align__(16) WaveWarp {
    int front[2][kWaveFrontier];
    WaveLeaf leaves[kWaveLeaves];
    unsigned long long out[kWaveOut + 32];
    long long qk[32][6];
    float qb[32][8];     // lo xyz, pad, hi xyz, pad (two float4 loads)
    float sub[4][8];     // union boxes of queries 8g .. 8g+7
    uint32_t qs[32];
    uint32_t qp[32];
    int nout;
    unsigned qhit; // queries of the current packet that produced a pair
};
constexpr size_t kWaveSmem = sizeof(WaveWarp) * kWaveWarps;
static_assert(sizeof(WaveWarp) % 16 == 0 && offsetof(WaveWarp, qb) % 16 == 0 && offsetof(WaveWarp, sub) % 16 == 0,
    "float4 shared-memory loads of the query boxes need 16-byte alignment");

// SPLIT = false: one packet per work item, the walk starting at the top cut;
// a packet still far from done after `split_round` rounds is split into
// entries (its queries in groups of 8 x its remaining subtree roots in
// chunks of 32) for the second launch. SPLIT = true: one entry per work item.
template <bool SPLIT>
__global__ void __launch_bounds__(kBlock) k_traverse_wave(Problem P, const double* __restrict__ fbox,
    const uint32_t* __restrict__ qface, const uint2* __restrict__ packets, const uint32_t* __restrict__ leaf_face,
    const uint32_t* __restrict__ cl_start, const uint8_t* __restrict__ cl_n, const WaveTop* __restrict__ top,
    int nleaf, const Node* __restrict__ nodes, unsigned long long* __restrict__ pairs, uint64_t cap,
    uint32_t* __restrict__ counters, uint8_t* __restrict__ cand, uint32_t* __restrict__ pair_status,
    SplitEntry* __restrict__ split, uint32_t split_cap, int split_round, const int32_t* __restrict__ pair_root)
{
    extern __shared__ __align__(16) unsigned char wave_smem[];
    const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
    WaveWarp& W = reinterpret_cast<WaveWarp*>(wave_smem)[wib];
    const unsigned full = 0xFFFFFFFFu;
    const unsigned lt = (1u << lane) - 1u;
    const uint32_t npackets = counters[9];
    if (lane == 0) W.nout = 0;
    __syncwarp();
    auto flush_out = [&]() {
        __syncwarp();
        const int nout = min(W.nout, kWaveOut + 32);
        uint32_t base = 0;
        if (lane == 0 && nout) base = atomicAdd(&counters[0], (uint32_t)nout);
        base = __shfl_sync(full, base, 0);
        for (int k = lane; k < nout; k += 32)
            if ((uint64_t)base + k < cap) pairs[base + k] = W.out[k];
        __syncwarp();
        if (lane == 0) W.nout = 0;
        __syncwarp();
    };
    const uint32_t nitems = SPLIT ? min(counters[14], split_cap) : npackets;
    for (;;) {
        uint32_t it = 0;
        if (lane == 0) it = atomicAdd(&counters[SPLIT ? 15 : 8], 1u);
        it = __shfl_sync(full, it, 0);
        if (it >= nitems) break;
        const uint32_t pk = SPLIT ? split[it].packet : it;
        const uint32_t qmask = SPLIT ? split[it].qmask : 0xFFFFFFFFu;
        const uint2 range = packets[pk];
        const int psize = (int)(range.y - range.x + 1);
        const uint32_t t = range.x + lane;
        const bool active = lane < psize && ((qmask >> lane) & 1u);
        uint32_t p = 0xFFFFu;
        float ql[3], qh[3];
        if (!active) {
            // a query this item does not walk for matches nothing
            for (int j = 0; j < 3; ++j) { W.qb[lane][j] = 3.4e38f; W.qb[lane][4 + j] = -3.4e38f; }
            W.qp[lane] = 0xFFFFFFFFu;
        }
        if (active) {
            const uint32_t s = qface[t];
            p = P.face_pair[s] & ~kCutBit;
            const Box qb = load_box(fbox, s);
            for (int j = 0; j < 3; ++j) {
                W.qk[lane][j] = dkey(qb.mn[j]);
                W.qk[lane][3 + j] = dkey(qb.mx[j]);
                ql[j] = f32_rd(qb.mn[j]);
                qh[j] = f32_ru(qb.mx[j]);
                W.qb[lane][j] = ql[j];
                W.qb[lane][4 + j] = qh[j];
            }
            W.qs[lane] = s;
            W.qp[lane] = p;
        } else {
            for (int j = 0; j < 3; ++j) { ql[j] = 3.4e38f; qh[j] = -3.4e38f; }
        }
        float ul[3] = { ql[0], ql[1], ql[2] }, uh[3] = { qh[0], qh[1], qh[2] };
        uint32_t pmin = active ? p : 0xFFFFu, pmax = active ? p : 0u;
        for (int off = 1; off < 32; off <<= 1) {
            if (off == 8) {
                // lanes 8g .. 8g+7 now hold their group's union: lane 8g writes it
                if ((lane & 7) == 0)
                    for (int j = 0; j < 3; ++j) { W.sub[lane >> 3][j] = ul[j]; W.sub[lane >> 3][4 + j] = uh[j]; }
            }
            for (int j = 0; j < 3; ++j) {
                ul[j] = fminf(ul[j], __shfl_xor_sync(full, ul[j], off));
                uh[j] = fmaxf(uh[j], __shfl_xor_sync(full, uh[j], off));
            }
            pmin = min(pmin, __shfl_xor_sync(full, pmin, off));
            pmax = max(pmax, __shfl_xor_sync(full, pmax, off));
        }
        if (lane == 0) W.qhit = 0;
        __syncwarp();
        bool overflow = false;
        int nl = 0;         // queued leaves (uniform across the warp)
        // lane k takes queued leaf k: a 32-bit mask of the packet's queries
        // whose fp32 box meets the leaf's box, then exact tests of those
        // queries against the leaf's faces; hits go to the warp's staging
        // buffer through shared-memory atomics (global atomics past it)
        auto drain = [&]() {
            __syncwarp();
            for (int base = 0; base < nl; base += 32) {
                const int k = base + lane;
                if (k < nl) {
                    const WaveLeaf L = W.leaves[k];
                    // the cluster's faces: first position from the pair tables (as
                    // k_clusters lays clusters out); their ids are requested before
                    // the box tests so the loads overlap them
                    const uint32_t lp = L.pr & 0xFFFFu;
                    const uint32_t s0 = P.pair_cbase[lp] + ((uint32_t)L.id - P.pair_clbase[lp]) * P.leaf_size;
                    const uint32_t cn = min(P.leaf_size, P.pair_cbase[lp + 1] - s0);
                    uint32_t cf0[4];
#pragma unroll
                    for (int u = 0; u < 4; ++u) cf0[u] = (uint32_t)u < cn ? __ldg(&leaf_face[s0 + u]) : 0u;
                    // queries whose fp32 box meets the leaf box, group by group of 8
                    // (a group whose union misses the leaf is skipped)
                    unsigned mask = 0;
                    for (int g = 0; g * 8 < psize; ++g) {
                        const float4 ga = *reinterpret_cast<const float4*>(&W.sub[g][0]);
                        const float4 gb = *reinterpret_cast<const float4*>(&W.sub[g][4]);
                        if (!(ga.x <= L.hi[0] && gb.x >= L.lo[0] && ga.y <= L.hi[1] && gb.y >= L.lo[1]
                                && ga.z <= L.hi[2] && gb.z >= L.lo[2]))
                            continue;
                        const int je = min(psize, g * 8 + 8);
                        for (int j = g * 8; j < je; ++j) {
                            const float4 qa = *reinterpret_cast<const float4*>(&W.qb[j][0]);
                            const float4 qb4 = *reinterpret_cast<const float4*>(&W.qb[j][4]);
                            const bool ov = W.qp[j] == lp && qa.x <= L.hi[0] && qb4.x >= L.lo[0] && qa.y <= L.hi[1]
                                && qb4.y >= L.lo[1] && qa.z <= L.hi[2] && qb4.z >= L.lo[2];
                            mask |= (ov ? 1u : 0u) << j;
                        }
                    }
                    if (mask) {
                        // exact boxes tested first with no stores in the loop, the next
                        // face's box loading while the current one is tested; pairs
                        // are emitted after
                        for (uint32_t u0 = 0; u0 < cn; u0 += 4) {
                            const uint32_t m = min(4u, cn - u0);
                            uint32_t cfs[4];
#pragma unroll
                            for (int u = 0; u < 4; ++u)
                                cfs[u] = u0 == 0 ? cf0[u] : ((uint32_t)u < m ? __ldg(&leaf_face[s0 + u0 + u]) : 0u);
                            unsigned hits[4] = { 0u, 0u, 0u, 0u };
                            longlong2 na, nb, nc;
                            load_key_box(fbox, cfs[0], na, nb, nc);
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                if ((uint32_t)u >= m) break;
                                const longlong2 ka = na, kb = nb, kc = nc;
                                if ((uint32_t)u + 1 < m) load_key_box(fbox, cfs[u + 1], na, nb, nc);
                                unsigned h = 0;
                                for (unsigned mm = mask; mm; mm &= mm - 1) {
                                    const int j = __ffs(mm) - 1;
                                    const long long* q = W.qk[j];
                                    if (q[0] <= kb.y && q[3] >= ka.x && q[1] <= kc.x && q[4] >= ka.y && q[2] <= kc.y
                                        && q[5] >= kb.x)
                                        h |= 1u << j;
                                }
                                hits[u] = h;
                            }
#pragma unroll
                            for (int u = 0; u < 4; ++u) {
                                if (!hits[u]) continue;
                                const uint32_t cf = cfs[u];
                                for (unsigned mm = hits[u]; mm; mm &= mm - 1) {
                                    const int j = __ffs(mm) - 1;
                                    const unsigned long long pr = ((unsigned long long)W.qs[j] << 32) | cf;
                                    const int pos = atomicAdd(&W.nout, 1);
                                    if (pos < kWaveOut + 32) {
                                        W.out[pos] = pr;
                                    } else {
                                        const uint32_t g = atomicAdd(&counters[0], 1u);
                                        if (g < cap) pairs[g] = pr;
                                    }
                                }
                                atomicOr(&W.qhit, hits[u]);
                                cand[cf] = 1;
                            }
                        }
                    }
                }
                __syncwarp();
                if (W.nout >= kWaveOut) flush_out();
            }
            nl = 0;
            __syncwarp();
        };
        if (nleaf == 1) {
            if (lane == 0) {
                WaveLeaf& L = W.leaves[0];
                for (int j = 0; j < 3; ++j) { L.lo[j] = -3.4e38f; L.hi[j] = 3.4e38f; }
                L.id = 0;
                L.pr = (P.face_pair[leaf_face[0]] & ~kCutBit) * 0x10001u;
            }
            nl = 1;
            drain();
        } else {
            // Nodes to expand sit on a warp-wide stack (both frontier arrays as one
            // 512-entry array); each round pops up to 32 and pushes the children
            // that meet the packet's union box, deepest first, which bounds the
            // stack by the tree depth times 32 instead of by the widest level.
            int* stk = &W.front[0][0];
            constexpr int kStk = 2 * kWaveFrontier;
            int sp = 0;
            if (SPLIT) {
                const int cnt = (int)split[it].count;
                if (lane < cnt) stk[lane] = split[it].nodes[lane];
                sp = cnt;
            }
            // first: the listed top cut of the tree -- or, for a packet of one
            // pair in a batch, that pair's own subtree (the levels above it hold
            // other pairs' clusters only)
            int ntop = SPLIT ? 0 : (int)counters[13];
            if (!SPLIT && pair_root && pmin == pmax) {
                const int r0 = __ldg(&pair_root[pmin]);
                if (r0 >= 0) {
                    if (lane == 0) stk[0] = r0;
                    __syncwarp();
                    sp = 1;
                    ntop = 0;
                }
            }
            for (int base = 0; base < ntop; base += 32) {
                const int i = base + lane;
                bool hit = false;
                int ch = 0;
                float bx[6];
                uint32_t prr = 0;
                if (i < ntop) {
                    const WaveTop e = top[i];
                    ch = e.id;
                    prr = e.pr;
                    for (int j = 0; j < 3; ++j) { bx[j] = e.lo[j]; bx[3 + j] = e.hi[j]; }
                    hit = (prr & 0xFFFFu) <= pmax && pmin <= (prr >> 16) && ul[0] <= bx[3] && uh[0] >= bx[0]
                        && ul[1] <= bx[4] && uh[1] >= bx[1] && ul[2] <= bx[5] && uh[2] >= bx[2];
                }
                const bool inner = hit && ch >= 0, leaf = hit && ch < 0;
                const unsigned mi = __ballot_sync(full, inner), ml = __ballot_sync(full, leaf);
                if (sp + __popc(mi) > kStk) {
                    overflow = true;
                } else {
                    if (inner) stk[sp + __popc(mi & lt)] = ch;
                    sp += __popc(mi);
                }
                if (nl + __popc(ml) > kWaveLeaves) drain();
                if (leaf) {
                    WaveLeaf& L = W.leaves[nl + __popc(ml & lt)];
                    for (int j = 0; j < 3; ++j) { L.lo[j] = bx[j]; L.hi[j] = bx[3 + j]; }
                    L.id = ~ch;
                    L.pr = prr;
                }
                nl += __popc(ml);
            }
            __syncwarp();
            int rounds = 0;
            while (sp > 0) {
                if (!SPLIT && split_round > 0 && ++rounds > split_round && sp > MCGPU_SPLIT_STACK) {
                    // a slow packet: its groups of 8 queries x chunks of 32 roots go
                    // to the second launch, each walked by its own warp
                    constexpr int kG = MCGPU_SPLIT_GROUP;
                    constexpr unsigned kGm = kG == 32 ? 0xFFFFFFFFu : ((1u << kG) - 1u);
                    unsigned am = __ballot_sync(full, active);
                    const int chunks = (sp + 31) / 32;
                    int ng = 0;
                    for (int g = 0; g < 32 / kG; ++g) ng += ((am >> (kG * g)) & kGm) ? 1 : 0;
                    uint32_t base_e = 0;
                    if (lane == 0) base_e = atomicAdd(&counters[14], (uint32_t)(ng * chunks));
                    base_e = __shfl_sync(full, base_e, 0);
                    if (base_e + (uint32_t)(ng * chunks) > split_cap) {
                        // no room: the reserved entries below the cap are left empty
                        // and this packet finishes its own walk
                        for (uint32_t e = base_e + lane; e < split_cap && e < base_e + (uint32_t)(ng * chunks); e += 32) {
                            split[e].packet = pk;
                            split[e].qmask = 0u;
                            split[e].count = 0u;
                        }
                        rounds = -(1 << 30);
                    } else {
                        uint32_t e = base_e;
                        for (int g = 0; g < 32 / kG; ++g) {
                            const uint32_t gm = am & (kGm << (kG * g));
                            if (!gm) continue;
                            for (int c = 0; c < chunks; ++c, ++e) {
                                const int cnt = min(32, sp - 32 * c);
                                if (lane == 0) {
                                    split[e].packet = pk;
                                    split[e].qmask = gm;
                                    split[e].count = (uint32_t)cnt;
                                }
                                if (lane < cnt) split[e].nodes[lane] = stk[32 * c + lane];
                            }
                        }
                    }
                    __syncwarp();
                    if (rounds >= 0) {
                        sp = 0;
                        break;
                    }
                }
                const int take = min(sp, 32);
                const int base = sp - take;
                const bool v = lane < take;
                bool hit[2] = { false, false };
                int ch[2] = { 0, 0 };
                float bx[2][6];
                uint32_t prr[2] = { 0, 0 };
                const int nd = v ? stk[base + lane] : 0;
                __syncwarp(); // every lane holds its entry before the pushes reuse the slots
                sp = base;
                if (v) {
                    const float4 a = __ldg(&nodes[nd].b0), b = __ldg(&nodes[nd].b1), c = __ldg(&nodes[nd].b2);
                    const int2 cc = __ldg(reinterpret_cast<const int2*>(&nodes[nd].child[0]));
                    const uint2 pr = __ldg(reinterpret_cast<const uint2*>(&nodes[nd].prange[0]));
                    ch[0] = cc.x; ch[1] = cc.y; prr[0] = pr.x; prr[1] = pr.y;
                    bx[0][0] = a.x; bx[0][1] = a.y; bx[0][2] = a.z; bx[0][3] = a.w; bx[0][4] = b.x; bx[0][5] = b.y;
                    bx[1][0] = b.z; bx[1][1] = b.w; bx[1][2] = c.x; bx[1][3] = c.y; bx[1][4] = c.z; bx[1][5] = c.w;
                    for (int k = 0; k < 2; ++k)
                        hit[k] = (prr[k] & 0xFFFFu) <= pmax && pmin <= (prr[k] >> 16) && ul[0] <= bx[k][3]
                            && uh[0] >= bx[k][0] && ul[1] <= bx[k][4] && uh[1] >= bx[k][1] && ul[2] <= bx[k][5]
                            && uh[2] >= bx[k][2];
                }
                for (int k = 0; k < 2; ++k) {
                    const bool inner = hit[k] && ch[k] >= 0, leaf = hit[k] && ch[k] < 0;
                    const unsigned mi = __ballot_sync(full, inner), ml = __ballot_sync(full, leaf);
                    if (sp + __popc(mi) > kStk) {
                        overflow = true;
                    } else {
                        if (inner) stk[sp + __popc(mi & lt)] = ch[k];
                        sp += __popc(mi);
                    }
                    if (nl + __popc(ml) > kWaveLeaves) drain(); // nl is uniform
                    if (leaf) {
                        WaveLeaf& L = W.leaves[nl + __popc(ml & lt)];
                        for (int j = 0; j < 3; ++j) { L.lo[j] = bx[k][j]; L.hi[j] = bx[k][3 + j]; }
                        L.id = ~ch[k];
                        L.pr = prr[k];
                    }
                    nl += __popc(ml);
                }
                __syncwarp();
            }
            drain();
        }
        __syncwarp();
        if (active && (W.qhit >> lane) & 1u) cand[W.qs[lane]] = 1;
        overflow = __any_sync(full, overflow);
        if (overflow && lane == 0) atomicOr(&pair_status[pmin == 0xFFFFu ? 0 : pmin], ST_STACK);
        __syncwarp();
    }
    flush_out();
}

// ---------------------------------------------------------------------------
// traversal: every source face queries the cut-face LBVH (intersectOIBVHs,
// bvh.cpp:638-783). Queries run in Morton order so neighbouring threads walk
// similar paths. Leaf tests are the reference's exact closed fp64 test.
// ---------------------------------------------------------------------------
template <int STACK>
__global__ void __launch_bounds__(kBlock) k_traverse(Problem P, const double* __restrict__ fbox,
    const uint32_t* __restrict__ qface, const uint32_t* __restrict__ leaf_face, const uint32_t* __restrict__ cl_start,
    const uint8_t* __restrict__ cl_n, const long long* __restrict__ leaf_key_box, int nleaf,
    const Node* __restrict__ nodes, unsigned long long* __restrict__ pairs, uint64_t cap,
    uint32_t* __restrict__ counters, uint8_t* __restrict__ cand, uint32_t* __restrict__ pair_status)
{
    // queries cost very different amounts (far faces stop at the root), so
    // warps take the next 32 Morton-ordered queries from a shared counter
    const int lane = threadIdx.x & 31;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(&counters[8], 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= P.ns) break;
        const uint32_t t = base + lane;
        if (t >= P.ns) continue;
        const uint32_t s = qface[t];
        const uint32_t p = P.face_pair[s] & ~kCutBit;
        const Box qb = load_box(fbox, s);
        float ql[3], qh[3];
        long long qk[6];
        for (int j = 0; j < 3; ++j) {
            ql[j] = f32_rd(qb.mn[j]);
            qh[j] = f32_ru(qb.mx[j]);
            qk[j] = dkey(qb.mn[j]);
            qk[3 + j] = dkey(qb.mx[j]);
        }
        unsigned long long buf[8];
        int nb = 0;
        bool any = false;
        auto flush = [&]() {
            if (nb == 0) return;
            const uint32_t pos = atomicAdd(&counters[0], (uint32_t)nb);
            for (int k = 0; k < nb; ++k)
                if ((uint64_t)pos + k < cap) pairs[pos + k] = buf[k];
            nb = 0;
        };
        // a leaf cluster's faces, tested exactly: the closed fp64 overlap of
        // intersect_bounding_boxes (math.h:931-943) on dkey() integers. The
        // cluster's pair was checked with its box (prange).
        auto leaf = [&](int li) {
            const uint32_t s0 = __ldg(&cl_start[li]), cn = __ldg(&cl_n[li]);
            for (uint32_t u = 0; u < cn; ++u) {
                const uint32_t cf = __ldg(&leaf_face[s0 + u]);
                longlong2 a, b, c;
                load_key_box(fbox, cf, a, b, c);
                if (qk[0] <= b.y && qk[3] >= a.x && qk[1] <= c.x && qk[4] >= a.y && qk[2] <= c.y && qk[5] >= b.x) {
                    buf[nb++] = ((unsigned long long)s << 32) | cf;
                    cand[cf] = 1;
                    any = true;
                    if (nb == 8) flush();
                }
            }
        };
        if (nleaf == 1) {
            if ((P.face_pair[__ldg(&leaf_face[0])] & ~kCutBit) == p) leaf(0);
        } else {
            int stack[STACK];
            int sp = 0;
            stack[sp++] = 0;
            bool overflow = false;
            while (sp > 0) {
                const int nd = stack[--sp];
                const float4 a = __ldg(&nodes[nd].b0), b = __ldg(&nodes[nd].b1), c = __ldg(&nodes[nd].b2);
                const int2 ch = __ldg(reinterpret_cast<const int2*>(&nodes[nd].child[0]));
                const uint2 pr = __ldg(reinterpret_cast<const uint2*>(&nodes[nd].prange[0]));
                const bool hit0 = (pr.x & 0xFFFFu) <= p && p <= (pr.x >> 16) && ql[0] <= a.w && qh[0] >= a.x
                    && ql[1] <= b.x && qh[1] >= a.y && ql[2] <= b.y && qh[2] >= a.z;
                const bool hit1 = (pr.y & 0xFFFFu) <= p && p <= (pr.y >> 16) && ql[0] <= c.y && qh[0] >= b.z
                    && ql[1] <= c.z && qh[1] >= b.w && ql[2] <= c.w && qh[2] >= c.x;
                if (hit0) {
                    if (ch.x < 0) leaf(~ch.x);
                    else if (sp < STACK) stack[sp++] = ch.x;
                    else overflow = true;
                }
                if (hit1) {
                    if (ch.y < 0) leaf(~ch.y);
                    else if (sp < STACK) stack[sp++] = ch.y;
                    else overflow = true;
                }
            }
            if (overflow) atomicOr(&pair_status[p], ST_STACK);
        }
        flush();
        if (any) cand[s] = 1;
    }
}

// Source faces of pairs with a resident cut tree (ResPair) walk that tree,
// one thread per face. The tree's boxes are in the mesh's user coordinates;
// the pair's cut vertices are x' = (x - com) + t, so a cut face whose
// enlarged pair-frame box meets the query box has a user box meeting the
// query box shifted by com - t and widened by the cut-box enlargement and a
// margin that covers the roundings of x' and of the shift (far below the
// fp32 boxes' own outward rounding). At the leaves the faces are tested
// exactly on their pair-frame fp64 boxes, as every other candidate, so the
// pair set is the one the batch tree gives.
template <int STACK>
__global__ void __launch_bounds__(kBlock) k_traverse_resident(Problem P, const double* __restrict__ fbox,
    const uint32_t* __restrict__ qface, unsigned long long* __restrict__ pairs, uint64_t cap,
    uint32_t* __restrict__ counters, uint8_t* __restrict__ cand, uint32_t* __restrict__ pair_status)
{
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < P.ns; t += gridDim.x * blockDim.x) {
        const uint32_t s = qface[t];
        const uint32_t p = face_pair_of(P, s) & ~kCutBit;
        const ResPair R = P.res_pairs[p];
        if (R.ncl == 0) continue;
        const Box qb = load_box(fbox, s);
        const double* fr = P.pair_frames + 6 * (size_t)p;
        const double eps = P.pair_eps[p];
        float ql[3], qh[3];
        long long qk[6];
        for (int j = 0; j < 3; ++j) {
            const double sh = fr[j] - fr[3 + j];
            const double m = 0x1p-48 * (fabs(qb.mn[j]) + fabs(qb.mx[j]) + eps + 2.0 * (fabs(fr[j]) + fabs(fr[3 + j]))
                + 2.0 * R.mag[j]);
            ql[j] = f32_rd(((qb.mn[j] - eps) + sh) - m);
            qh[j] = f32_ru(((qb.mx[j] + eps) + sh) + m);
            qk[j] = dkey(qb.mn[j]);
            qk[3 + j] = dkey(qb.mx[j]);
        }
        const uint32_t cbase = P.pair_fbase[p] + P.pair_fs[p]; // the pair's first cut face (ps id)
        unsigned long long buf[8];
        int nb = 0;
        bool any = false;
        auto flush = [&]() {
            if (nb == 0) return;
            const uint32_t pos = atomicAdd(&counters[0], (uint32_t)nb);
            for (int k = 0; k < nb; ++k)
                if ((uint64_t)pos + k < cap) pairs[pos + k] = buf[k];
            nb = 0;
        };
        auto leaf = [&](int li) {
            const uint32_t s0 = __ldg(&R.cl_start[li]), cn = __ldg(&R.cl_n[li]);
            for (uint32_t u = 0; u < cn; ++u) {
                const uint32_t cf = cbase + __ldg(&R.leaf_face[s0 + u]);
                longlong2 a, b, c;
                load_key_box(fbox, cf, a, b, c);
                if (qk[0] <= b.y && qk[3] >= a.x && qk[1] <= c.x && qk[4] >= a.y && qk[2] <= c.y && qk[5] >= b.x) {
                    buf[nb++] = ((unsigned long long)s << 32) | cf;
                    cand[cf] = 1;
                    any = true;
                    if (nb == 8) flush();
                }
            }
        };
        if (R.ncl == 1) {
            leaf(0);
        } else {
            int stack[STACK];
            int sp = 0;
            stack[sp++] = 0;
            bool overflow = false;
            while (sp > 0) {
                const int nd = stack[--sp];
                const float4 a = __ldg(&R.nodes[nd].b0), b = __ldg(&R.nodes[nd].b1), c = __ldg(&R.nodes[nd].b2);
                const int2 ch = __ldg(reinterpret_cast<const int2*>(&R.nodes[nd].child[0]));
                const bool hit0 = ql[0] <= a.w && qh[0] >= a.x && ql[1] <= b.x && qh[1] >= a.y && ql[2] <= b.y
                    && qh[2] >= a.z;
                const bool hit1 = ql[0] <= c.y && qh[0] >= b.z && ql[1] <= c.z && qh[1] >= b.w && ql[2] <= c.w
                    && qh[2] >= c.x;
                if (hit0) {
                    if (ch.x < 0) leaf(~ch.x);
                    else if (sp < STACK) stack[sp++] = ch.x;
                    else overflow = true;
                }
                if (hit1) {
                    if (ch.y < 0) leaf(~ch.y);
                    else if (sp < STACK) stack[sp++] = ch.y;
                    else overflow = true;
                }
            }
            if (overflow) atomicOr(&pair_status[p], ST_STACK);
        }
        flush();
        if (any) cand[s] = 1;
    }
}

// A resident mesh's faces: fp32 boxes rounded outward from its fp64 user
// coordinates and 23-bit Morton keys in the frame of its vertex bounds
// mn / mx; thread 0 writes the one-pair tables the cluster pass reads.
__global__ void __launch_bounds__(kBlock) k_res_faces(const double* __restrict__ X, const uint32_t* __restrict__ idx,
    uint32_t nv, uint32_t nf, double mn0, double mn1, double mn2, double mx0, double mx1, double mx2,
    float* __restrict__ fbox32, uint32_t* __restrict__ key, uint32_t* __restrict__ val, uint32_t* __restrict__ tab,
    uint32_t ncl)
{
    const double mn[3] = { mn0, mn1, mn2 }, mx[3] = { mx0, mx1, mx2 };
    float flo[3], fsc[3];
    for (int j = 0; j < 3; ++j) {
        flo[j] = f32_rd(mn[j]);
        const float ext = f32_ru(mx[j]) - flo[j];
        fsc[j] = ext > 0.0f ? __fdiv_rn(1023.0f, ext) : 0.0f;
    }
    if (blockIdx.x == 0 && threadIdx.x == 0) {
        tab[0] = 0; tab[1] = nf; // pair_cbase
        tab[2] = 0; tab[3] = ncl; // pair_clbase
    }
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
        double lo[3] = { 1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308 };
        double hi[3] = { -1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308 };
        for (int k = 0; k < 3; ++k) {
            uint32_t v = idx[3 * (size_t)f + k];
            if (v >= nv) v = 0;
            for (int j = 0; j < 3; ++j) {
                const double x = X[3 * (size_t)v + j];
                lo[j] = fmin(lo[j], x);
                hi[j] = fmax(hi[j], x);
            }
        }
        float b[6];
        for (int j = 0; j < 3; ++j) { b[j] = f32_rd(lo[j]); b[3 + j] = f32_ru(hi[j]); }
        float2* d32 = reinterpret_cast<float2*>(fbox32 + (size_t)f * 6);
        d32[0] = make_float2(b[0], b[1]);
        d32[1] = make_float2(b[2], b[3]);
        d32[2] = make_float2(b[4], b[5]);
        key[f] = morton_code((0.5f * (b[0] + b[3]) - flo[0]) * fsc[0], (0.5f * (b[1] + b[4]) - flo[1]) * fsc[1],
            (0.5f * (b[2] + b[5]) - flo[2]) * fsc[2]);
        val[f] = f;
    }
}

// ---------------------------------------------------------------------------
// candidate-face properties: vertex needs, face planes, degenerate check
// (kernel.cpp:2184-2356, math.cpp:130-239)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(kBlock) k_mark_vertices(Problem P, const uint8_t* __restrict__ cand,
    uint8_t* __restrict__ vneed)
{
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < P.nf; f += gridDim.x * blockDim.x) {
        if (!cand[f]) continue;
        const uint32_t o = face_o(P, f), n = face_n(P, f);
        for (uint32_t k = 0; k < n; ++k) vneed[P.fidx[o + k]] = 1;
    }
}

__global__ void __launch_bounds__(kBlock) k_vf_count(Problem P, const uint8_t* __restrict__ vneed,
    uint32_t* __restrict__ vdeg)
{
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < P.nf; f += gridDim.x * blockDim.x) {
        const uint32_t o = face_o(P, f), n = face_n(P, f);
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t v = P.fidx[o + k];
            if (vneed[v]) atomicAdd(&vdeg[v], 1u);
        }
    }
}

// Fixed-width incidence: up to K faces per needed vertex in vslot[v K ..]
// with its count in vdeg[v], in one pass (no count, scan and fill). A vertex
// with more than K incident faces sets counters[12]; the host then reruns
// the call with the CSR lists.
__global__ void __launch_bounds__(kBlock) k_vf_slots(Problem P, const uint8_t* __restrict__ vneed,
    uint32_t* __restrict__ vdeg, uint32_t* __restrict__ vslot, uint32_t K, uint32_t* __restrict__ counters)
{
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < P.nf; f += gridDim.x * blockDim.x) {
        const uint32_t o = face_o(P, f), n = face_n(P, f);
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t v = P.fidx[o + k];
            if (!vneed[v]) continue;
            const uint32_t j = atomicAdd(&vdeg[v], 1u);
            if (j < K) vslot[(size_t)v * K + j] = f;
            else counters[12] = 1u;
        }
    }
}

__global__ void __launch_bounds__(kBlock) k_vf_fill(Problem P, const uint8_t* __restrict__ vneed,
    const uint32_t* __restrict__ voff, uint32_t* __restrict__ vcur, uint32_t* __restrict__ vface, uint64_t cap)
{
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < P.nf; f += gridDim.x * blockDim.x) {
        const uint32_t o = face_o(P, f), n = face_n(P, f);
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t v = P.fidx[o + k];
            if (vneed[v]) {
                const uint32_t pos = voff[v] + atomicAdd(&vcur[v], 1u);
                if (pos < cap) vface[pos] = f;
            }
        }
    }
}

// vertex k of the face's list as the reference's narrow phase sees it: the
// polygon soup's get_vertices_around_face returns the TARGETS of the face's
// halfedges (hmesh.cpp:722-733). The soup copies the source mesh, so a
// source face lists its input corners rotated by one; it adds each cut face
// as the cut mesh's own get_vertices_around_face lists it (kernel.cpp:
// 1650-1700), so a cut face lists them rotated by two. rot = face_rot(P, f).
__device__ __forceinline__ uint32_t face_rot(const Problem& P, uint32_t f)
{
    return (face_pair_of(P, f) & kCutBit) ? 2u : 1u;
}
__device__ __forceinline__ uint32_t face_vertex(const Problem& P, uint32_t o, uint32_t n, uint32_t k, uint32_t rot)
{
    uint32_t j = k + rot; // k < n and rot <= 2 < n + 1: one wrap at most
    if (j >= n) j -= n;
    return P.fidx[o + j];
}

// unit normal, d and the largest component from the raw Newell normal in
// pl.n (compute_polygon_plane_coefficients, math.cpp:130-239)
__device__ __forceinline__ void finish_plane(FacePlane& pl, const double* first)
{
    const double nn[3] = { pl.n[0], pl.n[1], pl.n[2] };
    const double len = sqrt(dot3(nn, nn));
    pl.n[0] = nn[0] / len; pl.n[1] = nn[1] / len; pl.n[2] = nn[2] / len;
    pl.d = dot3(first, pl.n);
    double big = 0.0;
    pl.mc = 0;
    for (int i = 0; i < 3; ++i) {
        const double t = fabs(pl.n[i]);
        if (t > big) { big = t; pl.mc = i; }
    }
}

#ifndef MCGPU_PL_MINB
#define MCGPU_PL_MINB 1
#endif
// Candidate faces -> dense plane slots, and the slot -> face list (slot_face)
// the plane kernel walks: its fp64 work then runs in full warps however
// sparsely the candidates lie among the faces.
__global__ void __launch_bounds__(kBlock) k_plane_slots(Problem P, const uint8_t* __restrict__ cand,
    uint32_t* __restrict__ plane_slot, uint64_t plane_cap, uint32_t* __restrict__ counters,
    uint32_t* __restrict__ slot_face, uint32_t* __restrict__ proj_flag)
{
    for (uint32_t f0 = blockIdx.x * blockDim.x; f0 < P.nf; f0 += gridDim.x * blockDim.x) {
        const uint32_t f = f0 + threadIdx.x;
        const bool c = f < P.nf && cand[f] != 0;
        const uint32_t slot = warp_append(&counters[3], c);
        if (!c) continue;
        plane_slot[f] = slot;
        if (slot >= plane_cap) continue;
        slot_face[slot] = f;
        proj_flag[slot] = 0u; // the narrow phase queues the slot's projection once
    }
}

__global__ void __launch_bounds__(kBlock, MCGPU_PL_MINB) k_planes(Problem P, const uint32_t* __restrict__ slot_face,
    FacePlane* __restrict__ planes, uint64_t plane_cap, uint32_t* __restrict__ counters,
    uint32_t* __restrict__ poly_list, int32_t* __restrict__ pair_bad)
{
    const uint32_t nslots = (uint32_t)min((uint64_t)counters[3], plane_cap);
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < nslots; slot += gridDim.x * blockDim.x) {
        const uint32_t f = slot_face[slot];
        const uint32_t o = face_o(P, f), n = face_n(P, f), rot = face_rot(P, f);
        // Newell's normal over the rotated vertex list
        double nx = 0.0, ny = 0.0, nz = 0.0;
        double cur[3], nxt[3], first[3];
        load_v(P, face_vertex(P, o, n, 0, rot), first);
        cur[0] = first[0]; cur[1] = first[1]; cur[2] = first[2];
        for (uint32_t k = 0; k < n; ++k) {
            if (k + 1 < n) load_v(P, face_vertex(P, o, n, k + 1, rot), nxt);
            else { nxt[0] = first[0]; nxt[1] = first[1]; nxt[2] = first[2]; }
            nx = nx + (cur[1] - nxt[1]) * (cur[2] + nxt[2]);
            ny = ny + (cur[2] - nxt[2]) * (cur[0] + nxt[0]);
            nz = nz + (cur[0] - nxt[0]) * (cur[1] + nxt[1]);
            cur[0] = nxt[0]; cur[1] = nxt[1]; cur[2] = nxt[2];
        }
        FacePlane pl;
        const double nn[3] = { nx, ny, nz };
        const double sq = dot3(nn, nn);
        const uint32_t p = P.face_pair[f] & ~kCutBit;
        if (isnan(nx) || isnan(ny) || isnan(nz) || sq < 1e-9 || sq == 0.0) {
            atomicMin(&pair_bad[p], (int32_t)(f - P.pair_fbase[p]));
            pl.tri[0] = -1;
            planes[slot] = pl;
            continue;
        }
        pl.tri[0] = 0; pl.tri[1] = 1; pl.tri[2] = 2;
        pl.n[0] = nx; pl.n[1] = ny; pl.n[2] = nz;
        if (n == 3) {
            // a triangle keeps its raw Newell normal: the unit normal, d, the
            // largest component and the projection are only needed if a
            // segment meets its plane (k_finish_planes, once per such face)
            planes[slot] = pl;
            continue;
        }
        finish_plane(pl, first);
        // the triplet ranking of polygons needs the projection now
        projection_matrix(pl.n, pl.mc, pl.P);
        planes[slot] = pl;
        if (n > 3) {
            const uint32_t k = atomicAdd(&counters[4], 1u);
            poly_list[k] = f;
        }
    }
}

// ---------------------------------------------------------------------------
// plane-defining triplet of polygons with > 3 vertices
// (determine_three_noncollinear_vertices, math.cpp:289-389): every triplet's
// orient2d value in the projected frame, the first after libstdc++'s
// std::sort by |value| descending (its introsort + insertion-sort schedule
// decides ties, so it is replayed), entries in global scratch.
// ---------------------------------------------------------------------------
struct Trip { double v; int i, j, k, pad; };
__device__ __forceinline__ bool tless(const Trip& a, const Trip& b) { return fabs(a.v) > fabs(b.v); }
__device__ void t_swap(Trip* a, Trip* b) { Trip t = *a; *a = *b; *b = t; }
__device__ void t_ins_sort(Trip* f, long n)
{
    for (long i = 1; i < n; ++i) {
        Trip v = f[i];
        if (tless(v, f[0])) {
            for (long j = i; j > 0; --j) f[j] = f[j - 1];
            f[0] = v;
        } else {
            long j = i;
            while (tless(v, f[j - 1])) { f[j] = f[j - 1]; --j; }
            f[j] = v;
        }
    }
}
__device__ void t_unguarded_ins(Trip* f, long from, long n)
{
    for (long i = from; i < n; ++i) {
        Trip v = f[i];
        long j = i;
        while (tless(v, f[j - 1])) { f[j] = f[j - 1]; --j; }
        f[j] = v;
    }
}
__device__ void t_median(Trip* r, Trip* a, Trip* b, Trip* c)
{
    if (tless(*a, *b)) {
        if (tless(*b, *c)) t_swap(r, b);
        else if (tless(*a, *c)) t_swap(r, c);
        else t_swap(r, a);
    } else if (tless(*a, *c)) t_swap(r, a);
    else if (tless(*b, *c)) t_swap(r, c);
    else t_swap(r, b);
}
__device__ void t_sift(Trip* f, long hole, long len, Trip v)
{
    const long top = hole;
    long child = hole;
    while (child < (len - 1) / 2) {
        child = 2 * (child + 1);
        if (tless(f[child], f[child - 1])) child--;
        f[hole] = f[child];
        hole = child;
    }
    if ((len & 1) == 0 && child == (len - 2) / 2) {
        child = 2 * (child + 1);
        f[hole] = f[child - 1];
        hole = child - 1;
    }
    long par = (hole - 1) / 2;
    while (hole > top && tless(f[par], v)) {
        f[hole] = f[par];
        hole = par;
        par = (hole - 1) / 2;
    }
    f[hole] = v;
}
__device__ void t_heap_sort(Trip* f, long n)
{
    if (n < 2) return;
    for (long par = (n - 2) / 2;; --par) {
        t_sift(f, par, n, f[par]);
        if (par == 0) break;
    }
    for (long last = n - 1; last > 0; --last) {
        Trip v = f[last];
        f[last] = f[0];
        t_sift(f, 0, last, v);
    }
}
__device__ void t_std_sort(Trip* f, long n)
{
    if (n < 2) return;
    // introsort loop, iterative on the left part, explicit stack for the right parts
    struct Seg { long off, n; int depth; };
    Seg st[64];
    int sp = 0;
    int depth0 = 2 * (63 - __clzll((long long)n));
    long off = 0, len = n;
    int depth = depth0;
    for (;;) {
        while (len > 16) {
            if (depth == 0) { t_heap_sort(f + off, len); len = 0; break; }
            --depth;
            Trip* g = f + off;
            const long mid = len / 2;
            t_median(&g[0], &g[1], &g[mid], &g[len - 1]);
            long lo = 1, hi = len;
            for (;;) {
                while (tless(g[lo], g[0])) ++lo;
                --hi;
                while (tless(g[0], g[hi])) --hi;
                if (!(lo < hi)) break;
                t_swap(&g[lo], &g[hi]);
                ++lo;
            }
            // the reference recurses into [lo, len) first, then loops on [0, lo)
            if (sp < 64) st[sp++] = Seg { off + lo, len - lo, depth };
            len = lo;
        }
        // left part done (len <= 16 is left for the final insertion sort);
        // continue with the most recently deferred right part -- the
        // recursion order does not change the result, each segment is
        // partitioned independently
        if (sp == 0) break;
        --sp;
        off = st[sp].off;
        len = st[sp].n;
        depth = st[sp].depth;
    }
    if (n > 16) {
        t_ins_sort(f, 16);
        t_unguarded_ins(f, 16, n);
    } else {
        t_ins_sort(f, n);
    }
}

__global__ void k_triplets(Problem P, const uint32_t* __restrict__ poly_list, const uint32_t* __restrict__ counters,
    const uint32_t* __restrict__ plane_slot, FacePlane* __restrict__ planes, Trip* __restrict__ scratch,
    uint64_t scratch_cap, uint64_t stride, uint32_t* __restrict__ pair_status)
{
    const uint32_t npoly = counters[4];
    for (uint32_t t = blockIdx.x * blockDim.x + threadIdx.x; t < npoly; t += gridDim.x * blockDim.x) {
        const uint32_t f = poly_list[t];
        FacePlane& pl = planes[plane_slot[f]];
        const uint32_t o = face_o(P, f), n = face_n(P, f), rot = face_rot(P, f);
        // scratch: one region of `stride` triplets (the largest polygon's count) per polygon
        const uint64_t per = (uint64_t)n * (n - 1) * (n - 2) / 6;
        const uint64_t base = (uint64_t)t * stride;
        if (base + per > scratch_cap || per == 0) {
            atomicOr(&pair_status[P.face_pair[f] & ~kCutBit], ST_INVALID);
            pl.tri[0] = -1;
            continue;
        }
        Trip* tr = scratch + base;
        long m = 0;
        for (uint32_t i = 0; i < n; ++i) {
            double vi[3], xi[2];
            load_v(P, face_vertex(P, o, n, i, rot), vi);
            project2(pl.P, vi, xi);
            for (uint32_t j = i + 1; j < n; ++j) {
                double vj[3], xj[2];
                load_v(P, face_vertex(P, o, n, j, rot), vj);
                project2(pl.P, vj, xj);
                for (uint32_t k = j + 1; k < n; ++k) {
                    double vk[3], xk[2];
                    load_v(P, face_vertex(P, o, n, k, rot), vk);
                    project2(pl.P, vk, xk);
                    const double r = orient2d(xi, xj, xk);
                    if (!(r == 0.0)) tr[m++] = Trip { r, (int)i, (int)j, (int)k, 0 };
                }
            }
        }
        if (m == 0) { pl.tri[0] = -1; continue; }
        t_std_sort(tr, m);
        pl.tri[0] = tr[0].i; pl.tri[1] = tr[0].j; pl.tri[2] = tr[0].k;
    }
}

// ---------------------------------------------------------------------------
// candidate pair -> culled edge-face tests (kernel.cpp:1781-2177)
//
// The reference tests each edge of a candidate face against the union of the
// partners of the (up to two) candidate faces containing it. Here every pair
// (s, c) proposes (edge of s, c) and (edge of c, s); the proposal is dropped
// when the edge's other face F' is lower-numbered and also a partner of the
// tested face -- and "partner" is exactly "face boxes overlap" (the pair set
// is all overlapping face-box pairs), so no pair lookup is needed. Edge boxes
// cull as kernel.cpp:2074-2177 does.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t other_face(const Problem& P, const uint32_t* __restrict__ voff,
    const uint32_t* __restrict__ vface, uint32_t K, uint32_t F, uint32_t a, uint32_t b, uint32_t& slot_out)
{
    // faces incident to a that hold the halfedge b -> a: CSR lists (K == 0),
    // or K slots per vertex with voff[a] the count
    uint64_t lo, hi;
    if (K) {
        lo = (uint64_t)a * K;
        hi = lo + min(voff[a], K);
    } else {
        lo = voff[a];
        hi = voff[a + 1];
    }
    for (uint64_t i = lo; i < hi; ++i) {
        const uint32_t G = vface[i];
        if (G == F) continue;
        const uint32_t o = face_o(P, G), n = face_n(P, G);
        for (uint32_t k = 0; k < n; ++k) {
            const uint32_t x = P.fidx[o + k];
            const uint32_t y = P.fidx[o + (k + 1 == n ? 0 : k + 1)];
            if (x == b && y == a) { slot_out = o + k; return G; }
        }
    }
    return kNone;
}

__global__ void __launch_bounds__(kBlock) k_pair_tests(Problem P, const double* __restrict__ fbox,
    const unsigned long long* __restrict__ pairs, const uint32_t* __restrict__ counters_ro, uint64_t pair_cap,
    const uint32_t* __restrict__ voff, const uint32_t* __restrict__ vface, uint32_t inc_slots, Test* __restrict__ tests,
    uint64_t test_cap, uint32_t* __restrict__ counters, const int32_t* __restrict__ pair_bad,
    uint32_t* __restrict__ pair_status, uint32_t* __restrict__ pair_cnt)
{
    __shared__ uint32_t s_nmax;
    const uint64_t np = min((uint64_t)counters_ro[0], pair_cap);
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x; i0 < np; i0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = i0 + threadIdx.x;
        bool live = i < np;
        uint32_t sface = 0, cface = 0, p = 0;
        if (live) {
            const unsigned long long pr = pairs[i];
            sface = (uint32_t)(pr >> 32);
            cface = (uint32_t)pr;
            p = P.face_pair[sface] & ~kCutBit;
        }
        if (pair_cnt) {
            const uint32_t one[1] = { 1u };
            pair_add<1>(pair_cnt, live ? p : kNone, 0, one);
        }
        if (live) live = pair_bad[p] == kNoBad; // the reference stops before the narrow phase
        // edges of the source face against the cut face, then the reverse;
        // the loop runs to the block's longest face so every thread reaches
        // each block_append
        uint32_t ns = live ? face_n(P, sface) : 0u, nc = live ? face_n(P, cface) : 0u;
        if (P.all_triangles) {
            if (threadIdx.x == 0) s_nmax = 3;
        } else {
            if (threadIdx.x == 0) s_nmax = 0;
            __syncthreads();
            atomicMax(&s_nmax, max(ns, nc));
        }
        __syncthreads();
        const uint32_t nmax = s_nmax;
        __syncthreads();
        for (int side = 0; side < 2; ++side) {
            const uint32_t F = side == 0 ? sface : cface;
            const uint32_t g = side == 0 ? cface : sface;
            const uint32_t n = side == 0 ? ns : nc;
            Box gb;
            if (live) gb = load_box(fbox, g);
            const uint32_t o = live ? face_o(P, F) : 0u;
            for (uint32_t k = 0; k < nmax; ++k) {
                bool emit = k < n;
                uint32_t a = 0, b = 0, oslot = kNone, G = kNone;
                if (emit) {
                    a = P.fidx[o + k];
                    b = P.fidx[o + (k + 1 == n ? 0 : k + 1)];
                    G = other_face(P, voff, vface, inc_slots, F, a, b, oslot);
                    if (G != kNone && G < F && box_overlap(load_box(fbox, G), gb)) emit = false;
                }
                if (emit) {
                    double xa[3], xb[3];
                    load_v(P, a, xa);
                    load_v(P, b, xb);
                    Box eb;
                    for (int j = 0; j < 3; ++j) {
                        eb.mx[j] = dmax_ref(dmax_ref(-1.7976931348623157e308, xa[j]), xb[j]);
                        eb.mn[j] = dmin_ref(dmin_ref(1.7976931348623157e308, xa[j]), xb[j]);
                    }
                    emit = box_overlap(eb, gb);
                }
                const uint32_t pos = warp_append(&counters[1], emit);
                if (!emit) continue;
                if (pos >= test_cap) { atomicOr(&pair_status[p], ST_OVERFLOW_TESTS); continue; }
                Test t;
                t.g = g;
                if (G != kNone && G < F) {
                    t.q = b; t.r = a; t.f0 = G; t.f1 = F; t.slot = oslot;
                } else {
                    t.q = a; t.r = b; t.f0 = F; t.f1 = G; t.slot = o + k;
                }
                tests[pos] = t;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// narrow phase (kernel.cpp:2456-2658; math.cpp:249-287, 391-427, 643-703, 851-902)
// ---------------------------------------------------------------------------
__device__ char pip_face(const Problem& P, const double* Pm, uint32_t o, uint32_t n, uint32_t rot, const double* pt)
{
    double q[2];
    project2(Pm, pt, q);
    int rc = 0, lc = 0;
    double prv[2];
    {
        double v[3];
        load_v(P, face_vertex(P, o, n, n - 1, rot), v);
        project2(Pm, v, prv);
    }
    for (uint32_t i = 0; i < n; ++i) {
        double v[3], c[2];
        load_v(P, face_vertex(P, o, n, i, rot), v);
        project2(Pm, v, c);
        const double xi = c[0] - q[0], yi = c[1] - q[1];
        if (xi == 0.0 && yi == 0.0) return 'v';
        const double xl = prv[0] - q[0], yl = prv[1] - q[1];
        const bool rs = (yi > 0.0) != (yl > 0.0);
        const bool ls = (yi < 0.0) != (yl < 0.0);
        if (rs || ls) {
            const double x = (xi * yl - xl * yi) / (yl - yi);
            if (rs && x > 0.0) rc++;
            if (ls && x < 0.0) lc++;
        }
        prv[0] = c[0]; prv[1] = c[1];
    }
    if ((rc & 1) != (lc & 1)) return 'e';
    return (rc & 1) ? 'i' : 'o';
}

// Narrow phase, pass 1 (every culled test): both orient3d signs and the
// type char (compute_segment_plane_intersection_type, math.cpp:391-427).
// Tests whose segment meets the plane ('1', 'q', 'r', 'p') go to a compact
// hit list for pass 2, so its fp64 work runs on full warps.
#ifndef MCGPU_NS_MINB
#define MCGPU_NS_MINB 2
#endif
__global__ void __launch_bounds__(kBlock, MCGPU_NS_MINB) k_narrow_signs(Problem P, const Test* __restrict__ tests,
    const uint32_t* __restrict__ counters_ro, uint64_t test_cap, const uint32_t* __restrict__ plane_slot,
    const FacePlane* __restrict__ planes, int keep_tests, int8_t* __restrict__ test_info, uint2* __restrict__ hits,
    uint32_t* __restrict__ proj_flag, uint32_t* __restrict__ proj_list, uint32_t* __restrict__ counters,
    uint32_t* __restrict__ pair_cnt)
{
    const uint64_t nt = min((uint64_t)counters_ro[1], test_cap);
    uint32_t esc[3] = { 0, 0, 0 };
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x; i0 < nt; i0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t i = i0 + threadIdx.x;
        bool hit = false, first_hit = false;
        uint32_t code = 0, slot = 0;
        uint32_t e[3] = { 0, 0, 0 }; // this test's signs by deciding stage
        uint32_t pid = kNone;
        if (i < nt) {
            const Test t = tests[i];
            if (pair_cnt) pid = P.face_pair[t.g] & ~kCutBit;
            const uint32_t o = face_o(P, t.g), n = face_n(P, t.g);
            // a triangle's plane-defining vertices are its own three (a
            // degenerate triangle makes its whole pair degenerate, and the hit
            // pass drops that pair's results); a polygon's come from k_triplets
            int t0 = 0, t1 = 1, t2 = 2;
            if (n != 3) {
                const int* tri = planes[plane_slot[t.g]].tri;
                t0 = tri[0];
                t1 = tri[1];
                t2 = tri[2];
            }
            int8_t sq = 0, sr = 0;
            char type = '0';
            if (t0 >= 0) {
                const uint32_t rot = face_rot(P, t.g);
                const uint32_t va = face_vertex(P, o, n, t0, rot), vb = face_vertex(P, o, n, t1, rot),
                               vc = face_vertex(P, o, n, t2, rot);
                // the fp32-vertex filter first; the fp64 coordinates only for
                // the signs it leaves undecided
                int dq = 0, dr = 0;
                if (P.X32) {
                    const float4 fa = P.X32[va], fb = P.X32[vb], fc = P.X32[vc];
                    dq = orient3d_sign_f32v(fa, fb, fc, P.X32[t.q]);
                    dr = orient3d_sign_f32v(fa, fb, fc, P.X32[t.r]);
                    e[ESC_F32] += (dq != 0) + (dr != 0);
                }
                sq = (int8_t)dq;
                sr = (int8_t)dr;
                if (dq == 0 || dr == 0) {
                    double a[3], b[3], c[3], x[3];
                    load_v(P, va, a);
                    load_v(P, vb, b);
                    load_v(P, vc, c);
                    int st;
                    if (dq == 0) {
                        load_v(P, t.q, x);
                        sq = (int8_t)orient3d_sign_filtered(a, b, c, x, st);
                        e[st]++;
                    }
                    if (dr == 0) {
                        load_v(P, t.r, x);
                        sr = (int8_t)orient3d_sign_filtered(a, b, c, x, st);
                        e[st]++;
                    }
                }
                if (sq == 0 && sr == 0) type = 'p';
                else if (sq == 0) type = 'q';
                else if (sr == 0) type = 'r';
                else if ((sr < 0 && sq < 0) || (sr > 0 && sq > 0)) type = '0';
                else type = '1';
            }
            code = (uint32_t)(uint8_t)sq | ((uint32_t)(uint8_t)sr << 8) | ((uint32_t)(uint8_t)type << 16);
            hit = type != '0';
            if (!hit && keep_tests) reinterpret_cast<char4*>(test_info)[i] = make_char4(sq, sr, type, 0);
            // the first hit on a triangle queues the rest of its plane
            if (hit && n == 3) {
                first_hit = atomicExch(&proj_flag[plane_slot[t.g]], 1u) == 0u;
                slot = t.g;
            }
        }
        const uint32_t pos = warp_append(&counters[10], hit);
        if (hit && pos < test_cap) hits[pos] = make_uint2((uint32_t)i, code);
        const uint32_t k = warp_append(&counters[11], first_hit);
        if (first_hit) proj_list[k] = slot;
        for (int j = 0; j < 3; ++j) esc[j] += e[j];
        if (pair_cnt) {
            const uint32_t v[4] = { 1u, e[0], e[1], e[2] };
            pair_add<4>(pair_cnt, pid, 1, v);
        }
    }
    for (int k = 0; k < 3; ++k) {
        uint32_t v = esc[k];
        for (int off = 16; off; off >>= 1) v += __shfl_down_sync(0xFFFFFFFFu, v, off);
        if ((threadIdx.x & 31) == 0 && v) atomicAdd(&counters[5 + k], v);
    }
}

// The triangles that pass 1 queued (a segment meets their plane): unit
// normal, d, largest component and projection matrix, once per face
// (polygons got theirs with the plane).
// Narrow-phase kernels over short lists run long fp64 chains per item: the
// hit triangles' plane finishing is launched in blocks of kSpread threads so
// that a list of a few thousand items still occupies every SM (the hit list
// itself does best in blocks of 256, measured).
constexpr int kSpread = 64;
#ifndef MCGPU_NH_BLOCK
#define MCGPU_NH_BLOCK 256
#endif
constexpr int kNarrowHitsBlock = MCGPU_NH_BLOCK;
__global__ void __launch_bounds__(kSpread) k_finish_planes(Problem P, FacePlane* __restrict__ planes,
    const uint32_t* __restrict__ plane_slot, const uint32_t* __restrict__ proj_list,
    const uint32_t* __restrict__ counters)
{
    const uint32_t n = counters[11];
    for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < n; k += gridDim.x * blockDim.x) {
        const uint32_t f = proj_list[k];
        FacePlane& plr = planes[plane_slot[f]];
        FacePlane pl = plr;
        double first[3];
        load_v(P, face_vertex(P, face_o(P, f), 3, 0, face_rot(P, f)), first);
        finish_plane(pl, first);
        projection_matrix(pl.n, pl.mc, pl.P);
        plr = pl;
    }
}

// Narrow phase, pass 2 (the hit list): segment-plane point
// (compute_segment_plane_intersection, math.cpp:249-287), point-in-polygon
// (math.cpp:851-902), general-position violations and records
// (kernel.cpp:2456-2658).
#ifndef MCGPU_NH_MINB
#define MCGPU_NH_MINB 1
#endif
__global__ void __launch_bounds__(kNarrowHitsBlock, MCGPU_NH_MINB) k_narrow_hits(Problem P, const Test* __restrict__ tests,
    const uint2* __restrict__ hits, uint64_t test_cap, const uint32_t* __restrict__ plane_slot,
    const FacePlane* __restrict__ planes, int keep_tests, int8_t* __restrict__ test_info,
    unsigned long long* __restrict__ rec_key, uint32_t* __restrict__ rec_val, double* __restrict__ rec_pt,
    uint32_t* __restrict__ counters, uint32_t* __restrict__ pair_status, const int32_t* __restrict__ pair_bad)
{
    const uint64_t nh = min((uint64_t)counters[10], test_cap);
    for (uint64_t h0 = blockIdx.x * (uint64_t)blockDim.x; h0 < nh; h0 += (uint64_t)gridDim.x * blockDim.x) {
        const uint64_t h = h0 + threadIdx.x;
        bool rec = false;
        Test t;
        uint32_t i = 0;
        double pt[3] = { 0.0, 0.0, 0.0 };
        if (h < nh) {
            const uint2 hv = hits[h];
            i = hv.x;
            const int8_t sq = (int8_t)(hv.y & 0xFFu), sr = (int8_t)((hv.y >> 8) & 0xFFu);
            const char type = (char)((hv.y >> 16) & 0xFFu);
            t = tests[i];
            const FacePlane pl = planes[plane_slot[t.g]];
            const uint32_t o = face_o(P, t.g), n = face_n(P, t.g), rot = face_rot(P, t.g);
            const double* Pm = pl.P;
            double q[3], r[3];
            load_v(P, t.q, q);
            load_v(P, t.r, r);
            char pip = 0;
            if (type == 'q' || type == 'r') {
                pip = pip_face(P, Pm, o, n, rot, type == 'q' ? q : r);
            } else if (type == 'p') {
                pip = pip_face(P, Pm, o, n, rot, q);
                if (!(pip == 'i' || pip == 'v' || pip == 'e')) pip = pip_face(P, Pm, o, n, rot, r);
            } else {
                const double num = pl.d - dot3(q, pl.n);
                const double rq[3] = { r[0] - q[0], r[1] - q[1], r[2] - q[2] };
                const double den = dot3(rq, pl.n);
                if (!(den == 0.0)) {
                    const double tt = num / den;
                    for (int k = 0; k < 3; ++k) pt[k] = q[k] + tt * (r[k] - q[k]);
                }
                pip = pip_face(P, Pm, o, n, rot, pt);
                rec = pip == 'i';
            }
            const uint32_t p = P.face_pair[t.g] & ~kCutBit;
            if (pair_bad[p] != kNoBad) {
                // a pair with a degenerate face has no narrow phase (the reference
                // stops before it): no records, no flags
                rec = false;
                pip = 0;
            } else if (((type == 'q' || type == 'r' || type == 'p') && (pip == 'i' || pip == 'v' || pip == 'e'))
                || (type == '1' && (pip == 'v' || pip == 'e'))) {
                if (!(*(volatile uint32_t*)&pair_status[p] & ST_GP)) atomicOr(&pair_status[p], ST_GP);
            }
            if (keep_tests) reinterpret_cast<char4*>(test_info)[i] = make_char4(sq, sr, type, pip);
        }
        const uint32_t pos = warp_append(&counters[2], rec);
        if (rec) {
            rec_key[pos] = ((unsigned long long)t.slot << 32) | t.g;
            rec_val[pos] = i;
            rec_pt[(size_t)i * 3 + 0] = pt[0];
            rec_pt[(size_t)i * 3 + 1] = pt[1];
            rec_pt[(size_t)i * 3 + 2] = pt[2];
        }
    }
}

// records: (slot << 32 | face) -> (slot << gbits | face)
__global__ void __launch_bounds__(kBlock) k_record_pack(unsigned long long* __restrict__ rec_key, uint32_t nrec,
    int gbits)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nrec; i += gridDim.x * blockDim.x) {
        const unsigned long long k = rec_key[i];
        rec_key[i] = ((k >> 32) << gbits) | (k & 0xFFFFFFFFull);
    }
}

// first sorted record of every pair (and the total at n_pairs): the records
// are grouped by pair, so a binary search over the sorted keys finds them
// record count: the host's, or (ndev) the device's when it is within cap (else 0)
__device__ __forceinline__ uint32_t record_count(uint32_t n, const uint32_t* ndev, uint32_t cap)
{
    if (!ndev) return n;
    const uint32_t v = *ndev;
    return v <= cap ? v : 0u;
}

__global__ void __launch_bounds__(kBlock) k_pair_record_ranges(Problem P, const unsigned long long* __restrict__ key,
    uint32_t nrec_host, const uint32_t* __restrict__ ndev, uint32_t cap, int gbits, uint32_t* __restrict__ rec_begin)
{
    const uint32_t nrec = record_count(nrec_host, ndev, cap);
    const unsigned long long gmask = (1ull << gbits) - 1ull;
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p <= P.n_pairs; p += gridDim.x * blockDim.x) {
        uint32_t lo = 0, hi = nrec;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            const uint32_t mp = P.face_pair[(uint32_t)(key[mid] & gmask)] & ~kCutBit;
            if (mp < p) lo = mid + 1; else hi = mid;
        }
        rec_begin[p] = lo;
    }
}

// Record order in two steps. k_sort_slices sorts each slice of kRankChunk
// (key, value) pairs in place, in shared memory (bitonic network; padding
// keys are all ones and sort last). k_rank_records then gives every record
// its rank among all keys (unique: one record per (edge, face)): block (x, y)
// stages sorted slice y in shared memory and each of its 256 records counts
// the slice's smaller keys by binary search, adding the count into rank[].
// The scatter that follows moves each record to its rank.
#ifndef MCGPU_RANK_CHUNK
#define MCGPU_RANK_CHUNK 512
#endif
constexpr int kRankChunk = MCGPU_RANK_CHUNK;
static_assert((kRankChunk & (kRankChunk - 1)) == 0 && kRankChunk == 2 * kBlock, "one compare-exchange per thread");
__global__ void __launch_bounds__(kBlock) k_sort_slices(unsigned long long* __restrict__ key, uint32_t* __restrict__ val,
    uint32_t n_host, const uint32_t* __restrict__ ndev, uint32_t cap)
{
    __shared__ unsigned long long sk[kRankChunk];
    __shared__ uint32_t sv[kRankChunk];
    const uint32_t n = record_count(n_host, ndev, cap);
    const uint32_t lo = blockIdx.x * kRankChunk;
    if (lo >= n) return; // grids sized for a capacity
    const uint32_t m = min(n - lo, (uint32_t)kRankChunk);
    for (uint32_t j = threadIdx.x; j < kRankChunk; j += kBlock) {
        sk[j] = j < m ? key[lo + j] : ~0ull;
        sv[j] = j < m ? val[lo + j] : 0u;
    }
    __syncthreads();
    for (uint32_t size = 2; size <= (uint32_t)kRankChunk; size <<= 1) {
        for (uint32_t stride = size >> 1; stride > 0; stride >>= 1) {
            // thread t compares element a with its partner a + stride
            const uint32_t t = threadIdx.x;
            const uint32_t a = 2 * t - (t & (stride - 1));
            const uint32_t b = a + stride;
            const bool up = (a & size) == 0;
            const unsigned long long ka = sk[a], kb = sk[b];
            if ((ka > kb) == up) {
                sk[a] = kb;
                sk[b] = ka;
                const uint32_t v = sv[a];
                sv[a] = sv[b];
                sv[b] = v;
            }
            __syncthreads();
        }
    }
    for (uint32_t j = threadIdx.x; j < m; j += kBlock) {
        key[lo + j] = sk[j];
        val[lo + j] = sv[j];
    }
}

__global__ void __launch_bounds__(kBlock) k_rank_records(const unsigned long long* __restrict__ key, uint32_t n_host,
    const uint32_t* __restrict__ ndev, uint32_t cap, uint32_t* __restrict__ rank)
{
    __shared__ unsigned long long sk[kRankChunk];
    const uint32_t n = record_count(n_host, ndev, cap);
    const uint32_t lo = blockIdx.y * kRankChunk;
    if (lo >= n || blockIdx.x * kBlock >= n) return; // grids sized for a capacity
    const uint32_t m = min(n, lo + kRankChunk) - lo;
    for (uint32_t j = threadIdx.x; j < m; j += kBlock) sk[j] = key[lo + j];
    __syncthreads();
    const uint32_t i = blockIdx.x * kBlock + threadIdx.x;
    if (i >= n) return;
    const unsigned long long k = key[i];
    uint32_t a = 0, b = m; // the slice's keys below k: lower bound in the sorted slice
    while (a < b) {
        const uint32_t mid = (a + b) >> 1;
        if (sk[mid] < k) a = mid + 1; else b = mid;
    }
    if (a) atomicAdd(&rank[i], a);
}

// records in rank order -> sorted keys and output arrays with per-pair local ids
__global__ void __launch_bounds__(kBlock) k_scatter_records(Problem P, const unsigned long long* __restrict__ key,
    const uint32_t* __restrict__ val, const uint32_t* __restrict__ rank, uint32_t nrec_host,
    const uint32_t* __restrict__ ndev, uint32_t cap, const Test* __restrict__ tests, const double* __restrict__ rec_pt,
    unsigned long long* __restrict__ skey, uint32_t* __restrict__ rec_ids, double* __restrict__ rec_pts)
{
    const uint32_t nrec = record_count(nrec_host, ndev, cap);
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nrec; i += gridDim.x * blockDim.x) {
        const uint32_t r = rank[i];
        const uint32_t ti = val[i];
        skey[r] = key[i];
        const Test t = tests[ti];
        const uint32_t p = P.face_pair[t.g] & ~kCutBit;
        const uint32_t vb = P.pair_vbase[p], fb = P.pair_fbase[p];
        rec_ids[(size_t)r * 5 + 0] = t.q - vb;
        rec_ids[(size_t)r * 5 + 1] = t.r - vb;
        rec_ids[(size_t)r * 5 + 2] = t.g - fb;
        rec_ids[(size_t)r * 5 + 3] = t.f0 - fb;
        rec_ids[(size_t)r * 5 + 4] = t.f1 == kNone ? kNone : t.f1 - fb;
        rec_pts[(size_t)r * 3 + 0] = rec_pt[(size_t)ti * 3 + 0];
        rec_pts[(size_t)r * 3 + 1] = rec_pt[(size_t)ti * 3 + 1];
        rec_pts[(size_t)r * 3 + 2] = rec_pt[(size_t)ti * 3 + 2];
    }
}

// sorted record order -> output arrays with per-pair local ids
__global__ void __launch_bounds__(kBlock) k_gather_records(Problem P, const uint32_t* __restrict__ order,
    uint32_t nrec, const Test* __restrict__ tests, const double* __restrict__ rec_pt, uint32_t* __restrict__ rec_ids,
    double* __restrict__ rec_pts)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nrec; i += gridDim.x * blockDim.x) {
        const uint32_t ti = order[i];
        const Test t = tests[ti];
        const uint32_t p = P.face_pair[t.g] & ~kCutBit;
        const uint32_t vb = P.pair_vbase[p], fb = P.pair_fbase[p];
        rec_ids[(size_t)i * 5 + 0] = t.q - vb;
        rec_ids[(size_t)i * 5 + 1] = t.r - vb;
        rec_ids[(size_t)i * 5 + 2] = t.g - fb;
        rec_ids[(size_t)i * 5 + 3] = t.f0 - fb;
        rec_ids[(size_t)i * 5 + 4] = t.f1 == kNone ? kNone : t.f1 - fb;
        rec_pts[(size_t)i * 3 + 0] = rec_pt[(size_t)ti * 3 + 0];
        rec_pts[(size_t)i * 3 + 1] = rec_pt[(size_t)ti * 3 + 1];
        rec_pts[(size_t)i * 3 + 2] = rec_pt[(size_t)ti * 3 + 2];
    }
}

// clear status bits of every pair (a rerun of a stage clears that stage's own
// bits and keeps the others, e.g. the bounds kernel's ST_INVALID)
__global__ void k_clear_status(uint32_t* __restrict__ st, uint32_t n, uint32_t mask)
{
    for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x) st[p] &= ~mask;
}

static int sm_count()
{
    static int sms = 0;
    if (!sms) {
        int dev = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        if (sms <= 0) sms = 148;
    }
    return sms;
}

int grid_for(uint64_t n)
{
    const uint64_t want = (n + kBlock - 1) / kBlock;
    const uint64_t cap = (uint64_t)sm_count() * 8;
    return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

// blocks of kSpread threads for n items, at most 32 per SM
int grid_spread(uint64_t n)
{
    const uint64_t want = (n + kSpread - 1) / kSpread;
    const uint64_t cap = (uint64_t)sm_count() * 32;
    return (int)(want < 1 ? 1 : (want > cap ? cap : want));
}

} // namespace

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
void launch_bounds_morton(const Problem& P, const Problem& Pin, Work& W, bool wide, int key_bits, cudaStream_t s)
{
    float4* frame = reinterpret_cast<float4*>(W.mesh_frame);
    g_launches += 3;
    k_vertex_bounds<<<grid_for(P.nv / kBoundsItems + 1), kBlock, 0, s>>>(P, W.mesh_box, W.x32, W.hx_src, W.hx_cut,
        W.hx_out, W.x_raw, W.raw_float, W.frames);
    k_mesh_frames<<<(2 * P.n_pairs + 255) / 256, 256, 0, s>>>(W.mesh_box, 2 * P.n_pairs, frame);
    const int g = grid_for(P.nf);
    if (wide)
        k_face_bounds<unsigned long long><<<g, kBlock, 0, s>>>(Pin, W.fbox, W.fbox32, frame,
            (unsigned long long*)W.skeys[0], W.svals[0], (unsigned long long*)W.ckeys[0], W.cvals[0], key_bits,
            W.pair_status, W.cand, W.fidx_out, W.face_pair_out, W.fidx_fix);
    else
        k_face_bounds<uint32_t><<<g, kBlock, 0, s>>>(Pin, W.fbox, W.fbox32, frame, (uint32_t*)W.skeys[0], W.svals[0],
            (uint32_t*)W.ckeys[0], W.cvals[0], key_bits, W.pair_status, W.cand, W.fidx_out, W.face_pair_out,
            W.fidx_fix);
}

int launch_sort(const Problem& P, Work& W, bool wide, int key_bits, cudaStream_t s, int& cut_buf)
{
    // source and cut keys sit back to back (ckeys[b] == skeys[b] + ns) and the
    // mesh bit above the key orders them apart: one sort for both meshes
    const uint32_t n = P.ns + P.nc;
    int buf;
    if (wide)
        buf = radix_sort_pairs<unsigned long long>((unsigned long long*)W.skeys[0], W.svals[0],
            (unsigned long long*)W.skeys[1], W.svals[1], n, 0, key_bits + 1, W.sort_temp, s);
    else
        buf = radix_sort_pairs<uint32_t>((uint32_t*)W.skeys[0], W.svals[0], (uint32_t*)W.skeys[1], W.svals[1], n, 0,
            key_bits + 1, W.sort_temp, s);
    cut_buf = buf;
    return buf;
}

void launch_hierarchy(const Problem& P, Work& W, bool wide, int cut_buf, cudaStream_t s)
{
    const int n = (int)P.ncl;
    const int gc = grid_for(n);
    g_launches++;
    if (wide)
        k_clusters<unsigned long long><<<gc, kBlock, 0, s>>>(P, (const unsigned long long*)W.ckeys[cut_buf],
            (unsigned long long*)W.cl_key, W.cl_start, W.cl_n, W.split_far);
    else
        k_clusters<uint32_t><<<gc, kBlock, 0, s>>>(P, (const uint32_t*)W.ckeys[cut_buf], (uint32_t*)W.cl_key,
            W.cl_start, W.cl_n, W.split_far);
    if (n < 2) return;
    g_launches++;
    const int g = (n + kRefitWin - 1) / kRefitWin;
    if (wide)
        k_build<unsigned long long><<<g, kRefitWin, 0, s>>>(P, (const unsigned long long*)W.cl_key, n, W.fbox32,
            W.cvals[cut_buf], W.cl_start, W.cl_n, W.nodes, W.split_far, (FBox*)W.split_box, W.pair_root);
    else
        k_build<uint32_t><<<g, kRefitWin, 0, s>>>(P, (const uint32_t*)W.cl_key, n, W.fbox32, W.cvals[cut_buf],
            W.cl_start, W.cl_n, W.nodes, W.split_far, (FBox*)W.split_box, W.pair_root);
}

void launch_packets(const Problem& P, Work& W, int src_buf, cudaStream_t s)
{
    g_launches++;
    if (P.n_pairs > 1)
        k_src_packets<unsigned long long><<<grid_for(P.ns), kBlock, 0, s>>>(
            (const unsigned long long*)W.skeys[src_buf], (int)P.ns, W.packets, W.counters, (int)W.packet_faces);
    else
        k_src_packets<uint32_t><<<grid_for(P.ns), kBlock, 0, s>>>((const uint32_t*)W.skeys[src_buf], (int)P.ns,
            W.packets, W.counters, (int)W.packet_faces);
}

static void launch_traverse_tree(const Problem& P, Work& W, int src_buf, int cut_buf, bool deep, cudaStream_t s)
{
    // W.traversal: 0 (default) one warp per query packet (a compact source
    // subtree of <= W.packet_faces faces), breadth-first; 1 the same
    // depth-first; 2 one thread per source face with a W.stack_depth stack.
    // launch_packets must have run since the counters were cleared (0, 1).
    // The deep re-run after a stack overflow is per thread, 512 entries.
    const bool per_thread = W.traversal == 2;
    if (deep || per_thread) {
        const int g = grid_for(P.ns);
        g_launches++;
        if (deep || W.stack_depth > 64)
            k_traverse<512><<<g, kBlock, 0, s>>>(P, W.fbox, W.svals[src_buf], W.cvals[cut_buf], W.cl_start, W.cl_n,
                W.leaf_key_box, (int)P.ncl, W.nodes, W.pairs, W.pair_cap, W.counters, W.cand, W.pair_status);
        else
            k_traverse<64><<<g, kBlock, 0, s>>>(P, W.fbox, W.svals[src_buf], W.cvals[cut_buf], W.cl_start, W.cl_n,
                W.leaf_key_box, (int)P.ncl, W.nodes, W.pairs, W.pair_cap, W.counters, W.cand, W.pair_status);
        return;
    }
    g_launches++;
    const bool dfs = W.traversal == 1;
    if (dfs)
        k_traverse_packet<<<grid_for(P.ns), kBlock, 0, s>>>(P, W.fbox, W.svals[src_buf], W.packets,
            W.cvals[cut_buf], W.cl_start, W.cl_n, W.leaf_key_box, (int)P.ncl, W.nodes, W.pairs, W.pair_cap,
            W.counters, W.cand, W.pair_status);
    else {
        static std::atomic<unsigned long long> attr { 0 }, attr2 { 0 };
        set_smem_once((const void*)k_traverse_wave<false>, (int)kWaveSmem, attr);
        set_smem_once((const void*)k_traverse_wave<true>, (int)kWaveSmem, attr2);
        WaveTop* top = reinterpret_cast<WaveTop*>(W.top);
        SplitEntry* split = reinterpret_cast<SplitEntry*>(W.split);
        g_launches += 2; // top cut + first walk
        k_top_cut<<<1, 32, 0, s>>>(W.nodes, (int)P.ncl, top, W.counters);
        k_traverse_wave<false><<<grid_for(P.ns), kBlock, kWaveSmem, s>>>(P, W.fbox, W.svals[src_buf], W.packets,
            W.cvals[cut_buf], W.cl_start, W.cl_n, top, (int)P.ncl, W.nodes, W.pairs, W.pair_cap, W.counters, W.cand,
            W.pair_status, split, (uint32_t)W.split_cap, (int)W.split_round, W.pair_root);
        if (W.split_round > 0) {
            g_launches++;
            k_traverse_wave<true><<<grid_for(P.ns), kBlock, kWaveSmem, s>>>(P, W.fbox, W.svals[src_buf], W.packets,
                W.cvals[cut_buf], W.cl_start, W.cl_n, top, (int)P.ncl, W.nodes, W.pairs, W.pair_cap, W.counters,
                W.cand, W.pair_status, split, (uint32_t)W.split_cap, 0, nullptr);
        }
    }
}

void launch_traverse(const Problem& P, Work& W, int src_buf, int cut_buf, bool deep, cudaStream_t s)
{
    // the batch tree (absent when every pair's cut tree is resident), then
    // the resident trees
    if (P.ncl > 0) launch_traverse_tree(P, W, src_buf, cut_buf, deep, s);
    if (P.res_pairs) {
        const int g = grid_for(P.ns);
        g_launches++;
        if (deep)
            k_traverse_resident<512><<<g, kBlock, 0, s>>>(P, W.fbox, W.svals[src_buf], W.pairs, W.pair_cap, W.counters,
                W.cand, W.pair_status);
        else
            k_traverse_resident<64><<<g, kBlock, 0, s>>>(P, W.fbox, W.svals[src_buf], W.pairs, W.pair_cap, W.counters,
                W.cand, W.pair_status);
    }
}

ResTreeSizes resident_tree_sizes(uint32_t nf, uint32_t leaf_size)
{
    auto al = [](uint64_t b) { return (b + 255) & ~255ull; };
    ResTreeSizes z {};
    z.ncl = ((uint64_t)nf + leaf_size - 1) / leaf_size;
    const uint64_t nc2 = std::max<uint64_t>(z.ncl, 2);
    z.nodes_bytes = (nc2 - 1) * sizeof(Node);
    z.leaf_bytes = (uint64_t)nf * 4;
    z.start_bytes = z.ncl * 4;
    z.n_bytes = z.ncl;
    // fp32 boxes, keys and values (double-buffered), sort scratch, cluster
    // keys, the build's split records, the one-pair tables
    z.scratch_bytes = al((uint64_t)nf * 24) + 4 * al((uint64_t)nf * 4) + al(radix_sort_temp_bytes(nf))
        + al(z.ncl * 4) + al(nc2 * 4) + al(nc2 * 64) + al(16);
    return z;
}

void build_resident_tree(const double* X, const uint32_t* idx, uint32_t nv, uint32_t nf, const double* mn,
    const double* mx, uint32_t leaf_size, void* scratch, const ResTreeOut& out, cudaStream_t s)
{
    auto al = [](uint64_t b) { return (b + 255) & ~255ull; };
    const ResTreeSizes z = resident_tree_sizes(nf, leaf_size);
    const uint64_t nc2 = std::max<uint64_t>(z.ncl, 2);
    uint8_t* b = static_cast<uint8_t*>(scratch);
    auto take = [&](uint64_t bytes) { uint8_t* r = b; b += al(bytes); return r; };
    float* fbox32 = reinterpret_cast<float*>(take((uint64_t)nf * 24));
    uint32_t* keys[2] = { reinterpret_cast<uint32_t*>(take((uint64_t)nf * 4)), reinterpret_cast<uint32_t*>(take((uint64_t)nf * 4)) };
    uint32_t* vals[2] = { reinterpret_cast<uint32_t*>(take((uint64_t)nf * 4)), reinterpret_cast<uint32_t*>(take((uint64_t)nf * 4)) };
    uint32_t* temp = reinterpret_cast<uint32_t*>(take(radix_sort_temp_bytes(nf)));
    uint32_t* clkey = reinterpret_cast<uint32_t*>(take(z.ncl * 4));
    uint32_t* split_far = reinterpret_cast<uint32_t*>(take(nc2 * 4));
    void* split_box = take(nc2 * 64);
    uint32_t* tab = reinterpret_cast<uint32_t*>(take(16));
    g_launches++;
    k_res_faces<<<grid_for(nf), kBlock, 0, s>>>(X, idx, nv, nf, mn[0], mn[1], mn[2], mx[0], mx[1], mx[2], fbox32,
        keys[0], vals[0], tab, (uint32_t)z.ncl);
    const int buf = radix_sort_pairs<uint32_t>(keys[0], vals[0], keys[1], vals[1], nf, 0, kMortonBits, temp, s);
    cudaMemcpyAsync(out.leaf_face, vals[buf], (size_t)nf * 4, cudaMemcpyDeviceToDevice, s);
    Problem P1 {};
    P1.n_pairs = 1;
    P1.nf = nf;
    P1.nc = nf;
    P1.face_split = 0; // every face a cut face of pair 0
    P1.pair_cbase = tab;
    P1.pair_clbase = tab + 2;
    P1.leaf_size = leaf_size;
    P1.ncl = (uint32_t)z.ncl;
    const int n = (int)z.ncl;
    g_launches++;
    k_clusters<uint32_t><<<grid_for(n), kBlock, 0, s>>>(P1, keys[buf], clkey, out.cl_start, out.cl_n, split_far);
    if (n < 2) return;
    g_launches++;
    k_build<uint32_t><<<(n + kRefitWin - 1) / kRefitWin, kRefitWin, 0, s>>>(P1, clkey, n, fbox32, vals[buf],
        out.cl_start, out.cl_n, out.nodes, split_far, (FBox*)split_box, nullptr);
}

void launch_planes(const Problem& P, Work& W, cudaStream_t s)
{
    const int g = grid_for(P.nf);
    g_launches += 2;
    // the slot -> face list lives in proj_list until the narrow phase queues projections there
    k_plane_slots<<<g, kBlock, 0, s>>>(P, W.cand, W.plane_slot, W.plane_cap, W.counters, W.proj_list, W.proj_flag);
    k_planes<<<grid_for(W.plane_cap), kBlock, 0, s>>>(P, W.proj_list, (FacePlane*)W.planes, W.plane_cap, W.counters,
        W.poly_list, W.pair_bad);
    if (W.tri_stride) g_launches++;
    if (W.tri_stride)
        k_triplets<<<grid_for(1024), kBlock, 0, s>>>(P, W.poly_list, W.counters, W.plane_slot, (FacePlane*)W.planes,
            (Trip*)W.tri_scratch, W.tri_scratch_cap, W.tri_stride, W.pair_status);
}

void launch_incidence(const Problem& P, Work& W, cudaStream_t s)
{
    const int g = grid_for(P.nf);
    cudaMemsetAsync(W.vneed, 0, (size_t)P.nv, s);
    g_launches++;
    k_mark_vertices<<<g, kBlock, 0, s>>>(P, W.cand, W.vneed);
    cudaMemsetAsync(W.voff, 0, sizeof(uint32_t) * ((size_t)P.nv + 1), s);
    if (W.inc_slots) {
        g_launches++;
        k_vf_slots<<<g, kBlock, 0, s>>>(P, W.vneed, W.voff, W.vface, W.inc_slots, W.counters);
        return;
    }
    g_launches++;
    k_vf_count<<<g, kBlock, 0, s>>>(P, W.vneed, W.voff);
    exclusive_scan(W.voff, P.nv + 1, nullptr, W.scan_temp, s);
    cudaMemsetAsync(W.vcur, 0, sizeof(uint32_t) * (size_t)P.nv, s);
    g_launches++;
    k_vf_fill<<<g, kBlock, 0, s>>>(P, W.vneed, W.voff, W.vcur, W.vface, W.inc_cap);
}

void launch_adjacency_planes(const Problem& P, Work& W, cudaStream_t s)
{
    launch_planes(P, W, s);
    launch_incidence(P, W, s);
}

void launch_tests(const Problem& P, Work& W, cudaStream_t s)
{
    const int g = grid_for(W.pair_cap);
    g_launches++;
    k_pair_tests<<<g, kBlock, 0, s>>>(P, W.fbox, W.pairs, W.counters, W.pair_cap, W.voff, W.vface, W.inc_slots,
        W.tests, W.test_cap, W.counters, W.pair_bad, W.pair_status, W.pair_cnt);
}

void launch_narrow(const Problem& P, Work& W, bool keep_tests, cudaStream_t s)
{
    const int g = grid_for(W.test_cap);
    // the hit list lives in rec_key[1] (uint2 per test), free until the record sort
    uint2* hits = reinterpret_cast<uint2*>(W.rec_key[1]);
    g_launches += 3;
    k_narrow_signs<<<g, kBlock, 0, s>>>(P, W.tests, W.counters, W.test_cap, W.plane_slot, (const FacePlane*)W.planes,
        keep_tests ? 1 : 0, W.test_info, hits, W.proj_flag, W.proj_list, W.counters, W.pair_cnt);
    k_finish_planes<<<grid_spread(W.plane_cap), kSpread, 0, s>>>(P, (FacePlane*)W.planes, W.plane_slot,
        W.proj_list, W.counters);
    const int gh = std::max(1, grid_spread(W.test_cap) * kSpread / kNarrowHitsBlock);
    k_narrow_hits<<<gh, kNarrowHitsBlock, 0, s>>>(P, W.tests, hits, W.test_cap, W.plane_slot,
        (const FacePlane*)W.planes, keep_tests ? 1 : 0, W.test_info, W.rec_key[0], W.rec_val[0], W.rec_pt_raw, W.counters, W.pair_status,
        W.pair_bad);
}

void launch_clear_status(uint32_t* pair_status, uint32_t n_pairs, uint32_t mask, cudaStream_t s)
{
    g_launches++;
    k_clear_status<<<grid_for(n_pairs), kBlock, 0, s>>>(pair_status, n_pairs, mask);
}

// Records up to kRankSortMax are ordered by k_rank_records (one launch). With
// one pair W.pair_nrec is left alone: that pair owns records [0, nrec).

int launch_records(const Problem& P, Work& W, uint32_t nrec, cudaStream_t s)
{
    if (nrec == 0) return 0;
    // key = halfedge slot (the edge's first face corner in the source-then-cut
    // face arrays), then face: both global and monotone in the pair index,
    // so records come out grouped by pair. The
    // key is packed to the bits the ids need, which sets the radix passes.
    const uint32_t nidx = P.all_triangles ? 3u * P.nf : 0xFFFFFFFFu;
    const int sbits = nidx == 0xFFFFFFFFu ? 32 : 32 - __builtin_clz(nidx | 1u);
    const int gbits = 32 - __builtin_clz(P.nf | 1u);
    const int g = grid_for(nrec);
    if (nrec <= kRankSortMax) {
        // raw keys (slot << 32 | face) order like the packed ones
        uint32_t* rank = W.rec_val[1];
        cudaMemsetAsync(rank, 0, sizeof(uint32_t) * nrec, s);
        g_launches += 3;
        k_sort_slices<<<(nrec + kRankChunk - 1) / kRankChunk, kBlock, 0, s>>>(W.rec_key[0], W.rec_val[0], nrec,
            nullptr, 0);
        k_rank_records<<<dim3((nrec + kBlock - 1) / kBlock, (nrec + kRankChunk - 1) / kRankChunk), kBlock, 0, s>>>(
            W.rec_key[0], nrec, nullptr, 0, rank);
        k_scatter_records<<<g, kBlock, 0, s>>>(P, W.rec_key[0], W.rec_val[0], rank, nrec, nullptr, 0, W.tests,
            W.rec_pt_raw, W.rec_key[1], W.rec_ids, W.rec_pts);
        if (P.n_pairs > 1) { // one pair owns every record (the caller knows the range)
            g_launches++;
            k_pair_record_ranges<<<grid_for(P.n_pairs + 1), kBlock, 0, s>>>(P, W.rec_key[1], nrec, nullptr, 0, 32,
                W.pair_nrec);
        }
        return 1;
    }
    g_launches++;
    k_record_pack<<<g, kBlock, 0, s>>>(W.rec_key[0], nrec, gbits);
    const int buf = radix_sort_pairs<unsigned long long>(W.rec_key[0], W.rec_val[0], W.rec_key[1], W.rec_val[1], nrec,
        0, sbits + gbits, W.sort_temp, s);
    g_launches += 2;
    k_gather_records<<<g, kBlock, 0, s>>>(P, W.rec_val[buf], nrec, W.tests, W.rec_pt_raw, W.rec_ids, W.rec_pts);
    if (P.n_pairs > 1)
        k_pair_record_ranges<<<grid_for(P.n_pairs + 1), kBlock, 0, s>>>(P, W.rec_key[buf], nrec, nullptr, 0, gbits,
            W.pair_nrec);
    else
        g_launches--;
    return buf;
}

// The same one-launch ordering with the record count left on the device
// (counters[2]): grids are sized for `cap` records, and a count above it
// leaves everything untouched for the host to order from its own count.
int launch_records_dev(const Problem& P, Work& W, uint32_t cap, cudaStream_t s)
{
    const uint32_t* nd = W.counters + 2;
    uint32_t* rank = W.rec_val[1];
    cudaMemsetAsync(rank, 0, sizeof(uint32_t) * cap, s);
    g_launches += 3;
    k_sort_slices<<<(cap + kRankChunk - 1) / kRankChunk, kBlock, 0, s>>>(W.rec_key[0], W.rec_val[0], 0, nd, cap);
    k_rank_records<<<dim3((cap + kBlock - 1) / kBlock, (cap + kRankChunk - 1) / kRankChunk), kBlock, 0, s>>>(
        W.rec_key[0], 0, nd, cap, rank);
    k_scatter_records<<<grid_for(cap), kBlock, 0, s>>>(P, W.rec_key[0], W.rec_val[0], rank, 0, nd, cap, W.tests,
        W.rec_pt_raw, W.rec_key[1], W.rec_ids, W.rec_pts);
    if (P.n_pairs > 1) {
        g_launches++;
        k_pair_record_ranges<<<grid_for(P.n_pairs + 1), kBlock, 0, s>>>(P, W.rec_key[1], 0, nd, cap, 32, W.pair_nrec);
    }
    return 1;
}

} // namespace mcgpu
