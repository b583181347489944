// The record hand-over on the device: the maps dispatch()'s host stages read
// from the narrow phase (kernel.cpp:2599-2655, merged at kernel.cpp:2673-2714),
// built from one dispatch's sorted records.
//
// Record i (canonical order: the tested edge's first face corner, then the
// tested face) is the intersection vertex Vs + Vc + i of MCUT's m0. From the
// records' (q, r, tested face g, f0, f1):
//   edges    ps_intersecting_edges: a run of records with the same (q, r)
//   cutpath  cutpath_edge_creation_info: {source face, cut face} of g and each
//            face of the edge; MCUT's pair<> orders the two faces and source
//            faces come first, so the key is (source, cut)
//   faces    ps_iface_to_ivtx_list: g, f0 and f1
//   border   cm_border_reentrant_ivtx_list: cut-mesh edges with one face
// The reference keys its maps with std::map / unordered_map and appends each
// vertex as its thread meets it; here keys ascend and each key's vertices
// ascend.
//
// Work per record: one emit thread writes 2 cutpath and 3 face (key, vertex)
// entries (absent faces get a key that sorts last), two stable radix sorts
// order them, one kernel flags run heads, ONE exclusive scan over the four
// flag segments (edge heads, border records, cutpath heads, face heads) gives
// every output position, and one kernel writes the outputs and the counts.
#include <cstdint>

#include "fe_common.cuh"
#include "fe_derived.cuh"
#include "fe_sort.cuh"

namespace mcgpu {

namespace {

constexpr int kDBlock = 256;
constexpr unsigned long long kNoKey64 = ~0ull;
constexpr uint32_t kNoKey32 = 0xFFFFFFFFu;

__global__ void __launch_bounds__(kDBlock) k_derive_emit(const uint32_t* __restrict__ rec, uint32_t nrec, uint32_t vs,
    uint32_t nv, int cbits, unsigned long long* __restrict__ ck, uint32_t* __restrict__ cv, uint32_t* __restrict__ fk,
    uint32_t* __restrict__ fv, uint32_t* __restrict__ flags)
{
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nrec; i += gridDim.x * blockDim.x) {
        const uint32_t q = rec[5 * (size_t)i], r = rec[5 * (size_t)i + 1], g = rec[5 * (size_t)i + 2];
        const uint32_t f0 = rec[5 * (size_t)i + 3], f1 = rec[5 * (size_t)i + 4];
        const uint32_t vtx = nv + i;
        // the edge's vertices (and faces) are the cut mesh's
        const bool cut_edge = q >= vs;
        flags[i] = (i == 0 || rec[5 * (size_t)(i - 1)] != q || rec[5 * (size_t)(i - 1) + 1] != r) ? 1u : 0u;
        flags[nrec + i] = (cut_edge && f1 == kNone) ? 1u : 0u;
        const uint32_t ef[2] = { f0, f1 };
        for (int k = 0; k < 2; ++k) {
            unsigned long long key = kNoKey64;
            if (ef[k] != kNone) {
                const uint32_t sface = cut_edge ? g : ef[k], cface = cut_edge ? ef[k] : g;
                key = ((unsigned long long)sface << cbits) | cface;
            }
            ck[2 * (size_t)i + k] = key;
            cv[2 * (size_t)i + k] = vtx;
        }
        fk[3 * (size_t)i] = g;
        fk[3 * (size_t)i + 1] = f0;
        fk[3 * (size_t)i + 2] = f1 == kNone ? kNoKey32 : f1;
        fv[3 * (size_t)i] = fv[3 * (size_t)i + 1] = fv[3 * (size_t)i + 2] = vtx;
    }
}

// run heads of the sorted entries, and the number of entries with a key
__global__ void __launch_bounds__(kDBlock) k_derive_heads(const unsigned long long* __restrict__ ck, uint32_t ncp,
    const uint32_t* __restrict__ fk, uint32_t nfc, uint32_t* __restrict__ cp_head, uint32_t* __restrict__ fc_head,
    uint32_t* __restrict__ counts)
{
    const uint32_t n = max(ncp, nfc);
    for (uint32_t j = blockIdx.x * blockDim.x + threadIdx.x; j < n; j += gridDim.x * blockDim.x) {
        if (j < ncp) {
            const unsigned long long k = ck[j];
            const bool valid = k != kNoKey64;
            cp_head[j] = (valid && (j == 0 || ck[j - 1] != k)) ? 1u : 0u;
            if (valid && (j + 1 == ncp || ck[j + 1] == kNoKey64)) counts[kDerivedCutpathEntries] = j + 1;
        }
        if (j < nfc) {
            const uint32_t k = fk[j];
            const bool valid = k != kNoKey32;
            fc_head[j] = (valid && (j == 0 || fk[j - 1] != k)) ? 1u : 0u;
            if (valid && (j + 1 == nfc || fk[j + 1] == kNoKey32)) counts[kDerivedFaceEntries] = j + 1;
        }
    }
}

// S: the exclusive scan of the flags [edge heads R | border R | cutpath heads 2R
// | face heads 3R | 0]; flag(x) = S[x+1] - S[x]
__global__ void __launch_bounds__(kDBlock) k_derive_write(const uint32_t* __restrict__ S, uint32_t nrec, uint32_t nv,
    int cbits, const unsigned long long* __restrict__ ck, const uint32_t* __restrict__ fk, DerivedOut o,
    uint32_t* __restrict__ counts)
{
    const uint32_t R = nrec;
    const uint64_t n = 7ull * R;
    const unsigned long long cmask = (1ull << cbits) - 1ull;
    for (uint64_t x = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; x < n; x += (uint64_t)gridDim.x * blockDim.x) {
        const bool flag = S[x + 1] != S[x];
        if (x < R) {
            if (flag) o.edge_off[S[x]] = (uint32_t)x;
            if (x == R - 1) {
                o.edge_off[S[R]] = R;
                counts[kDerivedEdges] = S[R];
            }
        } else if (x < 2ull * R) {
            const uint32_t i = (uint32_t)(x - R);
            if (flag) o.border[S[x] - S[R]] = nv + i;
            if (i == R - 1) counts[kDerivedBorder] = S[2 * R] - S[R];
        } else if (x < 4ull * R) {
            const uint32_t j = (uint32_t)(x - 2ull * R);
            if (flag) {
                const uint32_t idx = S[x] - S[2 * R];
                const unsigned long long k = ck[j];
                o.cp_pairs[2 * (size_t)idx] = (uint32_t)(k >> cbits);
                o.cp_pairs[2 * (size_t)idx + 1] = (uint32_t)(k & cmask);
                o.cp_off[idx] = j;
            }
            if (j == 2 * R - 1) {
                const uint32_t K = S[4 * R] - S[2 * R];
                o.cp_off[K] = counts[kDerivedCutpathEntries];
                counts[kDerivedCutpath] = K;
            }
        } else {
            const uint32_t j = (uint32_t)(x - 4ull * R);
            if (flag) {
                const uint32_t idx = S[x] - S[4 * R];
                o.face_keys[idx] = fk[j];
                o.face_off[idx] = j;
            }
            if (j == 3 * R - 1) {
                const uint32_t M = S[7 * R] - S[4 * R];
                o.face_off[M] = counts[kDerivedFaceEntries];
                counts[kDerivedFaces] = M;
            }
        }
    }
}

int dgrid(uint64_t n)
{
    const uint64_t g = (n + kDBlock - 1) / kDBlock;
    return (int)(g < 1 ? 1 : (g > 152 * 8 ? 152 * 8 : g));
}

int bits_for(uint32_t n) { return 32 - __builtin_clz(n | 1u); }

} // namespace

size_t derived_sort_temp_bytes(uint32_t nrec) { return radix_sort_temp_bytes(3u * nrec); }
size_t derived_scan_temp_bytes(uint32_t nrec) { return scan_temp_bytes(7u * nrec + 1u); }

void launch_derived(const uint32_t* rec_ids, uint32_t nrec, uint32_t vs, uint32_t nv, uint32_t fs, uint32_t nf,
    DerivedScratch& w, DerivedOut& o, cudaStream_t s)
{
    // counts start at zero (a run of no entries leaves its count untouched)
    cudaMemsetAsync(o.counts, 0, sizeof(uint32_t) * kDerivedCounts, s);
    if (nrec == 0) return;
    // keys: source face above cbits bits of cut face; source faces < fs, so a
    // key never has all of its sbits + cbits bits set, and the absent-face key
    // (all ones) sorts after every key
    const int cbits = bits_for(nf), sbits = bits_for(fs), fbits = bits_for(nf);
    g_launches += 3;
    k_derive_emit<<<dgrid(nrec), kDBlock, 0, s>>>(rec_ids, nrec, vs, nv, cbits, w.ck[0], w.cv[0], w.fk[0], w.fv[0],
        w.flags);
    const int cb = radix_sort_pairs<unsigned long long>(w.ck[0], w.cv[0], w.ck[1], w.cv[1], 2 * nrec, 0,
        sbits + cbits, w.sort_temp, s);
    const int fb = radix_sort_pairs<uint32_t>(w.fk[0], w.fv[0], w.fk[1], w.fv[1], 3 * nrec, 0, fbits, w.sort_temp, s);
    o.cp_vtx = w.cv[cb];
    o.face_vtx = w.fv[fb];
    k_derive_heads<<<dgrid(3ull * nrec), kDBlock, 0, s>>>(w.ck[cb], 2 * nrec, w.fk[fb], 3 * nrec,
        w.flags + 2 * (size_t)nrec, w.flags + 4 * (size_t)nrec, o.counts);
    cudaMemsetAsync(w.flags + 7 * (size_t)nrec, 0, sizeof(uint32_t), s);
    exclusive_scan(w.flags, 7 * nrec + 1, nullptr, w.scan_temp, s);
    k_derive_write<<<dgrid(7ull * nrec), kDBlock, 0, s>>>(w.flags, nrec, nv, cbits, w.ck[cb], w.fk[fb], o, o.counts);
}

} // namespace mcgpu
