// mcgpu_dispatch_noalloc: the single-pair front end for callers that cannot
// allocate GPU memory.
//
// Who needs it: code that may not call cudaMalloc at the moment it wants the
// intersection records -- a plugin living inside an application that hands
// out device memory only through its own arena and treats any other
// allocation as a leak, a process whose device memory another framework's
// caching allocator has already reserved (a fresh cudaMalloc would fail
// there), or a frame loop with a hard latency budget that must never wait on
// the driver's allocator (cudaMalloc and cudaFree can wait for the device).
//
// What it does instead: every scratch buffer of the front end (face boxes,
// sort keys, tree nodes, candidate pairs, planes, incidence, edge-face tests,
// record keys) lives in ONE file-scope __device__ array of fixed size,
// kScratchBytes (about 12 MB). Every GPU that loads this library holds that
// array until the process exits. The caller passes the inputs (device
// pointers to the internal, recentred coordinates and triangle indices) and
// the outputs (device buffers for the records). No cudaMalloc, cudaFree,
// cudaMallocHost or allocating library call is made; status readbacks copy
// into host stack variables, so the call waits for its stream three or four
// times and returns when its GPU work is done.
//
// Limits (anything larger is rejected with MCGPU_TOO_LARGE before any GPU
// work): triangles only, at most kMaxVerts vertices and kMaxFaces faces over
// both meshes, kMaxPairs candidate face pairs, kMaxTests edge-face tests.
//
// Sharing: all calls in the process use the same array, on every stream. The
// array keeps whatever the previous call left in it; this file clears every
// counter and flag a call depends on before using it. Two calls whose GPU
// work overlaps (different streams, or different host threads on the same
// device) overwrite each other's scratch and give wrong results: serialise
// them.
//
// Set-up: the device address of the array is looked up with
// cudaGetSymbolAddress the first time the entry point runs on a device (with
// that device current) and cached. Make that first call before any stream
// capture begins.
#include <cstring>
#include <mutex>

#include "fe_common.cuh"
#include "fe_kernels.cuh"
#include "fe_sort.cuh"
#include "mcut_gb300.h"

namespace {

using namespace mcgpu;

constexpr uint32_t kMaxVerts = 16384;
constexpr uint32_t kMaxFaces = 16384;
constexpr uint32_t kMaxPairs = 32768;
constexpr uint32_t kMaxTests = 65536;
constexpr uint32_t kLeafSize = 4;

constexpr size_t al(size_t x) { return (x + 255) & ~size_t(255); }

// byte offsets of every buffer inside the scratch array
constexpr size_t oX = 0;
constexpr size_t oFidx = oX + al(kMaxVerts * 24ull);
constexpr size_t oFpair = oFidx + al(kMaxFaces * 12ull);
constexpr size_t oTab = oFpair + al(kMaxFaces * 4ull);
constexpr size_t oEps = oTab + al(8 * 2 * 4);
constexpr size_t oClKey = oEps + al(8);
constexpr size_t oClStart = oClKey + al(kMaxFaces * 4ull);
constexpr size_t oClN = oClStart + al(kMaxFaces * 4ull);
constexpr size_t oLkb = oClN + al(kMaxFaces);
constexpr size_t oPackets = oLkb + al(kMaxFaces * 48ull);
constexpr size_t oFbox = oPackets + al(kMaxFaces * 8ull);
constexpr size_t oMbox = oFbox + al(kMaxFaces * 48ull);
constexpr size_t oKeys = oMbox + al(12 * 8);             // 8 arrays of kMaxFaces x 4 B
constexpr size_t oSortTmp = oKeys + al(8ull * kMaxFaces * 4);
constexpr size_t kSortTmpBytes = radix_sort_temp_bytes(kMaxTests) + 4096; // table + scan block sums
constexpr size_t oNodes = oSortTmp + al(kSortTmpBytes);
constexpr size_t oParent = oNodes + al(kMaxFaces * sizeof(Node)); // split_far
constexpr size_t oPairs = oParent + al(kMaxFaces * 4ull);
constexpr size_t oCounters = oPairs + al(kMaxPairs * 8ull);
constexpr size_t oCand = oCounters + al(16 * 4);
constexpr size_t oPslot = oCand + al(kMaxFaces);
constexpr size_t oPlanes = oPslot + al(kMaxFaces * 4ull);
constexpr size_t oVneed = oPlanes + al(kMaxFaces * sizeof(FacePlane));
constexpr size_t oVoff = oVneed + al(kMaxVerts);
constexpr size_t oVcur = oVoff + al((kMaxVerts + 1) * 4ull);
constexpr size_t oVface = oVcur + al(kMaxVerts * 4ull);
constexpr size_t oScanTmp = oVface + al(kMaxFaces * 12ull);
constexpr size_t oTests = oScanTmp + al(4096);
constexpr size_t oTinfo = oTests + al(kMaxTests * sizeof(Test));
constexpr size_t oRkey = oTinfo + al(4);
constexpr size_t oRval = oRkey + al(2ull * kMaxTests * 8);
constexpr size_t oRpt = oRval + al(2ull * kMaxTests * 4);
constexpr size_t oPstat = oRpt + al(kMaxTests * 24ull);
constexpr size_t oPflag = oPstat + al(3 * 4);
constexpr size_t oPlist = oPflag + al(kMaxFaces * 4ull);
constexpr size_t oTop = oPlist + al(kMaxFaces * 4ull);
constexpr size_t kSplitCap = 2048;
constexpr size_t oSplit = oTop + al(64 * 32);
constexpr size_t oNrange = oSplit + al(kSplitCap * 144ull);
constexpr size_t oFrame = oNrange + al(kMaxFaces * 64ull); // split_box
constexpr size_t oX32 = oFrame + al(64);
constexpr size_t kScratchBytes = oX32 + al(kMaxVerts * 16ull);

__device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_addr_mu;
void* g_addr[64] = {};

// device address of the scratch array on the current device (looked up once per device)
int scratch_address(unsigned char** out)
{
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return MCGPU_CUDA_ERROR;
    std::lock_guard<std::mutex> lk(g_addr_mu);
    if (!g_addr[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) return MCGPU_CUDA_ERROR;
        g_addr[dev] = p;
    }
    *out = static_cast<unsigned char*>(g_addr[dev]);
    return MCGPU_OK;
}

// copy the caller's indices into scratch with the cut mesh's vertex offset,
// tag faces with their mesh, reset the mesh boxes
__global__ void k_na_prep(const uint32_t* __restrict__ si, const uint32_t* __restrict__ ci, uint32_t nsi,
    uint32_t nci, uint32_t vs, uint32_t fs, uint32_t nf, uint32_t* __restrict__ fidx, uint32_t* __restrict__ fpair,
    unsigned long long* __restrict__ mbox)
{
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nsi + nci; i += stride)
        fidx[i] = i < nsi ? si[i] : ci[i - nsi] + vs;
    for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += stride)
        fpair[f] = f >= fs ? kCutBit : 0u;
    if (blockIdx.x == 0 && threadIdx.x < 12) mbox[threadIdx.x] = (threadIdx.x % 6) < 3 ? ~0ull : 0ull;
}

int na_fail(mcgpu_summary* out, int code)
{
    if (out) out->status = code;
    return code;
}

} // namespace

extern "C" int mcgpu_dispatch_noalloc(void* stream, const mcgpu_mesh* src, const mcgpu_mesh* cut, double cut_eps,
    uint32_t* record_ids, double* record_points, uint64_t record_capacity, mcgpu_summary* out)
{
    if (out) memset(out, 0, sizeof(*out));
    if (!src || !cut || !src->vertices || !src->face_indices || !cut->vertices || !cut->face_indices)
        return na_fail(out, MCGPU_INVALID_VALUE);
    // an error left by the caller's earlier, unrelated work is not this call's
    (void)cudaGetLastError();
    // the call waits for its stream between stages, which a stream being
    // captured into a CUDA graph cannot do: refuse before any GPU call, so
    // the caller's capture stays valid
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(static_cast<cudaStream_t>(stream), &cap) != cudaSuccess
        || cap != cudaStreamCaptureStatusNone) {
        (void)cudaGetLastError();
        return na_fail(out, MCGPU_INVALID_VALUE);
    }
    if (src->face_sizes || cut->face_sizes) return na_fail(out, MCGPU_TOO_LARGE); // triangles only
    const uint64_t nv = (uint64_t)src->num_vertices + cut->num_vertices;
    const uint64_t nf = (uint64_t)src->num_faces + cut->num_faces;
    if (src->num_vertices < 3 || cut->num_vertices < 3 || src->num_faces < 1 || cut->num_faces < 1)
        return na_fail(out, MCGPU_INVALID_INPUT);
    if (nv > kMaxVerts || nf > kMaxFaces) return na_fail(out, MCGPU_TOO_LARGE);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned char* base = nullptr;
    if (scratch_address(&base) != MCGPU_OK) return na_fail(out, MCGPU_CUDA_ERROR);

    const uint32_t Vs = src->num_vertices, Fs = src->num_faces;
    Problem P {};
    P.n_pairs = 1;
    P.nv = (uint32_t)nv;
    P.nf = (uint32_t)nf;
    P.ns = Fs;
    P.nc = cut->num_faces;
    P.X = reinterpret_cast<double*>(base + oX);
    P.Xc = nullptr;
    P.xsplit = 0xFFFFFFFFu;
    P.foff = nullptr;
    P.fidx = reinterpret_cast<uint32_t*>(base + oFidx);
    P.face_pair = reinterpret_cast<uint32_t*>(base + oFpair);
    // per-pair table, two entries per row (pair 0, end): fbase | fs | vbase | vs | sbase | cbase | clbase
    const uint32_t ncl = (P.nc + kLeafSize - 1) / kLeafSize;
    const uint32_t htab[14] = { 0, (uint32_t)nf, Fs, 0, 0, (uint32_t)nv, Vs, 0, 0, Fs, 0, P.nc, 0, ncl };
    uint32_t* tab = reinterpret_cast<uint32_t*>(base + oTab);
    P.pair_fbase = tab;
    P.pair_fs = tab + 2;
    P.pair_vbase = tab + 4;
    P.pair_vs = tab + 6;
    P.pair_sbase = tab + 8;
    P.pair_cbase = tab + 10;
    P.pair_eps = reinterpret_cast<double*>(base + oEps);
    P.pair_clbase = tab + 12;
    P.X32 = reinterpret_cast<float4*>(base + oX32);
    P.all_triangles = 1;
    P.leaf_size = kLeafSize;
    P.ncl = ncl;

    Work W {};
    W.traversal = 0;
    W.packet_faces = 32;
    W.stack_depth = 64;
    W.split_round = 2;
    W.fbox = reinterpret_cast<double*>(base + oFbox);
    W.x32 = reinterpret_cast<float4*>(base + oX32);
    W.mesh_box = reinterpret_cast<unsigned long long*>(base + oMbox);
    uint32_t* keys = reinterpret_cast<uint32_t*>(base + oKeys);
    // source then cut keys in one array per buffer (one sort orders both meshes)
    W.skeys[0] = keys;
    W.skeys[1] = keys + kMaxFaces;
    W.svals[0] = keys + 2 * kMaxFaces;
    W.svals[1] = keys + 3 * kMaxFaces;
    W.ckeys[0] = keys + Fs;
    W.ckeys[1] = keys + kMaxFaces + Fs;
    W.cvals[0] = keys + 2 * kMaxFaces + Fs;
    W.cvals[1] = keys + 3 * kMaxFaces + Fs;
    W.sort_temp = reinterpret_cast<uint32_t*>(base + oSortTmp);
    W.cl_key = base + oClKey;
    W.cl_start = reinterpret_cast<uint32_t*>(base + oClStart);
    W.cl_n = base + oClN;
    W.leaf_key_box = nullptr;
    W.fbox32 = reinterpret_cast<float*>(base + oLkb);
    W.packets = reinterpret_cast<uint2*>(base + oPackets);
    W.nodes = reinterpret_cast<Node*>(base + oNodes);
    W.split_far = reinterpret_cast<uint32_t*>(base + oParent);
    W.pairs = reinterpret_cast<unsigned long long*>(base + oPairs);
    W.pair_cap = kMaxPairs;
    W.counters = reinterpret_cast<uint32_t*>(base + oCounters);
    W.cand = base + oCand;
    W.plane_slot = reinterpret_cast<uint32_t*>(base + oPslot);
    W.planes = base + oPlanes;
    W.plane_cap = kMaxFaces;
    W.proj_flag = reinterpret_cast<uint32_t*>(base + oPflag);
    W.proj_list = reinterpret_cast<uint32_t*>(base + oPlist);
    W.top = base + oTop;
    W.split = base + oSplit;
    W.split_cap = kSplitCap;
    W.split_box = base + oNrange;
    W.mesh_frame = base + oFrame;
    W.poly_list = nullptr;
    W.vneed = base + oVneed;
    W.voff = reinterpret_cast<uint32_t*>(base + oVoff);
    W.vcur = reinterpret_cast<uint32_t*>(base + oVcur);
    W.vface = reinterpret_cast<uint32_t*>(base + oVface);
    W.inc_cap = 3ull * nf;
    W.scan_temp = reinterpret_cast<uint32_t*>(base + oScanTmp);
    W.tests = reinterpret_cast<Test*>(base + oTests);
    W.test_cap = kMaxTests;
    W.test_info = reinterpret_cast<int8_t*>(base + oTinfo);
    W.rec_key[0] = reinterpret_cast<unsigned long long*>(base + oRkey);
    W.rec_key[1] = W.rec_key[0] + kMaxTests;
    W.rec_val[0] = reinterpret_cast<uint32_t*>(base + oRval);
    W.rec_val[1] = W.rec_val[0] + kMaxTests;
    W.rec_pt_raw = reinterpret_cast<double*>(base + oRpt);
    W.rec_ids = record_ids;
    W.rec_pts = record_points;
    W.pair_status = reinterpret_cast<uint32_t*>(base + oPstat);
    W.pair_bad = reinterpret_cast<int32_t*>(base + oPstat + 4);
    W.pair_nrec = reinterpret_cast<uint32_t*>(base + oPstat + 8);
    W.tri_scratch = nullptr;
    W.tri_scratch_cap = 0;
    W.tri_stride = 0;
    // the bounds kernel replaces an index outside its mesh in the table it reads
    W.fidx_fix = reinterpret_cast<uint32_t*>(base + oFidx);

    auto ok = [](cudaError_t e) { return e == cudaSuccess; };
    // inputs and the per-pair table into scratch; clear what must start at zero
    if (!ok(cudaMemcpyAsync(base + oX, src->vertices, (size_t)Vs * 24, cudaMemcpyDeviceToDevice, s))
        || !ok(cudaMemcpyAsync(base + oX + (size_t)Vs * 24, cut->vertices, (size_t)cut->num_vertices * 24,
            cudaMemcpyDeviceToDevice, s))
        || !ok(cudaMemcpyAsync(tab, htab, sizeof(uint32_t) * 14, cudaMemcpyHostToDevice, s))
        || !ok(cudaMemcpyAsync(base + oEps, &cut_eps, sizeof(double), cudaMemcpyHostToDevice, s))
        || !ok(cudaMemsetAsync(W.counters, 0, 64, s)) || !ok(cudaMemsetAsync(W.cand, 0, nf, s))
        || !ok(cudaMemsetAsync(W.vneed, 0, nv, s)) || !ok(cudaMemsetAsync(W.pair_status, 0, 4, s))
        || !ok(cudaMemsetAsync(W.pair_bad, 0x7F, 4, s)) || !ok(cudaMemsetAsync(W.pair_nrec, 0, 4, s)))
        return na_fail(out, MCGPU_CUDA_ERROR);
    k_na_prep<<<64, 256, 0, s>>>(src->face_indices, cut->face_indices, 3 * Fs, 3 * cut->num_faces, Vs, Fs,
        (uint32_t)nf, reinterpret_cast<uint32_t*>(base + oFidx), reinterpret_cast<uint32_t*>(base + oFpair),
        W.mesh_box);

    launch_bounds_morton(P, P, W, false, kMortonBits, s);
    int cut_buf = 0;
    const int src_buf = launch_sort(P, W, false, kMortonBits, s, cut_buf);
    launch_hierarchy(P, W, false, cut_buf, s);
    launch_packets(P, W, src_buf, s);
    launch_traverse(P, W, src_buf, cut_buf, false, s);
    uint32_t hc[16 + 3];
    if (!ok(cudaMemcpyAsync(hc, W.counters, 64, cudaMemcpyDeviceToHost, s))
        || !ok(cudaMemcpyAsync(hc + 16, W.pair_status, 4, cudaMemcpyDeviceToHost, s))
        || !ok(cudaStreamSynchronize(s)))
        return na_fail(out, MCGPU_CUDA_ERROR);
    if (hc[16] & ST_STACK) {
        // the walk again with 512-entry stacks; its own bits are cleared first and
        // the bounds kernel's ST_INVALID stays
        if (!ok(cudaMemsetAsync(W.counters, 0, 64, s)) || !ok(cudaMemsetAsync(W.cand, 0, nf, s)))
            return na_fail(out, MCGPU_CUDA_ERROR);
        launch_clear_status(W.pair_status, 1, ST_STACK | ST_OVERFLOW_PAIRS, s);
        launch_traverse(P, W, src_buf, cut_buf, true, s);
        if (!ok(cudaMemcpyAsync(hc, W.counters, 64, cudaMemcpyDeviceToHost, s))
            || !ok(cudaMemcpyAsync(hc + 16, W.pair_status, 4, cudaMemcpyDeviceToHost, s))
            || !ok(cudaStreamSynchronize(s)))
            return na_fail(out, MCGPU_CUDA_ERROR);
        // a tree deeper than the long stacks: the pair list would be incomplete
        if (hc[16] & ST_STACK) return na_fail(out, MCGPU_TOO_LARGE);
    }
    if (out) out->num_pairs = hc[0];
    if (hc[0] > kMaxPairs) return na_fail(out, MCGPU_TOO_LARGE);

    launch_adjacency_planes(P, W, s);
    launch_tests(P, W, s);
    launch_narrow(P, W, false, s);
    if (!ok(cudaMemcpyAsync(hc, W.counters, 64, cudaMemcpyDeviceToHost, s))
        || !ok(cudaMemcpyAsync(hc + 16, W.pair_status, 12, cudaMemcpyDeviceToHost, s))
        || !ok(cudaStreamSynchronize(s)))
        return na_fail(out, MCGPU_CUDA_ERROR);
    const uint32_t st = hc[16];
    const int32_t bad = (int32_t)hc[17];
    if (out) {
        out->num_tests = hc[1];
        out->num_records = hc[2];
        out->escalations[0] = hc[5];
        out->escalations[1] = hc[6];
        out->escalations[2] = hc[7];
        out->cut_eps = cut_eps;
        out->bad_face = -1;
    }
    if ((st & ST_OVERFLOW_TESTS) || hc[1] > kMaxTests) return na_fail(out, MCGPU_TOO_LARGE);
    if (hc[2] > record_capacity || (hc[2] && (!record_ids || !record_points))) return na_fail(out, MCGPU_TOO_LARGE);
    launch_records(P, W, hc[2], s);
    if (!ok(cudaStreamSynchronize(s)) || !ok(cudaGetLastError())) return na_fail(out, MCGPU_CUDA_ERROR);
    if (out) {
        if (st & ST_INVALID) out->status = MCGPU_INVALID_INPUT;
        else if (bad != kNoBad) {
            out->bad_face = bad;
            out->status = (uint32_t)bad >= Fs ? MCGPU_DEGENERATE_CUT_FACE : MCGPU_DEGENERATE_SRC_FACE;
        } else if (st & ST_GP) out->status = MCGPU_GP_VIOLATION;
        else out->status = MCGPU_OK;
    }
    return MCGPU_OK;
}
