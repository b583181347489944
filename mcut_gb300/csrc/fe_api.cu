// C ABI of the GB300 intersection front end: contexts, device memory,
// stage orchestration, result retrieval.
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <random>
#include <atomic>
#include <chrono>
#include <string>
#include <thread>
#include <vector>

#include "fe_common.cuh"
#include "fe_cutpath.cuh"
#include "fe_derived.cuh"
#include "fe_hmesh.cuh"
#include "fe_host.h"
#include "fe_kernels.cuh"
#include "fe_sort.cuh"
#include "mcut_gb300.h"

namespace {

thread_local std::string g_last_error;

int fail(int code, const std::string& msg)
{
    g_last_error = msg;
    return code;
}

struct CudaError {
    cudaError_t e;
    std::string where;
};

inline void ck(cudaError_t e, const char* where)
{
    if (e != cudaSuccess) throw CudaError { e, where };
}

// grow-only device buffer of a context's pool; `held` sums the pool's bytes,
// and a growth that would take it past a nonzero `limit` fails as an
// allocation failure before anything is freed
// A grow-only device buffer of a context's pool, allocated and freed in
// stream order on the context's stream (cudaMallocAsync / cudaFreeAsync): a
// context that grows its pool neither waits for nor stalls the device work
// of other contexts, as cudaFree's device-wide synchronisation would.
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    uint64_t* held = nullptr;
    const uint64_t* limit = nullptr;
    const cudaStream_t* stream = nullptr;
    template <typename T>
    T* get(size_t count)
    {
        const size_t bytes = std::max<size_t>(count * sizeof(T), 256);
        if (bytes > cap) {
            const size_t want = bytes + bytes / 4;
            if (limit && *limit && *held - cap + want > *limit)
                throw CudaError { cudaErrorMemoryAllocation, "context memory limit" };
            release();
            ck(cudaMallocAsync(&p, want, *stream), "cudaMallocAsync");
            cap = want;
            *held += want;
        }
        return reinterpret_cast<T*>(p);
    }
    void release()
    {
        if (p) cudaFreeAsync(p, *stream);
        if (held) *held -= cap;
        p = nullptr;
        cap = 0;
    }
};

struct PinBuf {
    void* p = nullptr;
    size_t cap = 0;
    template <typename T>
    T* get(size_t count)
    {
        const size_t bytes = std::max<size_t>(count * sizeof(T), 256);
        if (bytes > cap) {
            if (p) cudaFreeHost(p);
            p = nullptr;
            cap = 0;
            size_t want = bytes + bytes / 4;
            ck(cudaMallocHost(&p, want), "cudaMallocHost");
            cap = want;
        }
        return reinterpret_cast<T*>(p);
    }
    void release()
    {
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
    }
};

enum BufId {
    B_X, B_FOFF, B_FIDX, B_FPAIR, B_PTAB, B_EPS, B_FBOX, B_MESHBOX, B_SK0, B_SK1, B_SV0, B_SV1, B_CK0, B_CK1, B_CV0,
    B_CV1, B_SORTTMP, B_NODES, B_PARENT, B_PAIRS, B_COUNTERS, B_CAND, B_PSLOT, B_PLANES, B_POLY, B_VNEED,
    B_VOFF, B_VCUR, B_VFACE, B_SCANTMP, B_TESTS, B_TINFO, B_RK0, B_RK1, B_RV0, B_RV1, B_RPTRAW, B_RIDS, B_RPTS,
    B_PSTAT, B_PBAD, B_PNREC, B_TRI, B_SEG, B_CLKEY, B_CLSTART, B_CLN, B_LKB, B_PACKETS, B_PFLAG, B_PLIST, B_TOP, B_NRANGE, B_SPLIT, B_FRAME, B_XPERT, B_FIDXG,
    // the record hand-over (built at the first query for it)
    B_DCK0, B_DCK1, B_DCV0, B_DCV1, B_DFK0, B_DFK1, B_DFV0, B_DFV1, B_DFLAGS, B_DSORT, B_DSCAN, B_DOUT,
    B_X32, B_PCNT, B_XRAW, B_GSEG, B_FRAMES, B_COM, B_RAWB, B_RESP, B_PROOT,
    // the cut path (built at the first query for it)
    B_CP_CAND, B_CP_INSIDE, B_CP_SORTED, B_CP_PROJ, B_CP_PK0, B_CP_PK1, B_CP_PV0, B_CP_PV1, B_CP_MADE, B_CP_FK0,
    B_CP_FK1, B_CP_FV0, B_CP_FV1, B_CP_HK0, B_CP_HK1, B_CP_HV0, B_CP_HV1, B_CP_FLAGS, B_CP_SORT, B_CP_SCAN, B_CP_OUT,
    B_FP_PARENT, B_FP_FLAGS, B_FP_SIZE, B_FP_K0, B_FP_K1, B_FP_V0, B_FP_V1, B_FP_SORT, B_FP_SCAN, B_FP_OUT, B_FP_NRM,
    // the halfedge mesh (mcgpu_halfedge_mesh)
    B_HM_IDX, B_HM_FOFF, B_HM_KEY, B_HM_FIRST, B_HM_DIR, B_HM_SLOTFACE, B_HM_BUCKET, B_HM_EID, B_HM_VCUR,
    B_HM_PARENT, B_HM_SCAN, B_HM_SMALL, B_HM_TGT, B_HM_FACE, B_HM_NEXT, B_HM_PREV, B_HM_CORNER, B_HM_VOFF,
    B_HM_VHE, B_CW_FACE, B_CW_POS, B_CW_ADJ, B_CW_ADJN, B_CW_SCAN, B_CW_VF, B_CW_XD, B_COUNT
};

// host per-pair tables and results of the last dispatch
struct Layout {
    uint32_t n_pairs = 0;
    std::vector<uint32_t> vbase, vs, fbase, fs, sbase, cbase, ibase, is, clbase; // ibase: index base, is: src index count
    std::vector<double> eps;
    uint64_t nv = 0, nf = 0, ns = 0, nc = 0, nidx = 0, ncl = 0;
    uint32_t leaf_size = 4;
    bool all_tri = true;
    uint64_t tri_stride = 0, n_poly = 0;
    uint32_t max_face = 3;
    uint32_t res_trees = 0; // pairs whose cut tree is resident
};

} // namespace

struct mcgpu_context_t {
    int device = 0;
    cudaStream_t s = nullptr;
    cudaStream_t s2 = nullptr; // independent launches run here beside s (fork / join by events)
    cudaEvent_t fork[2] = {}, join[2] = {};
    cudaEvent_t ev[16] = {};  // begin / end of each stage (MCGPU_PROFILE)
    DevBuf buf[B_COUNT];
    uint64_t dev_held = 0;   // bytes the pool holds (every buf)
    uint64_t dev_limit = 0;  // 0: no cap (mcgpu_context_set_memory_limit)
    PinBuf pin_counters, pin_tab, pin_stage, pin_idx, pin_seg, pin_frames, pin_eps, pin_res;
    bool eps_on_device = false; // the last upload's cut-box enlargements come from the device (pin_eps)
    Layout L;
    mcgpu::Problem P {};
    mcgpu::Problem Pin {}; // the bounds kernel's view of the indices
    mcgpu::Work W {};
    std::vector<mcgpu_summary> sums;
    std::vector<uint64_t> rec_begin;  // per pair, +1
    uint64_t n_pairs_found = 0, n_tests = 0, n_records = 0;
    uint32_t flags = 0;
    int rec_buf = 0;
    mcgpu_tuning tune { 4, 0, 32, 64, 2 };  // MCGPU_LEAF_SIZE / MCGPU_TRAVERSAL / MCGPU_PACKET_FACES override at creation
    bool use_graphs = true;               // MCGPU_GRAPHS=0 disables
    bool use_fuse = true;                 // MCGPU_FUSE=0: every call stage by stage
    bool host_reads = false;              // the device reads pageable host memory (MCGPU_HOST_READS=0: never)
    uint32_t inc_slots = 16;              // vertex -> face slots per vertex (MCGPU_INC_SLOTS; 0: CSR lists)
    // general-position enforcement (frontend.h:596-597) and the perturbation
    // sequence: the reference's thread_local engines of the context's API
    // thread (preproc.cpp:2621-2627), one sequence per context
    double gp_constant = 1e-4;
    uint32_t gp_attempts = 4;
    std::mt19937 gp_rng { std::default_random_engine(1)() };
    std::uniform_real_distribution<double> gp_uniform { -1.0, 1.0 };
    bool csr_incidence = false;           // a vertex of this layout had more faces than slots
    uint64_t split_cap = 0;               // MCGPU_SPLIT_CAP: fixed split-entry capacity (0: by size)
    struct Graph {
        std::vector<unsigned char> key;
        cudaGraphExec_t exec = nullptr;
        int seen = 0;
        unsigned long long launches = 0;
        int aux[3] = { 0, 0, 0 };
    } graphs[4];
    // the fused call (one graph, one readback) follows a call with the same segment-0 key
    std::vector<unsigned char> fuse_key;
    bool fuse_ok = false;
    uint64_t fuse_nrec = 0, fuse_npairs = 0;
    bool have_results = false; // a dispatch completed since the last trim (queries 1-17 read it)
    // the floating polygons of the last single dispatch (built on demand)
    bool floating_ready = false;
    mcgpu::FloatingOut floating {};
    uint32_t floating_counts[mcgpu::kFpCounts] = {};
    mcgpu::CutpathInput cutpath_in {};
    // the cut path of the last single dispatch (built on demand)
    bool cutpath_ready = false;
    mcgpu::CutpathOut cutpath {};
    uint32_t cutpath_counts[mcgpu::kCpCounts] = {};
    // the record hand-over of the last single dispatch (built on demand)
    bool derived_ready = false;
    mcgpu::DerivedOut derived {};
    uint32_t derived_counts[mcgpu::kDerivedCounts] = {};
    // the last halfedge mesh (mcgpu_halfedge_mesh); valid when hm_ready
    bool hm_ready = false;
    uint32_t hm_ne = 0, hm_nv = 0;
    uint64_t hm_nidx = 0;
    // the last halfedge mesh's face offsets (null: triangles) and face count,
    // and the component wire arrays derived from it (built at the first query)
    const uint32_t* hm_foff = nullptr;
    uint32_t hm_nf = 0;
    bool cw_ready = false, hm_has_vf = false;
    mcgpu::CcWireOut cw {};
    uint32_t cw_total = 0;
    mcgpu::HmeshOut hm {};
};

namespace {

using namespace mcgpu;

// ---------------------------------------------------------------------------
// host recentring (calculate_vertex_parameters + client_input_arrays_to_hmesh,
// preproc.cpp:2124-2290, 147-181)
// ---------------------------------------------------------------------------
double dmaxr(double a, double b) { return (a < b) ? b : a; }
double dminr(double a, double b) { return (b < a) ? b : a; }
float fmaxr(float a, float b) { return (a < b) ? b : a; }
float fminr(float a, float b) { return (b < a) ? b : a; }

// the accumulators are locals: the compiler cannot keep values it must
// assume the vertex array aliases in registers
void vertex_bounds(const void* v, bool fin, uint32_t n, double* mn_out, double* mx_out, double* com_out)
{
    double mn[3], mx[3], com[3];
    for (int j = 0; j < 3; ++j) {
        mn[j] = 1.7976931348623157e308;
        mx[j] = -1.7976931348623157e308;
        com[j] = 0.0;
    }
    if (fin) {
        const float* p = (const float*)v;
        for (uint32_t i = 0; i < n; ++i)
            for (int j = 0; j < 3; ++j) {
                const float x = p[(size_t)i * 3 + j];
                mx[j] = (double)fmaxr((float)mx[j], x);
                mn[j] = (double)fminr((float)mn[j], x);
                com[j] += (double)x;
            }
    } else {
        const double* p = (const double*)v;
        for (uint32_t i = 0; i < n; ++i)
            for (int j = 0; j < 3; ++j) {
                const double x = p[(size_t)i * 3 + j];
                mx[j] = dmaxr(mx[j], x);
                mn[j] = dminr(mn[j], x);
                com[j] += x;
            }
    }
    for (int j = 0; j < 3; ++j) {
        mn_out[j] = mn[j];
        mx_out[j] = mx[j];
        com_out[j] = com[j] / (double)n;
    }
}

// a mesh's centroid sums, each coordinate summed in vertex order (the
// reference's accumulation; the bounds are taken on the device): one pass,
// three independent chains
void mesh_sums(const void* v, bool fin, uint32_t n, double* out)
{
    double a = 0.0, b = 0.0, c = 0.0;
    if (fin) {
        const float* p = (const float*)v;
        for (uint32_t i = 0; i < n; ++i) {
            a += (double)p[3 * (size_t)i];
            b += (double)p[3 * (size_t)i + 1];
            c += (double)p[3 * (size_t)i + 2];
        }
    } else {
        const double* p = (const double*)v;
        for (uint32_t i = 0; i < n; ++i) {
            a += p[3 * (size_t)i];
            b += p[3 * (size_t)i + 1];
            c += p[3 * (size_t)i + 2];
        }
    }
    out[0] = a;
    out[1] = b;
    out[2] = c;
}

double hdot(const double* a, const double* b)
{
    double o = 0.0;
    o = o + a[0] * b[0];
    o = o + a[1] * b[1];
    o = o + a[2] * b[2];
    return o;
}

} // namespace

namespace mcgpu {

void mesh_stats(const void* v, bool fin, uint32_t n, MeshStats& st) { vertex_bounds(v, fin, n, st.mn, st.mx, st.com); }

// the pair's frame: com of the two centroids, t = (com - gmin) + its unit
// vector (preproc.cpp:2124-2290)
void pair_frame(const MeshStats& S, const MeshStats& Cm, double* com, double* t)
{
    double tp[3];
    for (int j = 0; j < 3; ++j) {
        com[j] = (S.com[j] + Cm.com[j]) / 2.0;
        tp[j] = com[j] - dminr(S.mn[j], Cm.mn[j]);
    }
    const double len = std::sqrt(hdot(tp, tp));
    for (int j = 0; j < 3; ++j) t[j] = tp[j] + tp[j] / len;
}

// x' = (x - com) + t per coordinate (preproc.cpp:147-181)
void apply_frame(bool fin, const mcgpu_mesh& m, const double* com, const double* t, double* out)
{
    if (fin) {
        const float* p = (const float*)m.vertices;
        for (size_t k = 0; k < (size_t)m.num_vertices * 3; ++k) {
            const int j = (int)(k % 3);
            const float x = (p[k] - (float)com[j]) + (float)t[j];
            out[k] = (double)x;
        }
    } else {
        const double* p = (const double*)m.vertices;
        for (size_t k = 0; k < (size_t)m.num_vertices * 3; ++k) {
            const int j = (int)(k % 3);
            out[k] = (p[k] - com[j]) + t[j];
        }
    }
}

double frame_eps(const MeshStats& Cm, const double* t, double constant, bool absolute)
{
    double d[3];
    for (int j = 0; j < 3; ++j) d[j] = (Cm.mx[j] + t[j]) - (Cm.mn[j] + t[j]);
    return (absolute ? 1.0 : std::sqrt(hdot(d, d))) * constant;
}

} // namespace mcgpu

namespace {

void recentre_pair(bool fin, const mcgpu_mesh& S, const mcgpu_mesh& Cm, double* sx, double* cx, double* eps_out,
    double gp_constant = 1e-4, bool gp_absolute = false)
{
    MeshStats ss, cs;
    mesh_stats(S.vertices, fin, S.num_vertices, ss);
    mesh_stats(Cm.vertices, fin, Cm.num_vertices, cs);
    double com[3], t[3];
    pair_frame(ss, cs, com, t);
    apply_frame(fin, S, com, t, sx);
    apply_frame(fin, Cm, com, t, cx);
    *eps_out = frame_eps(cs, t, gp_constant, gp_absolute);
}

// memcpy on several host threads (large staging copies)
void memcpy_mt(void* dst, const void* src, size_t bytes, unsigned threads)
{
    if (bytes < (8u << 20) || threads < 2) {
        memcpy(dst, src, bytes);
        return;
    }
    const size_t chunk = ((bytes + threads - 1) / threads + 4095) & ~size_t(4095);
    std::vector<std::thread> ts;
    for (size_t lo = 0; lo < bytes; lo += chunk) {
        const size_t len = std::min(chunk, bytes - lo);
        ts.emplace_back([=] { memcpy(static_cast<char*>(dst) + lo, static_cast<const char*>(src) + lo, len); });
    }
    for (auto& t : ts) t.join();
}

// recentre_pair for one large pair on several host threads: the two meshes'
// stats run side by side (each centroid is still summed in vertex order, as
// the reference sums it), then the coordinate maps run in chunks
void recentre_pair_mt(bool fin, const mcgpu_mesh& S, const mcgpu_mesh& Cm, double* sx, double* cx, double* eps_out,
    unsigned threads, double gp_constant, bool gp_absolute)
{
    MeshStats ss, cs;
    std::thread tc([&] { mesh_stats(Cm.vertices, fin, Cm.num_vertices, cs); });
    mesh_stats(S.vertices, fin, S.num_vertices, ss);
    tc.join();
    double com[3], t[3];
    pair_frame(ss, cs, com, t);
    const uint64_t ns = S.num_vertices, nc = Cm.num_vertices, total = ns + nc;
    const uint64_t chunk = (total + threads - 1) / threads;
    std::vector<std::thread> ts;
    for (unsigned k = 0; k < threads; ++k) {
        const uint64_t lo = k * chunk, hi = std::min(total, lo + chunk);
        if (lo >= hi) break;
        ts.emplace_back([&, lo, hi] {
            // vertices [lo, hi) of the concatenation (source then cut)
            auto part = [&](const mcgpu_mesh& m, uint64_t base, double* out) {
                const uint64_t a = std::max(lo, base), b = std::min(hi, base + m.num_vertices);
                if (a >= b) return;
                mcgpu_mesh sub = m;
                const size_t vsz = fin ? 12 : 24;
                sub.vertices = static_cast<const char*>(m.vertices) + (a - base) * vsz;
                sub.num_vertices = (uint32_t)(b - a);
                apply_frame(fin, sub, com, t, out + (a - base) * 3);
            };
            part(S, 0, sx);
            part(Cm, ns, cx);
        });
    }
    for (auto& th : ts) th.join();
    *eps_out = frame_eps(cs, t, gp_constant, gp_absolute);
}

// the cut vertices of one general-position enforcement attempt: the
// recentred coordinate plus the perturbation, one rounding
// (preproc.cpp:131-133, 176-180)
__global__ void k_perturb(const double* __restrict__ in, double* __restrict__ out, uint64_t n3, double p0, double p1,
    double p2)
{
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n3; k += (uint64_t)gridDim.x * blockDim.x) {
        const int j = (int)(k % 3);
        out[k] = in[k] + (j == 0 ? p0 : (j == 1 ? p1 : p2));
    }
}

// Gathers segments of 4-byte words (host arrays the device reads over the
// link, or device arrays) into device buffers, one launch for every pair's
// arrays. segs[k].begin is the first word of segment k in the concatenation,
// segs[nseg].begin the total.
struct GatherSeg {
    const uint32_t* src;
    uint32_t* dst;
    uint64_t begin;
};
__global__ void __launch_bounds__(256) k_gather(const GatherSeg* __restrict__ segs, uint32_t nseg)
{
    const uint64_t total = segs[nseg].begin, stride = (uint64_t)gridDim.x * blockDim.x;
    uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
    if (i >= total) return;
    uint32_t lo = 0, hi = nseg; // the last segment starting at or before i
    while (hi - lo > 1) {
        const uint32_t mid = (lo + hi) >> 1;
        if (segs[mid].begin <= i) lo = mid; else hi = mid;
    }
    uint32_t k = lo;
    for (; i < total; i += stride) {
        while (i >= segs[k + 1].begin) ++k;
        const uint64_t o = i - segs[k].begin;
        segs[k].dst[o] = segs[k].src[o];
    }
}

// Bounds of every mesh's raw user coordinates, per (pair, mesh, axis), with
// the reference's sequential rule: max = (m < x) ? x : m and min =
// (x < m) ? x : m from +-DBL_MAX (+-inf for float input, the float cast of
// DBL_MAX), so NaNs never enter and of equal values the first in vertex
// order stays -- which only shows for zeros of either sign. Keys order the
// values with -0 and +0 equal; the first zero of each (pair, mesh, axis)
// (vertex << 1 | sign) gives the sign when a bound is zero.
__device__ __forceinline__ unsigned long long raw_key(double x)
{
    const long long b = __double_as_longlong(x == 0.0 ? 0.0 : x);
    return b < 0 ? ~(unsigned long long)b : ((unsigned long long)b | 0x8000000000000000ull);
}
__device__ __forceinline__ double raw_value(unsigned long long k)
{
    return __longlong_as_double((long long)((k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k));
}
constexpr int kRawChunk = 16; // consecutive vertices per thread
__global__ void __launch_bounds__(256) k_raw_bounds(const void* __restrict__ xraw, int fin, uint32_t nv,
    uint32_t n_pairs, const uint32_t* __restrict__ vbase, const uint32_t* __restrict__ vs,
    unsigned long long* __restrict__ lo, unsigned long long* __restrict__ hi, unsigned long long* __restrict__ zero)
{
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x * kRawChunk;
    for (uint64_t v0 = (blockIdx.x * (uint64_t)blockDim.x + threadIdx.x) * kRawChunk; v0 < nv; v0 += stride) {
        uint32_t l = 0, h = n_pairs; // the pair of v0
        while (h - l > 1) {
            const uint32_t mid = (l + h) >> 1;
            if (vbase[mid] <= v0) l = mid; else h = mid;
        }
        uint32_t p = l, seg = kNone;
        unsigned long long a[3], b[3], z[3];
        auto flush = [&]() {
            if (seg == kNone) return;
            for (int j = 0; j < 3; ++j) {
                if (a[j] != ~0ull) atomicMin(&lo[3 * (size_t)seg + j], a[j]);
                if (b[j] != 0ull) atomicMax(&hi[3 * (size_t)seg + j], b[j]);
                if (z[j] != ~0ull) atomicMin(&zero[3 * (size_t)seg + j], z[j]);
            }
        };
        const uint64_t v1 = v0 + kRawChunk < nv ? v0 + kRawChunk : (uint64_t)nv;
        for (uint64_t v = v0; v < v1; ++v) {
            while (v >= vbase[p + 1]) ++p;
            const uint32_t sg = 2 * p + ((v - vbase[p]) >= vs[p] ? 1u : 0u);
            if (sg != seg) {
                flush();
                seg = sg;
                for (int j = 0; j < 3; ++j) { a[j] = ~0ull; b[j] = 0ull; z[j] = ~0ull; }
            }
            for (int j = 0; j < 3; ++j) {
                const double x = fin ? (double)static_cast<const float*>(xraw)[3 * v + j]
                                     : static_cast<const double*>(xraw)[3 * v + j];
                if (x != x) continue;
                const unsigned long long k = raw_key(x);
                a[j] = min(a[j], k);
                b[j] = max(b[j], k);
                if (x == 0.0) z[j] = min(z[j], (v << 1) | (__double_as_longlong(x) < 0 ? 1ull : 0ull));
            }
        }
        flush();
    }
}

// Each pair's frame from its centroid (summed on the host) and the device's
// bounds (pair_frame and frame_eps of the host path, operation for
// operation: preproc.cpp:2124-2290, 2518, 2664-2676): frames[6p..] = com,
// t; eps[p] the cut-box enlargement.
__global__ void k_frames(uint32_t n_pairs, const double* __restrict__ com, const unsigned long long* __restrict__ lo,
    const unsigned long long* __restrict__ hi, const unsigned long long* __restrict__ zero, int fin,
    double constant, int absolute, double* __restrict__ frames, double* __restrict__ eps)
{
    const uint32_t p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n_pairs) return;
    const double top = fin ? __longlong_as_double(0x7FF0000000000000ll) : 1.7976931348623157e308;
    double mn[2][3], mx[2][3];
    for (int m = 0; m < 2; ++m)
        for (int j = 0; j < 3; ++j) {
            const size_t k = 3 * (2 * (size_t)p + m) + j;
            const double zs = (zero[k] != ~0ull && (zero[k] & 1ull)) ? -0.0 : 0.0;
            double a = lo[k] == ~0ull ? top : raw_value(lo[k]);
            double b = hi[k] == 0ull ? -top : raw_value(hi[k]);
            if (a == 0.0) a = zs;
            if (b == 0.0) b = zs;
            mn[m][j] = (a < top) ? a : top;   // the start value stays unless passed
            mx[m][j] = (-top < b) ? b : -top;
        }
    double tp[3], t[3], d[3];
    const double* c = com + 3 * (size_t)p;
    for (int j = 0; j < 3; ++j) {
        const double g = (mn[1][j] < mn[0][j]) ? mn[1][j] : mn[0][j];
        tp[j] = __dsub_rn(c[j], g);
    }
    double o = 0.0;
    for (int j = 0; j < 3; ++j) o = __dadd_rn(o, __dmul_rn(tp[j], tp[j]));
    const double len = __dsqrt_rn(o);
    for (int j = 0; j < 3; ++j) t[j] = __dadd_rn(tp[j], __ddiv_rn(tp[j], len));
    for (int j = 0; j < 3; ++j) d[j] = __dsub_rn(__dadd_rn(mx[1][j], t[j]), __dadd_rn(mn[1][j], t[j]));
    double q = 0.0;
    for (int j = 0; j < 3; ++j) q = __dadd_rn(q, __dmul_rn(d[j], d[j]));
    eps[p] = __dmul_rn(absolute ? 1.0 : __dsqrt_rn(q), constant);
    for (int j = 0; j < 3; ++j) {
        frames[6 * (size_t)p + j] = c[j];
        frames[6 * (size_t)p + 3 + j] = t[j];
    }
}

// the fp64 arithmetic rate: independent chains of a separately rounded
// multiply and add (as the library's fp64 code runs, --fmad=false)
constexpr int kFp64Chains = 8;
__global__ void __launch_bounds__(256) k_fp64_rate(double* __restrict__ out, int iters, double a, double b)
{
    const uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    double x[kFp64Chains];
    for (int k = 0; k < kFp64Chains; ++k) x[k] = 1.0 + 1e-3 * (double)(t + k);
    for (int i = 0; i < iters; ++i)
#pragma unroll
        for (int k = 0; k < kFp64Chains; ++k) x[k] = __dadd_rn(__dmul_rn(x[k], a), b);
    double s = 0.0;
    for (int k = 0; k < kFp64Chains; ++k) s += x[k];
    out[t] = s;
}

// resident cut mesh: its stored user coordinates mapped into the pair's frame
__global__ void k_apply_frame(const double* __restrict__ in, double* __restrict__ out, uint64_t n3, double c0,
    double c1, double c2, double t0, double t1, double t2)
{
    for (uint64_t k = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; k < n3; k += (uint64_t)gridDim.x * blockDim.x) {
        const int j = (int)(k % 3);
        const double c = j == 0 ? c0 : (j == 1 ? c1 : c2);
        const double t = j == 0 ? t0 : (j == 1 ? t1 : t2);
        out[k] = __dadd_rn(__dsub_rn(in[k], c), t);
    }
}

// ---------------------------------------------------------------------------
// device helpers
// ---------------------------------------------------------------------------
// ps indices (local -> global vertex ids) and the face -> pair table. With
// src_in / cut_in (a single pair from device arrays) the indices are read
// from the caller's arrays; otherwise they were copied into fidx already.
__global__ void k_prep(uint32_t n_pairs, const uint32_t* __restrict__ tab, uint32_t* __restrict__ fidx, uint64_t nidx,
    uint32_t* __restrict__ face_pair, uint64_t nf, const uint32_t* __restrict__ src_in,
    const uint32_t* __restrict__ cut_in)
{
    // tab rows (n_pairs+1 each): ibase, is, vbase, vs, fbase, fs
    const uint32_t* ibase = tab;
    const uint32_t* is = tab + (n_pairs + 1);
    const uint32_t* vbase = tab + 2 * (n_pairs + 1);
    const uint32_t* vs = tab + 3 * (n_pairs + 1);
    const uint32_t* fbase = tab + 4 * (n_pairs + 1);
    const uint32_t* fs = tab + 5 * (n_pairs + 1);
    const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
    // four independent elements per thread and step: their loads are in flight together
    for (uint64_t i0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i0 < nidx; i0 += 4 * stride) {
        uint32_t local[4], add[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint64_t i = i0 + k * stride;
            local[k] = 0u;
            add[k] = 0u;
            if (i >= nidx) continue;
            uint32_t lo = 0, hi = n_pairs; // last pair with ibase <= i
            while (hi - lo > 1) {
                const uint32_t mid = (lo + hi) >> 1;
                if (ibase[mid] <= i) lo = mid; else hi = mid;
            }
            const uint32_t p = lo;
            const bool cut = (i - ibase[p]) >= is[p];
            local[k] = src_in ? (cut ? cut_in[i - is[0]] : src_in[i]) : fidx[i];
            add[k] = vbase[p] + (cut ? vs[p] : 0u);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const uint64_t i = i0 + k * stride;
            if (i < nidx) fidx[i] = local[k] + add[k];
        }
    }
    for (uint64_t f = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; f < nf; f += stride) {
        uint32_t lo = 0, hi = n_pairs;
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (fbase[mid] <= f) lo = mid; else hi = mid;
        }
        const uint32_t p = lo;
        face_pair[f] = p | (((f - fbase[p]) >= fs[p]) ? kCutBit : 0u);
    }
}

// a dispatch's starting state in one launch: empty mesh boxes (min at the
// top, max at the bottom of the ordered-uint64 encoding), zero counters,
// statuses and record ranges, no degenerate face
__global__ void k_init_dispatch(unsigned long long* __restrict__ mb, uint32_t n_pairs, uint32_t* __restrict__ counters,
    uint32_t* __restrict__ pair_status, int32_t* __restrict__ pair_bad, uint32_t* __restrict__ pair_nrec,
    uint32_t* __restrict__ pair_cnt, int32_t* __restrict__ pair_root)
{
    const uint64_t n12 = (uint64_t)n_pairs * 12;
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n12 + 16; i += (uint64_t)gridDim.x * blockDim.x) {
        if (i < n12) mb[i] = (i % 6) < 3 ? ~0ull : 0ull;
        else counters[i - n12] = 0u;
        if (i < n_pairs) {
            pair_status[i] = 0u;
            pair_bad[i] = kNoBad;
        }
        if (i <= n_pairs) pair_nrec[i] = 0u;
        if (pair_cnt && i < (uint64_t)n_pairs * 5) pair_cnt[i] = 0u;
        if (pair_root && i < n_pairs) pair_root[i] = kNoRoot;
    }
}

int grid1(uint64_t n)
{
    const uint64_t g = (n + 255) / 256;
    return (int)std::max<uint64_t>(1, std::min<uint64_t>(g, 152 * 16));
}

uint32_t face_size(const mcgpu_mesh& m, uint32_t f) { return m.face_sizes ? m.face_sizes[f] : 3u; }

int build_layout(mcgpu_context_t* c, uint32_t flags, uint32_t n, const mcgpu_mesh* srcs, const mcgpu_mesh* cuts,
    const double* eps, const ResidentCut* const* res)
{
    Layout& L = c->L;
    L = Layout();
    L.n_pairs = n;
    L.vbase.resize(n + 1); L.vs.resize(n + 1); L.fbase.resize(n + 1); L.fs.resize(n + 1);
    L.sbase.resize(n + 1); L.cbase.resize(n + 1); L.ibase.resize(n + 1); L.is.resize(n + 1);
    L.clbase.resize(n + 1);
    L.leaf_size = c->tune.leaf_size;
    uint64_t cl = 0;
    L.eps.assign(n, 0.0);
    uint64_t v = 0, f = 0, sf = 0, cf = 0, ix = 0;
    for (uint32_t p = 0; p < n; ++p) {
        const mcgpu_mesh &S = srcs[p], &C = cuts[p];
        if (!S.vertices || !S.face_indices || !C.vertices || !C.face_indices)
            return fail(MCGPU_INVALID_VALUE, "null mesh array");
        if (S.num_vertices < 3 || C.num_vertices < 3 || S.num_faces < 1 || C.num_faces < 1)
            return fail(MCGPU_INVALID_INPUT, "mesh needs >= 3 vertices and >= 1 face");
        L.vbase[p] = (uint32_t)v; L.vs[p] = S.num_vertices;
        L.fbase[p] = (uint32_t)f; L.fs[p] = S.num_faces;
        L.sbase[p] = (uint32_t)sf; L.cbase[p] = (uint32_t)cf; L.ibase[p] = (uint32_t)ix;
        L.clbase[p] = (uint32_t)cl;
        // a resident cut tree keeps the pair's cut faces out of the sorted list and the batch tree
        const bool own_tree = res && res[p] && res[p]->tree_ncl > 0;
        if (!own_tree) cl += (C.num_faces + L.leaf_size - 1) / L.leaf_size;
        L.res_trees += own_tree ? 1 : 0;
        uint64_t is = 0, ic = 0;
        for (int side = 0; side < 2; ++side) {
            const mcgpu_mesh& m = side ? C : S;
            if (m.face_sizes) {
                L.all_tri = false;
                for (uint32_t k = 0; k < m.num_faces; ++k) {
                    const uint32_t sz = m.face_sizes[k];
                    if (sz < 3) return fail(MCGPU_INVALID_INPUT, "face with fewer than 3 vertices");
                    (side ? ic : is) += sz;
                    L.max_face = std::max(L.max_face, sz);
                    if (sz > 3) {
                        L.n_poly++;
                        L.tri_stride = std::max<uint64_t>(L.tri_stride, (uint64_t)sz * (sz - 1) * (sz - 2) / 6);
                    }
                }
            } else {
                (side ? ic : is) += 3ull * m.num_faces;
            }
        }
        L.is[p] = (uint32_t)is;
        v += (uint64_t)S.num_vertices + C.num_vertices;
        f += (uint64_t)S.num_faces + C.num_faces;
        sf += S.num_faces;
        if (!own_tree) cf += C.num_faces;
        ix += is + ic;
        if (eps && !(flags & MCGPU_RECENTRE)) L.eps[p] = eps[p];
    }
    if (v >= 0x7FFFFFFFull || f >= 0x7FFFFFFFull || ix >= 0xFFFFFFFFull)
        return fail(MCGPU_TOO_LARGE, "more than 2^31 vertices / faces in one dispatch");
    if (n > 65535) return fail(MCGPU_TOO_LARGE, "more than 65535 pairs in one batch");
    L.vbase[n] = (uint32_t)v; L.fbase[n] = (uint32_t)f; L.sbase[n] = (uint32_t)sf; L.cbase[n] = (uint32_t)cf;
    L.ibase[n] = (uint32_t)ix;
    L.clbase[n] = (uint32_t)cl;
    L.nv = v; L.nf = f; L.ns = sf; L.nc = cf; L.nidx = ix; L.ncl = cl;
    return MCGPU_OK;
}

// body(p) for p in [0, n) on up to `threads` host threads (dynamic, one pair at a time)
template <typename F>
void parallel_pairs(uint32_t n, uint64_t work, F body)
{
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const unsigned want = (unsigned)std::min<uint64_t>({ (uint64_t)std::min(hw / 2u, 8u), n, work / 100000 + 1 });
    if (want <= 1) {
        for (uint32_t p = 0; p < n; ++p) body(p);
        return;
    }
    std::atomic<uint32_t> next { 0 };
    auto loop = [&] {
        for (uint32_t p; (p = next.fetch_add(1)) < n;) body(p);
    };
    std::vector<std::thread> ts;
    for (unsigned k = 1; k < want; ++k) ts.emplace_back(loop);
    loop();
    for (auto& t : ts) t.join();
}

// a packed batch: the caller's arrays already follow the internal layout
struct Packed {
    const void* X;
    const uint32_t* idx;
};

// upload ps arrays: coordinates (recentred on the host when asked), indices, offsets
void upload(mcgpu_context_t* c, uint32_t flags, const mcgpu_mesh* srcs, const mcgpu_mesh* cuts, const Packed* pk,
    const ResidentCut* const* res)
{
    Layout& L = c->L;
    const uint32_t n = L.n_pairs;
    cudaStream_t s = c->s;
    const bool fin = (flags & MCGPU_VERTEX_ARRAY_FLOAT) != 0;
    const bool dev = (flags & MCGPU_DEVICE_POINTERS) != 0;
    const bool gp_absolute = (flags & MCGPU_ENFORCE_GENERAL_POSITION_ABSOLUTE) != 0;
    // device inputs are read in place (a packed batch as one array, a single
    // pair as its two arrays); everything else is copied
    const bool split = dev && !pk && n == 1;
    const double* X = (pk && dev) ? static_cast<const double*>(pk->X)
        : split ? static_cast<const double*>(srcs[0].vertices) : c->buf[B_X].get<double>(L.nv * 3);
    uint32_t* fidx = c->buf[B_FIDX].get<uint32_t>(L.nidx);
    // a single pair from host arrays, copied by the device reading them
    const bool host_read = c->host_reads && !dev && !pk && !res && n == 1 && !(flags & MCGPU_RECENTRE)
        && ((uintptr_t)srcs[0].vertices & 7) == 0 && ((uintptr_t)cuts[0].vertices & 7) == 0
        && ((uintptr_t)srcs[0].face_indices & 3) == 0 && ((uintptr_t)cuts[0].face_indices & 3) == 0;
    // With host_read the bounds kernels read the caller's arrays over the host
    // link themselves -- the vertex kernel the coordinates (writing the device
    // copy X), the face kernel the indices (writing the global table) -- so
    // the upload runs at the link's rate with their work hidden under it.
    c->W.hx_src = host_read ? static_cast<const double*>(srcs[0].vertices) : nullptr;
    c->W.hx_cut = host_read ? static_cast<const double*>(cuts[0].vertices) : nullptr;
    c->W.hx_out = host_read ? const_cast<double*>(X) : nullptr;
    c->W.x_raw = nullptr;
    c->W.raw_float = 0;
    c->W.frames = nullptr;
    // user coordinates from host arrays: gathered raw to the device by one
    // launch while the host sums the centroids, mapped by the bounds kernel
    bool gathered = c->host_reads && !dev && !pk && (flags & MCGPU_RECENTRE) && !(fin && res);
    for (uint32_t p = 0; gathered && p < n; ++p) {
        const uintptr_t a = (uintptr_t)srcs[p].vertices | (uintptr_t)srcs[p].face_indices
            | ((res && res[p]) ? 0 : ((uintptr_t)cuts[p].vertices | (uintptr_t)cuts[p].face_indices));
        gathered = (a & 3) == 0;
    }
    if ((pk && dev) || split || host_read) {
        // read in place
    } else if (gathered) {
        const size_t vsz = fin ? 12 : 24;
        uint8_t* xraw = c->buf[B_XRAW].get<uint8_t>(L.nv * vsz);
        GatherSeg* gs = c->pin_seg.get<GatherSeg>(4 * (size_t)n + 1);
        uint64_t words = 0;
        uint32_t k = 0;
        auto add = [&](const void* src, void* dst, uint64_t bytes) {
            gs[k++] = GatherSeg { static_cast<const uint32_t*>(src), static_cast<uint32_t*>(dst), words };
            words += bytes / 4;
        };
        for (uint32_t p = 0; p < n; ++p) {
            const bool r = res && res[p];
            const uint64_t nvc = (uint64_t)L.vbase[p + 1] - L.vbase[p] - L.vs[p];
            const uint64_t ic = (uint64_t)L.ibase[p + 1] - L.ibase[p] - L.is[p];
            add(srcs[p].vertices, xraw + (size_t)L.vbase[p] * vsz, (uint64_t)L.vs[p] * vsz);
            add(r ? static_cast<const void*>(res[p]->X) : cuts[p].vertices,
                xraw + ((size_t)L.vbase[p] + L.vs[p]) * vsz, nvc * vsz);
            add(srcs[p].face_indices, fidx + L.ibase[p], (uint64_t)L.is[p] * 4);
            add(r ? static_cast<const void*>(res[p]->idx) : cuts[p].face_indices, fidx + L.ibase[p] + L.is[p],
                ic * 4);
        }
        gs[k] = GatherSeg { nullptr, nullptr, words };
        GatherSeg* dseg = c->buf[B_GSEG].get<GatherSeg>((size_t)k + 1);
        ck(cudaMemcpyAsync(dseg, gs, sizeof(GatherSeg) * (k + 1), cudaMemcpyHostToDevice, s), "H2D segments");
        g_launches++;
        k_gather<<<grid1(words), 256, 0, s>>>(dseg, k);
        // meanwhile: each pair's centroid, summed in vertex order on the host
        // (a large pair: one thread per mesh and axis); the bounds and the
        // frame follow on the device once the tables are up
        double* hcom = c->pin_frames.get<double>(3 * (size_t)n);
        parallel_pairs(n, L.nv, [&](uint32_t p) {
            const bool r = res && res[p];
            const mcgpu_mesh* m[2] = { &srcs[p], &cuts[p] };
            double sum[2][3];
            if (!r && n == 1 && L.nv > 200000) {
                // the meshes side by side (each pass is bound by one core's reads)
                std::thread tc([&] { mesh_sums(m[1]->vertices, fin, m[1]->num_vertices, sum[1]); });
                mesh_sums(m[0]->vertices, fin, m[0]->num_vertices, sum[0]);
                tc.join();
            } else {
                mesh_sums(m[0]->vertices, fin, m[0]->num_vertices, sum[0]);
                if (!r) mesh_sums(m[1]->vertices, fin, m[1]->num_vertices, sum[1]);
            }
            for (int j = 0; j < 3; ++j) {
                const double cs = sum[0][j] / (double)srcs[p].num_vertices;
                const double cc = r ? res[p]->st.com[j] : sum[1][j] / (double)cuts[p].num_vertices;
                hcom[3 * (size_t)p + j] = (cs + cc) / 2.0;
            }
        });
        c->W.x_raw = xraw;
        c->W.raw_float = fin ? 1 : 0;
        c->W.frames = c->buf[B_FRAMES].get<double>(6 * (size_t)n);
        c->W.hx_out = const_cast<double*>(X);
    } else if (pk && !(flags & MCGPU_RECENTRE)) {
        ck(cudaMemcpyAsync(const_cast<double*>(X), pk->X, L.nv * 3 * sizeof(double), cudaMemcpyHostToDevice, s),
            "H2D X");
    } else if (flags & MCGPU_RECENTRE) {
        // host recentring (and the index copy into one pinned stage) in
        // parallel over the pairs; one H2D copy per array
        double* st = c->pin_stage.get<double>(L.nv * 3);
        uint32_t* ist = dev ? nullptr : c->pin_idx.get<uint32_t>(L.nidx);
        struct Job { double com[3], t[3]; };
        std::vector<Job> jobs(res ? n : 0);
        // resident cut trees: the frames of their pairs, for the tree walk
        double* hfr = L.res_trees ? c->pin_frames.get<double>(6 * (size_t)n) : nullptr;
        parallel_pairs(n, L.nv + L.nidx, [&](uint32_t p) {
            double* sx = st + (size_t)L.vbase[p] * 3;
            if (res && res[p]) {
                // resident cut: only the source is mapped on the host
                Job& j = jobs[p];
                MeshStats ss;
                mesh_stats(srcs[p].vertices, fin, srcs[p].num_vertices, ss);
                pair_frame(ss, res[p]->st, j.com, j.t);
                apply_frame(fin, srcs[p], j.com, j.t, sx);
                if (hfr)
                    for (int k = 0; k < 3; ++k) { hfr[6 * (size_t)p + k] = j.com[k]; hfr[6 * (size_t)p + 3 + k] = j.t[k]; }
                L.eps[p] = frame_eps(res[p]->st, j.t, c->gp_constant, gp_absolute);
            } else if (n == 1 && L.nv > 200000) {
                const unsigned hw = std::max(2u, std::min(16u, std::thread::hardware_concurrency()));
                recentre_pair_mt(fin, srcs[p], cuts[p], sx, st + ((size_t)L.vbase[p] + L.vs[p]) * 3, &L.eps[p], hw,
                    c->gp_constant, gp_absolute);
            } else {
                recentre_pair(fin, srcs[p], cuts[p], sx, st + ((size_t)L.vbase[p] + L.vs[p]) * 3, &L.eps[p],
                    c->gp_constant, gp_absolute);
            }
            if (ist) {
                const uint64_t ic = (uint64_t)L.ibase[p + 1] - L.ibase[p] - L.is[p];
                const unsigned th = n == 1 ? std::max(1u, std::min(16u, std::thread::hardware_concurrency())) : 1u;
                memcpy_mt(ist + L.ibase[p], srcs[p].face_indices, (size_t)L.is[p] * 4, th);
                if (!(res && res[p])) memcpy_mt(ist + L.ibase[p] + L.is[p], cuts[p].face_indices, (size_t)ic * 4, th);
            }
        });
        ck(cudaMemcpyAsync(const_cast<double*>(X), st, L.nv * 3 * sizeof(double), cudaMemcpyHostToDevice, s),
            "H2D X");
        if (ist) ck(cudaMemcpyAsync(fidx, ist, (size_t)L.nidx * 4, cudaMemcpyHostToDevice, s), "H2D idx");
        for (uint32_t p = 0; res && p < n; ++p) {
            if (!res[p]) continue;
            const Job& j = jobs[p];
            const ResidentCut& r = *res[p];
            const uint64_t n3 = 3ull * r.nv;
            g_launches++;
            k_apply_frame<<<grid1(n3), 256, 0, s>>>(r.X, const_cast<double*>(X) + ((size_t)L.vbase[p] + L.vs[p]) * 3,
                n3, j.com[0], j.com[1], j.com[2], j.t[0], j.t[1], j.t[2]);
        }
    } else {
        const cudaMemcpyKind kind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
        for (uint32_t p = 0; p < n; ++p) {
            ck(cudaMemcpyAsync(const_cast<double*>(X) + (size_t)L.vbase[p] * 3, srcs[p].vertices,
                   (size_t)L.vs[p] * 3 * sizeof(double), kind, s), "H2D Xs");
            ck(cudaMemcpyAsync(const_cast<double*>(X) + ((size_t)L.vbase[p] + L.vs[p]) * 3, cuts[p].vertices,
                   (size_t)cuts[p].num_vertices * 3 * sizeof(double), kind, s), "H2D Xc");
        }
    }
    const cudaMemcpyKind ikind = dev ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
    const bool staged = (flags & MCGPU_RECENTRE) != 0; // indices went up with the recentred coordinates
    if (split || host_read || gathered) {
        // the bounds kernel reads the caller's index arrays, or they were gathered above
    } else if (pk && !staged)
        ck(cudaMemcpyAsync(fidx, pk->idx, (size_t)L.nidx * 4, ikind, s), "H2D idx");
    else for (uint32_t p = 0; p < n; ++p) {
        const uint64_t ic = (uint64_t)L.ibase[p + 1] - L.ibase[p] - L.is[p];
        if (!staged)
            ck(cudaMemcpyAsync(fidx + L.ibase[p], srcs[p].face_indices, (size_t)L.is[p] * 4, ikind, s), "H2D Is");
        if (res && res[p])
            ck(cudaMemcpyAsync(fidx + L.ibase[p] + L.is[p], res[p]->idx, (size_t)ic * 4, cudaMemcpyDeviceToDevice, s),
                "D2D Ic");
        else if (!staged)
            ck(cudaMemcpyAsync(fidx + L.ibase[p] + L.is[p], cuts[p].face_indices, (size_t)ic * 4, ikind, s),
                "H2D Ic");
    }
    // per pair tables: ibase, is, vbase, vs, fbase, fs, sbase, cbase, clbase (n+1 each), eps
    constexpr int kRows = 9;
    const size_t rows_u32 = (size_t)kRows * (n + 1), eps_off = (rows_u32 + 1) & ~size_t(1);
    uint32_t* tab = c->pin_tab.get<uint32_t>(eps_off + 2 * (size_t)(n + 1));
    const std::vector<uint32_t>* rows[kRows] = { &L.ibase, &L.is, &L.vbase, &L.vs, &L.fbase, &L.fs, &L.sbase,
        &L.cbase, &L.clbase };
    for (int r = 0; r < kRows; ++r) memcpy(tab + (size_t)r * (n + 1), rows[r]->data(), sizeof(uint32_t) * (n + 1));
    double* teps = reinterpret_cast<double*>(tab + eps_off);
    memcpy(teps, L.eps.data(), sizeof(double) * n);
    uint32_t* dtab = c->buf[B_PTAB].get<uint32_t>(rows_u32);
    double* deps = c->buf[B_EPS].get<double>(n);
    ck(cudaMemcpyAsync(dtab, tab, sizeof(uint32_t) * rows_u32, cudaMemcpyHostToDevice, s), "H2D tab");
    c->eps_on_device = gathered;
    if (gathered) {
        // bounds of the gathered raw coordinates, then each pair's frame and
        // cut-box enlargement on the device; the enlargements come back with
        // the first readback
        double* dcom = c->buf[B_COM].get<double>(3 * (size_t)n);
        unsigned long long* rb = c->buf[B_RAWB].get<unsigned long long>(18 * (size_t)n);
        ck(cudaMemcpyAsync(dcom, c->pin_frames.get<double>(3 * (size_t)n), sizeof(double) * 3 * n,
               cudaMemcpyHostToDevice, s), "H2D centroids");
        ck(cudaMemsetAsync(rb, 0xFF, sizeof(unsigned long long) * 12 * n, s), "memset");
        ck(cudaMemsetAsync(rb + 12 * (size_t)n, 0, sizeof(unsigned long long) * 6 * n, s), "memset");
        g_launches += 2;
        k_raw_bounds<<<grid1((L.nv + kRawChunk - 1) / kRawChunk), 256, 0, s>>>(c->W.x_raw, fin ? 1 : 0,
            (uint32_t)L.nv, n, dtab + 2 * (n + 1), dtab + 3 * (n + 1), rb, rb + 12 * (size_t)n, rb + 6 * (size_t)n);
        k_frames<<<(n + 127) / 128, 128, 0, s>>>(n, dcom, rb, rb + 12 * (size_t)n, rb + 6 * (size_t)n, fin ? 1 : 0,
            c->gp_constant, gp_absolute ? 1 : 0, const_cast<double*>(c->W.frames), deps);
        ck(cudaMemcpyAsync(c->pin_eps.get<double>(n), deps, sizeof(double) * n, cudaMemcpyDeviceToHost, s),
            "D2H eps");
    } else {
        ck(cudaMemcpyAsync(deps, teps, sizeof(double) * n, cudaMemcpyHostToDevice, s), "H2D eps");
    }
    uint32_t* foff = nullptr;
    if (!L.all_tri) {
        std::vector<uint32_t> off(L.nf + 1);
        uint64_t o = 0, f = 0;
        for (uint32_t p = 0; p < n; ++p)
            for (int side = 0; side < 2; ++side) {
                const mcgpu_mesh& m = side ? cuts[p] : srcs[p];
                for (uint32_t k = 0; k < m.num_faces; ++k) {
                    off[f++] = (uint32_t)o;
                    o += face_size(m, k);
                }
            }
        off[f] = (uint32_t)o;
        foff = c->buf[B_FOFF].get<uint32_t>(L.nf + 1);
        ck(cudaMemcpyAsync(foff, off.data(), sizeof(uint32_t) * (L.nf + 1), cudaMemcpyHostToDevice, s), "H2D foff");
        ck(cudaStreamSynchronize(s), "sync foff"); // `off` is a pageable temporary
    }
    // A batch's indices are made global here, with its face -> pair table.
    // One pair's are made global by the bounds kernel, which reads the raw
    // indices (the caller's device arrays or the uploaded copy, left as they
    // are) and writes the global table and the face -> pair table as it goes.
    uint32_t* face_pair = c->buf[B_FPAIR].get<uint32_t>(L.nf);
    uint32_t* fidx_glob = fidx;
    if (n > 1) {
        g_launches++;
        k_prep<<<grid1(std::max(L.nidx, L.nf)), 256, 0, s>>>(n, dtab, fidx, L.nidx, face_pair, L.nf, nullptr,
            nullptr);
    } else {
        fidx_glob = c->buf[B_FIDXG].get<uint32_t>(std::max<uint64_t>(L.nidx, 1));
    }

    Problem& P = c->P;
    P.n_pairs = n;
    P.nv = (uint32_t)L.nv;
    P.nf = (uint32_t)L.nf;
    P.ns = (uint32_t)L.ns;
    P.nc = (uint32_t)L.nc;
    P.X = X;
    P.Xc = split ? static_cast<const double*>(cuts[0].vertices) : nullptr;
    P.xsplit = split ? L.vs[0] : 0xFFFFFFFFu;
    P.foff = foff;
    P.fidx = fidx_glob;
    P.face_pair = face_pair;
    P.fidx_cut = nullptr;
    P.fidx_split = P.cut_vbase = P.face_split = 0u;
    P.pair_fbase = dtab + 4 * (n + 1);
    P.pair_fs = dtab + 5 * (n + 1);
    P.pair_vbase = dtab + 2 * (n + 1);
    P.pair_vs = dtab + 3 * (n + 1);
    P.pair_sbase = dtab + 6 * (n + 1);
    P.pair_cbase = dtab + 7 * (n + 1);
    P.pair_eps = deps;
    P.pair_clbase = dtab + 8 * (n + 1);
    P.all_triangles = L.all_tri ? 1 : 0;
    P.leaf_size = L.leaf_size;
    P.ncl = (uint32_t)L.ncl;
    P.res_pairs = nullptr;
    P.pair_frames = nullptr;
    if (L.res_trees) {
        // each pair's resident tree (ncl 0 for the others) and frame
        ResPair* hr = c->pin_res.get<ResPair>(n);
        for (uint32_t p = 0; p < n; ++p) {
            ResPair r {};
            const ResidentCut* q = res[p];
            if (q && q->tree_ncl) {
                r.nodes = static_cast<const Node*>(q->tree_nodes);
                r.leaf_face = q->tree_leaf_face;
                r.cl_start = q->tree_cl_start;
                r.cl_n = q->tree_cl_n;
                r.ncl = q->tree_ncl;
                for (int j = 0; j < 3; ++j) r.mag[j] = std::max(std::fabs(q->st.mn[j]), std::fabs(q->st.mx[j]));
            }
            hr[p] = r;
        }
        ResPair* dr = c->buf[B_RESP].get<ResPair>(n);
        ck(cudaMemcpyAsync(dr, hr, sizeof(ResPair) * n, cudaMemcpyHostToDevice, s), "H2D resident trees");
        P.res_pairs = dr;
        if (gathered) {
            P.pair_frames = c->W.frames;
        } else {
            double* df = c->buf[B_FRAMES].get<double>(6 * (size_t)n);
            ck(cudaMemcpyAsync(df, c->pin_frames.get<double>(6 * (size_t)n), sizeof(double) * 6 * n,
                   cudaMemcpyHostToDevice, s), "H2D frames");
            P.pair_frames = df;
        }
    }
    // the bounds kernel's input view: one pair's raw indices, cut ones
    // offset by the source vertex count on the fly
    Problem& Pin = c->Pin;
    Pin = P;
    c->W.fidx_out = c->W.face_pair_out = nullptr;
    c->W.fidx_fix = n > 1 ? fidx : nullptr;
    if (n == 1) {
        Pin.fidx = (split || host_read) ? srcs[0].face_indices : fidx;
        Pin.face_pair = nullptr;
        Pin.fidx_cut = (split || host_read) ? cuts[0].face_indices : fidx + L.is[0];
        Pin.fidx_split = L.is[0];
        Pin.cut_vbase = L.vs[0];
        Pin.face_split = L.fs[0];
        c->W.fidx_out = fidx_glob;
        c->W.face_pair_out = face_pair;
    }
}

// stage events: 2k at the start of stage k, 2k+1 at its end; the host
// readbacks between stages fall outside every stage
inline void rec(mcgpu_context_t* c, int i)
{
    if (c->flags & MCGPU_PROFILE) ck(cudaEventRecord(c->ev[i], c->s), "event");
}

// Key of a launch segment: every value its launches read on the host.
template <typename... T>
std::vector<unsigned char> seg_key(const T&... v)
{
    std::vector<unsigned char> k;
    auto add = [&](const auto& x) {
        const unsigned char* b = reinterpret_cast<const unsigned char*>(&x);
        k.insert(k.end(), b, b + sizeof(x));
    };
    (add(v), ...);
    return k;
}

// Runs a launch segment. Without MCGPU_PROFILE: the first time a key is seen its launches run
// directly; the second time they are captured into a CUDA graph (thread-local
// capture: other threads' allocations are unaffected); after that the graph
// is replayed. A key holds the Problem/Work values and sizes the launches
// embed, so a replay sees the same buffers, sizes and parameters.
template <typename F>
void run_segment(mcgpu_context_t* c, int i, const std::vector<unsigned char>& key, F launches)
{
    auto& G = c->graphs[i];
    // stage events (MCGPU_PROFILE) are timed only on direct launches
    if (!c->use_graphs || (c->flags & MCGPU_PROFILE)) {
        launches(G.aux);
        return;
    }
    if (G.exec && G.key == key) {
        g_launches += G.launches;
        ck(cudaGraphLaunch(G.exec, c->s), "cudaGraphLaunch");
        return;
    }
    if (G.key != key) {
        if (G.exec) cudaGraphExecDestroy(G.exec);
        G.exec = nullptr;
        G.key = key;
        G.seen = 0;
    }
    if (++G.seen < 2) {
        launches(G.aux);
        return;
    }
    ck(cudaStreamBeginCapture(c->s, cudaStreamCaptureModeThreadLocal), "cudaStreamBeginCapture");
    const unsigned long long l0 = g_launches;
    launches(G.aux);
    cudaGraph_t graph = nullptr;
    ck(cudaStreamEndCapture(c->s, &graph), "cudaStreamEndCapture");
    G.launches = g_launches - l0;
    const cudaError_t e = cudaGraphInstantiate(&G.exec, graph, 0);
    cudaGraphDestroy(graph);
    ck(e, "cudaGraphInstantiate");
    ck(cudaGraphLaunch(G.exec, c->s), "cudaGraphLaunch");
}

int run(mcgpu_context_t* c, uint32_t flags, uint32_t n, const mcgpu_mesh* srcs, const mcgpu_mesh* cuts,
    const double* eps, mcgpu_summary* out, const Packed* pk = nullptr, const ResidentCut* const* res = nullptr)
{
    if (!c || !srcs || !cuts || n == 0) return fail(MCGPU_INVALID_VALUE, "null argument");
    if (flags & MCGPU_DEVICE_POINTERS && flags & (MCGPU_RECENTRE | MCGPU_VERTEX_ARRAY_FLOAT))
        return fail(MCGPU_INVALID_VALUE, "device pointers must hold recentred double coordinates");
    if (!(flags & MCGPU_RECENTRE) && !eps) return fail(MCGPU_INVALID_VALUE, "cut_eps required without RECENTRE");
    const bool enforce = (flags & (MCGPU_ENFORCE_GENERAL_POSITION | MCGPU_ENFORCE_GENERAL_POSITION_ABSOLUTE)) != 0;
    if (enforce && (n != 1 || pk || res))
        return fail(MCGPU_INVALID_VALUE, "general-position enforcement is per pair (mcgpu_dispatch)");
    if ((flags & MCGPU_VERTEX_ARRAY_FLOAT) && !(flags & MCGPU_RECENTRE))
        return fail(MCGPU_INVALID_VALUE, "float vertices need MCGPU_RECENTRE");
    ck(cudaSetDevice(c->device), "cudaSetDevice");
    c->flags = flags;
    c->derived_ready = false;
    c->cutpath_ready = false;
    c->floating_ready = false;
    c->have_results = false;
    const unsigned long long launches0 = g_launches;
    int rc = build_layout(c, flags, n, srcs, cuts, eps, res);
    if (rc != MCGPU_OK) return rc;
    Layout& L = c->L;
    cudaStream_t s = c->s;
    rec(c, 2 * MCGPU_STAGE_UPLOAD);
    upload(c, flags, srcs, cuts, pk, res);
    rec(c, 2 * MCGPU_STAGE_UPLOAD + 1);

    Problem& P = c->P;
    Work& W = c->W;
    const bool wide = n > 1;
    const int pbits = n > 1 ? 32 - __builtin_clz(n - 1) : 0;
    const int key_bits = kMortonBits + pbits;
    // stage-1 buffers
    W.fbox = c->buf[B_FBOX].get<double>(L.nf * 6);
    // fp32 vertex copies for orient3d's first filter (written by the bounds kernel)
    W.x32 = c->buf[B_X32].get<float4>(std::max<uint64_t>(L.nv, 1));
    P.X32 = W.x32;
    c->Pin.X32 = W.x32;
    W.fbox32 = c->buf[B_LKB].get<float>(L.nf * 6);
    W.mesh_box = c->buf[B_MESHBOX].get<unsigned long long>((size_t)n * 12);
    W.mesh_frame = c->buf[B_FRAME].get<uint8_t>((size_t)n * 64);
    const size_t ksz = wide ? 8 : 4;
    for (int b = 0; b < 2; ++b) {
        W.skeys[b] = c->buf[b ? B_SK1 : B_SK0].get<uint8_t>((L.ns + L.nc) * ksz);
        W.svals[b] = c->buf[b ? B_SV1 : B_SV0].get<uint32_t>(L.ns + L.nc);
        W.ckeys[b] = static_cast<uint8_t*>(W.skeys[b]) + L.ns * ksz;
        W.cvals[b] = W.svals[b] + L.ns;
    }
    W.cl_key = c->buf[B_CLKEY].get<uint8_t>(L.ncl * ksz);
    W.cl_start = c->buf[B_CLSTART].get<uint32_t>(L.ncl);
    W.cl_n = c->buf[B_CLN].get<uint8_t>(L.ncl);
    W.leaf_key_box = nullptr;
    W.packets = c->buf[B_PACKETS].get<uint2>(L.ns);
    W.top = c->buf[B_TOP].get<uint8_t>(64 * 32);
    // slow packets split for the second traversal launch (one entry per two
    // queries and 32 subtree roots; past the cap a packet finishes its own walk)
    W.split_cap = c->split_cap ? c->split_cap : std::min<uint64_t>(std::max<uint64_t>(4096, L.ns), 4u << 20);
    W.split = c->buf[B_SPLIT].get<uint8_t>(W.split_cap * 144);
    W.nodes = c->buf[B_NODES].get<Node>(std::max<uint64_t>(L.ncl, 2) - 1);
    W.split_far = c->buf[B_PARENT].get<uint32_t>(std::max<uint64_t>(L.ncl, 2));
    W.split_box = c->buf[B_NRANGE].get<uint8_t>(64 * std::max<uint64_t>(L.ncl, 2));
    W.counters = c->buf[B_COUNTERS].get<uint32_t>(16);
    W.cand = c->buf[B_CAND].get<uint8_t>(L.nf);
    W.pair_status = c->buf[B_PSTAT].get<uint32_t>(n);
    W.pair_bad = c->buf[B_PBAD].get<int32_t>(n);
    W.pair_nrec = c->buf[B_PNREC].get<uint32_t>(n + 1);
    W.pair_cnt = n > 1 ? c->buf[B_PCNT].get<uint32_t>((size_t)n * 5) : nullptr;
    W.pair_root = n > 1 ? c->buf[B_PROOT].get<int32_t>(n) : nullptr;
    W.scan_temp = c->buf[B_SCANTMP].get<uint32_t>(scan_temp_bytes((uint32_t)L.nv + 1) / 4 + 64);
    if (W.pair_cap == 0) W.pair_cap = std::max<uint64_t>(1 << 16, 2 * (L.ns + L.nc));
    W.pairs = c->buf[B_PAIRS].get<unsigned long long>(W.pair_cap);

    W.sort_temp = c->buf[B_SORTTMP].get<uint32_t>(radix_sort_temp_bytes((uint32_t)(L.ns + L.nc)) / 4 + 64);
    W.traversal = c->tune.traversal;
    W.packet_faces = c->tune.packet_faces;
    W.stack_depth = c->tune.stack_depth;
    W.split_round = c->tune.split_round;
    const uint32_t prof = flags & MCGPU_PROFILE;
    const uint32_t keep = flags & MCGPU_KEEP_TESTS;
    int src_buf = 0, cut_buf = 0;
    // host readback block: counters [0, 16), per-pair status, degenerate face,
    // record ranges (n + 1), then from hcnt a batch's per-pair counts (5 n)
    uint32_t* hc = c->pin_counters.get<uint32_t>(16 + 8 * (size_t)n + 8);
    uint32_t* const hcnt = hc + 16 + 3 * (size_t)n + 8;
    auto seg0 = [&](int* aux) {
        rec(c, 2 * MCGPU_STAGE_BOUNDS);
        g_launches++;
        k_init_dispatch<<<grid1((uint64_t)n * 12 + 16), 256, 0, s>>>(W.mesh_box, n, W.counters, W.pair_status,
            W.pair_bad, W.pair_nrec, W.pair_cnt, W.pair_root); // the candidate-face flags are cleared by the bounds kernel
        launch_bounds_morton(P, c->Pin, W, wide, key_bits, s);
        rec(c, 2 * MCGPU_STAGE_BOUNDS + 1);
        rec(c, 2 * MCGPU_STAGE_SORT);
        aux[0] = launch_sort(P, W, wide, key_bits, s, aux[1]);
        rec(c, 2 * MCGPU_STAGE_SORT + 1);
        rec(c, 2 * MCGPU_STAGE_HIERARCHY);
        // the query packets (source keys) beside the cut tree's build
        ck(cudaEventRecord(c->fork[0], s), "fork");
        ck(cudaStreamWaitEvent(c->s2, c->fork[0], 0), "fork");
        launch_packets(P, W, aux[0], c->s2);
        ck(cudaEventRecord(c->join[0], c->s2), "join");
        launch_hierarchy(P, W, wide, aux[1], s);
        ck(cudaStreamWaitEvent(s, c->join[0], 0), "join");
        rec(c, 2 * MCGPU_STAGE_HIERARCHY + 1);
        rec(c, 2 * MCGPU_STAGE_TRAVERSE);
        launch_traverse(P, W, aux[0], aux[1], false, s);
        rec(c, 2 * MCGPU_STAGE_TRAVERSE + 1);
    };
    auto seg1 = [&]() {
        rec(c, 2 * MCGPU_STAGE_ADJACENCY);
        // vertex -> face incidence beside the candidate-face planes
        ck(cudaEventRecord(c->fork[1], s), "fork");
        ck(cudaStreamWaitEvent(c->s2, c->fork[1], 0), "fork");
        launch_incidence(P, W, c->s2);
        ck(cudaEventRecord(c->join[1], c->s2), "join");
        launch_planes(P, W, s);
        ck(cudaStreamWaitEvent(s, c->join[1], 0), "join");
        rec(c, 2 * MCGPU_STAGE_ADJACENCY + 1);
        rec(c, 2 * MCGPU_STAGE_NARROW);
        launch_tests(P, W, s);
        launch_narrow(P, W, keep != 0, s);
        rec(c, 2 * MCGPU_STAGE_NARROW + 1);
    };
    // stage-3 buffers for np candidate pairs (all_planes: a plane slot for every face)
    auto size_stage3 = [&](uint64_t np, bool all_planes) -> int {
        W.plane_cap = all_planes ? std::max<uint64_t>(L.nf, 1) : std::min<uint64_t>(L.nf, 2 * np + 1);
        W.plane_slot = c->buf[B_PSLOT].get<uint32_t>(L.nf);
        W.planes = c->buf[B_PLANES].get<FacePlane>(W.plane_cap);
        W.proj_flag = c->buf[B_PFLAG].get<uint32_t>(W.plane_cap);
        W.proj_list = c->buf[B_PLIST].get<uint32_t>(W.plane_cap);
        W.poly_list = c->buf[B_POLY].get<uint32_t>(L.all_tri ? 1 : L.nf);
        W.tri_stride = L.all_tri ? 0 : L.tri_stride;
        W.tri_scratch_cap = W.tri_stride * std::max<uint64_t>(L.n_poly, 1);
        W.tri_scratch = c->buf[B_TRI].get<double>(W.tri_scratch_cap * 3 + 1);
        W.vneed = c->buf[B_VNEED].get<uint8_t>(L.nv);
        W.voff = c->buf[B_VOFF].get<uint32_t>(L.nv + 1);
        W.vcur = c->buf[B_VCUR].get<uint32_t>(L.nv);
        W.inc_slots = c->csr_incidence ? 0u : c->inc_slots;
        W.inc_cap = W.inc_slots ? (uint64_t)L.nv * W.inc_slots : L.nidx;
        W.vface = c->buf[B_VFACE].get<uint32_t>(std::max<uint64_t>(W.inc_cap, 1));
        W.test_cap = std::max<uint64_t>(1, 2ull * L.max_face * np);
        if (W.test_cap > 0xFFFFFFFFull) return fail(MCGPU_TOO_LARGE, "edge-face tests exceed 2^32");
        W.tests = c->buf[B_TESTS].get<Test>(W.test_cap);
        W.test_info = c->buf[B_TINFO].get<int8_t>((flags & MCGPU_KEEP_TESTS) ? W.test_cap * 4 : 4);
        W.rec_key[0] = c->buf[B_RK0].get<unsigned long long>(W.test_cap);
        W.rec_key[1] = c->buf[B_RK1].get<unsigned long long>(W.test_cap);
        W.rec_val[0] = c->buf[B_RV0].get<uint32_t>(W.test_cap);
        W.rec_val[1] = c->buf[B_RV1].get<uint32_t>(W.test_cap);
        W.rec_pt_raw = c->buf[B_RPTRAW].get<double>(W.test_cap * 3);
        W.sort_temp = c->buf[B_SORTTMP].get<uint32_t>(
            radix_sort_temp_bytes((uint32_t)std::max<uint64_t>(L.ns + L.nc, W.test_cap)) / 4 + 64);
        return MCGPU_OK;
    };
    // record segment from the host's record count, then the per-pair ranges
    auto record_segment = [&]() {
        W.rec_ids = c->buf[B_RIDS].get<uint32_t>(std::max<uint64_t>(c->n_records, 1) * 5);
        W.rec_pts = c->buf[B_RPTS].get<double>(std::max<uint64_t>(c->n_records, 1) * 3);
        const uint32_t nrec = (uint32_t)c->n_records;
        run_segment(c, 2, seg_key(P, W, n, nrec, prof), [&](int* aux) {
            rec(c, 2 * MCGPU_STAGE_DOWNLOAD); // record sort + gather (added to the narrow stage)
            aux[0] = launch_records(P, W, nrec, s);
            rec(c, 2 * MCGPU_STAGE_DOWNLOAD + 1);
        });
        c->rec_buf = c->graphs[2].aux[0];
        // per-pair record ranges (first sorted record of each pair, then the total)
        if (n > 1)
            ck(cudaMemcpyAsync(hc + 16 + 2 * (size_t)n, W.pair_nrec, 4 * (size_t)(n + 1), cudaMemcpyDeviceToHost, s),
                "D2H ranges");
        else {
            hc[16 + 2] = 0;
            hc[16 + 3] = (uint32_t)c->n_records;
        }
        ck(cudaStreamSynchronize(s), "sync records");
    };
    auto read_status = [&](bool ranges) {
        ck(cudaMemcpyAsync(hc, W.counters, 64, cudaMemcpyDeviceToHost, s), "D2H counters");
        ck(cudaMemcpyAsync(hc + 16, W.pair_status, 4 * (size_t)n, cudaMemcpyDeviceToHost, s), "D2H status");
        ck(cudaMemcpyAsync(hc + 16 + n, W.pair_bad, 4 * (size_t)n, cudaMemcpyDeviceToHost, s), "D2H bad");
        if (ranges)
            ck(cudaMemcpyAsync(hc + 16 + 2 * (size_t)n, W.pair_nrec, 4 * (size_t)(n + 1), cudaMemcpyDeviceToHost, s),
                "D2H ranges");
        if (W.pair_cnt)
            ck(cudaMemcpyAsync(hcnt, W.pair_cnt, 20 * (size_t)n, cudaMemcpyDeviceToHost, s), "D2H pair counts");
    };
    // the stage-3 buffers of the previous call stay out of the segment keys
    auto clear_stage3 = [&]() {
        W.plane_slot = W.proj_flag = W.proj_list = W.poly_list = W.voff = W.vcur = W.vface = W.rec_ids = nullptr;
        W.planes = nullptr;
        W.vneed = nullptr;
        W.tri_scratch = nullptr;
        W.tests = nullptr;
        W.test_info = nullptr;
        W.rec_key[0] = W.rec_key[1] = nullptr;
        W.rec_val[0] = W.rec_val[1] = nullptr;
        W.rec_pt_raw = W.rec_pts = nullptr;
        W.tri_scratch_cap = W.tri_stride = W.test_cap = W.inc_cap = W.plane_cap = 0;
        W.inc_slots = 0;
    };
    clear_stage3();
    if (seg_key(P, c->Pin, W, n, key_bits, prof) != c->fuse_key) c->csr_incidence = false; // a new layout
    uint64_t npairs = 0;
    std::vector<unsigned char> key0;
    // a vertex with more incident faces than the fixed incidence slots reruns
    // the call with CSR incidence (kept for the layout's later calls)
    for (;;) {
        clear_stage3();
        key0 = seg_key(P, c->Pin, W, n, key_bits, prof);
        bool done = false;
        // Fused call: after a call of the same shape, the three segments run as
        // one graph with one readback. Stage 3 is sized before the pair count is
        // known: a plane slot for every face, and tests for the previous call's
        // pairs plus a quarter (at most the pair capacity); every kernel guards
        // its capacity, and the records are ordered from the count left on the
        // device. A pair, test or traversal-stack overflow reruns the call stage
        // by stage; a record count past the one-launch ordering reruns only the
        // record segment.
        if (c->use_graphs && c->use_fuse && !prof && c->fuse_ok && c->fuse_key == key0) {
            rc = size_stage3(std::min<uint64_t>(W.pair_cap, c->fuse_npairs + c->fuse_npairs / 4 + 1024), true);
            if (rc != MCGPU_OK) return rc;
            const uint32_t rec_cap = (uint32_t)std::min<uint64_t>(W.test_cap, kRankSortMax);
            const bool dev_rec = c->fuse_nrec <= rec_cap;
            if (dev_rec) {
                W.rec_ids = c->buf[B_RIDS].get<uint32_t>((size_t)rec_cap * 5);
                W.rec_pts = c->buf[B_RPTS].get<double>((size_t)rec_cap * 3);
            }
            run_segment(c, 3, seg_key(P, c->Pin, W, n, key_bits, keep, dev_rec, rec_cap), [&](int* aux) {
                seg0(aux);
                seg1();
                aux[2] = dev_rec ? launch_records_dev(P, W, rec_cap, s) : 0;
            });
            src_buf = c->graphs[3].aux[0];
            cut_buf = c->graphs[3].aux[1];
            read_status(dev_rec && n > 1);
            ck(cudaStreamSynchronize(s), "sync fused");
            bool rerun = false;
            for (uint32_t p = 0; p < n; ++p) rerun |= (hc[16 + p] & (ST_STACK | ST_OVERFLOW_TESTS)) != 0;
            if (!rerun && hc[0] <= W.pair_cap) {
                npairs = hc[0];
                c->n_pairs_found = npairs;
                c->n_tests = hc[1];
                c->n_records = hc[2];
                if (dev_rec && c->n_records <= rec_cap) {
                    c->rec_buf = c->graphs[3].aux[2];
                    if (n == 1) {
                        hc[16 + 2] = 0;
                        hc[16 + 3] = (uint32_t)c->n_records;
                    }
                } else {
                    record_segment();
                }
                done = true;
            }
        }
        if (!done) {
            run_segment(c, 0, key0, seg0);
            src_buf = c->graphs[0].aux[0];
            cut_buf = c->graphs[0].aux[1];

            // readback 1: pair count and traversal flags
            ck(cudaMemcpyAsync(hc, W.counters, 64, cudaMemcpyDeviceToHost, s), "D2H counters");
            ck(cudaMemcpyAsync(hc + 16, W.pair_status, 4 * (size_t)n, cudaMemcpyDeviceToHost, s), "D2H status");
            ck(cudaStreamSynchronize(s), "sync traverse");
            bool deep = false;
            for (int attempt = 0; attempt < 4; ++attempt) {
                bool stack = false;
                for (uint32_t p = 0; p < n; ++p) stack |= (hc[16 + p] & ST_STACK) != 0;
                const uint64_t np = hc[0];
                if (!stack && np <= W.pair_cap) break;
                if (np > W.pair_cap) {
                    W.pair_cap = np + np / 8 + 1024;
                    W.pairs = c->buf[B_PAIRS].get<unsigned long long>(W.pair_cap);
                }
                deep = deep || stack;
                ck(cudaMemsetAsync(W.counters, 0, 64, s), "memset");
                ck(cudaMemsetAsync(W.cand, 0, L.nf, s), "memset");
                // the traversal's bits go; the bounds kernel's ST_INVALID stays
                launch_clear_status(W.pair_status, n, ST_STACK | ST_OVERFLOW_PAIRS, s);
                launch_packets(P, W, src_buf, s);
                launch_traverse(P, W, src_buf, cut_buf, deep, s);
                ck(cudaMemcpyAsync(hc, W.counters, 64, cudaMemcpyDeviceToHost, s), "D2H counters");
                ck(cudaMemcpyAsync(hc + 16, W.pair_status, 4 * (size_t)n, cudaMemcpyDeviceToHost, s), "D2H status");
                ck(cudaStreamSynchronize(s), "sync traverse");
            }
            npairs = hc[0];
            c->n_pairs_found = npairs;
            rc = size_stage3(npairs, false);
            if (rc != MCGPU_OK) return rc;
            run_segment(c, 1, seg_key(P, W, n, keep, prof), [&](int*) { seg1(); });

            // readback 2: counters, per-pair status / degenerate face / record count
            read_status(false);
            ck(cudaStreamSynchronize(s), "sync narrow");
            c->n_tests = hc[1];
            c->n_records = hc[2];
            record_segment();
        }
        if (hc[12] == 0 || W.inc_slots == 0) break;
        c->csr_incidence = true;
    }
    // the enlargements the device computed (the first readback has them on the host)
    if (c->eps_on_device) memcpy(L.eps.data(), c->pin_eps.get<double>(n), sizeof(double) * n);
    c->fuse_key = key0;
    c->fuse_ok = true;
    c->fuse_nrec = c->n_records;
    c->fuse_npairs = npairs;

    // General-position enforcement (preproc.cpp:2590-2699, 2933-2945): each
    // attempt perturbs the narrow phase's cut vertices by uniform(-1, 1) *
    // cut_eps per axis and runs stage 3 and the record order again. The pairs,
    // face boxes and cut tree of the unperturbed meshes stay: the reference
    // builds the cut BVH only on the first attempt (preproc.cpp:2680) and
    // traverses only after a rebuild (preproc.cpp:2820-2846); the boxes are
    // enlarged by cut_eps, so they still hold the perturbed faces.
    uint32_t perturbations = 0;
    double pert[3] = { 0.0, 0.0, 0.0 };
    auto violated = [&]() {
        if ((hc[16] & ST_INVALID) || (int32_t)hc[17] != kNoBad) return false;
        // a perturbed pass that meets nothing is a violation (kernel.cpp:3211-3225)
        return (hc[16] & ST_GP) != 0 || (perturbations > 0 && c->n_records == 0);
    };
    if (enforce && violated()) {
        const uint64_t nc3 = 3ull * (L.nv - L.vs[0]);
        const double* base = P.xsplit != 0xFFFFFFFFu ? P.Xc : P.X + (size_t)L.vs[0] * 3;
        double* xp = c->buf[B_XPERT].get<double>(std::max<uint64_t>(nc3, 3));
        P.Xc = xp; // the cut vertices the narrow phase reads from now on
        P.xsplit = L.vs[0];
        P.X32 = nullptr; // the fp32 copies are of the unperturbed vertices
        while (violated() && perturbations < c->gp_attempts) {
            for (int j = 0; j < 3; ++j) pert[j] = c->gp_uniform(c->gp_rng) * L.eps[0];
            ++perturbations;
            g_launches++;
            k_perturb<<<grid1(nc3), 256, 0, s>>>(base, xp, nc3, pert[0], pert[1], pert[2]);
            // stage 3 starts again from its own counters (the pair count and the
            // traversal's stay), statuses and record ranges
            ck(cudaMemsetAsync(W.counters + 1, 0, 7 * sizeof(uint32_t), s), "memset");
            ck(cudaMemsetAsync(W.counters + 10, 0, 3 * sizeof(uint32_t), s), "memset");
            ck(cudaMemsetAsync(W.pair_status, 0, 4, s), "memset");
            ck(cudaMemsetAsync(W.pair_bad, 0x7F, 4, s), "memset");
            ck(cudaMemsetAsync(W.pair_nrec, 0, 8, s), "memset");
            run_segment(c, 1, seg_key(P, W, n, keep, prof), [&](int*) { seg1(); });
            read_status(false);
            ck(cudaStreamSynchronize(s), "sync narrow");
            c->n_tests = hc[1];
            c->n_records = hc[2];
            record_segment();
        }
    }
    ck(cudaGetLastError(), "kernel launch");

    c->sums.assign(n, mcgpu_summary());
    c->rec_begin.assign(n + 1, 0);
    for (uint32_t p = 0; p < n; ++p) {
        mcgpu_summary& m = c->sums[p];
        memset(&m, 0, sizeof m);
        const uint32_t st = hc[16 + p];
        const int32_t bad = (int32_t)hc[16 + n + p];
        m.bad_face = -1;
        if (st & ST_INVALID) m.status = MCGPU_INVALID_INPUT;
        else if (bad != kNoBad) {
            m.bad_face = bad;
            m.status = (uint32_t)bad >= L.fs[p] ? MCGPU_DEGENERATE_CUT_FACE : MCGPU_DEGENERATE_SRC_FACE;
        } else if (st & ST_GP) m.status = MCGPU_GP_VIOLATION;
        else m.status = MCGPU_OK;
        m.cut_eps = L.eps[p];
        m.num_records = c->n_records ? hc[16 + 2 * n + p + 1] - hc[16 + 2 * n + p] : 0;
        c->rec_begin[p + 1] = c->rec_begin[p] + m.num_records;
    }
    if (perturbations) {
        mcgpu_summary& m = c->sums[0];
        if (m.status == MCGPU_OK && c->n_records == 0) m.status = MCGPU_GP_VIOLATION;
        m.perturbations = perturbations;
        memcpy(m.perturbation, pert, sizeof pert);
    }
    if (n == 1) {
        c->sums[0].num_pairs = npairs;
        c->sums[0].num_tests = c->n_tests;
        c->sums[0].escalations[0] = hc[5];
        c->sums[0].escalations[1] = hc[6];
        c->sums[0].escalations[2] = hc[7];
    } else {
        for (uint32_t p = 0; p < n; ++p) {
            mcgpu_summary& m = c->sums[p];
            const uint32_t* k = hcnt + 5 * (size_t)p;
            m.num_pairs = k[0];
            m.num_tests = k[1];
            for (int j = 0; j < 3; ++j) m.escalations[j] = k[2 + j];
        }
    }
    if (flags & MCGPU_PROFILE) {
        // stage times of the whole call (every summary of a batch carries them)
        float st[8];
        for (int k = 0; k < 8; ++k) {
            st[k] = 0.f;
            cudaEventElapsedTime(&st[k], c->ev[2 * k], c->ev[2 * k + 1]);
        }
        st[MCGPU_STAGE_NARROW] += st[MCGPU_STAGE_DOWNLOAD];
        st[MCGPU_STAGE_DOWNLOAD] = 0.f;
        for (auto& m : c->sums) memcpy(m.stage_ms, st, sizeof st);
    }
    for (auto& m : c->sums) m.kernel_launches = (uint32_t)(g_launches - launches0);
    c->have_results = true;
    if (out) {
        if (n == 1) *out = c->sums[0];
        else memcpy(out, c->sums.data(), sizeof(mcgpu_summary) * n);
    }
    return MCGPU_OK;
}

// The record hand-over of the last dispatch (one pair), built once per
// dispatch on the context stream; the counts are read back with it.
int ensure_derived(mcgpu_context_t* c)
{
    if (c->derived_ready) return MCGPU_OK;
    if (c->L.n_pairs != 1) return fail(MCGPU_INVALID_VALUE, "the record hand-over is built for a single dispatch");
    const uint64_t R64 = c->n_records;
    if (7 * R64 + 1 > 0xFFFFFFFFull) return fail(MCGPU_TOO_LARGE, "too many records for the hand-over maps");
    const uint32_t R = (uint32_t)R64;
    const size_t r = std::max<size_t>(R, 1);
    DerivedScratch w {};
    w.ck[0] = c->buf[B_DCK0].get<unsigned long long>(2 * r);
    w.ck[1] = c->buf[B_DCK1].get<unsigned long long>(2 * r);
    w.cv[0] = c->buf[B_DCV0].get<uint32_t>(2 * r);
    w.cv[1] = c->buf[B_DCV1].get<uint32_t>(2 * r);
    w.fk[0] = c->buf[B_DFK0].get<uint32_t>(3 * r);
    w.fk[1] = c->buf[B_DFK1].get<uint32_t>(3 * r);
    w.fv[0] = c->buf[B_DFV0].get<uint32_t>(3 * r);
    w.fv[1] = c->buf[B_DFV1].get<uint32_t>(3 * r);
    w.flags = c->buf[B_DFLAGS].get<uint32_t>(7 * r + 1);
    w.sort_temp = c->buf[B_DSORT].get<uint32_t>(derived_sort_temp_bytes(R) / 4 + 64);
    w.scan_temp = c->buf[B_DSCAN].get<uint32_t>(derived_scan_temp_bytes(R) / 4 + 64);
    // outputs back to back: edge_off R+1 | border R | cp_pairs 4R | cp_off 2R+1 | face_keys 3R | face_off 3R+1 |
    // counts: 14R + 3 + kDerivedCounts words
    uint32_t* o = c->buf[B_DOUT].get<uint32_t>(14 * r + 3 + kDerivedCounts);
    DerivedOut& d = c->derived;
    d.edge_off = o;
    d.border = d.edge_off + r + 1;
    d.cp_pairs = d.border + r;
    d.cp_off = d.cp_pairs + 4 * r;
    d.face_keys = d.cp_off + 2 * r + 1;
    d.face_off = d.face_keys + 3 * r;
    d.counts = d.face_off + 3 * r + 1; // == o + 14 r + 3
    d.cp_vtx = d.face_vtx = nullptr;
    const Layout& L = c->L;
    launch_derived(c->W.rec_ids, R, L.vs[0], (uint32_t)L.nv, L.fs[0], (uint32_t)L.nf, w, d, c->s);
    if (R == 0) { // no records: one edge offset (0), every list empty
        ck(cudaMemsetAsync(d.edge_off, 0, 4, c->s), "memset");
        ck(cudaMemsetAsync(d.cp_off, 0, 4, c->s), "memset");
        ck(cudaMemsetAsync(d.face_off, 0, 4, c->s), "memset");
    }
    ck(cudaMemcpyAsync(c->derived_counts, d.counts, sizeof(c->derived_counts), cudaMemcpyDeviceToHost, c->s),
        "D2H counts");
    ck(cudaStreamSynchronize(c->s), "sync hand-over");
    ck(cudaGetLastError(), "hand-over launch");
    c->derived_ready = true;
    return MCGPU_OK;
}

// The cut path of the last dispatch (one pair), from its record hand-over.
int ensure_cutpath(mcgpu_context_t* c)
{
    if (c->cutpath_ready) return MCGPU_OK;
    const int rc = ensure_derived(c);
    if (rc != MCGPU_OK) return rc;
    const uint32_t K = c->derived_counts[kDerivedCutpath], N = c->derived_counts[kDerivedCutpathEntries];
    const uint32_t R = (uint32_t)c->n_records;
    if (5ull * N + 1 > 0xFFFFFFFFull) return fail(MCGPU_TOO_LARGE, "too many intersection vertices for the cut path");
    const size_t cc = std::max<size_t>(N - K, 1), ne = std::max<size_t>(N, 1);
    CutpathScratch w {};
    w.cand = c->buf[B_CP_CAND].get<uint32_t>(4 * cc);
    w.inside = c->buf[B_CP_INSIDE].get<uint32_t>(2 * cc);
    w.sorted = c->buf[B_CP_SORTED].get<uint32_t>(ne);
    w.proj = c->buf[B_CP_PROJ].get<double>(ne);
    w.pk[0] = c->buf[B_CP_PK0].get<unsigned long long>(cc);
    w.pk[1] = c->buf[B_CP_PK1].get<unsigned long long>(cc);
    w.pv[0] = c->buf[B_CP_PV0].get<uint32_t>(cc);
    w.pv[1] = c->buf[B_CP_PV1].get<uint32_t>(cc);
    w.made = c->buf[B_CP_MADE].get<uint32_t>(cc + 1);
    w.fk[0] = c->buf[B_CP_FK0].get<unsigned long long>(5 * cc);
    w.fk[1] = c->buf[B_CP_FK1].get<unsigned long long>(5 * cc);
    w.fv[0] = c->buf[B_CP_FV0].get<uint32_t>(5 * cc);
    w.fv[1] = c->buf[B_CP_FV1].get<uint32_t>(5 * cc);
    w.hk[0] = c->buf[B_CP_HK0].get<unsigned long long>(2 * cc);
    w.hk[1] = c->buf[B_CP_HK1].get<unsigned long long>(2 * cc);
    w.hv[0] = c->buf[B_CP_HV0].get<uint32_t>(2 * cc);
    w.hv[1] = c->buf[B_CP_HV1].get<uint32_t>(2 * cc);
    w.flags = c->buf[B_CP_FLAGS].get<uint32_t>(5 * cc + 1);
    w.sort_temp = c->buf[B_CP_SORT].get<uint32_t>(cutpath_sort_temp_bytes((uint32_t)cc) / 4 + 64);
    w.scan_temp = c->buf[B_CP_SCAN].get<uint32_t>(cutpath_scan_temp_bytes((uint32_t)cc) / 4 + 64);
    // outputs back to back: edges 2C | face_keys 5C | face_off 5C+1 | face_edges 5C | ivtx_off R+1 | ivtx_he 2C |
    // counts
    const size_t r = (size_t)R;
    uint32_t* o = c->buf[B_CP_OUT].get<uint32_t>(19 * cc + r + 2 + kCpCounts);
    CutpathOut& d = c->cutpath;
    d.edges = o;
    d.face_keys = d.edges + 2 * cc;
    d.face_off = d.face_keys + 5 * cc;
    d.face_edges = d.face_off + 5 * cc + 1;
    d.ivtx_off = d.face_edges + 5 * cc;
    d.ivtx_he = d.ivtx_off + r + 1;
    d.counts = d.ivtx_he + 2 * cc; // == o + 19 cc + r + 2
    const Layout& L = c->L;
    const Problem& P = c->P;
    CutpathInput in {};
    in.X = P.X;
    in.Xc = P.Xc;
    in.xsplit = P.xsplit;
    in.fidx = P.fidx;
    in.foff = P.foff;
    in.nv = (uint32_t)L.nv;
    in.nf = (uint32_t)L.nf;
    in.fs = L.fs[0];
    in.rec_ids = c->W.rec_ids;
    in.rec_pts = c->W.rec_pts;
    in.nrec = R;
    in.cp_pairs = c->derived.cp_pairs;
    in.cp_off = c->derived.cp_off;
    in.cp_vtx = c->derived.cp_vtx;
    in.n_keys = K;
    in.n_entries = N;
    c->cutpath_in = in;
    launch_cutpath(in, w, d, c->s);
    ck(cudaMemcpyAsync(c->cutpath_counts, d.counts, sizeof(c->cutpath_counts), cudaMemcpyDeviceToHost, c->s),
        "D2H cut-path counts");
    ck(cudaStreamSynchronize(c->s), "sync cut path");
    ck(cudaGetLastError(), "cut-path launch");
    c->cutpath_ready = true;
    return MCGPU_OK;
}

// The wire arrays of the last halfedge mesh (a connected component given in
// its corner order): its faces' vertices and face adjacency.
void ensure_cc_wire(mcgpu_context_t* c)
{
    if (c->cw_ready) return;
    const uint64_t nidx = c->hm_nidx;
    CcWireOut& w = c->cw;
    w.face = c->buf[B_CW_FACE].get<uint32_t>(std::max<uint64_t>(nidx, 1));
    w.pos = c->buf[B_CW_POS].get<uint32_t>(nidx + 1);
    w.adj = c->buf[B_CW_ADJ].get<uint32_t>(std::max<uint64_t>(nidx, 1));
    w.adj_n = c->buf[B_CW_ADJN].get<uint32_t>(std::max<uint32_t>(c->hm_nf, 1));
    // the scan's block sums, then one word for the adjacency count
    const size_t sw = cc_wire_scan_bytes(nidx) / 4;
    uint32_t* scan = c->buf[B_CW_SCAN].get<uint32_t>(sw + 64);
    uint32_t* total = scan + sw + 32;
    launch_cc_wire(c->hm, c->hm_foff, c->hm_nf, nidx, w, scan, total, c->s);
    ck(cudaMemcpyAsync(&c->cw_total, total, 4, cudaMemcpyDeviceToHost, c->s), "D2H adjacency count");
    ck(cudaStreamSynchronize(c->s), "sync wire arrays");
    ck(cudaGetLastError(), "wire arrays");
    c->cw_ready = true;
}

// The floating polygons of the last dispatch (one pair), from its cut path.
int ensure_floating(mcgpu_context_t* c)
{
    if (c->floating_ready) return MCGPU_OK;
    const int rc = ensure_cutpath(c);
    if (rc != MCGPU_OK) return rc;
    const uint32_t R = (uint32_t)c->n_records;
    const size_t r = std::max<size_t>(R, 1);
    FloatingScratch w {};
    w.parent = c->buf[B_FP_PARENT].get<uint32_t>(r);
    w.flags = c->buf[B_FP_FLAGS].get<uint32_t>(r);
    w.size = c->buf[B_FP_SIZE].get<uint32_t>(r);
    w.k[0] = c->buf[B_FP_K0].get<unsigned long long>(r);
    w.k[1] = c->buf[B_FP_K1].get<unsigned long long>(r);
    w.v[0] = c->buf[B_FP_V0].get<uint32_t>(r);
    w.v[1] = c->buf[B_FP_V1].get<uint32_t>(r);
    w.sort_temp = c->buf[B_FP_SORT].get<uint32_t>(floating_sort_temp_bytes(R) / 4 + 64);
    w.scan_temp = c->buf[B_FP_SCAN].get<uint32_t>(floating_scan_temp_bytes(R) / 4 + 64);
    // outputs: faces R | off R+1 | vtx R | mc R | counts; normals apart (doubles)
    uint32_t* o = c->buf[B_FP_OUT].get<uint32_t>(4 * r + 1 + kFpCounts);
    FloatingOut& d = c->floating;
    d.faces = o;
    d.off = d.faces + r;
    d.vtx = d.off + r + 1;
    d.mc = reinterpret_cast<int32_t*>(d.vtx + r);
    d.counts = reinterpret_cast<uint32_t*>(d.mc + r);
    d.normals = c->buf[B_FP_NRM].get<double>(3 * r);
    launch_floating(c->cutpath_in, c->cutpath, w, d, c->s);
    ck(cudaMemcpyAsync(c->floating_counts, d.counts, sizeof(c->floating_counts), cudaMemcpyDeviceToHost, c->s),
        "D2H floating counts");
    ck(cudaStreamSynchronize(c->s), "sync floating polygons");
    ck(cudaGetLastError(), "floating-polygon launch");
    if (c->floating_counts[kFpError]) return fail(MCGPU_CUDA_ERROR, "floating polygons: union-find retry cap");
    c->floating_ready = true;
    return MCGPU_OK;
}

int copy_out(mcgpu_context_t* c, const void* dptr, uint64_t need, uint64_t bytes, void* mem, uint64_t* bytes_out)
{
    if (bytes_out) *bytes_out = need;
    if (!mem && bytes == 0) return MCGPU_OK;
    if (!mem || bytes < need) return fail(MCGPU_INVALID_VALUE, "output buffer too small");
    if (need) {
        ck(cudaMemcpyAsync(mem, dptr, need, cudaMemcpyDeviceToHost, c->s), "D2H data");
        ck(cudaStreamSynchronize(c->s), "sync data");
    }
    return MCGPU_OK;
}

} // namespace

extern "C" {

int mcgpu_context_create(mcgpu_context* out, int device)
{
    if (!out) return fail(MCGPU_INVALID_VALUE, "null context pointer");
    *out = nullptr;
    try {
        int n = 0;
        ck(cudaGetDeviceCount(&n), "cudaGetDeviceCount");
        if (device < 0 || device >= n) return fail(MCGPU_INVALID_VALUE, "no such CUDA device");
        ck(cudaSetDevice(device), "cudaSetDevice");
        mcgpu_context_t* c = new (std::nothrow) mcgpu_context_t();
        if (!c) return fail(MCGPU_OUT_OF_MEMORY, "host allocation");
        c->device = device;
        for (auto& b : c->buf) {
            b.held = &c->dev_held;
            b.limit = &c->dev_limit;
            b.stream = &c->s;
        }
        if (const char* e = getenv("MCGPU_LEAF_SIZE")) {
            const int v = atoi(e);
            if (v >= 1 && v <= 16) c->tune.leaf_size = (uint32_t)v;
        }
        if (const char* e = getenv("MCGPU_TRAVERSAL")) {
            if (!strcmp(e, "packet")) c->tune.traversal = 1;
            if (!strcmp(e, "thread")) c->tune.traversal = 2;
        }
        if (const char* e = getenv("MCGPU_PACKET_FACES")) {
            const int v = atoi(e);
            if (v >= 1 && v <= 32) c->tune.packet_faces = (uint32_t)v;
        }
        if (const char* e = getenv("MCGPU_GRAPHS")) c->use_graphs = atoi(e) != 0;
        if (const char* e = getenv("MCGPU_FUSE")) c->use_fuse = atoi(e) != 0;
        int pma = 0;
        if (cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, device) == cudaSuccess) c->host_reads = pma != 0;
        if (const char* e = getenv("MCGPU_HOST_READS")) c->host_reads = c->host_reads && atoi(e) != 0;
        if (const char* e = getenv("MCGPU_INC_SLOTS")) c->inc_slots = (uint32_t)std::min(64, std::max(0, atoi(e)));
        if (const char* e = getenv("MCGPU_SPLIT_CAP")) c->split_cap = strtoull(e, nullptr, 10);
        ck(cudaStreamCreateWithFlags(&c->s, cudaStreamNonBlocking), "stream");
        ck(cudaStreamCreateWithFlags(&c->s2, cudaStreamNonBlocking), "stream");
        for (int k = 0; k < 2; ++k) {
            ck(cudaEventCreateWithFlags(&c->fork[k], cudaEventDisableTiming), "event");
            ck(cudaEventCreateWithFlags(&c->join[k], cudaEventDisableTiming), "event");
        }
        for (auto& e : c->ev) ck(cudaEventCreate(&e), "event");
        *out = c;
        return MCGPU_OK;
    } catch (const CudaError& e) {
        return fail(e.e == cudaErrorMemoryAllocation ? MCGPU_OUT_OF_MEMORY : MCGPU_CUDA_ERROR,
            e.where + ": " + cudaGetErrorString(e.e));
    }
}

int mcgpu_measure_fp64_rate(int device, double* gops)
{
    if (!gops) return fail(MCGPU_INVALID_VALUE, "null output");
    *gops = 0.0;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || device < 0 || device >= n)
        return fail(MCGPU_INVALID_VALUE, "no such CUDA device");
    cudaSetDevice(device);
    int sms = 0;
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    const int blocks = std::max(1, sms) * 8, threads = 256, iters = 2048;
    double* out = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return fail(MCGPU_OUT_OF_MEMORY, "fp64 probe");
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) { // the first run warms up
        cudaEventRecord(e0);
        k_fp64_rate<<<blocks, threads>>>(out, iters, 0.999999, 1e-7);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    const cudaError_t err = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (err != cudaSuccess) return fail(MCGPU_CUDA_ERROR, std::string("fp64 probe: ") + cudaGetErrorString(err));
    *gops = (double)blocks * threads * iters * kFp64Chains * 2.0 / (best * 1e6);
    return MCGPU_OK;
}

int mcgpu_context_get_memory(mcgpu_context c, uint64_t* device_bytes, uint64_t* limit_bytes)
{
    if (!c) return fail(MCGPU_INVALID_VALUE, "null context");
    if (device_bytes) *device_bytes = c->dev_held;
    if (limit_bytes) *limit_bytes = c->dev_limit;
    return MCGPU_OK;
}

int mcgpu_context_set_memory_limit(mcgpu_context c, uint64_t limit_bytes)
{
    if (!c) return fail(MCGPU_INVALID_VALUE, "null context");
    c->dev_limit = limit_bytes;
    return MCGPU_OK;
}

int mcgpu_context_trim(mcgpu_context c)
{
    if (!c) return fail(MCGPU_INVALID_VALUE, "null context");
    cudaSetDevice(c->device);
    if (cudaStreamSynchronize(c->s) != cudaSuccess || cudaStreamSynchronize(c->s2) != cudaSuccess)
        return fail(MCGPU_CUDA_ERROR, "stream synchronize before trim");
    // the captured launch graphs hold the pool's addresses
    for (auto& g : c->graphs) {
        if (g.exec) cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
        g.key.clear();
        g.seen = 0;
    }
    c->fuse_key.clear();
    c->fuse_ok = false;
    c->derived_ready = false;
    c->cutpath_ready = false;
    c->floating_ready = false;
    c->hm_ready = false;
    c->have_results = false;
    c->W = mcgpu::Work {};
    for (auto& b : c->buf) b.release();
    // the frees are stream-ordered: the synchronize returns the memory
    if (cudaStreamSynchronize(c->s) != cudaSuccess) return fail(MCGPU_CUDA_ERROR, "stream synchronize after trim");
    return MCGPU_OK;
}

int mcgpu_context_release(mcgpu_context c)
{
    if (!c) return fail(MCGPU_INVALID_VALUE, "null context");
    cudaSetDevice(c->device);
    if (c->s) cudaStreamSynchronize(c->s);
    if (c->s)
        for (auto& b : c->buf) b.release();
    if (c->s) cudaStreamSynchronize(c->s);
    c->pin_counters.release();
    c->pin_tab.release();
    c->pin_stage.release();
    c->pin_res.release();
    c->pin_idx.release();
    c->pin_seg.release();
    c->pin_frames.release();
    c->pin_eps.release();
    for (auto& e : c->ev)
        if (e) cudaEventDestroy(e);
    for (auto& g : c->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    if (c->s2) cudaStreamSynchronize(c->s2);
    for (int k = 0; k < 2; ++k) {
        if (c->fork[k]) cudaEventDestroy(c->fork[k]);
        if (c->join[k]) cudaEventDestroy(c->join[k]);
    }
    if (c->s2) cudaStreamDestroy(c->s2);
    if (c->s) cudaStreamDestroy(c->s);
    delete c;
    return MCGPU_OK;
}

int mcgpu_dispatch(mcgpu_context c, uint32_t flags, const mcgpu_mesh* src, const mcgpu_mesh* cut, double cut_eps,
    mcgpu_summary* out)
{
    try {
        return run(c, flags, 1, src, cut, &cut_eps, out);
    } catch (const CudaError& e) {
        return fail(e.e == cudaErrorMemoryAllocation ? MCGPU_OUT_OF_MEMORY : MCGPU_CUDA_ERROR,
            e.where + ": " + cudaGetErrorString(e.e));
    }
}

int mcgpu_dispatch_batch(mcgpu_context c, uint32_t flags, uint32_t n_pairs, const mcgpu_mesh* srcs,
    const mcgpu_mesh* cuts, const double* cut_eps, mcgpu_summary* summaries)
{
    try {
        return run(c, flags, n_pairs, srcs, cuts, cut_eps, summaries);
    } catch (const CudaError& e) {
        return fail(e.e == cudaErrorMemoryAllocation ? MCGPU_OUT_OF_MEMORY : MCGPU_CUDA_ERROR,
            e.where + ": " + cudaGetErrorString(e.e));
    }
}

int mcgpu_dispatch_packed(mcgpu_context c, uint32_t flags, const mcgpu_batch* b, mcgpu_summary* summaries)
{
    if (!c || !b || !b->vertices || !b->face_indices || !b->mesh_counts || b->num_pairs == 0)
        return fail(MCGPU_INVALID_VALUE, "null argument");
    try {
        // per-pair views into the packed arrays (host side only: counts are host memory)
        const uint32_t n = b->num_pairs;
        std::vector<mcgpu_mesh> ms(n), mc(n);
        const size_t vsz = (flags & MCGPU_VERTEX_ARRAY_FLOAT) ? 12 : 24;
        const char* v = static_cast<const char*>(b->vertices);
        const uint32_t* ix = b->face_indices;
        const uint32_t* fs = b->face_sizes;
        for (uint32_t p = 0; p < n; ++p) {
            const uint32_t* k = b->mesh_counts + 4 * (size_t)p;
            for (int side = 0; side < 2; ++side) {
                mcgpu_mesh& m = side ? mc[p] : ms[p];
                m.num_vertices = k[2 * side];
                m.num_faces = k[2 * side + 1];
                m.vertices = v;
                m.face_indices = ix;
                m.face_sizes = fs;
                v += vsz * m.num_vertices;
                uint64_t ni = 3ull * m.num_faces;
                if (fs) {
                    if (flags & MCGPU_DEVICE_POINTERS)
                        return fail(MCGPU_INVALID_VALUE, "packed device batches hold triangles only");
                    ni = 0;
                    for (uint32_t f = 0; f < m.num_faces; ++f) ni += fs[f];
                    fs += m.num_faces;
                }
                ix += ni;
            }
        }
        // the per-mesh views are read one by one only by the host recentring;
        // build_layout reads counts, the upload copies each packed array once
        Packed pk { b->vertices, b->face_indices };
        return run(c, flags, n, ms.data(), mc.data(), b->cut_eps, summaries, &pk);
    } catch (const CudaError& e) {
        return fail(e.e == cudaErrorMemoryAllocation ? MCGPU_OUT_OF_MEMORY : MCGPU_CUDA_ERROR,
            e.where + ": " + cudaGetErrorString(e.e));
    }
}

int mcgpu_context_set_tuning(mcgpu_context c, const mcgpu_tuning* t)
{
    if (!c || !t) return fail(MCGPU_INVALID_VALUE, "null argument");
    if (t->leaf_size < 1 || t->leaf_size > 16 || t->traversal > 2 || t->packet_faces < 1 || t->packet_faces > 32
        || (t->stack_depth != 64 && t->stack_depth != 512) || t->split_round > 64)
        return fail(MCGPU_INVALID_VALUE, "tuning out of range");
    c->tune = *t;
    return MCGPU_OK;
}

int mcgpu_context_get_tuning(mcgpu_context c, mcgpu_tuning* t)
{
    if (!c || !t) return fail(MCGPU_INVALID_VALUE, "null argument");
    *t = c->tune;
    return MCGPU_OK;
}

int mcgpu_context_set_general_position(mcgpu_context c, double constant, uint32_t attempts)
{
    if (!c) return fail(MCGPU_INVALID_VALUE, "null argument");
    // the reference rejects a constant <= 0 and fewer than one attempt (frontend.cpp:390-410)
    if (!(constant > 0.0) || !std::isfinite(constant)) return fail(MCGPU_INVALID_VALUE, "invalid general position constant");
    if (attempts < 1) return fail(MCGPU_INVALID_VALUE, "invalid general position enforcement attempts");
    c->gp_constant = constant;
    c->gp_attempts = attempts;
    return MCGPU_OK;
}

int mcgpu_context_get_general_position(mcgpu_context c, double* constant, uint32_t* attempts)
{
    if (!c || !constant || !attempts) return fail(MCGPU_INVALID_VALUE, "null argument");
    *constant = c->gp_constant;
    *attempts = c->gp_attempts;
    return MCGPU_OK;
}

int mcgpu_autotune(mcgpu_context c, uint32_t flags, const mcgpu_batch* sample, uint32_t repeats, mcgpu_tuning* best,
    float* best_ms)
{
    if (!c || !sample || sample->num_pairs == 0) return fail(MCGPU_INVALID_VALUE, "null argument");
    if (repeats == 0) repeats = 3;
    std::vector<mcgpu_tuning> cand;
    for (uint32_t leaf : { 2u, 4u, 8u }) {
        cand.push_back({ leaf, 0, 32, 64, 2 });
        cand.push_back({ leaf, 0, 32, 64, 0 });
        cand.push_back({ leaf, 0, 16, 64, 2 });
        cand.push_back({ leaf, 1, 32, 64, 0 });
        cand.push_back({ leaf, 2, 32, 64, 0 });
        cand.push_back({ leaf, 2, 32, 512, 0 });
    }
    const mcgpu_tuning keep = c->tune;
    std::vector<mcgpu_summary> sums(sample->num_pairs);
    float best_t = 3.4e38f;
    mcgpu_tuning best_c = keep;
    for (const mcgpu_tuning& t : cand) {
        c->tune = t;
        for (int w = 0; w < 2; ++w) { // warm-up: pools sized, launch graph captured
            const int rc = mcgpu_dispatch_packed(c, flags & ~(uint32_t)MCGPU_PROFILE, sample, sums.data());
            if (rc != MCGPU_OK) {
                c->tune = keep;
                return rc;
            }
        }
        const auto t0 = std::chrono::steady_clock::now();
        for (uint32_t r = 0; r < repeats; ++r)
            if (mcgpu_dispatch_packed(c, flags & ~(uint32_t)MCGPU_PROFILE, sample, sums.data()) != MCGPU_OK) {
                c->tune = keep;
                return fail(MCGPU_CUDA_ERROR, "autotune dispatch failed");
            }
        const float ms =
            std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count() / repeats;
        if (ms < best_t) {
            best_t = ms;
            best_c = t;
        }
    }
    c->tune = best_c;
    if (best) *best = best_c;
    if (best_ms) *best_ms = best_t;
    return MCGPU_OK;
}

int mcgpu_get_data(mcgpu_context c, uint32_t query, uint64_t bytes, void* mem, uint64_t* bytes_out)
{
    if (!c) return fail(MCGPU_INVALID_VALUE, "null context");
    const bool hm_query = (query >= MCGPU_DATA_HE_TARGET && query < MCGPU_DATA_CUTPATH_STATUS)
        || (query >= MCGPU_DATA_CC_FACE && query <= MCGPU_DATA_CC_VERTEX_FLOAT);
    if (!hm_query && !c->have_results)
        return fail(MCGPU_INVALID_VALUE, "no dispatch results (none completed, or the pool was trimmed)");
    try {
        const Work& W = c->W;
        switch (query) {
        case MCGPU_DATA_RECORD_IDS:
            return copy_out(c, W.rec_ids, c->n_records * 5 * 4, bytes, mem, bytes_out);
        case MCGPU_DATA_RECORD_POINTS:
            return copy_out(c, W.rec_pts, c->n_records * 3 * 8, bytes, mem, bytes_out);
        case MCGPU_DATA_PAIRS: {
            // (source face, cut face) in per-pair local ids of a single dispatch
            const uint64_t need = c->n_pairs_found * 8;
            if (bytes_out) *bytes_out = need;
            if (!mem && bytes == 0) return MCGPU_OK;
            if (!mem || bytes < need) return fail(MCGPU_INVALID_VALUE, "output buffer too small");
            std::vector<unsigned long long> raw(c->n_pairs_found);
            ck(cudaMemcpyAsync(raw.data(), W.pairs, need, cudaMemcpyDeviceToHost, c->s), "D2H pairs");
            ck(cudaStreamSynchronize(c->s), "sync");
            uint32_t* o = (uint32_t*)mem;
            for (uint64_t i = 0; i < c->n_pairs_found; ++i) {
                const uint32_t sface = (uint32_t)(raw[i] >> 32), cface = (uint32_t)raw[i];
                // single dispatch: pair 0, cut faces follow the Fs source faces
                o[2 * i] = sface;
                o[2 * i + 1] = cface - c->L.fs[0];
            }
            return MCGPU_OK;
        }
        case MCGPU_DATA_TESTS: {
            if (!(c->flags & MCGPU_KEEP_TESTS)) return fail(MCGPU_INVALID_VALUE, "dispatch without MCGPU_KEEP_TESTS");
            const uint64_t need = c->n_tests * 12;
            if (bytes_out) *bytes_out = need;
            if (!mem && bytes == 0) return MCGPU_OK;
            if (!mem || bytes < need) return fail(MCGPU_INVALID_VALUE, "output buffer too small");
            std::vector<Test> raw(c->n_tests);
            ck(cudaMemcpyAsync(raw.data(), W.tests, c->n_tests * sizeof(Test), cudaMemcpyDeviceToHost, c->s), "D2H");
            ck(cudaStreamSynchronize(c->s), "sync");
            uint32_t* o = (uint32_t*)mem;
            for (uint64_t i = 0; i < c->n_tests; ++i) {
                o[3 * i] = raw[i].q;
                o[3 * i + 1] = raw[i].r;
                o[3 * i + 2] = raw[i].g;
            }
            return MCGPU_OK;
        }
        case MCGPU_DATA_TEST_INFO:
            if (!(c->flags & MCGPU_KEEP_TESTS)) return fail(MCGPU_INVALID_VALUE, "dispatch without MCGPU_KEEP_TESTS");
            return copy_out(c, W.test_info, c->n_tests * 4, bytes, mem, bytes_out);
        case MCGPU_DATA_VERTICES: {
            if (c->P.xsplit == 0xFFFFFFFFu) return copy_out(c, c->P.X, c->L.nv * 24, bytes, mem, bytes_out);
            // a single pair read in place from the caller's two device arrays
            const uint64_t need = c->L.nv * 24, first = (uint64_t)c->P.xsplit * 24;
            if (bytes_out) *bytes_out = need;
            if (!mem && bytes == 0) return MCGPU_OK;
            if (!mem || bytes < need) return fail(MCGPU_INVALID_VALUE, "output buffer too small");
            ck(cudaMemcpyAsync(mem, c->P.X, first, cudaMemcpyDeviceToHost, c->s), "D2H vertices");
            ck(cudaMemcpyAsync(static_cast<char*>(mem) + first, c->P.Xc, need - first, cudaMemcpyDeviceToHost, c->s),
                "D2H vertices");
            ck(cudaStreamSynchronize(c->s), "sync data");
            return MCGPU_OK;
        }
        case MCGPU_DATA_FACE_BOXES:
            return copy_out(c, W.fbox, c->L.nf * 48, bytes, mem, bytes_out);
        case MCGPU_DATA_EDGE_RECORD_OFFSETS:
        case MCGPU_DATA_CUTPATH_PAIRS:
        case MCGPU_DATA_CUTPATH_OFFSETS:
        case MCGPU_DATA_CUTPATH_VERTICES:
        case MCGPU_DATA_FACE_KEYS:
        case MCGPU_DATA_FACE_OFFSETS:
        case MCGPU_DATA_FACE_VERTICES:
        case MCGPU_DATA_BORDER_VERTICES:
        case MCGPU_DATA_PARTIAL_CUT: {
            const int rc = ensure_derived(c);
            if (rc != MCGPU_OK) return rc;
            const DerivedOut& d = c->derived;
            const uint32_t* n = c->derived_counts;
            switch (query) {
            case MCGPU_DATA_EDGE_RECORD_OFFSETS:
                return copy_out(c, d.edge_off, 4ull * (n[kDerivedEdges] + 1), bytes, mem, bytes_out);
            case MCGPU_DATA_CUTPATH_PAIRS:
                return copy_out(c, d.cp_pairs, 8ull * n[kDerivedCutpath], bytes, mem, bytes_out);
            case MCGPU_DATA_CUTPATH_OFFSETS:
                return copy_out(c, d.cp_off, 4ull * (n[kDerivedCutpath] + 1), bytes, mem, bytes_out);
            case MCGPU_DATA_CUTPATH_VERTICES:
                return copy_out(c, d.cp_vtx, 4ull * n[kDerivedCutpathEntries], bytes, mem, bytes_out);
            case MCGPU_DATA_FACE_KEYS:
                return copy_out(c, d.face_keys, 4ull * n[kDerivedFaces], bytes, mem, bytes_out);
            case MCGPU_DATA_FACE_OFFSETS:
                return copy_out(c, d.face_off, 4ull * (n[kDerivedFaces] + 1), bytes, mem, bytes_out);
            case MCGPU_DATA_FACE_VERTICES:
                return copy_out(c, d.face_vtx, 4ull * n[kDerivedFaceEntries], bytes, mem, bytes_out);
            case MCGPU_DATA_BORDER_VERTICES:
                return copy_out(c, d.border, 4ull * n[kDerivedBorder], bytes, mem, bytes_out);
            default: {
                if (bytes_out) *bytes_out = 4;
                if (!mem && bytes == 0) return MCGPU_OK;
                if (!mem || bytes < 4) return fail(MCGPU_INVALID_VALUE, "output buffer too small");
                const uint32_t partial = n[kDerivedBorder] > 0 ? 1u : 0u;
                memcpy(mem, &partial, 4);
                return MCGPU_OK;
            }
            }
        }
        case MCGPU_DATA_CUTPATH_STATUS:
        case MCGPU_DATA_CUTPATH_EDGES:
        case MCGPU_DATA_CUTPATH_FACE_KEYS:
        case MCGPU_DATA_CUTPATH_FACE_OFFSETS:
        case MCGPU_DATA_CUTPATH_FACE_EDGES:
        case MCGPU_DATA_CUTPATH_VERTEX_OFFSETS:
        case MCGPU_DATA_CUTPATH_VERTEX_HALFEDGES: {
            const int rc = ensure_cutpath(c);
            if (rc != MCGPU_OK) return rc;
            const CutpathOut& d = c->cutpath;
            const uint32_t* n = c->cutpath_counts;
            switch (query) {
            case MCGPU_DATA_CUTPATH_STATUS: {
                if (bytes_out) *bytes_out = 8;
                if (!mem && bytes == 0) return MCGPU_OK;
                if (!mem || bytes < 8) return fail(MCGPU_INVALID_VALUE, "output buffer too small");
                const uint32_t st[2] = { n[kCpBadKey] != 0xFFFFFFFFu ? 1u : 0u, n[kCpBadKey] };
                memcpy(mem, st, 8);
                return MCGPU_OK;
            }
            case MCGPU_DATA_CUTPATH_EDGES: return copy_out(c, d.edges, 8ull * n[kCpEdges], bytes, mem, bytes_out);
            case MCGPU_DATA_CUTPATH_FACE_KEYS:
                return copy_out(c, d.face_keys, 4ull * n[kCpFaces], bytes, mem, bytes_out);
            case MCGPU_DATA_CUTPATH_FACE_OFFSETS:
                return copy_out(c, d.face_off, 4ull * (n[kCpFaces] + 1), bytes, mem, bytes_out);
            case MCGPU_DATA_CUTPATH_FACE_EDGES:
                return copy_out(c, d.face_edges, 4ull * n[kCpFaceEntries], bytes, mem, bytes_out);
            case MCGPU_DATA_CUTPATH_VERTEX_OFFSETS:
                return copy_out(c, d.ivtx_off, 4ull * (c->n_records + 1), bytes, mem, bytes_out);
            default:
                return copy_out(c, d.ivtx_he, 4ull * n[kCpHalfedges], bytes, mem, bytes_out);
            }
        }
        case MCGPU_DATA_FLOATING_FACES:
        case MCGPU_DATA_FLOATING_OFFSETS:
        case MCGPU_DATA_FLOATING_VERTICES:
        case MCGPU_DATA_FLOATING_NORMALS:
        case MCGPU_DATA_FLOATING_NORMAL_COMPONENTS: {
            const int rc = ensure_floating(c);
            if (rc != MCGPU_OK) return rc;
            const FloatingOut& d = c->floating;
            const uint64_t np = c->floating_counts[kFpPolygons];
            switch (query) {
            case MCGPU_DATA_FLOATING_FACES: return copy_out(c, d.faces, 4 * np, bytes, mem, bytes_out);
            case MCGPU_DATA_FLOATING_OFFSETS: return copy_out(c, d.off, 4 * (np + 1), bytes, mem, bytes_out);
            case MCGPU_DATA_FLOATING_VERTICES:
                return copy_out(c, d.vtx, 4ull * c->floating_counts[kFpVertices], bytes, mem, bytes_out);
            case MCGPU_DATA_FLOATING_NORMALS: return copy_out(c, d.normals, 24 * np, bytes, mem, bytes_out);
            default: return copy_out(c, d.mc, 4 * np, bytes, mem, bytes_out);
            }
        }
        case MCGPU_DATA_HE_TARGET:
        case MCGPU_DATA_HE_FACE:
        case MCGPU_DATA_HE_NEXT:
        case MCGPU_DATA_HE_PREV:
        case MCGPU_DATA_CORNER_HE:
        case MCGPU_DATA_VERTEX_HE_OFFSETS:
        case MCGPU_DATA_VERTEX_HE: {
            if (!c->hm_ready) return fail(MCGPU_INVALID_VALUE, "no halfedge mesh (mcgpu_halfedge_mesh) built");
            const uint64_t nhe = 2ull * c->hm_ne;
            switch (query) {
            case MCGPU_DATA_HE_TARGET: return copy_out(c, c->hm.he_target, 4 * nhe, bytes, mem, bytes_out);
            case MCGPU_DATA_HE_FACE: return copy_out(c, c->hm.he_face, 4 * nhe, bytes, mem, bytes_out);
            case MCGPU_DATA_HE_NEXT: return copy_out(c, c->hm.he_next, 4 * nhe, bytes, mem, bytes_out);
            case MCGPU_DATA_HE_PREV: return copy_out(c, c->hm.he_prev, 4 * nhe, bytes, mem, bytes_out);
            case MCGPU_DATA_CORNER_HE: return copy_out(c, c->hm.corner_he, 4 * c->hm_nidx, bytes, mem, bytes_out);
            case MCGPU_DATA_VERTEX_HE_OFFSETS:
                return copy_out(c, c->hm.v_off, 4ull * (c->hm_nv + 1), bytes, mem, bytes_out);
            default: return copy_out(c, c->hm.v_he, 4 * nhe, bytes, mem, bytes_out);
            }
        }
        case MCGPU_DATA_CC_FACE:
        case MCGPU_DATA_CC_FACE_ADJACENT_FACE_SIZE:
        case MCGPU_DATA_CC_FACE_ADJACENT_FACE:
        case MCGPU_DATA_CC_EDGE:
        case MCGPU_DATA_CC_VERTEX_FLOAT: {
            if (!c->hm_ready) return fail(MCGPU_INVALID_VALUE, "no halfedge mesh (mcgpu_halfedge_mesh) built");
            if (query == MCGPU_DATA_CC_EDGE) return copy_out(c, c->hm.he_target, 8ull * c->hm_ne, bytes, mem, bytes_out);
            if (query == MCGPU_DATA_CC_VERTEX_FLOAT) {
                if (!c->hm_has_vf) return fail(MCGPU_INVALID_VALUE, "no double vertices given to mcgpu_halfedge_mesh");
                return copy_out(c, c->buf[B_CW_VF].get<float>(3ull * c->hm_nv), 12ull * c->hm_nv, bytes, mem, bytes_out);
            }
            ensure_cc_wire(c);
            switch (query) {
            case MCGPU_DATA_CC_FACE: return copy_out(c, c->cw.face, 4 * c->hm_nidx, bytes, mem, bytes_out);
            case MCGPU_DATA_CC_FACE_ADJACENT_FACE_SIZE: return copy_out(c, c->cw.adj_n, 4ull * c->hm_nf, bytes, mem, bytes_out);
            default: return copy_out(c, c->cw.adj, 4ull * c->cw_total, bytes, mem, bytes_out);
            }
        }
        case MCGPU_DATA_RECORD_OFFSETS: {
            const uint64_t need = c->rec_begin.size() * 8;
            if (bytes_out) *bytes_out = need;
            if (!mem && bytes == 0) return MCGPU_OK;
            if (!mem || bytes < need) return fail(MCGPU_INVALID_VALUE, "output buffer too small");
            memcpy(mem, c->rec_begin.data(), need);
            return MCGPU_OK;
        }
        default:
            return fail(MCGPU_INVALID_VALUE, "unknown query");
        }
    } catch (const CudaError& e) {
        return fail(MCGPU_CUDA_ERROR, e.where + ": " + cudaGetErrorString(e.e));
    }
}

int mcgpu_get_batch_data(mcgpu_context c, uint32_t pair, uint32_t query, uint64_t bytes, void* mem,
    uint64_t* bytes_out)
{
    if (!c) return fail(MCGPU_INVALID_VALUE, "null context");
    if (!c->have_results) return fail(MCGPU_INVALID_VALUE, "no dispatch results (none completed, or the pool was trimmed)");
    if (pair >= c->L.n_pairs) return fail(MCGPU_INVALID_VALUE, "pair index out of range");
    try {
        const uint64_t b = c->rec_begin[pair], n = c->rec_begin[pair + 1] - b;
        switch (query) {
        case MCGPU_DATA_RECORD_IDS:
            return copy_out(c, c->W.rec_ids + b * 5, n * 20, bytes, mem, bytes_out);
        case MCGPU_DATA_RECORD_POINTS:
            return copy_out(c, c->W.rec_pts + b * 3, n * 24, bytes, mem, bytes_out);
        default:
            return fail(MCGPU_INVALID_VALUE, "batch queries: record ids and points");
        }
    } catch (const CudaError& e) {
        return fail(MCGPU_CUDA_ERROR, e.where + ": " + cudaGetErrorString(e.e));
    }
}

int mcgpu_halfedge_mesh(mcgpu_context c, uint32_t flags, const mcgpu_mesh* m, mcgpu_hmesh_report* out)
{
    if (out) memset(out, 0, sizeof *out);
    if (!c || !m || !out) return fail(MCGPU_INVALID_VALUE, "null argument");
    out->bad_face = -1;
    if (m->num_faces && !m->face_indices) return fail(MCGPU_INVALID_VALUE, "null face indices");
    const bool dev = (flags & MCGPU_DEVICE_POINTERS) != 0;
    try {
        ck(cudaSetDevice(c->device), "cudaSetDevice");
        cudaStream_t s = c->s;
        c->hm_ready = false;
        const unsigned long long launches0 = g_launches;
        const uint32_t nf = m->num_faces, nv = m->num_vertices;
        uint32_t* foff = nullptr;
        uint64_t nidx = 3ull * nf;
        uint32_t* scan_temp = nullptr;
        auto scan_space = [&](uint64_t n) {
            scan_temp = c->buf[B_HM_SCAN].get<uint32_t>(scan_temp_bytes((uint32_t)std::min<uint64_t>(n, 0xFFFFFFFFull)) / 4 + 64);
        };
        if (m->face_sizes) {
            foff = c->buf[B_HM_FOFF].get<uint32_t>((size_t)nf + 1);
            if (dev) {
                // face offsets on the device: exclusive scan of the sizes, the corner count after them
                ck(cudaMemcpyAsync(foff, m->face_sizes, 4ull * nf, cudaMemcpyDeviceToDevice, s), "D2D sizes");
                ck(cudaMemsetAsync(foff + nf, 0, 4, s), "memset");
                scan_space((uint64_t)nf + 1);
                exclusive_scan(foff, nf + 1, nullptr, scan_temp, s);
                uint32_t tot = 0;
                ck(cudaMemcpyAsync(&tot, foff + nf, 4, cudaMemcpyDeviceToHost, s), "D2H corners");
                ck(cudaStreamSynchronize(s), "sync corners");
                nidx = tot;
            } else {
                std::vector<uint32_t> off((size_t)nf + 1);
                uint64_t o = 0;
                for (uint32_t f = 0; f < nf; ++f) {
                    off[f] = (uint32_t)o;
                    o += m->face_sizes[f];
                    if (o > 0x7FFFFFFFull) return fail(MCGPU_TOO_LARGE, "more than 2^31 face corners");
                }
                off[nf] = (uint32_t)o;
                nidx = o;
                ck(cudaMemcpyAsync(foff, off.data(), 4ull * (nf + 1), cudaMemcpyHostToDevice, s), "H2D offsets");
                ck(cudaStreamSynchronize(s), "sync offsets"); // `off` is a pageable temporary
            }
        }
        if (nidx > 0x7FFFFFFFull || nv >= 0x7FFFFFFFu) return fail(MCGPU_TOO_LARGE, "more than 2^31 corners or vertices");
        const uint32_t* idx = m->face_indices;
        if (!dev && nidx) {
            uint32_t* d = c->buf[B_HM_IDX].get<uint32_t>(nidx);
            ck(cudaMemcpyAsync(d, m->face_indices, 4 * nidx, cudaMemcpyHostToDevice, s), "H2D indices");
            idx = d;
        }
        HmeshInput in { idx, foff, nv, nf, nidx };
        uint64_t buckets = 64;
        while (buckets < 2 * nidx) buckets <<= 1;
        HmeshTable t {};
        t.key = c->buf[B_HM_KEY].get<unsigned long long>(buckets);
        t.first = c->buf[B_HM_FIRST].get<uint32_t>(buckets);
        t.dir_first = c->buf[B_HM_DIR].get<uint32_t>(2 * buckets);
        t.mask = buckets - 1;
        HmeshScratch w {};
        const size_t ni = std::max<uint64_t>(nidx, 1);
        w.slot_face = foff ? c->buf[B_HM_SLOTFACE].get<uint32_t>(ni) : nullptr;
        w.slot_bucket = c->buf[B_HM_BUCKET].get<uint32_t>(ni);
        w.eid = c->buf[B_HM_EID].get<uint32_t>(ni);
        w.vcur = c->buf[B_HM_VCUR].get<uint32_t>(std::max<uint32_t>(nv, 1));
        w.parent = c->buf[B_HM_PARENT].get<uint32_t>(std::max<uint32_t>(nv, 1));
        scan_space(std::max<uint64_t>(nidx, (uint64_t)nv + 1));
        w.scan_temp = scan_temp;
        uint32_t* small = c->buf[B_HM_SMALL].get<uint32_t>(16);
        w.err = reinterpret_cast<unsigned long long*>(small);
        w.counts = small + 2;
        ck(cudaMemsetAsync(t.key, 0, 8 * buckets, s), "memset");
        ck(cudaMemsetAsync(t.first, 0xFF, 4 * buckets, s), "memset");
        ck(cudaMemsetAsync(t.dir_first, 0xFF, 8 * buckets, s), "memset");
        ck(cudaMemsetAsync(small, 0, 64, s), "memset");
        ck(cudaMemsetAsync(w.err, 0xFF, 8, s), "memset");
        launch_hmesh_edges(in, t, w, s);
        uint32_t hs[16];
        ck(cudaMemcpyAsync(hs, small, 64, cudaMemcpyDeviceToHost, s), "D2H hmesh");
        ck(cudaStreamSynchronize(s), "sync hmesh");
        unsigned long long err;
        memcpy(&err, hs, 8);
        out->kernel_launches = (uint32_t)(g_launches - launches0);
        if (err == ~0ull - 1) return fail(MCGPU_CUDA_ERROR, "halfedge mesh: edge table probe bound reached");
        if (err != ~0ull) {
            out->status = (int32_t)(err & 7u);
            out->bad_face = (int32_t)(err >> 3);
            return MCGPU_OK;
        }
        const uint32_t ne = hs[2 + kHmEdges];
        const size_t nhe = std::max<uint64_t>(2ull * ne, 1);
        HmeshOut& o = c->hm;
        o.he_target = c->buf[B_HM_TGT].get<uint32_t>(nhe);
        o.he_face = c->buf[B_HM_FACE].get<int32_t>(nhe);
        o.he_next = c->buf[B_HM_NEXT].get<int32_t>(nhe);
        o.he_prev = c->buf[B_HM_PREV].get<int32_t>(nhe);
        o.corner_he = c->buf[B_HM_CORNER].get<uint32_t>(ni);
        o.v_off = c->buf[B_HM_VOFF].get<uint32_t>((size_t)nv + 1);
        o.v_he = c->buf[B_HM_VHE].get<uint32_t>(nhe);
        ck(cudaMemsetAsync(o.he_face, 0xFF, 4 * nhe, s), "memset");
        ck(cudaMemsetAsync(o.he_next, 0xFF, 4 * nhe, s), "memset");
        ck(cudaMemsetAsync(o.he_prev, 0xFF, 4 * nhe, s), "memset");
        ck(cudaMemsetAsync(o.v_off, 0, 4 * ((size_t)nv + 1), s), "memset");
        ck(cudaMemsetAsync(w.vcur, 0, 4ull * std::max<uint32_t>(nv, 1), s), "memset");
        launch_hmesh_build(in, t, w, o, ne, s);
        ck(cudaMemcpyAsync(hs, small, 64, cudaMemcpyDeviceToHost, s), "D2H hmesh");
        ck(cudaStreamSynchronize(s), "sync hmesh");
        ck(cudaGetLastError(), "hmesh launch");
        memcpy(&err, hs, 8);
        out->kernel_launches = (uint32_t)(g_launches - launches0);
        if (err != ~0ull) return fail(MCGPU_CUDA_ERROR, "halfedge mesh: union-find retry bound reached");
        c->hm_ready = true;
        c->hm_ne = ne;
        c->hm_nv = nv;
        c->hm_nidx = nidx;
        c->hm_nf = nf;
        c->hm_foff = foff;
        c->cw_ready = false;
        c->hm_has_vf = false;
        if (m->vertices && !(flags & MCGPU_VERTEX_ARRAY_FLOAT) && nv) {
            // MC_CONNECTED_COMPONENT_DATA_VERTEX_FLOAT: static_cast<float> of each coordinate
            const double* x = static_cast<const double*>(m->vertices);
            if (!dev) {
                double* d = c->buf[B_CW_XD].get<double>(3ull * nv);
                ck(cudaMemcpyAsync(d, m->vertices, 24ull * nv, cudaMemcpyHostToDevice, s), "H2D vertices");
                x = d;
            }
            launch_to_float(x, 3ull * nv, c->buf[B_CW_VF].get<float>(3ull * nv), s);
            ck(cudaStreamSynchronize(s), "sync vertices");
            ck(cudaGetLastError(), "vertex rounding");
            c->hm_has_vf = true;
        }
        out->num_edges = ne;
        out->closed = hs[2 + kHmBorder] ? 0 : 1;
        // check_input_mesh (preproc.cpp:505-579): after the conversion
        if (nv < 3 || nf < 1) {
            out->status = MCGPU_HMESH_TOO_SMALL;
            return MCGPU_OK;
        }
        out->num_components = hs[2 + kHmComponents];
        out->status = out->num_components == 1 ? MCGPU_HMESH_OK : MCGPU_HMESH_COMPONENTS;
        return MCGPU_OK;
    } catch (const CudaError& e) {
        return fail(e.e == cudaErrorMemoryAllocation ? MCGPU_OUT_OF_MEMORY : MCGPU_CUDA_ERROR,
            e.where + ": " + cudaGetErrorString(e.e));
    }
}

int mcgpu_recentre(uint32_t flags, const mcgpu_mesh* src, const mcgpu_mesh* cut, double* src_out, double* cut_out,
    double* cut_eps_out)
{
    if (!src || !cut || !src_out || !cut_out || !cut_eps_out) return fail(MCGPU_INVALID_VALUE, "null argument");
    if (src->num_vertices < 1 || cut->num_vertices < 1) return fail(MCGPU_INVALID_INPUT, "empty mesh");
    recentre_pair((flags & MCGPU_VERTEX_ARRAY_FLOAT) != 0, *src, *cut, src_out, cut_out, cut_eps_out);
    return MCGPU_OK;
}

const char* mcgpu_last_error(void) { return g_last_error.c_str(); }

} // extern "C"

namespace mcgpu {

int set_error(int code, const std::string& msg) { return fail(code, msg); }

int dispatch_with_resident(mcgpu_context c, uint32_t flags, uint32_t n, const mcgpu_mesh* srcs,
    const mcgpu_mesh* cuts, const ResidentCut* const* resident, mcgpu_summary* out)
{
    if (!(flags & MCGPU_RECENTRE) || (flags & (MCGPU_DEVICE_POINTERS | MCGPU_VERTEX_ARRAY_FLOAT)))
        return fail(MCGPU_INVALID_VALUE, "resident cut meshes take double user coordinates with MCGPU_RECENTRE");
    try {
        // stand-in views for resident cuts: counts for the layout, never dereferenced on the host
        std::vector<mcgpu_mesh> cv(cuts, cuts + n);
        for (uint32_t p = 0; p < n; ++p)
            if (resident[p]) cv[p] = mcgpu_mesh { resident[p]->X, resident[p]->idx, nullptr, resident[p]->nv,
                                                  resident[p]->nf };
        return run(c, flags, n, srcs, cv.data(), nullptr, out, nullptr, resident);
    } catch (const CudaError& e) {
        return fail(e.e == cudaErrorMemoryAllocation ? MCGPU_OUT_OF_MEMORY : MCGPU_CUDA_ERROR,
            e.where + ": " + cudaGetErrorString(e.e));
    }
}

} // namespace mcgpu
