// Request server: continuous batching of front-end dispatches on one GPU.
//
// MCUT runs each dispatch as a task on its context's API thread
// (frontend.h:548-580, mcEnqueueDispatch in mcut.cpp:459-552); a server
// instead keeps a queue of independent (source, cut) requests and a few
// worker threads, each owning one context (CUDA stream + device pool).
// A free worker takes as many queued requests as fit its batch limits and
// the HBM admission budget, runs them as one batched dispatch, copies each
// request's records to its own host buffers and wakes its waiters. Requests
// that arrive while batches are on the GPU join the next batch a worker
// forms, and the workers' batches overlap on the device.
//
// Cut meshes registered once stay on the device (double user coordinates +
// indices) with their bounds and centroid and their own tree, built once
// over the user coordinates; a request naming one uploads only its source
// mesh, the cut is mapped into the pair's frame on the device, and the
// source faces walk the resident tree instead of joining its faces to the
// batch's sort and tree.
//
// Device memory: each worker may hold an allowance of device bytes -- its
// context's pool while idle, its batch's cap while it runs one -- and the
// resident meshes plus every allowance stay within hbm_budget_bytes. A batch
// is formed from the requests whose estimated bytes fit what the other
// workers' allowances leave; its context cannot grow past the cap
// (mcgpu_context_set_memory_limit). Idle workers' pools are freed when a
// batch does not fit beside them. A batch that meets its cap runs again
// with the pool freed and the cap widened to all that is free, then in
// halves; a request that still does not fit fails with MCGPU_TOO_LARGE.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "fe_host.h"
#include "fe_kernels.cuh"
#include "mcut_gb300.h"

namespace {

using Clock = std::chrono::steady_clock;
constexpr uint32_t kNoCut = 0xFFFFFFFFu;

int sfail(int code, const std::string& msg) { return mcgpu::set_error(code, msg); }

struct Request {
    uint64_t id = 0;
    mcgpu_mesh src {}, cut {};
    uint32_t cut_id = kNoCut;
    uint64_t faces = 0, est_bytes = 0;
    Clock::time_point t_submit, t_done;
    bool done = false;
    int rc = MCGPU_OK;
    std::string err;
    bool cancelled = false;
    mcgpu_summary sum {};
    std::vector<uint32_t> ids;
    std::vector<double> pts;
};

struct Resident {
    mcgpu::ResidentCut rc {};
    void* dX = nullptr;
    void* dI = nullptr;
    void* dTree = nullptr; // nodes, leaf order, leaf starts and sizes in one allocation
    uint64_t bytes = 0;
};

// leaves of the resident trees (faces per leaf cluster)
#ifndef MCGPU_RESIDENT_LEAF
#define MCGPU_RESIDENT_LEAF 4
#endif
constexpr uint32_t kResLeaf = MCGPU_RESIDENT_LEAF;
uint64_t al256(uint64_t b) { return (b + 255) & ~255ull; }
uint64_t tree_bytes(const mcgpu::ResTreeSizes& z)
{
    return al256(z.nodes_bytes) + al256(z.leaf_bytes) + al256(z.start_bytes) + al256(z.n_bytes);
}

uint64_t mesh_faces(const mcgpu_mesh& m) { return m.num_faces; }

uint64_t mesh_indices(const mcgpu_mesh& m)
{
    if (!m.face_sizes) return 3ull * m.num_faces;
    uint64_t n = 0;
    for (uint32_t f = 0; f < m.num_faces; ++f) n += m.face_sizes[f];
    return n;
}

// Device bytes one request adds to a batch: the dispatch's per-face and
// per-vertex buffers (face boxes f64 + f32, keys, values, tree, pairs, tests
// and records at their usual sizes, a plane slot for every face, 104 B, as a
// repeated dispatch shape sizes them, and 16 incidence slots per vertex,
// 64 B) plus slack.
uint64_t estimate_bytes(uint64_t faces, uint64_t verts) { return (1ull << 20) + faces * 744 + verts * 128; }
// the cap a batch of estimated bytes e runs under: the pool grows each
// buffer by a quarter beyond its need, its smallest buffers have fixed
// minimum sizes, and the estimate is not a bound
uint64_t batch_cap(uint64_t e) { return 2 * e + (64ull << 20); }

} // namespace

struct mcgpu_server_t {
    mcgpu_server_config cfg {};
    std::mutex m;
    std::condition_variable cv_work, cv_done;
    std::deque<Request*> pending;
    std::unordered_map<uint64_t, std::unique_ptr<Request>> reqs;
    std::vector<std::unique_ptr<Resident>> cuts;
    std::vector<std::thread> workers;
    std::vector<mcgpu_context> ctxs;
    uint64_t next_id = 1, inflight = 0, peak_inflight = 0, resident_bytes = 0, pending_faces = 0;
    uint32_t busy = 0; // workers with a batch on the device
    uint64_t submitted = 0, completed = 0, batches = 0, batched_pairs = 0, cancelled = 0;
    // per worker: bytes its pool holds (read after each batch), the bytes it
    // may hold (its pool while idle, its batch's cap while running), running
    std::vector<uint64_t> pool, allow;
    std::vector<uint8_t> running;
    uint64_t peak_reserved = 0, trims = 0;
    bool stop = false;
};

namespace {

// the bytes every worker but w may hold (caller holds S->m)
uint64_t others_allowance(const mcgpu_server_t* S, size_t w)
{
    uint64_t a = 0;
    for (size_t k = 0; k < S->allow.size(); ++k)
        if (k != w) a += S->allow[k];
    return a;
}

uint64_t free_bytes(const mcgpu_server_t* S, size_t w)
{
    const uint64_t used = S->resident_bytes + others_allowance(S, w);
    return S->cfg.hbm_budget_bytes > used ? S->cfg.hbm_budget_bytes - used : 0;
}

void note_reserved(mcgpu_server_t* S)
{
    uint64_t r = S->resident_bytes;
    for (uint64_t a : S->allow) r += a;
    if (r > S->peak_reserved) S->peak_reserved = r;
}

// frees the pools of the idle workers other than w (caller holds S->m; an
// idle worker touches its context only after taking S->m to form a batch)
bool trim_idle(mcgpu_server_t* S, size_t w)
{
    bool any = false;
    for (size_t k = 0; k < S->ctxs.size(); ++k) {
        if (k == w || S->running[k] || S->pool[k] == 0) continue;
        mcgpu_context_trim(S->ctxs[k]);
        S->pool[k] = S->allow[k] = 0;
        S->trims++;
        any = true;
    }
    return any;
}

// one batched dispatch; on success each request gets its summary and records
int run_batch(mcgpu_context ctx, const std::vector<Request*>& batch, const std::vector<const mcgpu::ResidentCut*>& res)
{
    const uint32_t n = (uint32_t)batch.size();
    std::vector<mcgpu_mesh> srcs(n), cuts(n);
    for (uint32_t i = 0; i < n; ++i) {
        srcs[i] = batch[i]->src;
        cuts[i] = batch[i]->cut;
    }
    std::vector<mcgpu_summary> sums(n);
    int rc = mcgpu::dispatch_with_resident(ctx, MCGPU_RECENTRE, n, srcs.data(), cuts.data(), res.data(), sums.data());
    if (rc != MCGPU_OK) return rc;
    std::vector<uint64_t> off(n + 1);
    std::vector<uint32_t> ids;
    std::vector<double> pts;
    uint64_t b = 0;
    rc = mcgpu_get_data(ctx, MCGPU_DATA_RECORD_OFFSETS, (n + 1) * 8, off.data(), &b);
    if (rc != MCGPU_OK) return rc;
    ids.resize(off[n] * 5 + 1);
    pts.resize(off[n] * 3 + 1);
    rc = mcgpu_get_data(ctx, MCGPU_DATA_RECORD_IDS, ids.size() * 4, ids.data(), &b);
    if (rc == MCGPU_OK) rc = mcgpu_get_data(ctx, MCGPU_DATA_RECORD_POINTS, pts.size() * 8, pts.data(), &b);
    if (rc != MCGPU_OK) return rc;
    for (uint32_t i = 0; i < n; ++i) {
        Request* r = batch[i];
        r->rc = MCGPU_OK;
        r->sum = sums[i];
        r->ids.assign(ids.begin() + off[i] * 5, ids.begin() + off[i + 1] * 5);
        r->pts.assign(pts.begin() + off[i] * 3, pts.begin() + off[i + 1] * 3);
    }
    return MCGPU_OK;
}

// marks requests done and wakes their waiters (caller holds S->m)
void complete(mcgpu_server_t* S, const std::vector<Request*>& done)
{
    const Clock::time_point now = Clock::now();
    for (Request* r : done) {
        r->done = true;
        r->t_done = now;
    }
    S->completed += done.size();
}

void worker(mcgpu_server_t* S, int w)
{
    cudaSetDevice(S->cfg.device);
    mcgpu_context ctx = S->ctxs[w];
    std::vector<Request*> batch;
    std::vector<const mcgpu::ResidentCut*> res;
    for (;;) {
        uint64_t bytes = 0;
        {
            std::unique_lock<std::mutex> lk(S->m);
            for (;;) {
                if (S->stop && S->pending.empty()) return;
                // continuous batching: while other batches keep the device busy, a short
                // queue waits up to linger_us for more requests to join it
                if (!S->pending.empty() && S->busy > 0 && !S->stop && S->cfg.linger_us > 0) {
                    const auto until = Clock::now() + std::chrono::microseconds(S->cfg.linger_us);
                    while (S->busy > 0 && !S->stop && S->pending.size() < S->cfg.max_batch_pairs
                        && S->pending_faces < S->cfg.max_batch_faces / 2
                        && S->cv_work.wait_until(lk, until) != std::cv_status::timeout) {
                    }
                }
                batch.clear();
                res.clear();
                uint64_t faces = 0;
                bytes = 0;
                uint64_t avail = free_bytes(S, w);
                bool alone = false; // the first request runs with every byte the budget has
                while (!S->pending.empty() && batch.size() < S->cfg.max_batch_pairs) {
                    Request* r = S->pending.front();
                    if (!batch.empty() && faces + r->faces > S->cfg.max_batch_faces) break;
                    if (batch_cap(bytes + r->est_bytes) > avail) {
                        if (!batch.empty()) break;
                        // the first request does not fit beside the other workers' pools:
                        // free the idle ones, else wait for a running batch to end
                        if (trim_idle(S, w)) avail = free_bytes(S, w);
                        if (batch_cap(r->est_bytes) > avail) {
                            if (S->busy > 0) break;
                            alone = true;
                        }
                    }
                    S->pending.pop_front();
                    S->pending_faces -= r->faces;
                    batch.push_back(r);
                    res.push_back(r->cut_id == kNoCut ? nullptr : &S->cuts[r->cut_id]->rc);
                    faces += r->faces;
                    bytes += r->est_bytes;
                    if (alone) break;
                }
                if (!batch.empty()) {
                    S->busy++;
                    S->running[w] = 1;
                    S->allow[w] = std::max(S->pool[w], alone ? avail : std::min(avail, batch_cap(bytes)));
                    note_reserved(S);
                    S->inflight += bytes;
                    if (S->inflight > S->peak_inflight) S->peak_inflight = S->inflight;
                    break;
                }
                S->cv_work.wait(lk);
            }
        }
        mcgpu_context_set_memory_limit(ctx, S->allow[w]);
        int rc = run_batch(ctx, batch, res);
        std::string err = rc == MCGPU_OK ? std::string() : std::string(mcgpu_last_error());
        // a batch that met its cap runs again with the cap widened to all that
        // is free (the pool keeps what it grew), then with this pool and the
        // idle ones freed, then in halves (the later half goes back to the
        // front of the queue)
        for (int attempt = 0; rc == MCGPU_OUT_OF_MEMORY; ++attempt) {
            if (attempt >= 1) mcgpu_context_trim(ctx);
            {
                std::lock_guard<std::mutex> lk(S->m);
                if (attempt >= 1) {
                    S->pool[w] = 0;
                    S->trims++;
                    trim_idle(S, (size_t)w);
                }
                if (attempt >= 2) {
                    if (batch.size() < 2) break; // one request that does not fit the budget
                    const size_t half = batch.size() / 2;
                    for (size_t k = batch.size(); k-- > half;) {
                        S->pending.push_front(batch[k]);
                        S->pending_faces += batch[k]->faces;
                        S->inflight -= batch[k]->est_bytes;
                        bytes -= batch[k]->est_bytes;
                    }
                    batch.resize(half);
                    res.resize(half);
                }
                S->allow[w] = free_bytes(S, w);
                note_reserved(S);
            }
            S->cv_work.notify_all();
            mcgpu_context_set_memory_limit(ctx, S->allow[w]);
            rc = run_batch(ctx, batch, res);
            err = rc == MCGPU_OK ? std::string() : std::string(mcgpu_last_error());
        }
        uint64_t held = 0;
        mcgpu_context_get_memory(ctx, &held, nullptr);
        {
            std::lock_guard<std::mutex> lk(S->m);
            S->busy--;
            S->running[w] = 0;
            S->pool[w] = S->allow[w] = held;
            S->inflight -= bytes;
            for (Request* r : batch) {
                if (rc == MCGPU_OK) continue;
                r->rc = rc == MCGPU_OUT_OF_MEMORY ? MCGPU_TOO_LARGE : rc;
                r->err = rc == MCGPU_OUT_OF_MEMORY ? "the request does not fit the device memory budget: " + err : err;
            }
            complete(S, batch);
            S->batches++;
            S->batched_pairs += batch.size();
        }
        S->cv_done.notify_all();
        S->cv_work.notify_all();
    }
}

Request* find(mcgpu_server_t* S, uint64_t ticket)
{
    auto it = S->reqs.find(ticket);
    return it == S->reqs.end() ? nullptr : it->second.get();
}

} // namespace

extern "C" {

int mcgpu_server_create(mcgpu_server* out, const mcgpu_server_config* cfg)
{
    if (!out) return sfail(MCGPU_INVALID_VALUE, "null server pointer");
    *out = nullptr;
    mcgpu_server_t* S = new (std::nothrow) mcgpu_server_t();
    if (!S) return sfail(MCGPU_OUT_OF_MEMORY, "host allocation");
    if (cfg) S->cfg = *cfg;
    if (S->cfg.workers == 0) S->cfg.workers = 3;
    if (S->cfg.max_batch_pairs == 0) S->cfg.max_batch_pairs = 512;
    if (S->cfg.max_batch_faces == 0) S->cfg.max_batch_faces = 16ull << 20;
    if (S->cfg.hbm_budget_bytes == 0) S->cfg.hbm_budget_bytes = 150ull << 30;
    if (S->cfg.linger_us == 0) S->cfg.linger_us = 400;
    if (S->cfg.linger_us > 1000000) S->cfg.linger_us = 0; // "never linger"
    if (S->cfg.workers > 16 || S->cfg.max_batch_pairs > 65535) {
        delete S;
        return sfail(MCGPU_INVALID_VALUE, "workers <= 16, max_batch_pairs <= 65535");
    }
    for (uint32_t w = 0; w < S->cfg.workers; ++w) {
        mcgpu_context c = nullptr;
        const int rc = mcgpu_context_create(&c, S->cfg.device);
        if (rc != MCGPU_OK) {
            for (mcgpu_context x : S->ctxs) mcgpu_context_release(x);
            delete S;
            return rc;
        }
        S->ctxs.push_back(c);
    }
    S->pool.assign(S->cfg.workers, 0);
    S->allow.assign(S->cfg.workers, 0);
    S->running.assign(S->cfg.workers, 0);
    for (uint32_t w = 0; w < S->cfg.workers; ++w) S->workers.emplace_back(worker, S, (int)w);
    *out = S;
    return MCGPU_OK;
}

int mcgpu_server_release(mcgpu_server S)
{
    if (!S) return sfail(MCGPU_INVALID_VALUE, "null server");
    {
        std::lock_guard<std::mutex> lk(S->m);
        S->stop = true;
    }
    S->cv_work.notify_all();
    for (auto& t : S->workers) t.join();
    for (mcgpu_context c : S->ctxs) mcgpu_context_release(c);
    cudaSetDevice(S->cfg.device);
    for (auto& r : S->cuts) {
        cudaFree(r->dX);
        cudaFree(r->dI);
        cudaFree(r->dTree);
    }
    delete S;
    return MCGPU_OK;
}

int mcgpu_server_add_cut_mesh(mcgpu_server S, const mcgpu_mesh* cut, uint32_t* cut_id)
{
    if (!S || !cut || !cut_id || !cut->vertices || !cut->face_indices)
        return sfail(MCGPU_INVALID_VALUE, "null argument");
    if (cut->face_sizes) return sfail(MCGPU_INVALID_VALUE, "resident cut meshes hold triangles");
    if (cut->num_vertices < 3 || cut->num_faces < 1) return sfail(MCGPU_INVALID_INPUT, "empty cut mesh");
    std::unique_ptr<Resident> r(new Resident());
    const size_t xb = (size_t)cut->num_vertices * 24, ib = (size_t)cut->num_faces * 12;
    const mcgpu::ResTreeSizes z = mcgpu::resident_tree_sizes(cut->num_faces, kResLeaf);
    const uint64_t tb = tree_bytes(z);
    {
        // the resident bytes join the budget (the build's scratch for the
        // time of the build): free idle pools if they do not fit
        std::lock_guard<std::mutex> lk(S->m);
        const uint64_t size = (uint64_t)xb + ib + tb;
        if (free_bytes(S, S->allow.size()) < size + z.scratch_bytes) trim_idle(S, S->allow.size());
        if (free_bytes(S, S->allow.size()) < size + z.scratch_bytes)
            return sfail(MCGPU_OUT_OF_MEMORY, "resident cut mesh exceeds the device memory budget");
        S->resident_bytes += size + z.scratch_bytes; // reserved now, so no batch takes these bytes meanwhile
    }
    bool scratch_held = true;
    auto unreserve = [&] {
        std::lock_guard<std::mutex> lk(S->m);
        S->resident_bytes -= (uint64_t)xb + ib + tb + (scratch_held ? z.scratch_bytes : 0);
    };
    mcgpu::mesh_stats(cut->vertices, false, cut->num_vertices, r->rc.st);
    cudaSetDevice(S->cfg.device);
    if (cudaMalloc(&r->dX, xb) != cudaSuccess || cudaMalloc(&r->dI, ib) != cudaSuccess) {
        cudaFree(r->dX);
        cudaGetLastError();
        unreserve();
        return sfail(MCGPU_OUT_OF_MEMORY, "resident cut mesh");
    }
    if (cudaMemcpy(r->dX, cut->vertices, xb, cudaMemcpyHostToDevice) != cudaSuccess
        || cudaMemcpy(r->dI, cut->face_indices, ib, cudaMemcpyHostToDevice) != cudaSuccess) {
        cudaFree(r->dX);
        cudaFree(r->dI);
        unreserve();
        return sfail(MCGPU_CUDA_ERROR, "resident cut upload");
    }
    r->rc.X = static_cast<const double*>(r->dX);
    r->rc.idx = static_cast<const uint32_t*>(r->dI);
    r->rc.nv = cut->num_vertices;
    r->rc.nf = cut->num_faces;
    // the mesh's own tree over its user coordinates
    void* scratch = nullptr;
    cudaStream_t st = nullptr;
    const bool got = cudaMalloc(&r->dTree, tb) == cudaSuccess && cudaMalloc(&scratch, z.scratch_bytes) == cudaSuccess;
    bool ok = got && cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
    if (ok) {
        uint8_t* t = static_cast<uint8_t*>(r->dTree);
        mcgpu::ResTreeOut o {};
        o.nodes = reinterpret_cast<mcgpu::Node*>(t);
        o.leaf_face = reinterpret_cast<uint32_t*>(t + al256(z.nodes_bytes));
        o.cl_start = reinterpret_cast<uint32_t*>(t + al256(z.nodes_bytes) + al256(z.leaf_bytes));
        o.cl_n = t + al256(z.nodes_bytes) + al256(z.leaf_bytes) + al256(z.start_bytes);
        mcgpu::build_resident_tree(r->rc.X, r->rc.idx, r->rc.nv, r->rc.nf, r->rc.st.mn, r->rc.st.mx, kResLeaf,
            scratch, o, st);
        ok = cudaGetLastError() == cudaSuccess && cudaStreamSynchronize(st) == cudaSuccess;
        r->rc.tree_nodes = o.nodes;
        r->rc.tree_leaf_face = o.leaf_face;
        r->rc.tree_cl_start = o.cl_start;
        r->rc.tree_cl_n = o.cl_n;
        r->rc.tree_ncl = (uint32_t)z.ncl;
    }
    if (st) cudaStreamDestroy(st);
    cudaFree(scratch);
    {
        std::lock_guard<std::mutex> lk(S->m);
        S->resident_bytes -= z.scratch_bytes;
        scratch_held = false;
    }
    if (!ok) {
        cudaGetLastError();
        cudaFree(r->dX);
        cudaFree(r->dI);
        cudaFree(r->dTree);
        unreserve();
        return sfail(got ? MCGPU_CUDA_ERROR : MCGPU_OUT_OF_MEMORY, "resident cut tree");
    }
    r->bytes = xb + ib + tb;
    std::lock_guard<std::mutex> lk(S->m);
    *cut_id = (uint32_t)S->cuts.size();
    S->cuts.push_back(std::move(r));
    return MCGPU_OK;
}

int mcgpu_server_submit(mcgpu_server S, const mcgpu_mesh* src, const mcgpu_mesh* cut, uint32_t cut_id,
    uint64_t* ticket)
{
    if (!S || !src || !ticket || !src->vertices || !src->face_indices)
        return sfail(MCGPU_INVALID_VALUE, "null argument");
    if (!cut && cut_id == kNoCut) return sfail(MCGPU_INVALID_VALUE, "no cut mesh");
    if (cut && (!cut->vertices || !cut->face_indices)) return sfail(MCGPU_INVALID_VALUE, "null cut array");
    if (src->num_vertices < 3 || src->num_faces < 1 || (cut && (cut->num_vertices < 3 || cut->num_faces < 1)))
        return sfail(MCGPU_INVALID_INPUT, "mesh needs >= 3 vertices and >= 1 face");
    std::unique_ptr<Request> r(new Request());
    r->src = *src;
    uint64_t verts = src->num_vertices;
    r->faces = mesh_faces(*src);
    uint64_t idx = mesh_indices(*src);
    {
        std::lock_guard<std::mutex> lk(S->m);
        if (!cut) {
            if (cut_id >= S->cuts.size()) return sfail(MCGPU_INVALID_VALUE, "unknown cut mesh id");
            r->cut_id = cut_id;
            verts += S->cuts[cut_id]->rc.nv;
            r->faces += S->cuts[cut_id]->rc.nf;
            idx += 3ull * S->cuts[cut_id]->rc.nf;
        }
    }
    if (cut) {
        r->cut = *cut;
        verts += cut->num_vertices;
        r->faces += mesh_faces(*cut);
        idx += mesh_indices(*cut);
    }
    if (verts >= 0x7FFFFFFFull || idx >= 0xFFFFFFFFull) return sfail(MCGPU_TOO_LARGE, "request too large");
    r->est_bytes = estimate_bytes(r->faces, verts);
    {
        std::lock_guard<std::mutex> lk(S->m);
        if (r->est_bytes + S->resident_bytes > S->cfg.hbm_budget_bytes)
            return sfail(MCGPU_TOO_LARGE, "request exceeds the HBM budget");
        if (S->stop) return sfail(MCGPU_INVALID_VALUE, "server is stopping");
        r->id = S->next_id++;
        r->t_submit = Clock::now();
        *ticket = r->id;
        S->pending.push_back(r.get());
        S->pending_faces += r->faces;
        S->reqs.emplace(r->id, std::move(r));
        S->submitted++;
    }
    S->cv_work.notify_one();
    return MCGPU_OK;
}

int mcgpu_server_cancel(mcgpu_server S, uint64_t ticket)
{
    if (!S) return sfail(MCGPU_INVALID_VALUE, "null server");
    {
        std::lock_guard<std::mutex> lk(S->m);
        Request* r = find(S, ticket);
        if (!r) return sfail(MCGPU_INVALID_VALUE, "unknown ticket");
        if (r->done) return sfail(MCGPU_INVALID_VALUE, "request already completed");
        auto it = std::find(S->pending.begin(), S->pending.end(), r);
        if (it == S->pending.end()) return sfail(MCGPU_NOT_READY, "request is in a running batch");
        S->pending.erase(it);
        S->pending_faces -= r->faces;
        r->cancelled = true;
        r->rc = MCGPU_CANCELLED;
        r->err = "request was cancelled";
        r->done = true;
        r->t_done = Clock::now();
        S->cancelled++;
    }
    S->cv_done.notify_all();
    S->cv_work.notify_all();
    return MCGPU_OK;
}

int mcgpu_server_wait(mcgpu_server S, uint64_t ticket, int timeout_ms, mcgpu_summary* out, double* latency_ms)
{
    if (!S) return sfail(MCGPU_INVALID_VALUE, "null server");
    std::unique_lock<std::mutex> lk(S->m);
    Request* r = find(S, ticket);
    if (!r) return sfail(MCGPU_INVALID_VALUE, "unknown ticket");
    if (timeout_ms < 0)
        S->cv_done.wait(lk, [&] { return r->done; });
    else if (!S->cv_done.wait_for(lk, std::chrono::milliseconds(timeout_ms), [&] { return r->done; }))
        return sfail(MCGPU_NOT_READY, "request still running");
    if (out) *out = r->sum;
    if (latency_ms) *latency_ms = std::chrono::duration<double, std::milli>(r->t_done - r->t_submit).count();
    if (r->cancelled) return sfail(MCGPU_CANCELLED, r->err);
    if (r->rc != MCGPU_OK) return sfail(r->rc, "the batch holding this request failed: " + r->err);
    return MCGPU_OK;
}

int mcgpu_server_get_data(mcgpu_server S, uint64_t ticket, uint32_t query, uint64_t bytes, void* mem,
    uint64_t* bytes_out)
{
    if (!S) return sfail(MCGPU_INVALID_VALUE, "null server");
    std::lock_guard<std::mutex> lk(S->m);
    Request* r = find(S, ticket);
    if (!r) return sfail(MCGPU_INVALID_VALUE, "unknown ticket");
    if (!r->done) return sfail(MCGPU_NOT_READY, "request still running");
    if (r->rc != MCGPU_OK) return sfail(r->rc, "the request has no records: " + r->err);
    const void* src = nullptr;
    uint64_t need = 0;
    if (query == MCGPU_DATA_RECORD_IDS) {
        src = r->ids.data();
        need = r->ids.size() * 4;
    } else if (query == MCGPU_DATA_RECORD_POINTS) {
        src = r->pts.data();
        need = r->pts.size() * 8;
    } else
        return sfail(MCGPU_INVALID_VALUE, "server queries: record ids and points");
    if (bytes_out) *bytes_out = need;
    if (!mem && bytes == 0) return MCGPU_OK;
    if (!mem || bytes < need) return sfail(MCGPU_INVALID_VALUE, "output buffer too small");
    if (need) memcpy(mem, src, need);
    return MCGPU_OK;
}

int mcgpu_server_release_request(mcgpu_server S, uint64_t ticket)
{
    if (!S) return sfail(MCGPU_INVALID_VALUE, "null server");
    std::lock_guard<std::mutex> lk(S->m);
    Request* r = find(S, ticket);
    if (!r) return sfail(MCGPU_INVALID_VALUE, "unknown ticket");
    if (!r->done) return sfail(MCGPU_NOT_READY, "request still running");
    S->reqs.erase(ticket);
    return MCGPU_OK;
}

int mcgpu_server_get_stats(mcgpu_server S, mcgpu_server_stats* out)
{
    if (!S || !out) return sfail(MCGPU_INVALID_VALUE, "null argument");
    std::lock_guard<std::mutex> lk(S->m);
    out->submitted = S->submitted;
    out->completed = S->completed;
    out->batches = S->batches;
    out->pending = S->pending.size();
    out->inflight_bytes = S->inflight;
    out->peak_inflight_bytes = S->peak_inflight;
    out->resident_bytes = S->resident_bytes;
    out->resident_meshes = S->cuts.size();
    out->pool_bytes = 0;
    for (uint64_t b : S->pool) out->pool_bytes += b;
    out->peak_reserved_bytes = S->peak_reserved;
    out->pool_trims = S->trims;
    out->cancelled = S->cancelled;
    return MCGPU_OK;
}

} // extern "C"
