// Harness around the reference with its front-end seam opened (TEST
// INFRASTRUCTURE ONLY; nothing in the product links it).
//
// The reference sources are copied and edited by oracle/make_seam.py so that
// dispatch() (kernel.cpp) takes its narrow-phase outputs -- the intersection
// vertices of m0 and the maps built from them, kernel.cpp:2377-2413 -- from
// the hook below instead of computing them; everything after (cut-path edges,
// polygon clipping, connected components, the public API) is the reference's
// own code. The hook applies a record hand-over in the form the GPU library
// delivers it (mcgpu_get_data's record and hand-over queries; fe_seam in
// mcut_oracle.h):
//   live    every front-end pass of the dispatch is computed by the oracle
//           (oracle_front_end_internal over the polygon soup the hook is
//           given, then oracle_seam), so general-position perturbation and
//           floating-polygon re-entries are covered;
//   replay  one hand-over recorded elsewhere -- the GPU's, read back through
//           the C ABI -- is applied to the dispatch's single front-end pass,
//           after checking that the polygon soup's coordinates are the ones
//           it was computed from.
// seam_dispatch() runs mcCreateContext / mcDispatch / mcGetConnectedComponents
// as ref_dispatch() does and returns the result code and per-CC (type, vertex
// count, face count), to be compared with the unmodified reference's.
#include <mcut/mcut.h>
#include <mcut/internal/hmesh.h>
#include <mcut/internal/kernel.h>
#include <mcut/internal/math.h>
#include <mcut/internal/tpool.h>
#include <mcut/internal/utils.h>

#include <algorithm>
#include <cstdio>
#include <cstring>
#include <string>
#include <unistd.h>
#include <vector>

#include "mcut_oracle.h"
#include "seam_hook.h"

bool calculate_vertex_parameters(double& quantization_multiplier, vec3_<double>& pre_quantization_translation,
    vec3_<double>& srcmesh_cutmesh_com, vec3_<double>& srcmesh_bboxmin, vec3_<double>& srcmesh_bboxmax,
    vec3_<double>& cutmesh_bboxmin, vec3_<double>& cutmesh_bboxmax, McFlags dispatchFlags,
    const void* pSrcMeshVertices, McUint32 numSrcMeshVertices, const void* pCutMeshVertices,
    McUint32 numCutMeshVertices);

namespace {

int g_mode = 0;                   // 0 live, 1 replay
int g_numbering = 0;              // 0 the hand-over's own (canonical) order, 1 the reference's
int g_n_replay = 0;               // replay: one hand-over per front-end pass, in pass order
const fe_seam* g_replay = nullptr;
const uint64_t* g_replay_hash = nullptr; // FNV-1a of the soup's coordinates each was computed from (0: unchecked)
const int* g_replay_status = nullptr;    // 0 success, 1 general-position violation

// every pass's inputs as the hook saw them (the oracle's view of the soup)
struct PassInput {
    std::vector<double> x;
    std::vector<uint32_t> sidx, ssz, cidx, csz;
    uint32_t vs, fs;
    double eps;
};
std::vector<PassInput> g_passes;
double g_eps = 0.0;               // cut-box enlargement of the live oracle pass
int g_calls = 0;
int g_error = 0;
std::string g_msg;

bool fail(int code, const std::string& msg)
{
    if (!g_error) {
        g_error = code;
        g_msg = msg;
    }
    return false;
}

uint64_t fnv1a(const unsigned char* p, size_t n, uint64_t h = 1469598103934665603ull)
{
    for (size_t i = 0; i < n; ++i) {
        h ^= p[i];
        h *= 1099511628211ull;
    }
    return h;
}

// the hand-over into dispatch()'s containers, as kernel.cpp:2599-2714 leaves them
bool apply(const fe_seam& s, const hmesh_t& ps, hmesh_t& m0, std::vector<std::pair<ed_t, fd_t>>& registry,
    std::vector<vd_t>& border, std::unordered_map<ed_t, std::vector<vd_t>>& isect_edges,
    std::map<pair<fd_t>, std::vector<vd_t>>& cutpath, std::unordered_map<fd_t, std::vector<vd_t>>& iface,
    bool& partial)
{
    const uint32_t nv = (uint32_t)ps.number_of_vertices();
    for (int64_t i = 0; i < s.n_records; ++i) {
        const uint32_t* r = s.rec_ids + 5 * i;
        const double* p = s.rec_pts + 3 * i;
        const vd_t v = m0.add_vertex(vec3(p[0], p[1], p[2]));
        if ((uint32_t)v != nv + (uint32_t)i) return fail(3, "m0 vertex ids do not follow the records");
        const ed_t e = ps.edge(vd_t(r[0]), vd_t(r[1]));
        if (e == hmesh_t::null_edge()) return fail(2, "a record's edge is not in the polygon soup");
        registry.emplace_back(e, fd_t(r[2]));
    }
    for (uint32_t e = 0; e < s.n_edges; ++e) {
        std::vector<vd_t>& l = isect_edges[registry[s.edge_off[e]].first];
        for (uint32_t i = s.edge_off[e]; i < s.edge_off[e + 1]; ++i) l.push_back(vd_t(nv + i));
    }
    for (uint32_t k = 0; k < s.n_cutpath; ++k) {
        std::vector<vd_t>& l = cutpath[make_pair(fd_t(s.cp_pairs[2 * k]), fd_t(s.cp_pairs[2 * k + 1]))];
        for (uint32_t j = s.cp_off[k]; j < s.cp_off[k + 1]; ++j) l.push_back(vd_t(s.cp_vtx[j]));
    }
    for (uint32_t m = 0; m < s.n_faces; ++m) {
        std::vector<vd_t>& l = iface[fd_t(s.face_keys[m])];
        for (uint32_t j = s.face_off[m]; j < s.face_off[m + 1]; ++j) l.push_back(vd_t(s.face_vtx[j]));
    }
    for (uint32_t b = 0; b < s.n_border; ++b) border.push_back(vd_t(s.border[b]));
    partial = s.n_border > 0;
    return true;
}

// The same hand-over numbered as the reference's own narrow phase numbers it:
// edges in the iteration order of its edge -> tested faces map, cut into
// parallel_for's blocks (tpool.h:420-472) and merged master block first, then
// the workers' blocks in order (kernel.cpp:2664-2714); an edge's records in
// tested-face order (the map's face lists are sorted). Lists keep ascending
// ids, as each thread appends in its processing order.
struct Renumbered {
    std::vector<uint32_t> rec_ids, edge_off, cp_pairs, cp_off, cp_vtx, face_keys, face_off, face_vtx, border;
    std::vector<double> rec_pts;
    fe_seam view() const
    {
        fe_seam s;
        memset(&s, 0, sizeof s);
        s.n_records = (int64_t)(rec_ids.size() / 5);
        s.rec_ids = const_cast<uint32_t*>(rec_ids.data());
        s.rec_pts = const_cast<double*>(rec_pts.data());
        s.n_edges = (uint32_t)edge_off.size() - 1;
        s.edge_off = const_cast<uint32_t*>(edge_off.data());
        s.n_cutpath = (uint32_t)cp_off.size() - 1;
        s.cp_pairs = const_cast<uint32_t*>(cp_pairs.data());
        s.cp_off = const_cast<uint32_t*>(cp_off.data());
        s.cp_vtx = const_cast<uint32_t*>(cp_vtx.data());
        s.n_faces = (uint32_t)face_off.size() - 1;
        s.face_keys = const_cast<uint32_t*>(face_keys.data());
        s.face_off = const_cast<uint32_t*>(face_off.data());
        s.face_vtx = const_cast<uint32_t*>(face_vtx.data());
        s.n_border = (uint32_t)border.size();
        s.border = const_cast<uint32_t*>(border.data());
        return s;
    }
};

bool renumber_like_reference(const fe_seam& s, const hmesh_t& ps,
    const std::unordered_map<ed_t, std::vector<fd_t>>& edge_faces, int helper_threads, Renumbered& out)
{
    const uint32_t nv = (uint32_t)ps.number_of_vertices();
    // the hand-over's record groups by (undirected) edge
    std::map<std::pair<uint32_t, uint32_t>, uint32_t> group_of;
    for (uint32_t e = 0; e < s.n_edges; ++e) {
        const uint32_t* r = s.rec_ids + 5ull * s.edge_off[e];
        group_of[{ std::min(r[0], r[1]), std::max(r[0], r[1]) }] = e;
    }
    std::vector<ed_t> iter;
    for (const auto& kv : edge_faces) iter.push_back(kv.first);
    uint32_t num_threads = 1, max_threads = 0, block = 0;
    if (!iter.empty())
        get_scheduling_parameters(num_threads, max_threads, block, (uint32_t)iter.size(),
            (uint32_t)helper_threads + 1, 1u << 10);
    const size_t master_first = (size_t)(num_threads - 1) * block;
    std::vector<ed_t> order(iter.begin() + (std::ptrdiff_t)master_first, iter.end());
    order.insert(order.end(), iter.begin(), iter.begin() + (std::ptrdiff_t)master_first);
    std::vector<uint32_t> new_of_old(s.n_records, 0xFFFFFFFFu);
    uint32_t next = 0;
    out.edge_off.assign(1, 0);
    for (const ed_t e : order) {
        const hd_t h = ps.halfedge(e, 0);
        const uint32_t a = (uint32_t)ps.source(h), b = (uint32_t)ps.target(h);
        auto it = group_of.find({ std::min(a, b), std::max(a, b) });
        if (it == group_of.end()) continue;
        for (uint32_t i = s.edge_off[it->second]; i < s.edge_off[it->second + 1]; ++i) {
            new_of_old[i] = next++;
            out.rec_ids.insert(out.rec_ids.end(), s.rec_ids + 5ull * i, s.rec_ids + 5ull * i + 5);
            out.rec_pts.insert(out.rec_pts.end(), s.rec_pts + 3ull * i, s.rec_pts + 3ull * i + 3);
        }
        out.edge_off.push_back(next);
    }
    if (next != (uint32_t)s.n_records) {
        for (int64_t i = 0; i < s.n_records; ++i)
            if (new_of_old[i] == 0xFFFFFFFFu)
                return fail(6, "the edge of record (" + std::to_string(s.rec_ids[5 * i]) + ", " +
                        std::to_string(s.rec_ids[5 * i + 1]) + ", face " + std::to_string(s.rec_ids[5 * i + 2]) +
                        ") is not in the reference's edge map");
    }
    auto remap = [&](uint32_t v) { return nv + new_of_old[v - nv]; };
    auto lists = [&](uint32_t n, const uint32_t* keys, int kw, const uint32_t* off, const uint32_t* vtx,
                     std::vector<uint32_t>& okeys, std::vector<uint32_t>& ooff, std::vector<uint32_t>& ovtx) {
        okeys.assign(keys, keys + (size_t)n * kw);
        ooff.assign(off, off + n + 1);
        ovtx.resize(off[n]);
        for (uint32_t k = 0; k < n; ++k) {
            for (uint32_t j = off[k]; j < off[k + 1]; ++j) ovtx[j] = remap(vtx[j]);
            std::sort(ovtx.begin() + off[k], ovtx.begin() + off[k + 1]);
        }
    };
    lists(s.n_cutpath, s.cp_pairs, 2, s.cp_off, s.cp_vtx, out.cp_pairs, out.cp_off, out.cp_vtx);
    lists(s.n_faces, s.face_keys, 1, s.face_off, s.face_vtx, out.face_keys, out.face_off, out.face_vtx);
    for (uint32_t b = 0; b < s.n_border; ++b) out.border.push_back(remap(s.border[b]));
    std::sort(out.border.begin(), out.border.end());
    return true;
}

bool apply_numbered(const fe_seam& s, const hmesh_t& ps, hmesh_t& m0, std::vector<std::pair<ed_t, fd_t>>& registry,
    std::vector<vd_t>& border, std::unordered_map<ed_t, std::vector<vd_t>>& isect_edges,
    std::map<pair<fd_t>, std::vector<vd_t>>& cutpath, std::unordered_map<fd_t, std::vector<vd_t>>& iface,
    bool& partial, const std::unordered_map<ed_t, std::vector<fd_t>>& edge_faces, int helper_threads)
{
    if (g_numbering == 0) return apply(s, ps, m0, registry, border, isect_edges, cutpath, iface, partial);
    Renumbered r;
    if (!renumber_like_reference(s, ps, edge_faces, helper_threads, r)) return false;
    const fe_seam v = r.view();
    return apply(v, ps, m0, registry, border, isect_edges, cutpath, iface, partial);
}

uint64_t soup_hash(const hmesh_t& ps)
{
    uint64_t h = 1469598103934665603ull;
    for (int v = 0; v < ps.number_of_vertices(); ++v) {
        const vec3& x = ps.vertex(vd_t(v));
        const double c[3] = { x.x(), x.y(), x.z() };
        h = fnv1a(reinterpret_cast<const unsigned char*>(c), sizeof c, h);
    }
    return h;
}

bool hook(const hmesh_t& ps, int sm_vtx_cnt, int sm_face_count, hmesh_t& m0,
    std::vector<std::pair<ed_t, fd_t>>& registry, std::vector<vd_t>& border,
    std::unordered_map<ed_t, std::vector<vd_t>>& isect_edges, std::map<pair<fd_t>, std::vector<vd_t>>& cutpath,
    std::unordered_map<fd_t, std::vector<vd_t>>& iface, bool& partial, int& status,
    const std::unordered_map<ed_t, std::vector<fd_t>>& edge_faces, int helper_threads)
{
    const int pass = g_calls++;
    status = 0;
    // this pass's meshes as arrays, as the front end is given them: the soup's
    // source then cut vertices; a source face from its first corner (its
    // halfedges' sources in order); a cut face the soup holds from its second
    // corner (kernel.cpp:1650-1700 adds cs.get_vertices_around_face), so its
    // last halfedge's source comes first
    g_passes.emplace_back();
    PassInput& in = g_passes.back();
    const uint32_t nv = (uint32_t)ps.number_of_vertices(), nf = (uint32_t)ps.number_of_faces();
    const uint32_t vs = in.vs = (uint32_t)sm_vtx_cnt, fs = in.fs = (uint32_t)sm_face_count;
    in.eps = g_eps;
    std::vector<double>& x = in.x;
    x.resize((size_t)nv * 3);
    for (uint32_t v = 0; v < nv; ++v) {
        const vec3& p = ps.vertex(vd_t(v));
        x[3 * v] = p.x();
        x[3 * v + 1] = p.y();
        x[3 * v + 2] = p.z();
    }
    std::vector<uint32_t>&sidx = in.sidx, &cidx = in.cidx, &ssz = in.ssz, &csz = in.csz;
    for (uint32_t f = 0; f < nf; ++f) {
        const std::vector<hd_t>& hs = ps.get_halfedges_around_face(fd_t(f));
        const size_t n = hs.size();
        for (size_t k = 0; k < n; ++k) {
            if (f < fs) sidx.push_back((uint32_t)ps.source(hs[k]));
            else cidx.push_back((uint32_t)ps.source(hs[(k + n - 1) % n]) - vs);
        }
        (f < fs ? ssz : csz).push_back((uint32_t)n);
    }
    if (g_mode == 1) {
        if (pass >= g_n_replay) return fail(5, "the dispatch ran more front-end passes than the replay holds");
        if (g_replay_hash[pass] && soup_hash(ps) != g_replay_hash[pass])
            return fail(1, "pass " + std::to_string(pass) + ": the soup's coordinates differ from the replay's");
        if (g_replay_status[pass] != 0) {
            status = 1;
            return true;
        }
        return apply_numbered(g_replay[pass], ps, m0, registry, border, isect_edges, cutpath, iface, partial,
            edge_faces, helper_threads);
    }
    // live: the oracle's pass over this soup
    fe_result r;
    if (oracle_front_end_internal(x.data(), sidx.data(), ssz.data(), vs, fs, x.data() + (size_t)vs * 3, cidx.data(),
            csz.data(), nv - vs, nf - fs, g_eps, 0, &r) != 0)
        return fail(4, "oracle pass failed");
    bool ok = true;
    if (r.status == FE_GP_VIOLATION) {
        status = 1;
    } else if (r.status != FE_OK) {
        ok = fail(4, "oracle pass status " + std::to_string(r.status));
    } else {
        fe_seam s;
        if (oracle_seam(sidx.data(), ssz.data(), vs, fs, cidx.data(), csz.data(), nv - vs, nf - fs, r.rec_ids,
                r.rec_pts, r.n_records, &s) != 0)
            ok = fail(4, "oracle hand-over failed");
        else
            ok = apply_numbered(s, ps, m0, registry, border, isect_edges, cutpath, iface, partial, edge_faces,
                helper_threads);
        oracle_seam_free(&s);
    }
    oracle_free(&r);
    return ok;
}

// the reference's own records (observer): per record q, r, tested face
std::vector<uint32_t> g_observed;
std::vector<double> g_observed_pts;
void observer(const hmesh_t& ps, const hmesh_t& m0, const std::vector<std::pair<ed_t, fd_t>>& registry)
{
    ++g_calls;
    g_observed.clear();
    g_observed_pts.clear();
    const int nv = ps.number_of_vertices();
    for (size_t i = 0; i < registry.size(); ++i) {
        const hd_t h = ps.halfedge(registry[i].first, 0);
        g_observed.push_back((uint32_t)ps.source(h));
        g_observed.push_back((uint32_t)ps.target(h));
        g_observed.push_back((uint32_t)registry[i].second);
        const vec3& p = m0.vertex(vd_t(nv + (int)i));
        g_observed_pts.push_back(p.x());
        g_observed_pts.push_back(p.y());
        g_observed_pts.push_back(p.z());
    }
}

// The reference's cut-path edge creation, observed (each pass): its inputs in
// the form oracle_cutpath takes them and its outputs.
struct CutpathObs {
    uint32_t nv = 0;
    std::vector<double> x, ivtx_xyz;
    std::vector<uint32_t> soup_off, soup_idx, reg, key_pairs, key_off, key_vtx;
    std::vector<uint32_t> edges, face_keys, face_off, face_edges, ivtx_off, ivtx_he;
    int bad = 0; // an output the arrays cannot hold (an edge id out of creation order)
};
std::vector<CutpathObs> g_cutpath;

void cutpath_observer(const hmesh_t& ps, const hmesh_t& m0, const std::vector<std::pair<ed_t, fd_t>>& registry,
    const std::map<pair<fd_t>, std::vector<vd_t>>& info, const std::vector<ed_t>& edges,
    const std::unordered_map<fd_t, std::vector<ed_t>>& face_edges,
    const std::unordered_map<vd_t, std::vector<hd_t>>& incoming)
{
    g_cutpath.emplace_back();
    CutpathObs& o = g_cutpath.back();
    const uint32_t nv = o.nv = (uint32_t)ps.number_of_vertices();
    for (uint32_t v = 0; v < nv; ++v) {
        const vec3& p = ps.vertex(vd_t(v));
        o.x.insert(o.x.end(), { p.x(), p.y(), p.z() });
    }
    o.soup_off.push_back(0);
    for (uint32_t f = 0; f < (uint32_t)ps.number_of_faces(); ++f) {
        for (const vd_t v : ps.get_vertices_around_face(fd_t(f))) o.soup_idx.push_back((uint32_t)v);
        o.soup_off.push_back((uint32_t)o.soup_idx.size());
    }
    auto face_or_none = [](fd_t f) { return f == hmesh_t::null_face() ? 0xFFFFFFFFu : (uint32_t)f; };
    for (size_t i = 0; i < registry.size(); ++i) {
        o.reg.push_back((uint32_t)registry[i].second);
        o.reg.push_back(face_or_none(ps.face(ps.halfedge(registry[i].first, 0))));
        o.reg.push_back(face_or_none(ps.face(ps.halfedge(registry[i].first, 1))));
        const vec3& p = m0.vertex(vd_t(nv + (uint32_t)i));
        o.ivtx_xyz.insert(o.ivtx_xyz.end(), { p.x(), p.y(), p.z() });
    }
    o.key_off.push_back(0);
    for (const auto& kv : info) {
        o.key_pairs.push_back((uint32_t)kv.first.first);
        o.key_pairs.push_back((uint32_t)kv.first.second);
        for (const vd_t v : kv.second) o.key_vtx.push_back((uint32_t)v);
        o.key_off.push_back((uint32_t)o.key_vtx.size());
    }
    for (size_t e = 0; e < edges.size(); ++e) {
        if ((size_t)edges[e] != e) o.bad = 1;
        const hd_t h = m0.halfedge(edges[e], 0);
        o.edges.push_back((uint32_t)m0.source(h));
        o.edges.push_back((uint32_t)m0.target(h));
        if ((size_t)h != 2 * e) o.bad = 1;
    }
    std::vector<uint32_t> fk;
    for (const auto& kv : face_edges) fk.push_back((uint32_t)kv.first);
    std::sort(fk.begin(), fk.end());
    o.face_off.push_back(0);
    for (const uint32_t f : fk) {
        o.face_keys.push_back(f);
        for (const ed_t e : face_edges.at(fd_t(f))) o.face_edges.push_back((uint32_t)e);
        o.face_off.push_back((uint32_t)o.face_edges.size());
    }
    o.ivtx_off.assign(registry.size() + 1, 0);
    for (size_t i = 0; i < registry.size(); ++i) {
        auto it = incoming.find(vd_t(nv + (uint32_t)i));
        if (it != incoming.end())
            for (const hd_t h : it->second) o.ivtx_he.push_back((uint32_t)h);
        o.ivtx_off[i + 1] = (uint32_t)o.ivtx_he.size();
    }
    if (incoming.size() > 0)
        for (const auto& kv : incoming)
            if ((uint32_t)kv.first < nv || (uint32_t)kv.first >= nv + registry.size()) o.bad = 1;
}

// The floating polygons each pass detected: per polygon its ps face, normal,
// largest normal component and vertex coordinates in the reference's order.
struct FloatingObs {
    std::vector<uint32_t> faces, off, mc;
    std::vector<double> normals, xyz;
};
std::vector<FloatingObs> g_floating;
void floating_observer(const std::map<fd_t, std::vector<floating_polygon_info_t>>& polygons)
{
    g_floating.emplace_back();
    FloatingObs& o = g_floating.back();
    o.off.push_back(0);
    for (const auto& kv : polygons)
        for (const floating_polygon_info_t& p : kv.second) {
            o.faces.push_back((uint32_t)kv.first);
            o.mc.push_back((uint32_t)p.polygon_normal_largest_component);
            o.normals.insert(o.normals.end(), { p.polygon_normal.x(), p.polygon_normal.y(), p.polygon_normal.z() });
            for (const vec3& v : p.polygon_vertices) o.xyz.insert(o.xyz.end(), { v.x(), v.y(), v.z() });
            o.off.push_back((uint32_t)(o.xyz.size() / 3));
        }
}

} // namespace

extern "C" int seam_floating_count() { return (int)g_floating.size(); }

// Floating observation k: sizes[2] = polygons, vertices; then (non-null) the arrays.
extern "C" int seam_floating_observation(int k, uint64_t* sizes, uint32_t* faces, uint32_t* off, uint32_t* mc,
    double* normals, double* xyz)
{
    if (k < 0 || k >= (int)g_floating.size()) return -1;
    const FloatingObs& o = g_floating[k];
    sizes[0] = o.faces.size();
    sizes[1] = o.xyz.size() / 3;
    if (faces && !o.faces.empty()) memcpy(faces, o.faces.data(), o.faces.size() * 4);
    if (off) memcpy(off, o.off.data(), o.off.size() * 4);
    if (mc && !o.mc.empty()) memcpy(mc, o.mc.data(), o.mc.size() * 4);
    if (normals && !o.normals.empty()) memcpy(normals, o.normals.data(), o.normals.size() * 8);
    if (xyz && !o.xyz.empty()) memcpy(xyz, o.xyz.data(), o.xyz.size() * 8);
    return 0;
}

// The cut-path observations of the last seam_observe_reference call: how many.
extern "C" int seam_cutpath_count() { return (int)g_cutpath.size(); }

// Observation k: sizes[14] = nv, |x|, |soup_off|, |soup_idx|, |reg|, |ivtx_xyz|,
// |key_pairs|, |key_off|, |key_vtx|, |edges|, |face_keys|, |face_off|,
// |face_edges|, |ivtx_off|; then (arrays non-null) the arrays in that order
// (doubles: x, ivtx_xyz) with |ivtx_he| in sizes[14] and bad in sizes[15].
extern "C" int seam_cutpath_observation(int k, uint64_t* sizes, double* x, double* ivtx_xyz, uint32_t* soup_off,
    uint32_t* soup_idx, uint32_t* reg, uint32_t* key_pairs, uint32_t* key_off, uint32_t* key_vtx, uint32_t* edges,
    uint32_t* face_keys, uint32_t* face_off, uint32_t* face_edges, uint32_t* ivtx_off, uint32_t* ivtx_he)
{
    if (k < 0 || k >= (int)g_cutpath.size()) return -1;
    const CutpathObs& o = g_cutpath[k];
    const uint64_t sz[16] = { o.nv, o.x.size(), o.soup_off.size(), o.soup_idx.size(), o.reg.size(), o.ivtx_xyz.size(),
        o.key_pairs.size(), o.key_off.size(), o.key_vtx.size(), o.edges.size(), o.face_keys.size(), o.face_off.size(),
        o.face_edges.size(), o.ivtx_off.size(), o.ivtx_he.size(), (uint64_t)o.bad };
    memcpy(sizes, sz, sizeof sz);
    auto cp = [](auto* dst, const auto& v) {
        if (dst && !v.empty()) memcpy(dst, v.data(), v.size() * sizeof(v[0]));
    };
    cp(x, o.x); cp(ivtx_xyz, o.ivtx_xyz); cp(soup_off, o.soup_off); cp(soup_idx, o.soup_idx); cp(reg, o.reg);
    cp(key_pairs, o.key_pairs); cp(key_off, o.key_off); cp(key_vtx, o.key_vtx); cp(edges, o.edges);
    cp(face_keys, o.face_keys); cp(face_off, o.face_off); cp(face_edges, o.face_edges); cp(ivtx_off, o.ivtx_off);
    cp(ivtx_he, o.ivtx_he);
    return 0;
}

// The unmodified reference's dispatch, observed: its records of the last
// front-end pass in its own numbering (q, r, tested face; up to cap).
// Returns the McResult; *n the record count, *calls the passes observed.
extern "C" int seam_observe_reference(const void* sv, const uint32_t* sf, const uint32_t* sfs, uint32_t nsv,
    uint32_t nsf, const void* cv, const uint32_t* cf, const uint32_t* cfs, uint32_t ncv, uint32_t ncf, uint32_t flags,
    int n_helpers, const char* workdir, uint32_t* rec3, double* pts, int64_t cap, int64_t* n, int* calls)
{
    g_calls = 0;
    g_observed.clear();
    g_cutpath.clear();
    g_floating.clear();
    mcut_seam_install(nullptr);
    mcut_seam_observe(&observer);
    mcut_seam_observe_cutpath(&cutpath_observer);
    mcut_seam_observe_floating(&floating_observer);
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1000;
    if (workdir && chdir(workdir) != 0) return -1001;
    McContext ctx = MC_NULL_HANDLE;
    McResult err = n_helpers > 0 ? mcCreateContextWithHelpers(&ctx, MC_NULL_HANDLE, (McUint32)n_helpers)
                                 : mcCreateContext(&ctx, MC_NULL_HANDLE);
    if (err == MC_NO_ERROR) err = mcDispatch(ctx, flags, sv, sf, sfs, nsv, nsf, cv, cf, cfs, ncv, ncf);
    if (ctx != MC_NULL_HANDLE) mcReleaseContext(ctx);
    mcut_seam_observe(nullptr);
    mcut_seam_observe_cutpath(nullptr);
    mcut_seam_observe_floating(nullptr);
    if (workdir && chdir(cwd) != 0) return -1002;
    *n = (int64_t)(g_observed.size() / 3);
    for (int64_t i = 0; i < *n && i < cap; ++i) {
        memcpy(rec3 + 3 * i, g_observed.data() + 3 * i, 12);
        memcpy(pts + 3 * i, g_observed_pts.data() + 3 * i, 24);
    }
    *calls = g_calls;
    return (int)err;
}

// mode 0: live; mode 1: replay replay[0 .. n_replay), one per front-end pass
// in pass order (each computed from coordinates whose FNV-1a hash is
// replay_hash[k], 0 to skip the check; replay_status[k] 1 replays a
// general-position violation). Returns the McResult of mcDispatch; cc_info
// receives (type, vertex count, face count) per CC (capacity max_cc) and
// cc_used (if not null) the number of those vertices its faces use; *calls
// the front-end passes the dispatch ran; *error a nonzero code (with msg) if
// the hand-over could not be applied. numbering 0 applies the hand-over's
// canonical numbering, 1 renumbers it as the reference's narrow phase would.
extern "C" int seam_dispatch(int mode, int numbering, int n_replay, const fe_seam* replay,
    const uint64_t* replay_hash, const int* replay_status,
    const void* sv, const uint32_t* sf, const uint32_t* sfs, uint32_t nsv, uint32_t nsf, const void* cv,
    const uint32_t* cf, const uint32_t* cfs, uint32_t ncv, uint32_t ncf, uint32_t flags, int n_helpers,
    const char* workdir, int32_t* cc_info, int32_t* cc_used, int max_cc, int* n_cc, int* calls, int* error, char* msg,
    int msg_len)
{
    g_mode = mode;
    g_numbering = numbering;
    g_n_replay = n_replay;
    g_replay = replay;
    g_replay_hash = replay_hash;
    g_replay_status = replay_status;
    g_passes.clear();
    g_calls = 0;
    g_error = 0;
    g_msg.clear();
    {
        double multiplier = 1;
        vec3_<double> smin, smax, cmin, cmax, com, trans;
        calculate_vertex_parameters(multiplier, trans, com, smin, smax, cmin, cmax, flags, sv, nsv, cv, ncv);
        g_eps = length(cmax - cmin, 1) * 1e-4; // preproc.cpp:2518, 2664-2676
    }
    mcut_seam_install(&hook);
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd)) return -1000;
    if (workdir && chdir(workdir) != 0) return -1001;
    McContext ctx = MC_NULL_HANDLE;
    McResult err = n_helpers > 0 ? mcCreateContextWithHelpers(&ctx, MC_NULL_HANDLE, (McUint32)n_helpers)
                                 : mcCreateContext(&ctx, MC_NULL_HANDLE);
    if (err == MC_NO_ERROR) err = mcDispatch(ctx, flags, sv, sf, sfs, nsv, nsf, cv, cf, cfs, ncv, ncf);
    *n_cc = 0;
    if (err == MC_NO_ERROR) {
        McUint32 n = 0;
        mcGetConnectedComponents(ctx, MC_CONNECTED_COMPONENT_TYPE_ALL, 0, NULL, &n);
        std::vector<McConnectedComponent> ccs(n);
        if (n) mcGetConnectedComponents(ctx, MC_CONNECTED_COMPONENT_TYPE_ALL, n, ccs.data(), NULL);
        for (McUint32 i = 0; i < n && (int)i < max_cc; ++i) {
            McSize nb = 0;
            McConnectedComponentType t;
            mcGetConnectedComponentData(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_TYPE, sizeof(t), &t, NULL);
            mcGetConnectedComponentData(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_VERTEX_DOUBLE, 0, NULL, &nb);
            cc_info[i * 3 + 0] = (int32_t)t;
            cc_info[i * 3 + 1] = (int32_t)(nb / (3 * sizeof(double)));
            mcGetConnectedComponentData(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_FACE_SIZE, 0, NULL, &nb);
            cc_info[i * 3 + 2] = (int32_t)(nb / sizeof(McUint32));
            if (cc_used) { // vertices the CC's faces reference
                mcGetConnectedComponentData(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_FACE, 0, NULL, &nb);
                std::vector<McUint32> fi(nb / sizeof(McUint32));
                if (nb) mcGetConnectedComponentData(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_FACE, nb, fi.data(), NULL);
                std::vector<char> seen((size_t)cc_info[i * 3 + 1] + 1, 0);
                int32_t used = 0;
                for (McUint32 v : fi)
                    if (v < seen.size() && !seen[v]) { seen[v] = 1; ++used; }
                cc_used[i] = used;
            }
        }
        *n_cc = (int)n;
        if (n) mcReleaseConnectedComponents(ctx, 0, NULL);
    }
    if (ctx != MC_NULL_HANDLE) mcReleaseContext(ctx);
    mcut_seam_install(nullptr);
    if (workdir && chdir(cwd) != 0) return -1002;
    *calls = g_calls;
    *error = g_error;
    if (msg && msg_len > 0) snprintf(msg, (size_t)msg_len, "%s", g_msg.c_str());
    return (int)err;
}

// The inputs of front-end pass k of the last seam_dispatch, as the hook saw
// them: counts (vs, vc, fs, fc, source index count, cut index count) and eps;
// with non-null arrays (sized by a first call) the coordinates, faces and sizes.
extern "C" int seam_pass_input(int k, uint32_t* counts, double* eps, double* x, uint32_t* sidx, uint32_t* ssz,
    uint32_t* cidx, uint32_t* csz)
{
    if (k < 0 || k >= (int)g_passes.size()) return -1;
    const PassInput& p = g_passes[k];
    counts[0] = p.vs;
    counts[1] = (uint32_t)(p.x.size() / 3) - p.vs;
    counts[2] = p.fs;
    counts[3] = (uint32_t)p.csz.size();
    counts[4] = (uint32_t)p.sidx.size();
    counts[5] = (uint32_t)p.cidx.size();
    *eps = p.eps;
    if (x) memcpy(x, p.x.data(), p.x.size() * sizeof(double));
    if (sidx) memcpy(sidx, p.sidx.data(), p.sidx.size() * 4);
    if (ssz) memcpy(ssz, p.ssz.data(), p.ssz.size() * 4);
    if (cidx) memcpy(cidx, p.cidx.data(), p.cidx.size() * 4);
    if (csz) memcpy(csz, p.csz.data(), p.csz.size() * 4);
    return 0;
}

// FNV-1a of the soup's coordinates (source then cut vertices, x y z doubles),
// the check a replay makes
extern "C" uint64_t seam_coordinate_hash(const double* xyz, uint64_t n_doubles)
{
    return fnv1a(reinterpret_cast<const unsigned char*>(xyz), n_doubles * sizeof(double));
}
