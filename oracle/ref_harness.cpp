// Harness around the UNMODIFIED reference (MCUT 1.2.0) compiled into
// _ref/libmcut_ref.so from its own sources. Test infrastructure only: it is
// built where the reference checkout exists, pins the plain-C oracle and
// generates golden fixtures; nothing in the product links it.
//
// What it exposes (extern "C", consumed through ctypes by tests/golden/make_golden.py):
//   ref_front_end : the front end of one dispatch, step for step as
//                   preproc.cpp:2292-2926 and kernel.cpp:1593-2878 run it,
//                   calling the reference's own build_oibvh, intersectOIBVHs,
//                   compute_polygon_plane_coefficients,
//                   compute_segment_plane_intersection_type,
//                   compute_segment_plane_intersection,
//                   compute_point_in_polygon_test and ::orient3d.
//                   The only restated parts are the container plumbing of
//                   kernel.cpp (edge->faces map, culling loop), which the
//                   reference keeps inside dispatch().
//   ref_dispatch  : the full public API (mcCreateContext / mcDispatch /
//                   mcGetConnectedComponents / mcGetConnectedComponentData)
//                   returning status and per-CC type / vertex / face counts,
//                   plus the intersection-point count read back from the
//                   reference's own verbose dumps (kernel.cpp:1736-1738,3260-3266).
//   ref_cc_wire   : the full public API, then each connected component's
//                   arrays as mcGetConnectedComponentData returns them
//                   (vertices, faces, face sizes, face adjacency, edges).
//   ref_hmesh     : one mesh's halfedge mesh as the reference builds it (its
//                   own hmesh_t::add_vertex / add_face, preceded by the face
//                   checks of client_input_arrays_to_hmesh, preproc.cpp:390-460)
//                   and check_input_mesh's outcome (preproc.cpp:505-579, with
//                   the reference's find_connected_components) and
//                   mesh_is_closed (preproc.cpp:1957-1994), read back
//                   through hmesh_t's public accessors.
#include <mcut/mcut.h>
#include <mcut/internal/bvh.h>
#include <mcut/internal/hmesh.h>
#include <mcut/internal/kernel.h>
#include <mcut/internal/math.h>
#include <mcut/internal/tpool.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <set>
#include <string>
#include <tuple>
#include <unistd.h>
#include <vector>

#include "mcut_oracle.h"

bool calculate_vertex_parameters(double& quantization_multiplier, vec3_<double>& pre_quantization_translation,
    vec3_<double>& srcmesh_cutmesh_com, vec3_<double>& srcmesh_bboxmin, vec3_<double>& srcmesh_bboxmax,
    vec3_<double>& cutmesh_bboxmin, vec3_<double>& cutmesh_bboxmax, McFlags dispatchFlags,
    const void* pSrcMeshVertices, McUint32 numSrcMeshVertices, const void* pCutMeshVertices,
    McUint32 numCutMeshVertices);
bool mesh_is_closed(const hmesh_t& mesh);
bool determine_three_noncollinear_vertices(int& i, int& j, int& k, const std::vector<vec3>& polygon_vertices,
    const vec3& polygon_normal, const int polygon_normal_largest_component, const double multiplier);

namespace {

struct Mesh {
    const void* v; // double[3*nv], or float[3*nv] for float input
    const uint32_t* f;
    const uint32_t* fs; // nullable -> triangles
    uint32_t nv, nf;
};

// Recentring exactly as client_input_arrays_to_hmesh does it (preproc.cpp:100-181):
// float input is recentred in float arithmetic, then widened.
void recentre(const Mesh& m, bool fin, const vec3_<double>& com, const vec3_<double>& t, std::vector<double>& out)
{
    out.resize((size_t)m.nv * 3);
    for (uint32_t i = 0; i < m.nv; ++i)
        for (int j = 0; j < 3; ++j) {
            if (fin) {
                const float x = (((const float*)m.v)[i * 3 + j] - (float)com[j]) + (float)t[j];
                out[i * 3 + j] = double(x);
            } else {
                out[i * 3 + j] = (((const double*)m.v)[i * 3 + j] - com[j]) + t[j];
            }
        }
}

void add_faces(hmesh_t& h, const Mesh& m, uint32_t voff)
{
    size_t o = 0;
    std::vector<vd_t> fv;
    for (uint32_t f = 0; f < m.nf; ++f) {
        const uint32_t n = m.fs ? m.fs[f] : 3;
        fv.clear();
        for (uint32_t j = 0; j < n; ++j)
            fv.push_back(vd_t(m.f[o + j] + voff));
        o += n;
        h.add_face(fv);
    }
}

template <class T>
T* dup(const std::vector<T>& v)
{
    T* p = (T*)malloc(std::max<size_t>(1, v.size() * sizeof(T)));
    if (!v.empty())
        memcpy(p, v.data(), v.size() * sizeof(T));
    return p;
}

int sgn(double x) { return x > 0 ? 1 : (x < 0 ? -1 : 0); }

} // namespace

// With a perturbation (general-position enforcement) the polygon soup's cut
// vertices are the recentred ones plus the perturbation, as
// client_input_arrays_to_hmesh adds it (preproc.cpp:131-133, 176-180), while
// the BVHs, face boxes and candidate pairs stay those of the unperturbed
// meshes (preproc.cpp:2680, 2820-2846); a perturbed pass with no record is a
// general-position violation (kernel.cpp:3211-3225).
extern "C" int ref_front_end2(const void* sv, const uint32_t* sf, const uint32_t* sfs, uint32_t nsv, uint32_t nsf,
    const void* cv, const uint32_t* cf, const uint32_t* cfs, uint32_t ncv, uint32_t ncf,
    int float_input, int n_helpers, double gp_constant, int gp_absolute, const double* perturbation, fe_result* out)
{
    memset(out, 0, sizeof(*out));
    out->bad_face = -1;
    Mesh S { sv, sf, sfs, nsv, nsf }, C { cv, cf, cfs, ncv, ncf };

    double multiplier = 1;
    vec3_<double> smin, smax, cmin, cmax, com, trans;
    calculate_vertex_parameters(multiplier, trans, com, smin, smax, cmin, cmax,
        float_input ? MC_DISPATCH_VERTEX_ARRAY_FLOAT : MC_DISPATCH_VERTEX_ARRAY_DOUBLE, sv, nsv, cv, ncv);
    std::vector<double> sx, cx;
    recentre(S, float_input != 0, com, trans, sx);
    recentre(C, float_input != 0, com, trans, cx);
    std::vector<double> px = cx; // the narrow phase's cut coordinates
    if (perturbation)
        for (uint32_t i = 0; i < ncv; ++i)
            for (int j = 0; j < 3; ++j) px[i * 3 + j] = cx[i * 3 + j] + perturbation[j];
    out->src_xyz = dup(sx);
    out->cut_xyz = dup(px);

    // cut-mesh enlargement: diag length of the (translated) cut box, or 1 with
    // absolute enforcement, times the general-position constant
    // (preproc.cpp:2518, 2664-2676; frontend.h:596)
    const double cut_diag = length(cmax - cmin, 1);
    const double eps = (gp_absolute ? 1.0 : cut_diag) * gp_constant;
    out->cut_eps = eps;

    hmesh_t sm, cm, ps;
    for (uint32_t i = 0; i < nsv; ++i) {
        sm.add_vertex(sx[i * 3], sx[i * 3 + 1], sx[i * 3 + 2]);
        ps.add_vertex(sx[i * 3], sx[i * 3 + 1], sx[i * 3 + 2]);
    }
    for (uint32_t i = 0; i < ncv; ++i) {
        cm.add_vertex(cx[i * 3], cx[i * 3 + 1], cx[i * 3 + 2]);
        ps.add_vertex(px[i * 3], px[i * 3 + 1], px[i * 3 + 2]);
    }
    add_faces(sm, S, 0);
    add_faces(cm, C, 0);
    // the polygon soup as kernel.cpp:1593-1700 builds it: a copy of the
    // source mesh, then each cut-mesh face as cs.get_vertices_around_face
    // lists it (its corners from the second one on), offset by Vs
    add_faces(ps, S, 0);
    {
        std::vector<vd_t> fv;
        for (uint32_t f = 0; f < ncf; ++f) {
            fv.clear();
            cm.get_vertices_around_face(fv, fd_t(f), nsv);
            ps.add_face(fv);
        }
    }

    thread_pool pool((uint32_t)n_helpers, 0);
    std::vector<bounding_box_t<vec3_<double>>> sAABB, cAABB, sFB, cFB;
    std::vector<fd_t> sLeaf, cLeaf;
    build_oibvh(pool, sm, sAABB, sLeaf, sFB, 0.0, multiplier);
    build_oibvh(pool, cm, cAABB, cLeaf, cFB, eps, multiplier);

    std::vector<double> boxes;
    for (auto& b : sFB)
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < 3; ++j)
                boxes.push_back(k ? b.maximum()[j] : b.minimum()[j]);
    for (auto& b : cFB)
        for (int k = 0; k < 2; ++k)
            for (int j = 0; j < 3; ++j)
                boxes.push_back(k ? b.maximum()[j] : b.minimum()[j]);
    out->face_boxes = dup(boxes);

    std::map<fd_t, std::vector<fd_t>> cand;
    intersectOIBVHs(cand, sAABB, sLeaf, cAABB, cLeaf);

    std::vector<uint32_t> pairs;
    for (auto& kv : cand)
        if ((uint32_t)kv.first < nsf)
            for (fd_t g : kv.second) {
                pairs.push_back((uint32_t)kv.first);
                pairs.push_back((uint32_t)g - nsf);
            }
    {
        std::vector<std::pair<uint32_t, uint32_t>> pp;
        for (size_t i = 0; i < pairs.size(); i += 2)
            pp.emplace_back(pairs[i], pairs[i + 1]);
        std::sort(pp.begin(), pp.end());
        pairs.clear();
        for (auto& p : pp) {
            pairs.push_back(p.first);
            pairs.push_back(p.second);
        }
    }
    out->n_pairs = (int64_t)pairs.size() / 2;
    out->pairs = dup(pairs);
    if (cand.empty()) {
        out->tests = dup(std::vector<uint32_t>());
        out->test_info = dup(std::vector<int8_t>());
        out->rec_ids = dup(std::vector<uint32_t>());
        out->rec_pts = dup(std::vector<double>());
        return 0;
    }

    // edge -> sorted union of partner faces (kernel.cpp:1781-1983)
    std::map<uint32_t, std::set<uint32_t>> e2f;
    for (auto& kv : cand) {
        for (hd_t h : ps.get_halfedges_around_face(kv.first)) {
            auto& s = e2f[(uint32_t)ps.edge(h)];
            for (fd_t g : kv.second)
                s.insert((uint32_t)g);
        }
    }

    // face properties for every candidate face, degenerate check (kernel.cpp:2184-2356)
    std::map<uint32_t, std::tuple<vec3, double, int, std::vector<vec3>>> props;
    for (auto& kv : cand) {
        std::vector<vec3> fverts;
        for (vd_t v : ps.get_vertices_around_face(kv.first))
            fverts.push_back(ps.vertex(v));
        vec3 n(0.0);
        double d = 0;
        int mc = compute_polygon_plane_coefficients(n, d, fverts.data(), (int)fverts.size(), multiplier);
        if (squared_length(n) == 0 || std::isnan(n.x()) || std::isnan(n.y()) || std::isnan(n.z())) {
            if (out->bad_face < 0 || (int)kv.first < out->bad_face)
                out->bad_face = (int)kv.first;
        }
        props[(uint32_t)kv.first] = std::make_tuple(n, d, mc, fverts);
    }
    if (out->bad_face >= 0)
        out->status = (uint32_t)out->bad_face >= nsf ? FE_DEGENERATE_CUT_FACE : FE_DEGENERATE_SRC_FACE;

    // culling + narrow phase (kernel.cpp:2074-2177, 2456-2658)
    std::vector<std::tuple<uint32_t, uint32_t, uint32_t, int8_t, int8_t, int8_t, int8_t>> tests;
    std::vector<std::tuple<uint32_t, uint32_t, uint32_t, double, double, double>> recs;
    bool gp = false;
    for (auto& ef : e2f) {
        const ed_t e((uint32_t)ef.first);
        const hd_t h0 = ps.halfedge(e, 0);
        const vd_t qd = ps.source(h0), rd = ps.target(h0);
        const vec3 q = ps.vertex(qd), r = ps.vertex(rd);
        bounding_box_t<vec3_<double>> eb;
        eb.expand(ps.vertex(ps.vertex(e, 0)));
        eb.expand(ps.vertex(ps.vertex(e, 1)));
        for (uint32_t g : ef.second) {
            const bounding_box_t<vec3_<double>>& fb = g < nsf ? sFB[g] : cFB[g - nsf];
            if (!intersect_bounding_boxes(eb, fb))
                continue;
            if (out->status != FE_OK && out->status != FE_GP_VIOLATION)
                continue; // the reference stops before the narrow phase on a degenerate face
            auto& pr = props[g];
            const vec3& n = std::get<0>(pr);
            const double d = std::get<1>(pr);
            const int mc = std::get<2>(pr);
            const std::vector<vec3>& fv = std::get<3>(pr);
            int i = 0, j = 1, k = 2;
            if (fv.size() > 3)
                determine_three_noncollinear_vertices(i, j, k, fv, n, mc, multiplier);
            const int8_t sq = (int8_t)sgn(orient3d(fv[i], fv[j], fv[k], q));
            const int8_t sr = (int8_t)sgn(orient3d(fv[i], fv[j], fv[k], r));
            const char type = compute_segment_plane_intersection_type(q, r, fv, n, mc, multiplier);
            char pip = 0;
            if (type == 'q' || type == 'r') {
                pip = compute_point_in_polygon_test(type == 'q' ? q : r, fv, n, mc, multiplier);
            } else if (type == 'p') {
                pip = compute_point_in_polygon_test(q, fv, n, mc, multiplier);
                if (!(pip == 'i' || pip == 'v' || pip == 'e'))
                    pip = compute_point_in_polygon_test(r, fv, n, mc, multiplier);
            } else if (type == '1') {
                vec3 p(0., 0., 0.);
                compute_segment_plane_intersection(p, n, d, q, r);
                pip = compute_point_in_polygon_test(p, fv, n, mc, multiplier);
                if (pip == 'i')
                    recs.emplace_back((uint32_t)qd, (uint32_t)rd, g, p.x(), p.y(), p.z());
            }
            if ((type == 'q' || type == 'r' || type == 'p') && (pip == 'i' || pip == 'v' || pip == 'e'))
                gp = true;
            if (type == '1' && (pip == 'v' || pip == 'e'))
                gp = true;
            tests.emplace_back((uint32_t)qd, (uint32_t)rd, g, sq, sr, (int8_t)type, (int8_t)pip);
        }
    }
    if (out->status == FE_OK && gp)
        out->status = FE_GP_VIOLATION;
    std::sort(tests.begin(), tests.end());
    std::sort(recs.begin(), recs.end(), [](const auto& a, const auto& b) {
        return std::make_tuple(std::get<0>(a), std::get<1>(a), std::get<2>(a))
            < std::make_tuple(std::get<0>(b), std::get<1>(b), std::get<2>(b));
    });
    std::vector<uint32_t> tid, rid;
    std::vector<int8_t> tinfo;
    std::vector<double> rpt;
    for (auto& t : tests) {
        tid.push_back(std::get<0>(t));
        tid.push_back(std::get<1>(t));
        tid.push_back(std::get<2>(t));
        tinfo.push_back(std::get<3>(t));
        tinfo.push_back(std::get<4>(t));
        tinfo.push_back(std::get<5>(t));
        tinfo.push_back(std::get<6>(t));
    }
    for (auto& r : recs) {
        rid.push_back(std::get<0>(r));
        rid.push_back(std::get<1>(r));
        rid.push_back(std::get<2>(r));
        rpt.push_back(std::get<3>(r));
        rpt.push_back(std::get<4>(r));
        rpt.push_back(std::get<5>(r));
    }
    out->n_tests = (int64_t)tests.size();
    out->tests = dup(tid);
    out->test_info = dup(tinfo);
    out->n_records = (int64_t)recs.size();
    out->rec_ids = dup(rid);
    out->rec_pts = dup(rpt);
    if (perturbation && out->status == FE_OK && recs.empty()) out->status = FE_GP_VIOLATION;
    return 0;
}

extern "C" int ref_front_end(const void* sv, const uint32_t* sf, const uint32_t* sfs, uint32_t nsv, uint32_t nsf,
    const void* cv, const uint32_t* cf, const uint32_t* cfs, uint32_t ncv, uint32_t ncf,
    int float_input, int n_helpers, fe_result* out)
{
    return ref_front_end2(sv, sf, sfs, nsv, nsf, cv, cf, cfs, ncv, ncf, float_input, n_helpers, 1e-4, 0, nullptr, out);
}

extern "C" double ref_orient3d(const double* pa, const double* pb, const double* pc, const double* pd)
{
    return ::orient3d((double*)pa, (double*)pb, (double*)pc, (double*)pd);
}
extern "C" double ref_orient2d(const double* pa, const double* pb, const double* pc)
{
    return ::orient2d((double*)pa, (double*)pb, (double*)pc);
}

extern "C" void ref_free(fe_result* r)
{
    free(r->pairs);
    free(r->tests);
    free(r->test_info);
    free(r->rec_ids);
    free(r->rec_pts);
    free(r->face_boxes);
    free(r->src_xyz);
    free(r->cut_xyz);
    memset(r, 0, sizeof(*r));
}

static long off_vertex_count(const char* path)
{
    FILE* f = fopen(path, "r");
    if (!f)
        return -1;
    char line[256];
    long nv = -1;
    while (fgets(line, sizeof line, f)) {
        if (line[0] == '#' || line[0] == '\n' || strncmp(line, "OFF", 3) == 0)
            continue;
        nv = strtol(line, nullptr, 10);
        break;
    }
    fclose(f);
    return nv;
}

// Full public-API dispatch. cc_info receives, per connected component,
// (type, vertex count, face count), capacity max_cc. workdir receives the
// reference's verbose dumps. Returns the McResult of mcDispatch; *n_cc and
// *n_ivtx (intersection points of the last kernel invocation) are filled on
// success.
extern "C" int ref_dispatch(const void* sv, const uint32_t* sf, const uint32_t* sfs, uint32_t nsv, uint32_t nsf,
    const void* cv, const uint32_t* cf, const uint32_t* cfs, uint32_t ncv, uint32_t ncf, uint32_t flags,
    int n_helpers, const char* workdir, int32_t* cc_info, int max_cc, int* n_cc, long* n_ivtx)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd))
        return -1000;
    if (workdir && chdir(workdir) != 0)
        return -1001;
    McContext ctx = MC_NULL_HANDLE;
    McResult err = n_helpers > 0 ? mcCreateContextWithHelpers(&ctx, MC_NULL_HANDLE, (McUint32)n_helpers)
                                 : mcCreateContext(&ctx, MC_NULL_HANDLE);
    if (err == MC_NO_ERROR) {
        err = mcDispatch(ctx, flags, sv, sf, sfs, nsv, nsf, cv, cf, cfs, ncv, ncf);
    }
    *n_cc = 0;
    *n_ivtx = -1;
    if (err == MC_NO_ERROR) {
        McUint32 n = 0;
        mcGetConnectedComponents(ctx, MC_CONNECTED_COMPONENT_TYPE_ALL, 0, NULL, &n);
        std::vector<McConnectedComponent> ccs(n);
        if (n)
            mcGetConnectedComponents(ctx, MC_CONNECTED_COMPONENT_TYPE_ALL, n, ccs.data(), NULL);
        for (McUint32 i = 0; i < n && (int)i < max_cc; ++i) {
            McSize nb = 0;
            McConnectedComponentType t;
            mcGetConnectedComponentData(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_TYPE, sizeof(t), &t, NULL);
            mcGetConnectedComponentData(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_VERTEX_DOUBLE, 0, NULL, &nb);
            const long nvtx = (long)(nb / (3 * sizeof(double)));
            mcGetConnectedComponentData(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_FACE_SIZE, 0, NULL, &nb);
            const long nfc = (long)(nb / sizeof(McUint32));
            cc_info[i * 3 + 0] = (int32_t)t;
            cc_info[i * 3 + 1] = (int32_t)nvtx;
            cc_info[i * 3 + 2] = (int32_t)nfc;
        }
        *n_cc = (int)n;
        if (n)
            mcReleaseConnectedComponents(ctx, 0, NULL);
        const long m0v = off_vertex_count("m0.v.off");
        const long psv = off_vertex_count("polygon-soup.off");
        if (m0v >= 0 && psv >= 0)
            *n_ivtx = m0v - psv;
    }
    if (ctx != MC_NULL_HANDLE)
        mcReleaseContext(ctx);
    if (workdir && chdir(cwd) != 0)
        return -1002;
    return (int)err;
}

// One connected component as mcGetConnectedComponentData hands it to the
// caller (frontend.cpp:2006-2832): vertices as doubles and floats, faces
// (vertices around each face) with their sizes, the faces around each face
// with their counts, and the edges' vertex pairs.
struct cc_wire {
    int32_t type;
    uint32_t nv, nf, nidx, nadj, ne;
    double* vd;
    float* vf;
    uint32_t *face, *fsize, *adj, *adjsize, *edge;
};

template <typename T>
static T* cc_query(McContext ctx, McConnectedComponent cc, McFlags q, uint32_t* count)
{
    McSize nb = 0;
    if (mcGetConnectedComponentData(ctx, cc, q, 0, NULL, &nb) != MC_NO_ERROR)
        return nullptr;
    T* p = (T*)malloc(nb ? nb : sizeof(T));
    if (nb && mcGetConnectedComponentData(ctx, cc, q, nb, p, NULL) != MC_NO_ERROR) {
        free(p);
        return nullptr;
    }
    *count = (uint32_t)(nb / sizeof(T));
    return p;
}

// Full public-API dispatch, then every connected component's wire arrays
// through the reference's own mcGetConnectedComponentData. *out: n_cc
// entries (free with ref_cc_wire_free).
extern "C" int ref_cc_wire(const void* sv, const uint32_t* sf, const uint32_t* sfs, uint32_t nsv, uint32_t nsf,
    const void* cv, const uint32_t* cf, const uint32_t* cfs, uint32_t ncv, uint32_t ncf, uint32_t flags,
    const char* workdir, int* n_cc, cc_wire** out)
{
    char cwd[4096];
    if (!getcwd(cwd, sizeof cwd))
        return -1000;
    if (workdir && chdir(workdir) != 0)
        return -1001;
    *n_cc = 0;
    *out = nullptr;
    McContext ctx = MC_NULL_HANDLE;
    McResult err = mcCreateContext(&ctx, MC_NULL_HANDLE);
    if (err == MC_NO_ERROR)
        err = mcDispatch(ctx, flags, sv, sf, sfs, nsv, nsf, cv, cf, cfs, ncv, ncf);
    if (err == MC_NO_ERROR) {
        McUint32 n = 0;
        mcGetConnectedComponents(ctx, MC_CONNECTED_COMPONENT_TYPE_ALL, 0, NULL, &n);
        std::vector<McConnectedComponent> ccs(n);
        if (n)
            mcGetConnectedComponents(ctx, MC_CONNECTED_COMPONENT_TYPE_ALL, n, ccs.data(), NULL);
        cc_wire* w = (cc_wire*)calloc(n ? n : 1, sizeof(cc_wire));
        for (McUint32 i = 0; i < n; ++i) {
            McConnectedComponentType t;
            mcGetConnectedComponentData(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_TYPE, sizeof(t), &t, NULL);
            w[i].type = (int32_t)t;
            uint32_t k = 0;
            w[i].vd = cc_query<double>(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_VERTEX_DOUBLE, &k);
            w[i].nv = k / 3;
            w[i].vf = cc_query<float>(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_VERTEX_FLOAT, &k);
            w[i].face = cc_query<uint32_t>(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_FACE, &w[i].nidx);
            w[i].fsize = cc_query<uint32_t>(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_FACE_SIZE, &w[i].nf);
            w[i].adj = cc_query<uint32_t>(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_FACE_ADJACENT_FACE, &w[i].nadj);
            w[i].adjsize = cc_query<uint32_t>(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_FACE_ADJACENT_FACE_SIZE, &k);
            w[i].edge = cc_query<uint32_t>(ctx, ccs[i], MC_CONNECTED_COMPONENT_DATA_EDGE, &k);
            w[i].ne = k / 2;
        }
        *n_cc = (int)n;
        *out = w;
        if (n)
            mcReleaseConnectedComponents(ctx, 0, NULL);
    }
    if (ctx != MC_NULL_HANDLE)
        mcReleaseContext(ctx);
    if (workdir && chdir(cwd) != 0)
        return -1002;
    return (int)err;
}

extern "C" void ref_cc_wire_free(cc_wire* w, int n)
{
    for (int i = 0; i < n; ++i) {
        free(w[i].vd);
        free(w[i].vf);
        free(w[i].face);
        free(w[i].fsize);
        free(w[i].adj);
        free(w[i].adjsize);
        free(w[i].edge);
    }
    free(w);
}

// One mesh's halfedge mesh and input checks, step for step as the
// single-threaded branch of client_input_arrays_to_hmesh (preproc.cpp:390-460)
// and check_input_mesh (preproc.cpp:505-579) run them; the connectivity is the
// reference's own hmesh_t, read back through its public accessors.
extern "C" int ref_hmesh(const uint32_t* f, const uint32_t* fs, uint32_t nv, uint32_t nf, hm_result* out)
{
    memset(out, 0, sizeof(*out));
    out->bad_face = -1;
    hmesh_t m;
    for (uint32_t v = 0; v < nv; ++v)
        m.add_vertex(0.0, 0.0, 0.0);
    uint64_t o = 0;
    int st = HM_OK;
    std::vector<vd_t> fv;
    for (uint32_t i = 0; i < nf && st == HM_OK; ++i) {
        const uint32_t n = fs ? fs[i] : 3;
        if (n < 3) { st = HM_FACE_SIZE; out->bad_face = (int32_t)i; break; }
        fv.clear();
        for (uint32_t j = 0; j < n; ++j) {
            const uint32_t idx = f[o + j];
            if (idx >= nv) { st = HM_INDEX_RANGE; break; }
            const vd_t d(idx);
            if (std::find(fv.cbegin(), fv.cend(), d) != fv.cend()) { st = HM_DUPLICATE_INDEX; break; }
            fv.push_back(d);
        }
        if (st == HM_OK && m.add_face(fv) == hmesh_t::null_face())
            st = HM_NON_MANIFOLD;
        if (st != HM_OK)
            out->bad_face = (int32_t)i;
        o += n;
    }
    fflush(stdout); // add_face reports a non-manifold face on stdout
    out->status = st;
    if (st != HM_OK)
        return 0;
    const uint32_t ne = (uint32_t)m.number_of_edges();
    out->n_edges = ne;
    const size_t nh = 2 * (size_t)ne;
    out->he_target = (uint32_t*)malloc(4 * (nh ? nh : 1));
    out->he_face = (int32_t*)malloc(4 * (nh ? nh : 1));
    out->he_next = (int32_t*)malloc(4 * (nh ? nh : 1));
    out->he_prev = (int32_t*)malloc(4 * (nh ? nh : 1));
    if ((size_t)m.number_of_halfedges() != nh)
        return -1;
    for (uint32_t e = 0; e < ne; ++e)
        if ((uint32_t)m.halfedge(ed_t(e), 0) != 2 * e || (uint32_t)m.halfedge(ed_t(e), 1) != 2 * e + 1)
            return -2;
    for (size_t h = 0; h < nh; ++h) {
        const hd_t hd((uint32_t)h);
        out->he_target[h] = (uint32_t)m.target(hd);
        const fd_t fd = m.face(hd);
        out->he_face[h] = fd == hmesh_t::null_face() ? -1 : (int32_t)fd;
        const hd_t nx = m.next(hd), pv = m.prev(hd);
        out->he_next[h] = nx == hmesh_t::null_halfedge() ? -1 : (int32_t)nx;
        out->he_prev[h] = pv == hmesh_t::null_halfedge() ? -1 : (int32_t)pv;
    }
    out->corner_he = (uint32_t*)malloc(4 * (o ? o : 1));
    o = 0;
    for (uint32_t i = 0; i < nf; ++i) {
        const std::vector<hd_t>& hs = m.get_halfedges_around_face(fd_t(i));
        for (size_t j = 0; j < hs.size(); ++j)
            out->corner_he[o + j] = (uint32_t)hs[j];
        o += hs.size();
    }
    out->v_off = (uint32_t*)calloc((size_t)nv + 1, 4);
    out->v_he = (uint32_t*)malloc(4 * (nh ? nh : 1));
    for (uint32_t v = 0; v < nv; ++v) {
        const std::vector<hd_t>& hs = m.get_halfedges_around_vertex(vd_t(v));
        out->v_off[v + 1] = out->v_off[v] + (uint32_t)hs.size();
        for (size_t j = 0; j < hs.size(); ++j)
            out->v_he[out->v_off[v] + j] = (uint32_t)hs[j];
    }
    out->closed = mesh_is_closed(m) ? 1 : 0;
    if (nv < 3 || nf < 1) {
        out->status = HM_TOO_SMALL;
        return 0;
    }
    thread_pool pool(1, 0);
    std::vector<int> fccmap, ccv, ccf;
    const int nc = find_connected_components(pool, fccmap, m, ccv, ccf);
    out->n_components = (uint32_t)nc;
    if (nc != 1)
        out->status = HM_COMPONENTS;
    return 0;
}

extern "C" void ref_hmesh_free(hm_result* r)
{
    free(r->he_target);
    free(r->he_face);
    free(r->he_next);
    free(r->he_prev);
    free(r->corner_he);
    free(r->v_off);
    free(r->v_he);
    memset(r, 0, sizeof(*r));
}
