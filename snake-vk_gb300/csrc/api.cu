// api.cu -- the C ABI of include/snk_pt.h: context, scene upload, acceleration
// structure builds, frame dispatch and the per-ray test hook.
//
// Reference boundary: class RT (Core/headers/rendering/Raytracing.h:11-31),
// RT::Init / RT::RecordRenderCmdBuf (Core/src/rendering/Raytracing.cpp:227-278)
// and the scene buffer systems that fill its descriptor table
// (Core/src/rendering/Raytracing.cpp:72-145).
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <string>
#include <vector>

#include "../../include/snk_pt.h"
#include "snk_frame.h"
#include "snk_host.h"
#include "snk_mlp.h"
#include "snk_particles.h"

using namespace snk;

struct HostMesh {
    std::vector<float> pos, nrm;
    std::vector<uint32_t> idx;
    uint32_t nv = 0, nt = 0;
    bool has_normals = false;
};

// Host copy of the last bytes uploaded into a device buffer, so that per-frame
// scene updates skip re-uploading tables that did not change.
struct UploadMemo {
    std::vector<unsigned char> bytes;
    const void* dev = nullptr;
};

struct RestirState {
    uint32_t w = 0, h = 0;
    DBuf<float4> g_pos, g_normal, g_albedo, g_misc, prev_normal;
    DBuf<float4> res_a, res_b, res_c;   // temporal, history, spatial (48 B = 3 float4 per pixel)
    DBuf<float4> ris;                    // initial-pass state between its recording and replaying runs
    DBuf<uint4> memo_keys;               // initial-pass visibility tests reused by the spatial pass
    DBuf<uint32_t> plan;                 // final-shading answers, spatial phase 1 -> 2
    DBuf<float4> combo;                  // combine targets between the recording and replaying runs
    uint32_t history_valid = 0;
    uint32_t hist = 1, spat = 2;        // which of b/c holds history / receives spatial
};

struct snk_pt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    int num_sms = 1;
    std::string err;

    // host-side scene
    std::vector<HostMesh> meshes;
    std::vector<snk_instance> instances;
    std::vector<snk_material> materials;
    snk_directional_light dir_light{};
    std::vector<snk_point_light> point_lights;
    bool meshes_dirty = true, inst_dirty = true, mats_dirty = true, lights_dirty = true;
    bool built = false;

    // device scene
    DBuf<float> d_pos, d_nrm;
    DBuf<uint32_t> d_idx;
    std::vector<MeshInfo> h_meshes;
    DBuf<MeshInfo> d_meshes;
    DBuf<WideNode> d_blas;
    DBuf<TriRecord> d_tris;
    DBuf<WideNode> d_tlas;
    DBuf<uint32_t> d_tlas_prims;
    uint32_t tlas_root = INVALID;
    uint64_t blas_nodes = 0, tlas_nodes = 0, total_tris = 0, tlas_prim_count = 0;
    double blas_sah = 0.0;
    bool blas_leaf_single = true;      // the mesh BVHs were built with one primitive per leaf
    bool tlas_leaf_single = true;      // the instance BVH was built with one instance per leaf
    DBuf<InstTrace> d_inst_trace;
    DBuf<InstShade> d_inst_shade;
    DBuf<MaterialDev> d_mats;
    DBuf<PointLightDev> d_pls;
    DBuf<uint32_t> d_emissive;
    DBuf<snk_instance> d_inst_raw;     // the caller's instance records, as given
    DBuf<uint32_t> d_em_first;         // first NEE record of each emissive instance's triangles
    DBuf<EmissiveRec> d_em_recs;       // ReSTIR candidate record of each emissive instance
    DBuf<LocalLight> d_lights;
    DBuf<double> d_light_w;            // selection weight of every NEE record
    DBuf<float> d_cdf, d_pmf;
    LightCdfScratch cdf_scratch;
    bool inst_tables_valid = false;    // instance and NEE records match the uploaded inputs
    bool lights_changed = true;        // point lights or materials changed since the NEE records
    uint32_t n_emissive = 0, n_local = 0;
    DBuf<unsigned> d_err;
    DBuf<unsigned char> q_in, q_in2, q_out, q_out2;   // staging of the particle / contact queries
    DBuf<float4> rq_rays;                              // ReSTIR visibility queue (slots x pixels x 2)
    DBuf<uint8_t> rq_vis_a, rq_vis_b;                  // its results (initial / shading, spatial)
    DBuf<uint32_t> rq_work;                            // work counters of the three visibility traces
    UploadMemo memo[7];                // raw instances, emissive firsts, emissive list, -, -, -, BVH list
    DBuf<SmallBuildOut> d_small_out;   // result record of the single-launch instance BVH build
    bool tlas_small = false;           // built by the single-launch builder (<= 1024 instances)
    bool tlas_refittable = false;      // the last build left the record, depths and order a refit needs
    // instance BVH refit state: exact node boxes and depths, primitive order and
    // the mesh of every listed instance at the last full build
    DBuf<float4> d_tlas_box;
    DBuf<uint32_t> d_tlas_depth, d_tlas_order;
    std::vector<uint32_t> tlas_meshes;
    uint32_t tlas_updates_since_build = 0;
    uint64_t tlas_builds = 0, tlas_refits = 0;

    BuildScratch scratch;
    DBuf<float4> d_box_lo, d_box_hi;
    DBuf<uint32_t> d_prim_order, d_inst_list;

    // frame buffers
    DBuf<float4> rays0, rays1, beta, L, srays, scontrib;
    DBuf<uint32_t> pid0, pid1, counters;
    DBuf<HitDev> hits;
    DBuf<unsigned long long> trav;
    DBuf<ViewDev> d_views;
    std::map<uint64_t, DBuf<unsigned char>> staging;
    uint32_t* h_counters = nullptr;          // pinned copy of the last frame's counters
    // pinned copies, made at the end of each render, of the device error word and
    // the instance BVH's build record (read by snk_pt_get_stats without a copy)
    unsigned* h_err = nullptr;
    SmallBuildOut* h_small = nullptr;
    bool aux_pending = false;
    unsigned long long* h_trav = nullptr;    // pinned copy of traversal counters
    bool counters_pending = false;
    uint32_t last_mode = 0, last_depth = 0, last_count_nodes = 0;
    uint64_t last_paths = 0, last_pixels = 0;

    std::vector<RestirState> restir;
    DBuf<float4> indirect;             // SNK_MODE_RESTIR_PT: per-pixel path-traced indirect light
    DBuf<double2> accum;
    uint32_t accum_w = 0, accum_h = 0;
    uint64_t accum_frames = 0;

    DBuf<float4> tr_rays;
    DBuf<HitDev> tr_hits;
    DBuf<uint32_t> tr_work;

    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timing_pending = false;
    double last_ms = 0.0;

    // per-launch profiling (SNK_RENDER_PROFILE): event pairs and their stage
    std::vector<cudaEvent_t> prof_ev;
    struct ProfInterval { uint32_t begin, end; int stage; };
    std::vector<ProfInterval> prof_iv;   // stage timings of the last profiled frame (event indices)
    size_t prof_used = 0;
    bool prof_pending = false;
    bool prof_chain = false;   // the last recorded event ended a stage and nothing was enqueued since
    cudaStream_t prof_stream = nullptr;   // the stream of that event
    cudaStream_t side = nullptr;          // second wavefront stream (shadow rays)
    cudaEvent_t ev_fork[MAX_DEPTH] = {}, ev_join[MAX_DEPTH] = {};
    double stage_ms[SNK_NUM_STAGES] = {0};
    uint64_t stage_launches[SNK_NUM_STAGES] = {0};

    snk_tuning tune{};   // launch knobs (zero = defaults)
    cudaGraphExec_t graph_exec = nullptr;   // replayed frame (SNK_RENDER_USE_GRAPH)
    std::vector<unsigned char> graph_key;   // what the captured launches bake in
    uint64_t graph_launches = 0, graph_captures = 0;
    uint64_t graph_stage_launches[SNK_NUM_STAGES] = {0};   // kernel launches per stage of the captured frame
    DBuf<uint32_t> d_dyn;                   // per-frame seed, frame index, accumulate flag

    // MLP radiance cache
    MlpState mlp;
    EncodeParams cache_ep{};
    bool cache_bounds_set = false;
    float scene_lo[3] = {0, 0, 0}, scene_hi[3] = {1, 1, 1};
    bool scene_bounds_dirty = true;    // recomputed on the host when the cache needs them
    DBuf<float4> cache_in;
    DBuf<float> cache_out, cache_grad;
    DBuf<float2> c_spread;
    DBuf<float4> c_qrec, c_qbeta, c_trec, c_tbeta, c_tL, c_samples;
    uint64_t last_cache_samples = 0;
    // quality guard of the cache (snk_pt_cache_set_guard; check_every 0: off)
    snk_cache_guard guard{};
    uint64_t guard_frames = 0, guard_probes = 0, guard_fallback_frames = 0;
    double guard_last = -1.0;
    bool guard_fallback = false;
};

namespace {

EncodeParams cache_encode_params(snk_pt_ctx* ctx);
Status cache_ensure(snk_pt_ctx* ctx);

int fail(snk_pt_ctx* c, int code, const std::string& msg) {
    if (c) c->err = msg;
    return code;
}
int fail(snk_pt_ctx* c, const Status& s) { return fail(c, s.code, s.msg); }

#define API_TRY(expr)                          \
    do {                                       \
        Status s__ = (expr);                   \
        if (!s__.ok()) return fail(ctx, s__);  \
    } while (0)

Status set_device(snk_pt_ctx* ctx) {
    SNK_TRY_CUDA(cudaSetDevice(ctx->device));
    return Status::Ok();
}

template <class T>
Status upload(DBuf<T>& b, const T* src, size_t n, cudaStream_t s);

template <class T>
Status upload_changed(DBuf<T>& b, UploadMemo& memo, const T* src, size_t n, cudaStream_t s, bool* changed = nullptr) {
    const size_t bytes = n * sizeof(T);
    if (changed) *changed = false;
    if (b.p && memo.dev == b.p && memo.bytes.size() == bytes && (bytes == 0 || !std::memcmp(memo.bytes.data(), src, bytes)))
        return Status::Ok();
    if (changed) *changed = true;
    SNK_TRY(upload(b, src, n, s));
    memo.bytes.assign(reinterpret_cast<const unsigned char*>(src), reinterpret_cast<const unsigned char*>(src) + bytes);
    memo.dev = b.p;
    return Status::Ok();
}

template <class T>
Status upload(DBuf<T>& b, const T* src, size_t n, cudaStream_t s) {
    SNK_TRY_CUDA(b.reserve(n ? n : 1));
    if (n) SNK_TRY_CUDA(cudaMemcpyAsync(b.p, src, n * sizeof(T), cudaMemcpyHostToDevice, s));
    return Status::Ok();
}

uint32_t leaf_size(uint32_t knob, uint32_t dflt) { return knob ? knob : dflt; }

int treelet_passes(uint32_t knob, int dflt) {
    return knob == SNK_TREELET_PASSES_NONE ? 0 : (knob ? (int)knob : dflt);
}

Status build_meshes(snk_pt_ctx* ctx) {
    cudaStream_t st = ctx->stream;
    size_t nv = 0, ni = 0, nt = 0;
    ctx->h_meshes.assign(ctx->meshes.size(), MeshInfo{});
    for (size_t m = 0; m < ctx->meshes.size(); m++) {
        MeshInfo& mi = ctx->h_meshes[m];
        mi.vertex_offset = (uint32_t)nv;
        mi.index_offset = (uint32_t)ni;
        mi.num_triangles = ctx->meshes[m].nt;
        mi.has_normals = ctx->meshes[m].has_normals ? 1u : 0u;
        mi.blas_root = INVALID;
        nv += ctx->meshes[m].nv;
        ni += 3ull * ctx->meshes[m].nt;
        nt += ctx->meshes[m].nt;
    }
    if (nv > 0xFFFFFFFFull || ni > 0xFFFFFFFFull) return Status::Err(SNK_ERR_INVALID_ARG, "scene too large");
    std::vector<float> pos(3 * nv), nrm(3 * nv, 0.0f);
    std::vector<uint32_t> idx(ni);
    for (size_t m = 0; m < ctx->meshes.size(); m++) {
        const HostMesh& H = ctx->meshes[m];
        const MeshInfo& mi = ctx->h_meshes[m];
        std::memcpy(&pos[3ull * mi.vertex_offset], H.pos.data(), H.pos.size() * sizeof(float));
        if (H.has_normals) std::memcpy(&nrm[3ull * mi.vertex_offset], H.nrm.data(), H.nrm.size() * sizeof(float));
        std::memcpy(&idx[mi.index_offset], H.idx.data(), H.idx.size() * sizeof(uint32_t));
    }
    SNK_TRY(upload(ctx->d_pos, pos.data(), pos.size(), st));
    SNK_TRY(upload(ctx->d_nrm, nrm.data(), nrm.size(), st));
    SNK_TRY(upload(ctx->d_idx, idx.data(), idx.size(), st));
    size_t max_nt = 1;
    for (auto& H : ctx->meshes) max_nt = std::max<size_t>(max_nt, H.nt);
    SNK_TRY_CUDA(ctx->d_box_lo.reserve(max_nt));
    SNK_TRY_CUDA(ctx->d_box_hi.reserve(max_nt));
    SNK_TRY_CUDA(ctx->d_prim_order.reserve(max_nt));
    SNK_TRY_CUDA(ctx->d_blas.reserve(nt + ctx->meshes.size() + 1));
    SNK_TRY_CUDA(ctx->d_tris.reserve(nt ? nt : 1));
    uint32_t node_base = 0, prim_base = 0;
    double sah_sum = 0.0, sah_w = 0.0;
    for (size_t m = 0; m < ctx->meshes.size(); m++) {
        MeshInfo& mi = ctx->h_meshes[m];
        if (mi.num_triangles == 0) continue;
        SNK_TRY(launch_triangle_boxes(ctx->d_pos.p, ctx->d_idx.p, mi.vertex_offset, mi.index_offset, mi.num_triangles,
                                      ctx->d_box_lo.p, ctx->d_box_hi.p, st));
        BuildResult br;
        SNK_TRY(build_wide_bvh(ctx->scratch, ctx->d_box_lo.p, ctx->d_box_hi.p, mi.num_triangles, ctx->d_blas.p,
                               node_base, prim_base, ctx->d_prim_order.p, st, &br,
                               treelet_passes(ctx->tune.bvh_treelet_passes, 3), leaf_size(ctx->tune.bvh_leaf_max, 1),
                               std::max(leaf_size(ctx->tune.bvh_leaf_pack, 1), leaf_size(ctx->tune.bvh_leaf_max, 1)),
                               ctx->tune.bvh_collapse == 0));
        SNK_TRY(launch_fill_triangles(ctx->d_prim_order.p, mi.num_triangles, ctx->d_pos.p, ctx->d_idx.p,
                                      mi.vertex_offset, mi.index_offset, ctx->d_tris.p + prim_base, st));
        mi.blas_root = node_base;
        for (int a = 0; a < 3; a++) { mi.lo[a] = br.lo[a]; mi.hi[a] = br.hi[a]; }
        node_base += br.num_nodes;
        prim_base += mi.num_triangles;
        sah_sum += br.sah * mi.num_triangles;
        sah_w += mi.num_triangles;
    }
    ctx->blas_nodes = node_base;
    ctx->total_tris = prim_base;
    ctx->blas_leaf_single = leaf_size(ctx->tune.bvh_leaf_max, 1) == 1 && leaf_size(ctx->tune.bvh_leaf_pack, 1) <= 1;
    ctx->blas_sah = sah_w > 0 ? sah_sum / sah_w : 0.0;
    SNK_TRY(upload(ctx->d_meshes, ctx->h_meshes.data(), ctx->h_meshes.size(), st));
    SNK_TRY_CUDA(cudaStreamSynchronize(st));
    return Status::Ok();
}

// World bounds of the listed instances (positions of the radiance cache are
// normalised to them); computed on the host when the cache asks for them.
void update_scene_bounds(snk_pt_ctx* ctx) {
    if (!ctx->scene_bounds_dirty) return;
    double lo[3] = {1e300, 1e300, 1e300}, hi[3] = {-1e300, -1e300, -1e300};
    bool any = false;
    for (const snk_instance& in : ctx->instances) {
        if (in.mesh_id >= ctx->h_meshes.size()) continue;
        const MeshInfo& M = ctx->h_meshes[in.mesh_id];
        if (M.blas_root == INVALID) continue;
        any = true;
        for (int c = 0; c < 8; c++) {
            double p[3] = {(c & 1) ? M.hi[0] : M.lo[0], (c & 2) ? M.hi[1] : M.lo[1], (c & 4) ? M.hi[2] : M.lo[2]};
            for (int r = 0; r < 3; r++) {
                double v = in.transform[4 * r] * p[0] + in.transform[4 * r + 1] * p[1] + in.transform[4 * r + 2] * p[2] +
                           in.transform[4 * r + 3];
                lo[r] = std::min(lo[r], v);
                hi[r] = std::max(hi[r], v);
            }
        }
    }
    for (int r = 0; r < 3; r++) {
        ctx->scene_lo[r] = any ? (float)lo[r] : 0.0f;
        ctx->scene_hi[r] = any ? (float)hi[r] : 1.0f;
    }
    ctx->scene_bounds_dirty = false;
}

Status build_instances(snk_pt_ctx* ctx) {
    cudaStream_t st = ctx->stream;
    const size_t ni = ctx->instances.size();
    // host: index checks and the two instance lists (instances of empty meshes have
    // no triangle to hit or sample and are left out of both)
    std::vector<uint32_t> list, emissive, em_first;
    list.reserve(ni);
    uint64_t n_em_tris = 0;
    for (size_t i = 0; i < ni; i++) {
        const snk_instance& in = ctx->instances[i];
        if (in.mesh_id >= ctx->meshes.size()) return Status::Err(SNK_ERR_INVALID_ARG, "instance mesh_id out of range");
        if (in.material_id >= ctx->materials.size())
            return Status::Err(SNK_ERR_INVALID_ARG, "instance material_id out of range");
        const MeshInfo& M = ctx->h_meshes[in.mesh_id];
        if (M.blas_root == INVALID) continue;
        list.push_back((uint32_t)i);
        if (ctx->materials[in.material_id].flags & SNK_MAT_EMISSIVE) {
            emissive.push_back((uint32_t)i);
            em_first.push_back((uint32_t)n_em_tris);
            n_em_tris += M.num_triangles;
        }
    }
    ctx->scene_bounds_dirty = true;

    // path-tracer local lights: sphere lights (host, few), then every emissive
    // triangle (device), selected in proportion to emitted power
    std::vector<LocalLight> spheres;
    std::vector<double> sw;
    for (size_t k = 0; k < ctx->point_lights.size(); k++) {
        const snk_point_light& P = ctx->point_lights[k];
        if (!(P.radius > 0.0f)) continue;
        LocalLight L{};
        L.kind = 0;
        L.index = (uint32_t)k;
        L.p0[0] = P.pos[0]; L.p0[1] = P.pos[1]; L.p0[2] = P.pos[2];
        L.p1[0] = P.radius;
        double inv_area = 1.0 / (M_PI * (double)P.radius * (double)P.radius);
        L.L[0] = (float)(P.colour[0] * inv_area);
        L.L[1] = (float)(P.colour[1] * inv_area);
        L.L[2] = (float)(P.colour[2] * inv_area);
        spheres.push_back(L);
        sw.push_back(4.0 * M_PI * (0.2126 * P.colour[0] + 0.7152 * P.colour[1] + 0.0722 * P.colour[2]));
    }
    const uint64_t n_lights = spheres.size() + n_em_tris;
    if (n_lights > 0x7FFFFFFFull) return Status::Err(SNK_ERR_INVALID_ARG, "too many emissive triangles");

    // device: instance records and NEE records, redone when their inputs changed
    bool raw_changed = false, em_changed = false, first_changed = false;
    SNK_TRY(upload_changed(ctx->d_inst_raw, ctx->memo[0], ctx->instances.data(), ni, st, &raw_changed));
    SNK_TRY(upload_changed(ctx->d_emissive, ctx->memo[2], emissive.data(), emissive.size(), st, &em_changed));
    SNK_TRY(upload_changed(ctx->d_em_first, ctx->memo[1], em_first.data(), em_first.size(), st, &first_changed));
    ctx->n_emissive = (uint32_t)emissive.size();
    const bool redo = raw_changed || em_changed || first_changed || !ctx->inst_tables_valid;
    ctx->inst_tables_valid = false;
    if (redo) {
        SNK_TRY_CUDA(ctx->d_inst_trace.reserve(ni));
        SNK_TRY_CUDA(ctx->d_inst_shade.reserve(ni));
        SNK_TRY(launch_instance_records(ctx->d_inst_raw.p, (uint32_t)ni, ctx->d_meshes.p, ctx->d_inst_trace.p,
                                        ctx->d_inst_shade.p, st));
        SNK_TRY_CUDA(ctx->d_em_recs.reserve(emissive.size()));
        SNK_TRY(launch_emissive_records(ctx->d_emissive.p, (uint32_t)emissive.size(), ctx->d_inst_shade.p,
                                        ctx->d_meshes.p, ctx->d_mats.p, ctx->d_em_recs.p, st));
    }
    SNK_TRY_CUDA(ctx->d_lights.reserve(n_lights));
    SNK_TRY_CUDA(ctx->d_cdf.reserve(n_lights));
    SNK_TRY_CUDA(ctx->d_pmf.reserve(n_lights));
    if (n_em_tris == 0) {
        // sphere lights only: the whole table is known here (nothing to launch)
        std::vector<float> cdf(sw.size()), pmf(sw.size());
        light_cdf_host(sw.data(), (uint32_t)sw.size(), cdf.data(), pmf.data());
        SNK_TRY(upload_changed(ctx->d_lights, ctx->memo[3], spheres.data(), spheres.size(), st));
        SNK_TRY(upload_changed(ctx->d_cdf, ctx->memo[4], cdf.data(), cdf.size(), st));
        SNK_TRY(upload_changed(ctx->d_pmf, ctx->memo[5], pmf.data(), pmf.size(), st));
    } else if (redo || ctx->lights_changed) {
        for (int k = 3; k <= 5; k++) ctx->memo[k] = UploadMemo{};
        SNK_TRY_CUDA(ctx->d_light_w.reserve(n_lights));
        if (!spheres.empty()) {
            SNK_TRY_CUDA(cudaMemcpyAsync(ctx->d_lights.p, spheres.data(), spheres.size() * sizeof(LocalLight),
                                         cudaMemcpyHostToDevice, st));
            SNK_TRY_CUDA(
                cudaMemcpyAsync(ctx->d_light_w.p, sw.data(), sw.size() * sizeof(double), cudaMemcpyHostToDevice, st));
        }
        SNK_TRY(launch_emissive_lights(ctx->d_inst_raw.p, ctx->d_emissive.p, ctx->d_em_first.p,
                                       (uint32_t)emissive.size(), (uint32_t)n_em_tris, ctx->d_meshes.p, ctx->d_pos.p,
                                       ctx->d_idx.p, ctx->d_mats.p, ctx->d_lights.p + spheres.size(),
                                       ctx->d_light_w.p + spheres.size(), st));
        SNK_TRY(launch_light_cdf(ctx->d_light_w.p, (uint32_t)n_lights, ctx->cdf_scratch, ctx->d_cdf.p, ctx->d_pmf.p, st));
    }
    ctx->lights_changed = false;
    ctx->inst_tables_valid = true;
    // (a table whose weights are all zero has pmf 0 everywhere: no record is ever used)
    ctx->n_local = (uint32_t)n_lights;

    // instance BVH (rebuilt whenever instances change, as TlasSystem::BuildTlas,
    // or refitted when the tuning asks for it and the topology allows it)
    const uint32_t prev_root = ctx->tlas_root;
    const uint64_t prev_prims = ctx->tlas_prim_count;
    ctx->tlas_root = INVALID;
    ctx->tlas_nodes = 0;
    ctx->tlas_prim_count = 0;
    const uint32_t n = (uint32_t)list.size();
    if (n > 0) {
        SNK_TRY(upload_changed(ctx->d_inst_list, ctx->memo[6], list.data(), list.size(), st));
        SNK_TRY_CUDA(ctx->d_box_lo.reserve(n));
        SNK_TRY_CUDA(ctx->d_box_hi.reserve(n));
        SNK_TRY_CUDA(ctx->d_prim_order.reserve(n));
        SNK_TRY_CUDA(ctx->d_tlas.reserve(n + 1));
        SNK_TRY_CUDA(ctx->d_tlas_prims.reserve(n));
        SNK_TRY(launch_instance_boxes(ctx->d_inst_list.p, n, ctx->d_inst_shade.p, ctx->d_meshes.p, ctx->d_box_lo.p,
                                      ctx->d_box_hi.p, st));
        const int passes = treelet_passes(ctx->tune.tlas_treelet_passes, 0);
        std::vector<uint32_t> meshes_now(n);
        for (uint32_t k = 0; k < n; k++) meshes_now[k] = ctx->instances[list[k]].mesh_id;
        const uint32_t interval = ctx->tune.tlas_refit_interval;
        const bool refit = interval > 0 && ctx->tlas_refittable && prev_root != INVALID && prev_prims == n &&
                           meshes_now == ctx->tlas_meshes && ctx->tlas_updates_since_build + 1 < interval;
        if (refit) {
            // same instances on the same meshes: new boxes into the existing tree
            SNK_TRY(refit_wide_bvh(ctx->d_box_lo.p, ctx->d_box_hi.p, n, ctx->d_tlas.p, 0u, 0u, ctx->d_tlas_order.p,
                                   ctx->d_small_out.p, ctx->d_tlas_box.p, ctx->d_tlas_depth.p, ctx->d_err.p, st));
            ctx->tlas_updates_since_build++;
            ctx->tlas_refits++;
            ctx->tlas_root = prev_root;   // the primitive map and counts are unchanged
            ctx->tlas_nodes = n + 1;
            ctx->tlas_prim_count = n;
            return Status::Ok();
        }
        // the refit state of either builder: build record, node depths, primitive order
        SNK_TRY_CUDA(ctx->d_small_out.reserve(1));
        SNK_TRY_CUDA(ctx->d_tlas_box.reserve(2ull * (n + 1)));
        SNK_TRY_CUDA(ctx->d_tlas_depth.reserve(n + 1));
        SNK_TRY_CUDA(ctx->d_tlas_order.reserve(n));
        ctx->tlas_meshes = meshes_now;
        ctx->tlas_updates_since_build = 0;
        ctx->tlas_refittable = true;
        ctx->tlas_leaf_single = leaf_size(ctx->tune.tlas_leaf_max, 1) == 1;
        if (n <= (uint32_t)SMALL_BUILD_MAX) {
            // one launch, no host round trip; the node count stays on the device
            // (traversal bounds its node indices by the capacity, n + 1)
            SNK_TRY(build_wide_bvh_small(ctx->d_box_lo.p, ctx->d_box_hi.p, n, ctx->d_tlas.p, 0u, 0u,
                                         ctx->d_tlas_order.p, passes, ctx->d_small_out.p, ctx->d_err.p,
                                         ctx->d_tlas_box.p, ctx->d_tlas_depth.p, st,
                                         leaf_size(ctx->tune.tlas_leaf_max, 1), ctx->tune.bvh_collapse == 0));
            SNK_TRY(launch_map_prims(ctx->d_tlas_order.p, ctx->d_inst_list.p, n, ctx->d_tlas_prims.p, st));
            ctx->tlas_nodes = n + 1;
            ctx->tlas_small = true;
            ctx->tlas_builds++;
            ctx->tlas_root = 0;
            ctx->tlas_prim_count = n;
            return Status::Ok();
        } else {
            // multi-launch build, also without a host round trip (node count bounded by n + 1)
            SNK_TRY(build_wide_bvh_device(ctx->scratch, ctx->d_box_lo.p, ctx->d_box_hi.p, n, ctx->d_tlas.p, 0u, 0u,
                                          ctx->d_tlas_order.p, ctx->d_err.p, st, passes,
                                          leaf_size(ctx->tune.tlas_leaf_max, 1), leaf_size(ctx->tune.tlas_leaf_max, 1),
                                          ctx->d_small_out.p, ctx->d_tlas_depth.p, ctx->tune.bvh_collapse == 0));
            ctx->tlas_nodes = n + 1;
            ctx->tlas_small = false;
            ctx->tlas_builds++;
        }
        SNK_TRY(launch_map_prims(ctx->d_tlas_order.p, ctx->d_inst_list.p, n, ctx->d_tlas_prims.p, st));
        ctx->tlas_root = 0;
        ctx->tlas_prim_count = n;
    }
    return Status::Ok();
}

Status build_all(snk_pt_ctx* ctx) {
    SNK_TRY(set_device(ctx));
    if (ctx->meshes_dirty) {
        SNK_TRY(build_meshes(ctx));
        ctx->meshes_dirty = false;
        ctx->inst_dirty = true;
        ctx->inst_tables_valid = false;
    }
    if (ctx->mats_dirty) {
        std::vector<MaterialDev> m(ctx->materials.size());
        static_assert(sizeof(MaterialDev) == sizeof(snk_material), "material layout");
        std::memcpy(m.data(), ctx->materials.data(), m.size() * sizeof(MaterialDev));
        SNK_TRY(upload(ctx->d_mats, m.data(), m.size(), ctx->stream));
        ctx->mats_dirty = false;
        ctx->inst_dirty = true;
        ctx->inst_tables_valid = false;
    }
    if (ctx->lights_dirty) {
        static_assert(sizeof(PointLightDev) == sizeof(snk_point_light), "point light layout");
        SNK_TRY(upload(ctx->d_pls, reinterpret_cast<const PointLightDev*>(ctx->point_lights.data()),
                       ctx->point_lights.size(), ctx->stream));
        ctx->lights_dirty = false;
        ctx->inst_dirty = true;
        ctx->lights_changed = true;
    }
    if (ctx->inst_dirty) {
        SNK_TRY(build_instances(ctx));
        ctx->inst_dirty = false;
    }
    SNK_TRY_CUDA(ctx->d_err.reserve(1));
    ctx->built = true;
    return Status::Ok();
}

SceneDev scene_dev(snk_pt_ctx* ctx) {
    SceneDev S;
    std::memset(&S, 0, sizeof(S));
    S.blas_nodes = ctx->d_blas.p;
    S.tris = ctx->d_tris.p;
    S.tlas_nodes = ctx->d_tlas.p;
    S.tlas_prims = ctx->d_tlas_prims.p;
    S.tlas_root = ctx->tlas_root;
    S.num_instances = (uint32_t)ctx->instances.size();
    S.inst_trace = ctx->d_inst_trace.p;
    S.inst_shade = ctx->d_inst_shade.p;
    S.meshes = ctx->d_meshes.p;
    S.positions = ctx->d_pos.p;
    S.normals = ctx->d_nrm.p;
    S.indices = ctx->d_idx.p;
    S.materials = ctx->d_mats.p;
    S.point_lights = ctx->d_pls.p;
    S.num_point_lights = (uint32_t)ctx->point_lights.size();
    S.num_emissive_instances = ctx->n_emissive;
    S.emissive_instances = ctx->d_emissive.p;
    S.emissive_recs = ctx->d_em_recs.p;
    S.local_lights = ctx->d_lights.p;
    S.light_cdf = ctx->d_cdf.p;
    S.light_pmf = ctx->d_pmf.p;
    S.num_local_lights = ctx->n_local;
    S.single_leaf = ctx->blas_leaf_single && ctx->tlas_leaf_single ? 1u : 0u;
    std::memcpy(&S.dir_light, &ctx->dir_light, sizeof(S.dir_light));
    S.error_word = ctx->d_err.p;
    S.num_blas_nodes = (uint32_t)ctx->blas_nodes;
    S.num_tris = (uint32_t)ctx->total_tris;
    S.num_tlas_nodes = (uint32_t)ctx->tlas_nodes;
    S.num_tlas_prims = ctx->tlas_root == INVALID ? 0u : (uint32_t)ctx->tlas_prim_count;
    S.max_steps = ctx->tune.max_traversal_steps ? ctx->tune.max_traversal_steps : MAX_TRAVERSAL_STEPS;
    S.stack_max = ctx->tune.stack_limit ? (int)ctx->tune.stack_limit : STACK_MAX;
    return S;
}

Status ensure_built(snk_pt_ctx* ctx) {
    if (ctx->meshes_dirty || ctx->inst_dirty || ctx->mats_dirty || ctx->lights_dirty || !ctx->built)
        return build_all(ctx);
    return Status::Ok();
}

Status check_device_error(snk_pt_ctx* ctx) {
    unsigned e = 0;
    SNK_TRY_CUDA(cudaMemcpyAsync(&e, ctx->d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, ctx->stream));
    SNK_TRY_CUDA(cudaStreamSynchronize(ctx->stream));
    if (e) {
        SNK_TRY_CUDA(cudaMemsetAsync(ctx->d_err.p, 0, sizeof(unsigned), ctx->stream));
        return Status::Err(SNK_ERR_LIMIT, std::string("device traversal bound hit (error word ") + std::to_string(e) +
                                              "): bit 1 stack depth, bit 2 step limit, bit 4 bad index, bit 8 instance BVH build, "
                                              "bit 16 tensor-core wait, bit 32 its drain wait");
    }
    return Status::Ok();
}

float* stage(snk_pt_ctx* ctx, uint32_t view, uint32_t kind, size_t bytes, Status* st) {
    DBuf<unsigned char>& b = ctx->staging[((uint64_t)view << 8) | kind];
    cudaError_t e = b.reserve(bytes);
    if (e != cudaSuccess) { *st = Status::Err(SNK_ERR_OUT_OF_MEMORY, "staging allocation failed"); return nullptr; }
    return reinterpret_cast<float*>(b.p);
}

constexpr int NUM_OUT = 10;
// element sizes of the outputs in snk_view_outputs order
const size_t OUT_BYTES[NUM_OUT] = {16, 16, 16, 16, 16, 8, 4, 4, 4, 4};

void** out_slots(snk_view_outputs& o) { return reinterpret_cast<void**>(&o); }
void** dev_slots(ViewDev& v) { return reinterpret_cast<void**>(&v.radiance); }

int grid_of(snk_pt_ctx* ctx, int per_sm) { return ctx->num_sms * per_sm; }
int trace_grid(snk_pt_ctx* ctx) { return grid_of(ctx, ctx->tune.trace_blocks_per_sm ? (int)ctx->tune.trace_blocks_per_sm : 16); }
int shade_grid(snk_pt_ctx* ctx) { return grid_of(ctx, ctx->tune.shade_blocks_per_sm ? (int)ctx->tune.shade_blocks_per_sm : 8); }
// any-hit traversal grid (shadow and visibility rays): its own knob, else the closest-hit one
int any_grid(snk_pt_ctx* ctx) {
    return ctx->tune.shadow_blocks_per_sm ? grid_of(ctx, (int)ctx->tune.shadow_blocks_per_sm) : trace_grid(ctx);
}
TraceTuning trace_tuning(snk_pt_ctx* ctx) {
    TraceTuning t;
    t.chunk = ctx->tune.ray_chunk;
    t.refill_idle = ctx->tune.refill_idle;
    t.prim_bias = ctx->tune.prim_bias;
    t.variant = ctx->tune.trace_variant;
    return t;
}
// knobs of the any-hit kernels: each falls back to the closest-hit knob when 0
TraceTuning any_tuning(snk_pt_ctx* ctx) {
    TraceTuning t = trace_tuning(ctx);
    const snk_tuning& k = ctx->tune;
    if (k.shadow_ray_chunk) t.chunk = k.shadow_ray_chunk;
    if (k.shadow_refill_idle) t.refill_idle = k.shadow_refill_idle;
    if (k.shadow_prim_bias) t.prim_bias = k.shadow_prim_bias;
    if (k.shadow_variant) t.variant = k.shadow_variant - 1u;
    return t;
}

// Runs one stage's launches; when profiling, CUDA events bracket them on the stream
// they are issued to (the context's stream unless given).  Stages enqueued back to
// back on one stream share the event between them (the end of one is the start of
// the next), so a profiled frame records about one event per stage boundary.
template <class Fn>
cudaError_t staged(snk_pt_ctx* ctx, bool profile, int stage, Fn&& fn, cudaStream_t stream = nullptr) {
    ctx->stage_launches[stage]++;
    if (!profile) return fn();
    if (!stream) stream = ctx->stream;
    if (ctx->prof_used + 2 > ctx->prof_ev.size()) {
        for (int k = 0; k < 16; k++) {
            cudaEvent_t e;
            cudaError_t r = cudaEventCreate(&e);
            if (r != cudaSuccess) return r;
            ctx->prof_ev.push_back(e);
        }
    }
    uint32_t b;
    if (ctx->prof_chain && ctx->prof_used > 0 && ctx->prof_stream == stream) {
        b = (uint32_t)(ctx->prof_used - 1);
    } else {
        b = (uint32_t)ctx->prof_used++;
        cudaEventRecord(ctx->prof_ev[b], stream);
    }
    cudaError_t r = fn();
    const uint32_t e = (uint32_t)ctx->prof_used++;
    cudaEventRecord(ctx->prof_ev[e], stream);
    ctx->prof_iv.push_back({b, e, stage});
    ctx->prof_chain = true;
    ctx->prof_stream = stream;
    return r;
}

// The second stream of the wavefront (shadow rays of segment d traced while the
// closest hits of segment d + 1 are) and its fork / join events, made on first use.
cudaError_t ensure_side_stream(snk_pt_ctx* ctx) {
    if (ctx->side) return cudaSuccess;
    cudaError_t e = cudaStreamCreateWithFlags(&ctx->side, cudaStreamNonBlocking);
    for (uint32_t d = 0; d < MAX_DEPTH && e == cudaSuccess; d++) {
        e = cudaEventCreateWithFlags(&ctx->ev_fork[d], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ctx->ev_join[d], cudaEventDisableTiming);
    }
    return e;
}

}  // namespace

extern "C" {

int snk_pt_abi_version(uint32_t* version) {
    if (!version) return SNK_ERR_INVALID_ARG;
    *version = SNK_PT_ABI_VERSION;
    return SNK_OK;
}

int snk_pt_create(const snk_pt_config* config, snk_pt_ctx** out_ctx) {
    if (!out_ctx) return SNK_ERR_INVALID_ARG;
    *out_ctx = nullptr;
    snk_pt_ctx* ctx = new snk_pt_ctx();
    ctx->device = config ? config->device : 0;
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
        delete ctx;
        return SNK_ERR_CUDA;
    }
    if (ctx->device < 0 || ctx->device >= ndev) { delete ctx; return SNK_ERR_INVALID_ARG; }
    if (cudaSetDevice(ctx->device) != cudaSuccess) { delete ctx; return SNK_ERR_CUDA; }
    if (config && config->stream) {
        ctx->stream = (cudaStream_t)config->stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) { delete ctx; return SNK_ERR_CUDA; }
        ctx->own_stream = true;
    }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);
    if (cudaMallocHost(&ctx->h_counters, CNT_TOTAL * sizeof(uint32_t)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_trav, 4 * sizeof(unsigned long long)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_err, sizeof(unsigned)) != cudaSuccess ||
        cudaMallocHost(&ctx->h_small, sizeof(SmallBuildOut)) != cudaSuccess ||
        cudaEventCreate(&ctx->ev0) != cudaSuccess || cudaEventCreate(&ctx->ev1) != cudaSuccess ||
        ctx->d_err.reserve(1) != cudaSuccess || cudaMemset(ctx->d_err.p, 0, sizeof(unsigned)) != cudaSuccess) {
        snk_pt_destroy(ctx);
        return SNK_ERR_CUDA;
    }
    std::memset(ctx->h_counters, 0, CNT_TOTAL * sizeof(uint32_t));
    std::memset(ctx->h_trav, 0, 4 * sizeof(unsigned long long));
    *ctx->h_err = 0;
    std::memset(ctx->h_small, 0, sizeof(SmallBuildOut));
    *out_ctx = ctx;
    return SNK_OK;
}

int snk_pt_destroy(snk_pt_ctx* ctx) {
    if (!ctx) return SNK_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->h_counters) cudaFreeHost(ctx->h_counters);
    if (ctx->h_trav) cudaFreeHost(ctx->h_trav);
    if (ctx->h_err) cudaFreeHost(ctx->h_err);
    if (ctx->h_small) cudaFreeHost(ctx->h_small);
    if (ctx->ev0) cudaEventDestroy(ctx->ev0);
    if (ctx->ev1) cudaEventDestroy(ctx->ev1);
    for (cudaEvent_t e : ctx->prof_ev) cudaEventDestroy(e);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->side) cudaStreamSynchronize(ctx->side);
    for (uint32_t d = 0; d < MAX_DEPTH; d++) {
        if (ctx->ev_fork[d]) cudaEventDestroy(ctx->ev_fork[d]);
        if (ctx->ev_join[d]) cudaEventDestroy(ctx->ev_join[d]);
    }
    if (ctx->side) cudaStreamDestroy(ctx->side);
    cudaStream_t s = ctx->own_stream ? ctx->stream : nullptr;
    delete ctx;
    if (s) cudaStreamDestroy(s);
    return SNK_OK;
}

int snk_pt_set_stream(snk_pt_ctx* ctx, void* stream) {
    if (!ctx) return SNK_ERR_INVALID_ARG;
    cudaSetDevice(ctx->device);
    cudaStreamSynchronize(ctx->stream);
    if (ctx->own_stream) cudaStreamDestroy(ctx->stream);
    ctx->own_stream = false;
    if (stream) {
        ctx->stream = (cudaStream_t)stream;
    } else {
        if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess) return fail(ctx, SNK_ERR_CUDA, "stream");
        ctx->own_stream = true;
    }
    return SNK_OK;
}

int snk_pt_get_last_error(const snk_pt_ctx* ctx, char* buf, size_t len) {
    if (!ctx || !buf || len == 0) return SNK_ERR_INVALID_ARG;
    size_t n = std::min(len - 1, ctx->err.size());
    std::memcpy(buf, ctx->err.data(), n);
    buf[n] = 0;
    return SNK_OK;
}

int snk_pt_upload_meshes(snk_pt_ctx* ctx, const snk_mesh* meshes, uint32_t num_meshes) {
    if (!ctx || (num_meshes && !meshes)) return fail(ctx, SNK_ERR_INVALID_ARG, "upload_meshes: null argument");
    std::vector<HostMesh> hm(num_meshes);
    for (uint32_t m = 0; m < num_meshes; m++) {
        const snk_mesh& M = meshes[m];
        if ((M.num_vertices && !M.positions) || (M.num_triangles && !M.indices))
            return fail(ctx, SNK_ERR_INVALID_ARG, "upload_meshes: null mesh array");
        HostMesh& H = hm[m];
        H.nv = M.num_vertices;
        H.nt = M.num_triangles;
        H.pos.assign(M.positions, M.positions + 3ull * M.num_vertices);
        H.idx.assign(M.indices, M.indices + 3ull * M.num_triangles);
        for (uint32_t x : H.idx)
            if (x >= M.num_vertices) return fail(ctx, SNK_ERR_INVALID_ARG, "upload_meshes: index out of range");
        for (float f : H.pos)
            if (!std::isfinite(f)) return fail(ctx, SNK_ERR_INVALID_ARG, "upload_meshes: non-finite vertex position");
        if (M.normals) {
            H.has_normals = true;
            H.nrm.assign(M.normals, M.normals + 3ull * M.num_vertices);
        }
    }
    ctx->meshes.swap(hm);
    ctx->meshes_dirty = true;
    ctx->built = false;
    return SNK_OK;
}

int snk_pt_set_instances(snk_pt_ctx* ctx, const snk_instance* instances, uint32_t n) {
    if (!ctx || (n && !instances)) return fail(ctx, SNK_ERR_INVALID_ARG, "set_instances: null argument");
    for (uint32_t i = 0; i < n; i++)
        for (int k = 0; k < 12; k++)
            if (!std::isfinite(instances[i].transform[k]) || !std::isfinite(instances[i].prev_transform[k]))
                return fail(ctx, SNK_ERR_INVALID_ARG, "set_instances: non-finite transform");
    ctx->instances.assign(instances, instances + n);
    ctx->inst_dirty = true;
    return SNK_OK;
}

int snk_pt_set_materials(snk_pt_ctx* ctx, const snk_material* materials, uint32_t n) {
    if (!ctx || (n && !materials)) return fail(ctx, SNK_ERR_INVALID_ARG, "set_materials: null argument");
    ctx->materials.assign(materials, materials + n);
    ctx->mats_dirty = true;
    return SNK_OK;
}

int snk_pt_set_lights(snk_pt_ctx* ctx, const snk_directional_light* dl, const snk_point_light* pl, uint32_t n) {
    if (!ctx || (n && !pl)) return fail(ctx, SNK_ERR_INVALID_ARG, "set_lights: null argument");
    if (dl) ctx->dir_light = *dl;
    else std::memset(&ctx->dir_light, 0, sizeof(ctx->dir_light));
    ctx->point_lights.assign(pl, pl + n);
    ctx->lights_dirty = true;
    return SNK_OK;
}

int snk_pt_build(snk_pt_ctx* ctx) {
    if (!ctx) return SNK_ERR_INVALID_ARG;
    API_TRY(build_all(ctx));
    return SNK_OK;
}

}  // extern "C"

namespace {

// Error measure of the radiance-cache guard: the relative MSE, over block x block
// pixel means and the 3 channels, of the cached probe against the plain one:
// mean((c - p)^2 / (p^2 + 0.01)).  Block means divide the probes' own noise by the
// block area, so what remains is mostly the cache's bias.
double guard_relmse(const float* cached, const float* plain, uint32_t w, uint32_t h, uint32_t block) {
    const uint32_t b = std::max(1u, std::min(block, std::min(w, h)));
    const uint32_t bw = w / b, bh = h / b;
    double sum = 0.0;
    for (uint32_t by = 0; by < bh; by++)
        for (uint32_t bx = 0; bx < bw; bx++)
            for (int c = 0; c < 3; c++) {
                double mc = 0.0, mp = 0.0;
                for (uint32_t y = by * b; y < (by + 1) * b; y++)
                    for (uint32_t x = bx * b; x < (bx + 1) * b; x++) {
                        mc += cached[4 * ((size_t)y * w + x) + c];
                        mp += plain[4 * ((size_t)y * w + x) + c];
                    }
                mc /= (double)b * b;
                mp /= (double)b * b;
                sum += (mc - mp) * (mc - mp) / (mp * mp + 0.01);
            }
    return bw && bh ? sum / ((double)bw * bh * 3.0) : 0.0;
}

int render_impl(snk_pt_ctx* ctx, const snk_view* views, uint32_t num_views, const snk_render_settings* settings,
                const snk_view_outputs* outputs);

// The guard's probe of a cache frame: view 0 at 1/probe_scale resolution rendered
// with probe_spp samples per pixel twice, in cache mode without a training step
// (cache_lr < 0) and plainly (the unbiased estimator the cache stands in for),
// both with the frame's depth, roulette and frame index and seed + 0x5EED.
int guard_probe(snk_pt_ctx* ctx, const snk_view& view, const snk_render_settings& rs, double* relmse) {
    const snk_cache_guard& g = ctx->guard;
    snk_view pv = view;
    pv.width = std::max(1u, view.width / std::max(1u, g.probe_scale));
    pv.height = std::max(1u, view.height / std::max(1u, g.probe_scale));
    const size_t np = (size_t)pv.width * pv.height;
    std::vector<float> cached(4 * np), plain(4 * np);
    snk_render_settings ps = rs;
    ps.spp = std::max(1u, g.probe_spp);
    ps.seed = rs.seed + 0x5EEDu;
    ps.flags = 0;
    ps.cache_lr = -1.0f;
    snk_view_outputs o;
    std::memset(&o, 0, sizeof(o));
    o.memory = SNK_MEM_HOST;
    o.radiance = cached.data();
    int rc = render_impl(ctx, &pv, 1, &ps, &o);
    if (rc) return rc;
    ps.mode = SNK_MODE_PATH;
    o.radiance = plain.data();
    rc = render_impl(ctx, &pv, 1, &ps, &o);
    if (rc) return rc;
    *relmse = guard_relmse(cached.data(), plain.data(), pv.width, pv.height, g.block);
    return SNK_OK;
}

}  // namespace

extern "C" {

// RT::RecordRenderCmdBuf (Raytracing.cpp:227-267), with the radiance cache's
// quality guard around cache-mode frames (snk_pt_cache_set_guard): every
// check_every-th guarded frame is preceded by a probe; while the last probe was
// over budget, frames render with an infinite spread threshold (no path ends in
// the cache, so the image is the plain tracer's bit for bit) and keep training
// the network, which returns to service at the next passing probe.
int snk_pt_render(snk_pt_ctx* ctx, const snk_view* views, uint32_t num_views, const snk_render_settings* settings,
                  const snk_view_outputs* outputs) {
    if (!ctx) return SNK_ERR_INVALID_ARG;
    if (!views || !settings || !outputs || num_views == 0 || num_views > MAX_VIEWS)
        return fail(ctx, SNK_ERR_INVALID_ARG, "render: bad views/settings/outputs");
    if (settings->mode != SNK_MODE_PATH_CACHE || ctx->guard.check_every == 0)
        return render_impl(ctx, views, num_views, settings, outputs);
    if (ctx->guard_frames > 0 && ctx->guard_frames % ctx->guard.check_every == 0) {
        double e = 0.0;
        const int rc = guard_probe(ctx, views[0], *settings, &e);
        if (rc) return rc;
        ctx->guard_last = e;
        ctx->guard_probes++;
        ctx->guard_fallback = e > (double)ctx->guard.relmse_budget;
    }
    ctx->guard_frames++;
    snk_render_settings rs = *settings;
    if (ctx->guard_fallback) {
        rs.cache_spread = 1e30f;
        ctx->guard_fallback_frames++;
    }
    return render_impl(ctx, views, num_views, &rs, outputs);
}

}  // extern "C"

namespace {

int render_impl(snk_pt_ctx* ctx, const snk_view* views, uint32_t num_views, const snk_render_settings* settings,
                const snk_view_outputs* outputs) {
    const snk_render_settings& rs = *settings;
    if (rs.mode != SNK_MODE_PATH && rs.mode != SNK_MODE_RESTIR_DI && rs.mode != SNK_MODE_PATH_CACHE &&
        rs.mode != SNK_MODE_RESTIR_PT)
        return fail(ctx, SNK_ERR_UNSUPPORTED, "render: mode not supported by this entry point");
    const bool path_like = rs.mode == SNK_MODE_PATH || rs.mode == SNK_MODE_PATH_CACHE;
    // ReSTIR DI at the primary vertex + path-traced indirect light (the wavefront
    // paths start at the primary vertex and also write the ReSTIR surface records).
    // ReSTIR DI alone runs the same wavefront for one segment of one path per pixel:
    // the persistent traversal traces the primary rays and the first shading pass
    // writes the G-buffer and the surface records.
    const bool restir_pt = rs.mode == SNK_MODE_RESTIR_PT;
    const bool restir_di = rs.mode == SNK_MODE_RESTIR_DI;
    const uint32_t max_depth = restir_di ? 1u : rs.max_depth;
    if (!restir_di && (rs.spp == 0 || rs.max_depth == 0 || rs.max_depth > MAX_DEPTH))
        return fail(ctx, SNK_ERR_INVALID_ARG, "render: spp must be >= 1 and 1 <= max_depth <= 16");
    if (!path_like && (rs.restir_spatial < 0 || rs.restir_spatial > 32 || rs.restir_candidates > 4096))
        return fail(ctx, SNK_ERR_INVALID_ARG, "render: restir_spatial must be 0..32, restir_candidates <= 4096");
    uint64_t n_pixels = 0;
    for (uint32_t v = 0; v < num_views; v++) {
        if (views[v].width == 0 || views[v].height == 0) return fail(ctx, SNK_ERR_INVALID_ARG, "render: empty view");
        if (outputs[v].memory > SNK_MEM_HOST) return fail(ctx, SNK_ERR_INVALID_ARG, "render: bad memory space");
        n_pixels += (uint64_t)views[v].width * views[v].height;
    }
    const uint32_t spp = restir_di ? 1u : rs.spp;
    if (n_pixels * spp >= (1ull << 31)) return fail(ctx, SNK_ERR_INVALID_ARG, "render: too many paths");
    API_TRY(set_device(ctx));
    API_TRY(ensure_built(ctx));
    if (!path_like) {   // per-view ReSTIR state (G-buffer records, reservoirs, history)
        if (ctx->restir.size() < num_views) ctx->restir.resize(num_views);
        for (uint32_t v = 0; v < num_views; v++) {
            RestirState& R = ctx->restir[v];
            const uint32_t w = views[v].width, h = views[v].height;
            const size_t np = (size_t)w * h;
            if (R.w != w || R.h != h) {
                if (R.g_pos.reserve(np) || R.g_normal.reserve(np) || R.g_albedo.reserve(np) || R.g_misc.reserve(np) ||
                    R.prev_normal.reserve(np) || R.res_a.reserve(3 * np) || R.res_b.reserve(3 * np) ||
                    R.res_c.reserve(3 * np) || R.ris.reserve(2 * np) || R.memo_keys.reserve(4 * np) ||
                    R.plan.reserve(np))
                    return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "restir buffers");
                R.w = w; R.h = h; R.history_valid = 0; R.hist = 1; R.spat = 2;
            }
        }
    }
    cudaStream_t st = ctx->stream;
    const bool cache = rs.mode == SNK_MODE_PATH_CACHE;
    const uint32_t n_train = cache ? (rs.cache_train_paths ? rs.cache_train_paths : 16384u) : 0u;
    if (n_train > (1u << 22)) return fail(ctx, SNK_ERR_INVALID_ARG, "render: too many cache training paths");
    const uint32_t n_render = (uint32_t)(n_pixels * spp);
    const uint32_t n_paths = n_render + n_train;

    // per-view device descriptors.  Host outputs in page-locked memory (cudaHostAlloc /
    // cudaHostRegister) are written by the kernels in place over the CPU-GPU link;
    // other host outputs go through device staging buffers and a copy back.
    std::vector<ViewDev> vd(num_views);
    std::vector<uint32_t> direct(num_views, 0u);   // bit k: output k written in place
    uint64_t off = 0;
    Status sst = Status::Ok();
    for (uint32_t v = 0; v < num_views; v++) {
        ViewDev& D = vd[v];
        std::memset(&D, 0, sizeof(D));
        std::memcpy(&D.v, &views[v], sizeof(ViewParams));
        D.pixel_offset = (uint32_t)off;
        snk_view_outputs o = outputs[v];
        void** src = out_slots(o);
        void** dst = dev_slots(D);
        size_t np = (size_t)views[v].width * views[v].height;
        for (int k = 0; k < NUM_OUT; k++) {
            if (!src[k]) continue;
            if (o.memory == SNK_MEM_HOST) {
                cudaPointerAttributes pa;
                if (cudaPointerGetAttributes(&pa, src[k]) == cudaSuccess && pa.type == cudaMemoryTypeHost &&
                    pa.devicePointer && reinterpret_cast<uintptr_t>(pa.devicePointer) % 16 == 0) {
                    dst[k] = pa.devicePointer;
                    direct[v] |= 1u << k;
                    continue;
                }
                cudaGetLastError();
                dst[k] = stage(ctx, v, (uint32_t)k, np * OUT_BYTES[k], &sst);
                if (!sst.ok()) return fail(ctx, sst);
            } else {
                dst[k] = src[k];
            }
        }
        if (!path_like) {   // the first shading pass writes the ReSTIR surface records
            RestirState& R = ctx->restir[v];
            D.rs_pos = R.g_pos.p; D.rs_normal = R.g_normal.p; D.rs_albedo = R.g_albedo.p; D.rs_misc = R.g_misc.p;
        }
        off += np;
    }
    API_TRY(upload(ctx->d_views, vd.data(), vd.size(), st));

    FrameParams F;
    std::memset(&F, 0, sizeof(F));
    F.S = scene_dev(ctx);
    F.views = ctx->d_views.p;
    F.nviews = num_views;
    F.spp = spp;
    F.max_depth = max_depth;
    F.rr_depth = rs.rr_depth;
    // the indirect paths of the ReSTIR mode get new random streams every frame
    F.seed = restir_pt ? rs.seed + 0x9E3779B9u * rs.frame_index : rs.seed;
    F.n_paths = n_paths;
    F.n_pixels = (uint32_t)n_pixels;
    // camera packets: every view large, single-primitive leaves, the default
    // traversal bounds (their limits are per ray) and no counting of traversal work
    F.packet_primary = F.S.single_leaf && !(rs.flags & SNK_RENDER_COUNT_NODES) &&
                       F.S.max_steps == MAX_TRAVERSAL_STEPS && F.S.stack_max >= STACK_MAX;
    for (uint32_t v = 0; v < num_views; v++) {
        const uint32_t w = views[v].width, h = views[v].height;
        if (w % PACKET_TILE_W || h % PACKET_TILE_H || (uint64_t)w * h < PACKET_MIN_PIXELS) F.packet_primary = 0u;
    }
    F.tune = trace_tuning(ctx);
    F.tune_any = any_tuning(ctx);
    const bool count_nodes = (rs.flags & SNK_RENDER_COUNT_NODES) != 0;
    const bool profile = (rs.flags & SNK_RENDER_PROFILE) != 0;
    if (ctx->prof_pending) cudaStreamSynchronize(st);   // events of the previous frame are reused
    ctx->prof_used = 0;
    ctx->prof_iv.clear();
    ctx->prof_chain = false;
    ctx->prof_pending = profile;
    for (int k = 0; k < SNK_NUM_STAGES; k++) ctx->stage_launches[k] = 0;

    // FP64 accumulator of view 0
    if (rs.flags & SNK_RENDER_ACCUMULATE_F64) {
        uint32_t w = views[0].width, h = views[0].height;
        if (ctx->accum_w != w || ctx->accum_h != h || (rs.flags & SNK_RENDER_RESET_ACCUM) || !ctx->accum.p) {
            if (ctx->accum.reserve(2ull * w * h) != cudaSuccess) return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "accumulator");
            if (cudaMemsetAsync(ctx->accum.p, 0, 2ull * w * h * sizeof(double2), st) != cudaSuccess)
                return fail(ctx, SNK_ERR_CUDA, "accumulator reset");
            ctx->accum_w = w;
            ctx->accum_h = h;
            ctx->accum_frames = 0;
        }
        F.accumulate = 1;
        ctx->accum_frames++;
    }
    F.accum = ctx->accum.p;   // (read only when accumulating)

    if (ctx->counters.reserve(CNT_TOTAL) != cudaSuccess || ctx->trav.reserve(4) != cudaSuccess)
        return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "counters");
    F.counters = ctx->counters.p;
    F.trav_counters = count_nodes ? ctx->trav.p : nullptr;
    auto reset_counters = [&]() -> cudaError_t {
        cudaError_t r = cudaMemsetAsync(ctx->counters.p, 0, CNT_TOTAL * sizeof(uint32_t), st);
        if (r == cudaSuccess) r = cudaMemsetAsync(ctx->trav.p, 0, 4 * sizeof(unsigned long long), st);
        return r;
    };
    // CUDA-graph replay (path modes): the frame's memsets and kernels are captured
    // once and replayed as long as nothing they bake in changes (the per-frame seed,
    // frame index and accumulate flag are read from device memory, the views'
    // poses and outputs from the uploaded view table); otherwise the frame is
    // captured again and the instantiated graph updated in place
    // (cudaGraphExecUpdate) when the topology matches
    const bool use_graph = (rs.flags & SNK_RENDER_USE_GRAPH) && path_like && !profile;
    if (!use_graph && reset_counters() != cudaSuccess) return fail(ctx, SNK_ERR_CUDA, "counter reset");

    {
        if (!path_like) F.indirect = 1;   // ReSTIR shades the primary vertex
        // (host outputs keep the resolve pass: its coalesced writes to page-locked host
        // memory beat the scattered writes of paths as they end)
        bool host_out = false;
        for (uint32_t v = 0; v < num_views; v++) host_out = host_out || outputs[v].memory == SNK_MEM_HOST;
        F.early_resolve = (path_like && !cache && spp == 1u && !host_out) ? 1u : 0u;
        if (restir_pt) {
            if (ctx->indirect.reserve(n_pixels) != cudaSuccess)
                return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "render: indirect light buffer");
            F.indirect_out = ctx->indirect.p;
        }
        if (cache) {
            API_TRY(cache_ensure(ctx));
            const size_t nv = (size_t)n_train * TRAIN_V;
            if (ctx->c_spread.reserve(n_paths) || ctx->c_qrec.reserve(4ull * n_render) || ctx->c_qbeta.reserve(n_render) ||
                ctx->c_trec.reserve(4 * nv) || ctx->c_tbeta.reserve(nv) || ctx->c_tL.reserve(nv) ||
                ctx->c_samples.reserve(5 * nv))
                return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "render: cache buffers");
            F.cache = 1;
            F.n_render = n_render;
            F.n_train = n_train;
            F.frame = rs.frame_index;
            F.spread_c = rs.cache_spread > 0.0f ? rs.cache_spread : 0.01f;
            F.spread = ctx->c_spread.p;
            F.qrec = ctx->c_qrec.p;
            F.qbeta = ctx->c_qbeta.p;
            F.train_rec = ctx->c_trec.p;
            F.train_beta = ctx->c_tbeta.p;
            F.train_L = ctx->c_tL.p;
            F.samples = ctx->c_samples.p;
            if (cudaMemsetAsync(F.train_beta, 0, nv * sizeof(float4), st) ||
                cudaMemsetAsync(F.train_L, 0, nv * sizeof(float4), st))
                return fail(ctx, SNK_ERR_CUDA, "render: cache buffer reset");
            const uint32_t steps = rs.cache_train_steps ? rs.cache_train_steps : 4u;
            API_TRY(mlp_train_reserve(ctx->mlp, (uint32_t)((nv + steps - 1) / steps)));
        }
        if (ctx->rays0.reserve(2ull * n_paths) || ctx->rays1.reserve(2ull * n_paths) || ctx->pid0.reserve(n_paths) ||
            ctx->pid1.reserve(n_paths) || ctx->hits.reserve(n_paths) || ctx->beta.reserve(n_paths) ||
            ctx->L.reserve(n_paths) || ctx->srays.reserve(4ull * n_paths) || ctx->scontrib.reserve(2ull * n_paths))
            return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "frame buffers");
        F.rays[0] = ctx->rays0.p; F.rays[1] = ctx->rays1.p;
        F.path_ids[0] = ctx->pid0.p; F.path_ids[1] = ctx->pid1.p;
        F.hits = ctx->hits.p; F.beta = ctx->beta.p; F.L = ctx->L.p;
        F.shadow_rays = ctx->srays.p; F.shadow_contrib = ctx->scontrib.p;
        const uint32_t dyn[4] = {F.seed, F.frame, F.accumulate, 0u};
        if (ctx->d_dyn.reserve(4) != cudaSuccess ||
            cudaMemcpyAsync(ctx->d_dyn.p, dyn, sizeof(dyn), cudaMemcpyHostToDevice, st) != cudaSuccess)
            return fail(ctx, SNK_ERR_CUDA, "render: frame values upload");
        F.dyn = ctx->d_dyn.p;
        const int g8 = shade_grid(ctx), g16 = trace_grid(ctx), gany = any_grid(ctx);
        const uint32_t train_steps = rs.cache_train_steps ? rs.cache_train_steps : 4u;
        const float train_lr = rs.cache_lr > 0.0f ? rs.cache_lr : (rs.cache_lr < 0.0f ? 0.0f : 1e-2f);
        if (cache) ctx->last_cache_samples = (uint64_t)n_train * TRAIN_V;
        bool replay = false;
        if (use_graph) {   // the key: the frame parameters without the per-frame values, grids, training steps
            FrameParams K = F;
            K.seed = 0; K.frame = 0; K.accumulate = 0;
            const EncodeParams ep = cache ? cache_encode_params(ctx) : EncodeParams{};
            const int grids[3] = {g8, g16, gany};
            // (the Adam steps bake their bias corrections in: a cache frame is captured every time)
            const uint32_t adam_step = cache ? ctx->mlp.step : 0u;
            std::vector<unsigned char> key(sizeof(K) + sizeof(ep) + sizeof(grids) + 3 * sizeof(uint32_t) + sizeof(float));
            unsigned char* kp = key.data();
            auto put = [&](const void* x, size_t b) { std::memcpy(kp, x, b); kp += b; };
            put(&K, sizeof(K)); put(&ep, sizeof(ep)); put(grids, sizeof(grids));
            put(&max_depth, sizeof(max_depth)); put(&train_steps, sizeof(train_steps)); put(&train_lr, sizeof(train_lr));
            put(&adam_step, sizeof(adam_step));
            replay = ctx->graph_exec && key == ctx->graph_key;
            if (!replay) ctx->graph_key.swap(key);
        }
        if (!use_graph) cudaEventRecord(ctx->ev0, st);
        cudaError_t e = cudaSuccess;
        if (use_graph && !replay) {
            e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
            if (e == cudaSuccess) e = reset_counters();
        }
        if (!replay) {
        // Segment d: closest hits, shading, then its shadow rays.  The shadow rays of
        // segment d and the closest hits of segment d + 1 are independent (they read
        // the queues shade(d) wrote and write different outputs), so they run
        // concurrently on two streams; shade(d + 1), which reuses segment d's shadow
        // slots, waits for both.  The kernels that end a launch early overlap the
        // other's tail instead of leaving SMs idle.
        if (e == cudaSuccess) e = ensure_side_stream(ctx);
        cudaStream_t side = ctx->side;
        if (e == cudaSuccess) e = staged(ctx, profile, SNK_STAGE_GENERATE, [&] { return launch_generate(F, g8, st); });
        if (e == cudaSuccess)
            e = staged(ctx, profile, SNK_STAGE_TRACE_CLOSEST,
                       [&] { return launch_trace_closest(F, 0, g16, count_nodes, st); });
        for (uint32_t d = 0; d < max_depth && e == cudaSuccess; d++) {
            e = staged(ctx, profile, SNK_STAGE_SHADE, [&] { return launch_shade(F, d, g8, st); });
            // (in the ReSTIR modes the primary vertex queues no shadow rays: ReSTIR shades it)
            const bool shadows = !(F.indirect && d == 0);
            if (e == cudaSuccess && shadows) {
                e = cudaEventRecord(ctx->ev_fork[d], st);
                if (e == cudaSuccess) e = cudaStreamWaitEvent(side, ctx->ev_fork[d], 0);
                if (e == cudaSuccess)
                    e = staged(ctx, profile, SNK_STAGE_TRACE_SHADOW,
                               [&] { return launch_trace_shadow(F, d, gany, count_nodes, side); }, side);
                ctx->stage_launches[SNK_STAGE_TRACE_SHADOW]++;   // (its second kernel: the accumulation)
                if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_join[d], side);
            }
            if (e == cudaSuccess && d + 1 < max_depth)
                e = staged(ctx, profile, SNK_STAGE_TRACE_CLOSEST,
                           [&] { return launch_trace_closest(F, d + 1, g16, count_nodes, st); });
            if (e == cudaSuccess && shadows) {
                e = cudaStreamWaitEvent(st, ctx->ev_join[d], 0);
                ctx->prof_chain = false;   // the next stage starts after the wait, not at the last event
            }
        }
        if (cache && e == cudaSuccess) {
            const EncodeParams ep = cache_encode_params(ctx);
            e = staged(ctx, profile, SNK_STAGE_CACHE_INFER, [&] {
                Status s = mlp_infer(ctx->mlp, F.qrec, F.counters + CNT_CACHE_QUERIES, 0u, ep, nullptr, F.qbeta, F.L,
                                     grid_of(ctx, 4), ctx->d_err.p, st);
                return s.ok() ? cudaSuccess : cudaErrorLaunchFailure;
            });
        }
        if (e == cudaSuccess && !restir_di && !F.early_resolve)
            e = staged(ctx, profile, SNK_STAGE_RESOLVE, [&] { return launch_resolve(F, g8, st); });
        if (cache && e == cudaSuccess) {
            e = staged(ctx, profile, SNK_STAGE_CACHE_SAMPLES, [&] { return launch_make_samples(F, g8, st); });
            const EncodeParams ep = cache_encode_params(ctx);
            const uint32_t steps = rs.cache_train_steps ? rs.cache_train_steps : 4u;
            const uint32_t total = n_train * TRAIN_V, chunk = (total + steps - 1) / steps;
            // cache_lr: 0 -> 1e-2; negative -> the network is not updated (gradients only)
            const float lr = rs.cache_lr > 0.0f ? rs.cache_lr : (rs.cache_lr < 0.0f ? 0.0f : 1e-2f);
            for (uint32_t k = 0; k < steps && e == cudaSuccess; k++) {
                const uint32_t b = k * chunk, cnt = b < total ? std::min(chunk, total - b) : 0u;
                if (cnt == 0) break;
                e = staged(ctx, profile, SNK_STAGE_CACHE_TRAIN, [&] {
                    Status s = mlp_train_step(ctx->mlp, F.samples + 5ull * b, cnt, ep, lr, nullptr, nullptr,
                                              ctx->d_err.p, st);
                    return s.ok() ? cudaSuccess : cudaErrorLaunchFailure;
                });
                ctx->stage_launches[SNK_STAGE_CACHE_TRAIN]++;   // (its second kernel: the Adam step)
            }
        }
        }   // (!replay)
        // a replayed frame runs the launches its capture counted
        if (replay) std::memcpy(ctx->stage_launches, ctx->graph_stage_launches, sizeof(ctx->stage_launches));
        else if (use_graph) std::memcpy(ctx->graph_stage_launches, ctx->stage_launches, sizeof(ctx->stage_launches));
        if (use_graph && !replay) {
            ctx->graph_captures++;
            cudaGraph_t graph = nullptr;
            cudaError_t ec = cudaStreamEndCapture(st, &graph);
            if (e == cudaSuccess) e = ec;
            if (e == cudaSuccess && ctx->graph_exec) {
                cudaGraphExecUpdateResultInfo info;
                if (cudaGraphExecUpdate(ctx->graph_exec, graph, &info) != cudaSuccess) {
                    cudaGetLastError();
                    cudaGraphExecDestroy(ctx->graph_exec);
                    ctx->graph_exec = nullptr;
                }
            }
            if (e == cudaSuccess && !ctx->graph_exec) e = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
            if (graph) cudaGraphDestroy(graph);
            if (e != cudaSuccess) ctx->graph_key.clear();
        }
        if (use_graph && e == cudaSuccess) {
            cudaEventRecord(ctx->ev0, st);
            e = cudaGraphLaunch(ctx->graph_exec, st);
            ctx->graph_launches++;
        }
        if (path_like) cudaEventRecord(ctx->ev1, st);
        if (e != cudaSuccess) return fail(ctx, SNK_ERR_CUDA, std::string("render launch: ") + cudaGetErrorString(e));
    }
    if (!path_like) {
        for (uint32_t v = 0; v < num_views; v++) {
            RestirState& R = ctx->restir[v];
            const size_t np = (size_t)views[v].width * views[v].height;
            RestirView RV;
            RV.g_pos = R.g_pos.p; RV.g_normal = R.g_normal.p; RV.g_albedo = R.g_albedo.p; RV.g_misc = R.g_misc.p;
            RV.prev_normal = R.prev_normal.p;
            RV.temporal = R.res_a.p;
            RV.history = R.hist == 1 ? R.res_b.p : R.res_c.p;
            RV.spatial = R.spat == 1 ? R.res_b.p : R.res_c.p;
            RV.ris = R.ris.p;
            RV.memo_keys = R.memo_keys.p; RV.plan = R.plan.p;
            if (R.combo.reserve((RESTIR_TEMPORAL_COMBOS + 1u + (uint32_t)std::max(rs.restir_spatial, 0)) * np))
                return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "restir buffers");
            RV.combo = R.combo.p;
            RV.indirect = restir_pt ? ctx->indirect.p + vd[v].pixel_offset : nullptr;
            RV.history_valid = R.history_valid;
            RestirSettings s;
            s.frame_index = rs.frame_index; s.seed = rs.seed; s.candidates = rs.restir_candidates;
            s.mcap = rs.restir_mcap; s.temporal = rs.restir_temporal; s.spatial = rs.restir_spatial;
            s.radius = rs.restir_radius; s.pad = 0;
            // visibility queues: initial (K1 slots per pixel), spatial (K2), final shading (K3)
            const uint32_t K1 = RESTIR_INITIAL_SLOTS, K2 = restir_spatial_slots(s.spatial), K3 = RESTIR_SHADE_SLOTS;
            if (ctx->rq_rays.reserve(2ull * std::max(K1, K2) * np) || ctx->rq_vis_a.reserve(std::max(K1, K3) * np) ||
                ctx->rq_vis_b.reserve((size_t)K2 * np) || ctx->rq_work.reserve(3))
                return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "restir visibility queues");
            ctx->prof_chain = false;   // the queue reset below is not part of a stage
            if (cudaMemsetAsync(ctx->rq_work.p, 0, 3 * sizeof(uint32_t), st) != cudaSuccess)
                return fail(ctx, SNK_ERR_CUDA, "restir queue reset");
            const RestirQueue q1{ctx->rq_rays.p, ctx->rq_vis_a.p, K1, (uint32_t)np},
                q2{ctx->rq_rays.p, ctx->rq_vis_b.p, K2, (uint32_t)np}, q3{ctx->rq_rays.p, ctx->rq_vis_a.p, K3, (uint32_t)np};
            const int tg = trace_grid(ctx);
            const SceneDev SD = scene_dev(ctx);
            const TraceTuning tt = any_tuning(ctx);
            const int ta = any_grid(ctx);
            auto pass = [&](int stage, int phase, const RestirQueue& qa, const RestirQueue& qb) {
                return staged(ctx, profile, SNK_STAGE_RESTIR_GBUFFER + stage,
                              [&] { return launch_restir_stage(stage, phase, F, v, RV, s, qa, qb, tg, st); });
            };
            auto visibility = [&](uint32_t K, uint8_t* vis, int slot) {
                return staged(ctx, profile, SNK_STAGE_TRACE_SHADOW, [&] {
                    return launch_trace_visibility(SD, ctx->rq_rays.p, (uint32_t)(K * np), vis, ctx->rq_work.p + slot,
                                                   ta, tt, st);
                });
            };
            // (the first shading pass wrote the G-buffer and the surface records)
            cudaError_t e = pass(1, -1, q1, q3);   // the RIS candidates
            if (e == cudaSuccess) e = pass(1, 0, q1, q3);
            if (e == cudaSuccess) e = visibility(K1, ctx->rq_vis_a.p, 0);
            if (e == cudaSuccess) e = pass(1, 1, q1, q3);
            if (e == cudaSuccess) e = pass(2, 0, q2, q3);
            if (e == cudaSuccess) e = visibility(K2, ctx->rq_vis_b.p, 1);
            if (e == cudaSuccess) e = pass(2, 1, q2, q3);
            if (e == cudaSuccess) e = visibility(K3, ctx->rq_vis_a.p, 2);
            if (e == cudaSuccess) e = pass(2, 2, q2, q3);
            if (e != cudaSuccess) return fail(ctx, SNK_ERR_CUDA, std::string("restir launch: ") + cudaGetErrorString(e));
            std::swap(R.hist, R.spat);
            R.history_valid = 1;
        }
        cudaEventRecord(ctx->ev1, st);
    }
    ctx->timing_pending = true;
    cudaMemcpyAsync(ctx->h_counters, ctx->counters.p, CNT_TOTAL * sizeof(uint32_t), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(ctx->h_trav, ctx->trav.p, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st);
    cudaMemcpyAsync(ctx->h_err, ctx->d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, st);
    if (ctx->tlas_refittable && ctx->tlas_root != INVALID && ctx->d_small_out.p)
        cudaMemcpyAsync(ctx->h_small, ctx->d_small_out.p, sizeof(SmallBuildOut), cudaMemcpyDeviceToHost, st);
    ctx->counters_pending = true;
    ctx->aux_pending = true;
    ctx->last_mode = rs.mode;
    ctx->last_depth = max_depth;
    ctx->last_paths = n_paths;
    ctx->last_pixels = n_pixels;
    ctx->last_count_nodes = count_nodes;

    // host outputs: copy back and synchronise
    bool any_host = false;
    for (uint32_t v = 0; v < num_views; v++) {
        if (outputs[v].memory != SNK_MEM_HOST) continue;
        any_host = true;
        snk_view_outputs o = outputs[v];
        void** src = out_slots(o);
        void** dst = dev_slots(vd[v]);
        size_t np = (size_t)views[v].width * views[v].height;
        for (int k = 0; k < NUM_OUT; k++) {
            if (!src[k] || (direct[v] >> k) & 1u) continue;
            if (cudaMemcpyAsync(src[k], dst[k], np * OUT_BYTES[k], cudaMemcpyDeviceToHost, st) != cudaSuccess)
                return fail(ctx, SNK_ERR_CUDA, "render: output copy");
        }
    }
    if (any_host) API_TRY(check_device_error(ctx));
    return SNK_OK;
}

}  // namespace

extern "C" {

int snk_pt_cache_set_guard(snk_pt_ctx* ctx, const snk_cache_guard* g) {
    if (!ctx) return SNK_ERR_INVALID_ARG;
    if (!g || g->check_every == 0) {
        std::memset(&ctx->guard, 0, sizeof(ctx->guard));
    } else {
        if (!(g->relmse_budget > 0.0f) || g->probe_spp > 4096 || g->probe_scale > 64 || g->block > 64)
            return fail(ctx, SNK_ERR_INVALID_ARG, "cache_set_guard: budget must be > 0, probe_spp <= 4096, "
                                                  "probe_scale <= 64, block <= 64");
        ctx->guard = *g;
    }
    ctx->guard_frames = ctx->guard_probes = ctx->guard_fallback_frames = 0;
    ctx->guard_last = -1.0;
    ctx->guard_fallback = false;
    return SNK_OK;
}

int snk_pt_cache_get_guard_state(const snk_pt_ctx* ctx, snk_cache_guard_state* s) {
    if (!ctx || !s) return SNK_ERR_INVALID_ARG;
    std::memset(s, 0, sizeof(*s));
    s->frames = ctx->guard_frames;
    s->probes = ctx->guard_probes;
    s->fallback_frames = ctx->guard_fallback_frames;
    s->last_probe_relmse = ctx->guard_last;
    s->fallback = ctx->guard_fallback ? 1u : 0u;
    return SNK_OK;
}

int snk_cache_guard_relmse(const float* cached, const float* plain, uint32_t width, uint32_t height, uint32_t block,
                           double* relmse) {
    if (!cached || !plain || !relmse || width == 0 || height == 0) return SNK_ERR_INVALID_ARG;
    *relmse = guard_relmse(cached, plain, width, height, block);
    return SNK_OK;
}

int snk_pt_set_tuning(snk_pt_ctx* ctx, const snk_tuning* t) {
    if (!ctx || !t) return fail(ctx, SNK_ERR_INVALID_ARG, "set_tuning: null argument");
    if (t->trace_blocks_per_sm > 64 || t->shade_blocks_per_sm > 64 || t->ray_chunk > 4096 || t->refill_idle > 32 ||
        t->prim_bias > 64 || t->trace_variant > 2 || 
        (t->bvh_treelet_passes > 16 && t->bvh_treelet_passes != SNK_TREELET_PASSES_NONE) ||
        (t->tlas_treelet_passes > 16 && t->tlas_treelet_passes != SNK_TREELET_PASSES_NONE) ||
        t->bvh_leaf_max > LEAF_MAX_LIMIT || t->tlas_leaf_max > LEAF_MAX_LIMIT || t->bvh_leaf_pack > LEAF_MAX_LIMIT ||
        t->max_traversal_steps > MAX_TRAVERSAL_STEPS || t->stack_limit > (uint32_t)STACK_MAX ||
        t->shadow_blocks_per_sm > 64 || t->shadow_ray_chunk > 4096 || t->shadow_refill_idle > 32 ||
        t->shadow_prim_bias > 64 || t->shadow_variant > 3 || t->bvh_collapse > 1)
        return fail(ctx, SNK_ERR_INVALID_ARG, "set_tuning: knob out of range");
    ctx->tune = *t;
    return SNK_OK;
}

int snk_pt_get_tuning(const snk_pt_ctx* ctx, snk_tuning* t) {
    if (!ctx || !t) return SNK_ERR_INVALID_ARG;
    *t = ctx->tune;
    return SNK_OK;
}

int snk_pt_autotune(snk_pt_ctx* ctx, const snk_view* views, uint32_t num_views, const snk_render_settings* settings,
                    uint32_t frames, snk_tuning* best) {
    if (!ctx || !views || !settings || num_views == 0) return fail(ctx, SNK_ERR_INVALID_ARG, "autotune: bad arguments");
    if (settings->mode != SNK_MODE_PATH) return fail(ctx, SNK_ERR_UNSUPPORTED, "autotune: path mode only");
    if (frames == 0) frames = 3;
    std::vector<snk_view_outputs> outs(num_views);
    std::memset(outs.data(), 0, outs.size() * sizeof(snk_view_outputs));
    snk_render_settings rs = *settings;
    rs.flags &= ~(SNK_RENDER_ACCUMULATE_F64 | SNK_RENDER_RESET_ACCUM | SNK_RENDER_COUNT_NODES | SNK_RENDER_PROFILE);
    auto trial = [&](const snk_tuning& t, double* ms) -> int {
        ctx->tune = t;
        int rc = snk_pt_render(ctx, views, num_views, &rs, outs.data());   // warm-up
        if (rc) return rc;
        cudaEvent_t a, b;
        cudaEventCreate(&a);
        cudaEventCreate(&b);
        cudaEventRecord(a, ctx->stream);
        for (uint32_t f = 0; f < frames && rc == 0; f++) {
            rs.seed = settings->seed + 1 + f;
            rc = snk_pt_render(ctx, views, num_views, &rs, outs.data());
        }
        cudaEventRecord(b, ctx->stream);
        cudaEventSynchronize(b);
        float m = 0.0f;
        cudaEventElapsedTime(&m, a, b);
        cudaEventDestroy(a);
        cudaEventDestroy(b);
        *ms = m;
        return rc;
    };
    snk_tuning cur = ctx->tune;
    if (!cur.trace_blocks_per_sm) cur.trace_blocks_per_sm = 16;
    if (!cur.shade_blocks_per_sm) cur.shade_blocks_per_sm = 8;
    if (!cur.ray_chunk) cur.ray_chunk = 64;
    if (!cur.refill_idle) cur.refill_idle = 4;
    if (!cur.prim_bias) cur.prim_bias = 4;
    double best_ms = 0.0;
    int rc = trial(cur, &best_ms);
    if (rc) return rc;
    struct Knob { uint32_t* field; std::vector<uint32_t> values; };
    for (int pass = 0; pass < 2; pass++) {
        snk_tuning cand = cur;
        Knob knobs[] = {
            {&cand.trace_blocks_per_sm, {4, 8, 12, 16, 24, 32}},
            {&cand.trace_variant, {0, 1, 2}},
            {&cand.refill_idle, {1, 2, 4, 8, 16}},
            {&cand.ray_chunk, {32, 64, 128, 256}},
            {&cand.prim_bias, {2, 4, 8}},
            {&cand.shade_blocks_per_sm, {4, 8, 16}},
        };
        for (Knob& k : knobs) {
            uint32_t keep = *k.field;
            for (uint32_t v : k.values) {
                if (v == keep) continue;
                cand = cur;
                // the Knob pointers refer to `cand`; rewrite the field through the same offset
                *k.field = v;
                double ms = 0.0;
                rc = trial(cand, &ms);
                if (rc) return rc;
                if (ms < best_ms) { best_ms = ms; cur = cand; }
            }
            cand = cur;
        }
    }
    ctx->tune = cur;
    if (best) *best = cur;
    return SNK_OK;
}

extern "C++" {
namespace {

EncodeParams cache_encode_params(snk_pt_ctx* ctx) {
    EncodeParams ep;
    if (!ctx->cache_bounds_set) update_scene_bounds(ctx);
    const float* lo = ctx->cache_bounds_set ? ctx->cache_ep.lo : ctx->scene_lo;
    for (int a = 0; a < 3; a++) {
        ep.lo[a] = lo[a];
        if (ctx->cache_bounds_set) {
            ep.inv_ext[a] = ctx->cache_ep.inv_ext[a];
        } else {
            float ext = ctx->scene_hi[a] - ctx->scene_lo[a];
            ep.inv_ext[a] = ext > 0.0f ? 1.0f / ext : 1.0f;
        }
    }
    return ep;
}

Status cache_ensure(snk_pt_ctx* ctx) {
    if (ctx->mlp.ready) return Status::Ok();
    // He-uniform initialisation from a PCG32 stream (seed 1)
    std::vector<float> w(MLP_NW);
    Pcg rng = pcg_stream(0x4D4C5031u, 0u, 0u, 1u);
    for (int i = 0; i < MLP_NW; i++) {
        const float s = i < 4 * 4096 ? std::sqrt(6.0f / 64.0f) : std::sqrt(6.0f / 64.0f) * 0.1f;
        w[i] = (pcg_float(rng) * 2.0f - 1.0f) * s;
    }
    SNK_TRY(mlp_init(ctx->mlp, w.data(), ctx->stream));
    return Status::Ok();
}

// copies n*floats_per host records into the context's device staging buffer
Status cache_stage(snk_pt_ctx* ctx, const float* src, uint32_t n, uint32_t floats_per, uint32_t memory,
                   const float4** out) {
    if (memory == SNK_MEM_DEVICE) { *out = reinterpret_cast<const float4*>(src); return Status::Ok(); }
    SNK_TRY_CUDA(ctx->cache_in.reserve(((size_t)n * floats_per + 3) / 4));
    SNK_TRY_CUDA(cudaMemcpyAsync(ctx->cache_in.p, src, (size_t)n * floats_per * sizeof(float), cudaMemcpyHostToDevice,
                                 ctx->stream));
    *out = ctx->cache_in.p;
    return Status::Ok();
}

}  // namespace
}  // extern "C++"

int snk_pt_cache_reset(snk_pt_ctx* ctx, uint32_t seed) {
    if (!ctx) return SNK_ERR_INVALID_ARG;
    API_TRY(set_device(ctx));
    std::vector<float> w(MLP_NW);
    Pcg rng = pcg_stream(0x4D4C5031u, 0u, 0u, seed);
    for (int i = 0; i < MLP_NW; i++) {
        const float s = i < 4 * 4096 ? std::sqrt(6.0f / 64.0f) : std::sqrt(6.0f / 64.0f) * 0.1f;
        w[i] = (pcg_float(rng) * 2.0f - 1.0f) * s;
    }
    API_TRY(mlp_init(ctx->mlp, w.data(), ctx->stream));
    return SNK_OK;
}

int snk_pt_cache_set_weights(snk_pt_ctx* ctx, const float* w, uint32_t n) {
    if (!ctx || !w || n != (uint32_t)MLP_NW) return fail(ctx, SNK_ERR_INVALID_ARG, "cache_set_weights: need 16576 weights");
    API_TRY(set_device(ctx));
    API_TRY(mlp_init(ctx->mlp, w, ctx->stream));
    return SNK_OK;
}

int snk_pt_cache_get_weights(snk_pt_ctx* ctx, float* w, uint32_t n) {
    if (!ctx || !w || n != (uint32_t)MLP_NW) return fail(ctx, SNK_ERR_INVALID_ARG, "cache_get_weights: need 16576 weights");
    API_TRY(set_device(ctx));
    API_TRY(cache_ensure(ctx));
    if (cudaMemcpyAsync(w, ctx->mlp.w.p, MLP_NW * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream) ||
        cudaStreamSynchronize(ctx->stream))
        return fail(ctx, SNK_ERR_CUDA, "cache_get_weights: copy");
    return SNK_OK;
}

int snk_pt_cache_set_bounds(snk_pt_ctx* ctx, const float lo[3], const float hi[3]) {
    if (!ctx || !lo || !hi) return fail(ctx, SNK_ERR_INVALID_ARG, "cache_set_bounds: null argument");
    for (int a = 0; a < 3; a++) {
        if (!(hi[a] > lo[a])) return fail(ctx, SNK_ERR_INVALID_ARG, "cache_set_bounds: empty box");
        ctx->cache_ep.lo[a] = lo[a];
        ctx->cache_ep.inv_ext[a] = 1.0f / (hi[a] - lo[a]);
    }
    ctx->cache_bounds_set = true;
    return SNK_OK;
}

int snk_pt_cache_encode(snk_pt_ctx* ctx, const float* records, uint32_t n, float* features, uint32_t memory) {
    if (!ctx || (n && (!records || !features)) || memory > SNK_MEM_HOST) return fail(ctx, SNK_ERR_INVALID_ARG, "cache_encode: bad arguments");
    API_TRY(set_device(ctx));
    if (n == 0) return SNK_OK;
    const float4* rec;
    API_TRY(cache_stage(ctx, records, n, 16, memory, &rec));
    float* out = features;
    if (memory == SNK_MEM_HOST) {
        if (ctx->cache_out.reserve((size_t)n * 64)) return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "cache_encode: buffer");
        out = ctx->cache_out.p;
    }
    API_TRY(mlp_encode(rec, n, cache_encode_params(ctx), out, ctx->stream));
    if (memory == SNK_MEM_HOST &&
        cudaMemcpyAsync(features, out, (size_t)n * 64 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream))
        return fail(ctx, SNK_ERR_CUDA, "cache_encode: copy");
    if (cudaStreamSynchronize(ctx->stream)) return fail(ctx, SNK_ERR_CUDA, "cache_encode: sync");
    return SNK_OK;
}

int snk_pt_cache_infer(snk_pt_ctx* ctx, const float* records, uint32_t n, float* outp, uint32_t memory) {
    if (!ctx || (n && (!records || !outp)) || memory > SNK_MEM_HOST) return fail(ctx, SNK_ERR_INVALID_ARG, "cache_infer: bad arguments");
    API_TRY(set_device(ctx));
    API_TRY(cache_ensure(ctx));
    if (n == 0) return SNK_OK;
    const float4* rec;
    API_TRY(cache_stage(ctx, records, n, 16, memory, &rec));
    float* out = outp;
    if (memory == SNK_MEM_HOST) {
        if (ctx->cache_out.reserve((size_t)n * 3)) return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "cache_infer: buffer");
        out = ctx->cache_out.p;
    }
    API_TRY(mlp_infer(ctx->mlp, rec, nullptr, n, cache_encode_params(ctx), out, nullptr, nullptr, grid_of(ctx, 4),
                      ctx->d_err.p, ctx->stream));
    if (memory == SNK_MEM_HOST &&
        cudaMemcpyAsync(outp, out, (size_t)n * 3 * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream))
        return fail(ctx, SNK_ERR_CUDA, "cache_infer: copy");
    if (cudaStreamSynchronize(ctx->stream)) return fail(ctx, SNK_ERR_CUDA, "cache_infer: sync");
    API_TRY(check_device_error(ctx));
    return SNK_OK;
}

int snk_pt_cache_train(snk_pt_ctx* ctx, const float* samples, uint32_t n, float lr, float* grad, float* loss,
                       uint32_t memory) {
    if (!ctx || (n && !samples) || memory > SNK_MEM_HOST || !(lr >= 0.0f))
        return fail(ctx, SNK_ERR_INVALID_ARG, "cache_train: bad arguments");
    API_TRY(set_device(ctx));
    API_TRY(cache_ensure(ctx));
    if (n == 0) return SNK_OK;
    const float4* s;
    API_TRY(cache_stage(ctx, samples, n, 20, memory, &s));
    if (grad && ctx->cache_grad.reserve(MLP_NW)) return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "cache_train: buffer");
    float l = 0.0f;
    API_TRY(mlp_train_step(ctx->mlp, s, n, cache_encode_params(ctx), lr, grad ? ctx->cache_grad.p : nullptr, &l,
                           ctx->d_err.p, ctx->stream));
    if (grad && (cudaMemcpyAsync(grad, ctx->cache_grad.p, MLP_NW * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream) ||
                 cudaStreamSynchronize(ctx->stream)))
        return fail(ctx, SNK_ERR_CUDA, "cache_train: copy");
    API_TRY(check_device_error(ctx));
    if (loss) *loss = l;
    return SNK_OK;
}

int snk_pt_synchronize(snk_pt_ctx* ctx) {
    if (!ctx) return SNK_ERR_INVALID_ARG;
    API_TRY(set_device(ctx));
    if (!ctx->d_err.p) return SNK_OK;
    API_TRY(check_device_error(ctx));
    return SNK_OK;
}

int snk_pt_trace_rays(snk_pt_ctx* ctx, const snk_ray* rays, uint32_t n, snk_hit* hits, uint32_t flags,
                      uint32_t memory) {
    if (!ctx || (n && (!rays || !hits)) || memory > SNK_MEM_HOST)
        return fail(ctx, SNK_ERR_INVALID_ARG, "trace_rays: bad arguments");
    API_TRY(set_device(ctx));
    API_TRY(ensure_built(ctx));
    if (n == 0) return SNK_OK;
    cudaStream_t st = ctx->stream;
    const float4* d_rays;
    HitDev* d_hits;
    if (memory == SNK_MEM_HOST) {
        if (ctx->tr_rays.reserve(2ull * n) || ctx->tr_hits.reserve(n)) return fail(ctx, SNK_ERR_OUT_OF_MEMORY, "trace buffers");
        if (cudaMemcpyAsync(ctx->tr_rays.p, rays, sizeof(snk_ray) * (size_t)n, cudaMemcpyHostToDevice, st))
            return fail(ctx, SNK_ERR_CUDA, "trace_rays: ray upload");
        d_rays = ctx->tr_rays.p;
        d_hits = ctx->tr_hits.p;
    } else {
        d_rays = reinterpret_cast<const float4*>(rays);
        d_hits = reinterpret_cast<HitDev*>(hits);
    }
    if (ctx->tr_work.reserve(1) || cudaMemsetAsync(ctx->tr_work.p, 0, sizeof(uint32_t), st))
        return fail(ctx, SNK_ERR_CUDA, "trace_rays: work counter");
    const bool any = (flags & SNK_TRACE_ANY_HIT) != 0;
    cudaError_t e = launch_trace_rays(scene_dev(ctx), d_rays, n, d_hits, any, ctx->tr_work.p,
                                      any ? any_grid(ctx) : trace_grid(ctx), any ? any_tuning(ctx) : trace_tuning(ctx), st);
    if (e != cudaSuccess) return fail(ctx, SNK_ERR_CUDA, std::string("trace_rays: ") + cudaGetErrorString(e));
    if (memory == SNK_MEM_HOST &&
        cudaMemcpyAsync(hits, d_hits, sizeof(snk_hit) * (size_t)n, cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return fail(ctx, SNK_ERR_CUDA, "trace_rays: hit download");
    API_TRY(check_device_error(ctx));
    return SNK_OK;
}

extern "C++" {
namespace {
// device view of a caller buffer: the buffer itself, or a staging copy of it
template <class T>
T* stage_in(snk_pt_ctx* ctx, DBuf<unsigned char>& b, const void* src, size_t bytes, uint32_t memory, Status* st) {
    if (memory == SNK_MEM_DEVICE) return reinterpret_cast<T*>(const_cast<void*>(src));
    if (b.reserve(bytes ? bytes : 1)) { *st = Status::Err(SNK_ERR_OUT_OF_MEMORY, "query staging"); return nullptr; }
    if (bytes && cudaMemcpyAsync(b.p, src, bytes, cudaMemcpyHostToDevice, ctx->stream)) {
        *st = Status::Err(SNK_ERR_CUDA, "query upload");
        return nullptr;
    }
    return reinterpret_cast<T*>(b.p);
}
template <class T>
T* stage_out(DBuf<unsigned char>& b, void* dst, size_t bytes, uint32_t memory, Status* st) {
    if (memory == SNK_MEM_DEVICE) return reinterpret_cast<T*>(dst);
    if (b.reserve(bytes ? bytes : 1)) { *st = Status::Err(SNK_ERR_OUT_OF_MEMORY, "query staging"); return nullptr; }
    return reinterpret_cast<T*>(b.p);
}
Status download(snk_pt_ctx* ctx, void* dst, const void* src, size_t bytes, uint32_t memory) {
    if (memory == SNK_MEM_HOST && bytes)
        SNK_TRY_CUDA(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
    return Status::Ok();
}
}  // namespace
}  // extern "C++"

int snk_pt_contact_rays(snk_pt_ctx* ctx, const snk_ray* rays, uint32_t n, float timestep, snk_contact* out,
                        uint32_t memory) {
    if (!ctx || (n && (!rays || !out)) || memory > SNK_MEM_HOST || !(timestep > 0.0f))
        return fail(ctx, SNK_ERR_INVALID_ARG, "contact_rays: bad arguments");
    API_TRY(set_device(ctx));
    API_TRY(ensure_built(ctx));
    if (n == 0) return SNK_OK;
    Status st;
    const float4* d_rays = stage_in<const float4>(ctx, ctx->q_in, rays, sizeof(snk_ray) * (size_t)n, memory, &st);
    ContactOut* d_out = stage_out<ContactOut>(ctx->q_out, out, sizeof(snk_contact) * (size_t)n, memory, &st);
    if (!st.ok()) return fail(ctx, st);
    cudaError_t e = launch_contact_rays(scene_dev(ctx), d_rays, n, timestep, d_out, grid_of(ctx, 16), ctx->stream);
    if (e != cudaSuccess) return fail(ctx, SNK_ERR_CUDA, std::string("contact_rays: ") + cudaGetErrorString(e));
    API_TRY(download(ctx, out, d_out, sizeof(snk_contact) * (size_t)n, memory));
    API_TRY(check_device_error(ctx));
    return SNK_OK;
}

int snk_pt_particle_probe(snk_pt_ctx* ctx, const snk_particle* particles, uint32_t n, float timestep,
                          snk_contact* candidate, float* gravity_dv, uint32_t memory) {
    if (!ctx || (n && (!particles || !candidate || !gravity_dv)) || memory > SNK_MEM_HOST || !(timestep > 0.0f))
        return fail(ctx, SNK_ERR_INVALID_ARG, "particle_probe: bad arguments");
    API_TRY(set_device(ctx));
    API_TRY(ensure_built(ctx));
    if (n == 0) return SNK_OK;
    Status st;
    const ParticleDev* d_p =
        stage_in<const ParticleDev>(ctx, ctx->q_in, particles, sizeof(snk_particle) * (size_t)n, memory, &st);
    ContactOut* d_c = stage_out<ContactOut>(ctx->q_out, candidate, sizeof(snk_contact) * (size_t)n, memory, &st);
    float* d_g = stage_out<float>(ctx->q_out2, gravity_dv, sizeof(float) * (size_t)n, memory, &st);
    if (!st.ok()) return fail(ctx, st);
    cudaError_t e = launch_particle_probe(scene_dev(ctx), d_p, n, timestep, d_c, d_g, grid_of(ctx, 16), ctx->stream);
    if (e != cudaSuccess) return fail(ctx, SNK_ERR_CUDA, std::string("particle_probe: ") + cudaGetErrorString(e));
    API_TRY(download(ctx, candidate, d_c, sizeof(snk_contact) * (size_t)n, memory));
    API_TRY(download(ctx, gravity_dv, d_g, sizeof(float) * (size_t)n, memory));
    API_TRY(check_device_error(ctx));
    return SNK_OK;
}

int snk_pt_particle_constrain(snk_pt_ctx* ctx, const snk_particle* particles, const float* offsets, uint32_t n,
                              float timestep, float* out, uint32_t memory) {
    if (!ctx || (n && (!particles || !offsets || !out)) || memory > SNK_MEM_HOST || !(timestep > 0.0f))
        return fail(ctx, SNK_ERR_INVALID_ARG, "particle_constrain: bad arguments");
    API_TRY(set_device(ctx));
    API_TRY(ensure_built(ctx));
    if (n == 0) return SNK_OK;
    Status st;
    const ParticleDev* d_p =
        stage_in<const ParticleDev>(ctx, ctx->q_in, particles, sizeof(snk_particle) * (size_t)n, memory, &st);
    const float* d_off = stage_in<const float>(ctx, ctx->q_in2, offsets, 3 * sizeof(float) * (size_t)n, memory, &st);
    float* d_out = stage_out<float>(ctx->q_out, out, 3 * sizeof(float) * (size_t)n, memory, &st);
    if (!st.ok()) return fail(ctx, st);
    cudaError_t e =
        launch_particle_constrain(scene_dev(ctx), d_p, d_off, n, timestep, d_out, grid_of(ctx, 16), ctx->stream);
    if (e != cudaSuccess) return fail(ctx, SNK_ERR_CUDA, std::string("particle_constrain: ") + cudaGetErrorString(e));
    API_TRY(download(ctx, out, d_out, 3 * sizeof(float) * (size_t)n, memory));
    API_TRY(check_device_error(ctx));
    return SNK_OK;
}

int snk_pt_get_stats(const snk_pt_ctx* cctx, snk_pt_stats* out) {
    snk_pt_ctx* ctx = const_cast<snk_pt_ctx*>(cctx);
    if (!ctx || !out) return SNK_ERR_INVALID_ARG;
    std::memset(out, 0, sizeof(*out));
    cudaSetDevice(ctx->device);
    // the first call after a frame reads the error word and build record that the
    // frame copied at its end (later calls read them from the device)
    const bool aux = ctx->aux_pending && ctx->counters_pending;
    ctx->aux_pending = false;
    if (ctx->counters_pending || ctx->timing_pending) {
        if (cudaStreamSynchronize(ctx->stream) != cudaSuccess) return fail(ctx, SNK_ERR_CUDA, "get_stats: sync");
        if (ctx->timing_pending) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
            ctx->last_ms = ms;
            ctx->timing_pending = false;
        }
        ctx->counters_pending = false;
    }
    const uint32_t* c = ctx->h_counters;
    out->cache_queries = ctx->last_mode == SNK_MODE_PATH_CACHE ? c[CNT_CACHE_QUERIES] : 0;
    out->cache_samples = ctx->last_mode == SNK_MODE_PATH_CACHE ? ctx->last_cache_samples : 0;
    out->shadow_tests_reused =
        ctx->last_mode == SNK_MODE_RESTIR_DI || ctx->last_mode == SNK_MODE_RESTIR_PT ? c[CNT_SHADOW_REUSED] : 0;
    if (ctx->last_mode == SNK_MODE_PATH || ctx->last_mode == SNK_MODE_PATH_CACHE ||
        ctx->last_mode == SNK_MODE_RESTIR_PT) {
        out->rays_camera = ctx->last_paths;
        uint64_t ext = 0;
        for (uint32_t d = 1; d < ctx->last_depth; d++) ext += c[CNT_QUEUE + d];
        out->rays_extension = ext;
    } else {
        out->rays_camera = ctx->last_pixels;
    }
    out->rays_shadow = c[CNT_SHADOW_RAYS];
    out->node_visits = ctx->last_count_nodes ? ctx->h_trav[0] : 0;
    out->triangle_tests = ctx->last_count_nodes ? ctx->h_trav[1] : 0;
    out->shadow_node_visits = ctx->last_count_nodes ? ctx->h_trav[2] : 0;
    out->shadow_triangle_tests = ctx->last_count_nodes ? ctx->h_trav[3] : 0;
    if (ctx->prof_pending) {
        for (int k = 0; k < SNK_NUM_STAGES; k++) ctx->stage_ms[k] = 0.0;
        // traversal intervals (closest hits and shadow rays overlap on two streams),
        // as times from the frame's first event, for the union of their spans
        std::vector<std::pair<float, float>> trav;
        for (const auto& iv : ctx->prof_iv) {
            float ms = 0.0f;
            cudaEventElapsedTime(&ms, ctx->prof_ev[iv.begin], ctx->prof_ev[iv.end]);
            ctx->stage_ms[iv.stage] += ms;
            if (iv.stage == SNK_STAGE_TRACE_CLOSEST || iv.stage == SNK_STAGE_TRACE_SHADOW) {
                float t0 = 0.0f, t1 = 0.0f;
                cudaEventElapsedTime(&t0, ctx->prof_ev[0], ctx->prof_ev[iv.begin]);
                cudaEventElapsedTime(&t1, ctx->prof_ev[0], ctx->prof_ev[iv.end]);
                trav.emplace_back(t0, t1);
            }
        }
        std::sort(trav.begin(), trav.end());
        double uni = 0.0;
        float cur0 = 0.0f, cur1 = -1.0f;
        for (const auto& t : trav) {
            if (t.first > cur1) {
                if (cur1 > cur0) uni += cur1 - cur0;
                cur0 = t.first;
                cur1 = t.second;
            } else if (t.second > cur1) {
                cur1 = t.second;
            }
        }
        if (cur1 > cur0) uni += cur1 - cur0;
        ctx->stage_ms[SNK_STAGE_TRACE_ANY] = uni;
        ctx->prof_pending = false;
    }
    for (int k = 0; k < SNK_NUM_STAGES; k++) {
        out->stage_ms[k] = ctx->stage_ms[k];
        out->stage_launches[k] = ctx->stage_launches[k];
    }
    uint64_t tlas_nodes = ctx->tlas_nodes;
    if (ctx->tlas_refittable && ctx->tlas_root != INVALID && ctx->d_small_out.p) {
        if (aux) {
            tlas_nodes = ctx->h_small->num_nodes;
        } else {
            SmallBuildOut r{};
            if (cudaMemcpyAsync(&r, ctx->d_small_out.p, sizeof(r), cudaMemcpyDeviceToHost, ctx->stream) == cudaSuccess &&
                cudaStreamSynchronize(ctx->stream) == cudaSuccess)
                tlas_nodes = r.num_nodes;
        }
    }
    out->wide_nodes = ctx->blas_nodes + tlas_nodes;
    out->triangles = ctx->total_tris;
    out->instances = ctx->instances.size();
    out->blas_sah_cost = ctx->blas_sah;
    out->last_render_ms = ctx->last_ms;
    unsigned e = 0;
    if (aux) e = *ctx->h_err;
    else if (ctx->d_err.p) cudaMemcpy(&e, ctx->d_err.p, sizeof(unsigned), cudaMemcpyDeviceToHost);
    out->device_error = e;
    out->instance_bvh_refits = (uint32_t)ctx->tlas_refits;
    out->graph_launches = ctx->graph_launches;
    out->graph_captures = ctx->graph_captures;
    return SNK_OK;
}

int snk_pt_read_accumulator(snk_pt_ctx* ctx, float* out, uint32_t memory, uint64_t* num_frames) {
    if (!ctx || !out || memory > SNK_MEM_HOST) return fail(ctx, SNK_ERR_INVALID_ARG, "read_accumulator: bad arguments");
    if (!ctx->accum.p || ctx->accum_w == 0) return fail(ctx, SNK_ERR_STATE, "read_accumulator: nothing accumulated");
    API_TRY(set_device(ctx));
    size_t np = (size_t)ctx->accum_w * ctx->accum_h;
    std::vector<double2> h(2 * np);
    if (cudaMemcpyAsync(h.data(), ctx->accum.p, h.size() * sizeof(double2), cudaMemcpyDeviceToHost, ctx->stream) ||
        cudaStreamSynchronize(ctx->stream))
        return fail(ctx, SNK_ERR_CUDA, "read_accumulator: copy");
    std::vector<float> f(4 * np);
    for (size_t i = 0; i < np; i++) {
        double cnt = h[2 * i + 1].y > 0 ? h[2 * i + 1].y : 1.0;
        f[4 * i + 0] = (float)(h[2 * i].x / cnt);
        f[4 * i + 1] = (float)(h[2 * i].y / cnt);
        f[4 * i + 2] = (float)(h[2 * i + 1].x / cnt);
        f[4 * i + 3] = 1.0f;
    }
    if (memory == SNK_MEM_HOST) {
        std::memcpy(out, f.data(), f.size() * sizeof(float));
    } else if (cudaMemcpy(out, f.data(), f.size() * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess) {
        return fail(ctx, SNK_ERR_CUDA, "read_accumulator: upload");
    }
    if (num_frames) *num_frames = ctx->accum_frames;
    return SNK_OK;
}

}  // extern "C"

// ---- read-only access to a context for entry points in other translation units
namespace snk {

bool ctx_view(snk_pt_ctx* ctx, CtxView* out) {
    if (!ctx || !out) return false;
    out->device = ctx->device;
    out->stream = ctx->stream;
    out->num_sms = ctx->num_sms;
    out->built = ctx->built && !ctx->meshes_dirty && !ctx->inst_dirty && !ctx->mats_dirty && !ctx->lights_dirty;
    out->scene = scene_dev(ctx);
    out->h_counters = ctx->h_counters;
    out->h_trav = ctx->h_trav;
    out->tune = trace_tuning(ctx);
    out->tune_any = any_tuning(ctx);
    out->trace_grid = trace_grid(ctx);
    out->any_grid = any_grid(ctx);
    out->shade_grid = shade_grid(ctx);
    return true;
}

int ctx_fail(snk_pt_ctx* ctx, int code, const char* msg) { return fail(ctx, code, msg); }

void ctx_note_render(snk_pt_ctx* ctx, uint32_t mode, uint32_t depth, uint64_t paths, uint64_t pixels, bool counted) {
    ctx->counters_pending = true;
    ctx->timing_pending = false;
    ctx->prof_pending = false;
    ctx->last_mode = mode;
    ctx->last_depth = depth;
    ctx->last_paths = paths;
    ctx->last_pixels = pixels;
    ctx->last_count_nodes = counted ? 1u : 0u;
    for (int k = 0; k < SNK_NUM_STAGES; k++) { ctx->stage_launches[k] = 0; ctx->stage_ms[k] = 0.0; }
    ctx->stage_launches[SNK_STAGE_GENERATE] = 1;
    ctx->stage_launches[SNK_STAGE_TRACE_CLOSEST] = depth;
    ctx->stage_launches[SNK_STAGE_SHADE] = depth;
    ctx->stage_launches[SNK_STAGE_TRACE_SHADOW] = 2 * depth;   // the shadow rays and their accumulation
    ctx->stage_launches[SNK_STAGE_RESOLVE] = 1;
}

}  // namespace snk
