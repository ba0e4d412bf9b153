// restir.cu -- the reference's two-pass ReSTIR DI on CUDA.
// Compiled with --fmad=false (exact binary32 operation order, see snk_device.cuh).
//
// Reference: Core/res/shaders/RayGen.rgen
//   PixelReservoir ..................... :64-76 (48 bytes, FP32)
//   Update*Reservoir ................... :215-239
//   TriangleShadowTest / ComputeTriangleRadiance :241-282
//   DoInitialWRS ....................... :296-357 (LIGHT_RIS_ITERS candidates per light kind)
//   CombinePixelReservoir .............. :361-386
//   WriteInitialReservoirs (temporal) .. :411-468 (M cap, normal test 0.95)
//   ComputeAndWriteSpatialReservoirReuse :470-506
//   CalculateRadianceFromReservoirs .... :508-528, main :530-570
// dispatched by RT::RecordRenderCmdBuf (Core/src/rendering/Raytracing.cpp:250-263)
// as two full-screen launches with a barrier between them; here: the initial
// candidates (RIS) kernel, the visibility+temporal kernel and the spatial+shading
// kernel.  The G-buffer (the reference's raster G-buffer pass, read at :534-555) comes
// from the wavefront: camera rays through pixel centres traced by the persistent
// closest-hit kernel, whose first shading pass writes the G-buffer outputs and the
// surface records these passes read.  In the mode that adds path-traced indirect
// light (main, :565-566) the same paths continue from the primary vertex, and the
// final shading adds each surface pixel's indirect light.
//
// Deviations (the CPU oracle makes the same ones):
//   - gold_noise / random() are replaced by PCG32 streams keyed by
//     (pixel, frame, pass, seed); one number per decision, drawn in program order;
//   - the point-light visibility direction of DoInitialWRS (:346) is
//     (pos - biased_pos) / dist (the shader divides only biased_pos);
//   - when temporal reuse is not applied the initial reservoir is written (the
//     shader writes an empty one, :417-467), so the first frame is lit;
//   - neighbour and history normals are fetched at the nearest texel; spatial
//     reuse compares against this frame's normals (the shader samples the
//     previous frame's normal image at :490);
//   - FindNeighbourPixelCoord's unbounded retry loop (:400) is bounded to 8 tries.
//
// Visibility rays are not traced inline: the initial and spatial passes run twice
// (three times for the spatial pass) over the same pixels with the same random
// streams.  The first run records every shadow ray into a per-pixel slot queue
// (the rays' origins, directions and lengths never depend on earlier visibility
// results, and neither does the number of random draws), the queue is traced by
// the persistent any-hit kernel with ray replacement, and the next run replays
// the results in the same order.  The final shading rays depend on which samples
// the spatial reservoir kept, so they form a third queue.
#include "snk_frame.h"
#include "snk_trace.cuh"

namespace snk {
namespace {

constexpr int RBLK = 128;

struct Reservoir {
    float w_sum_pl, w_pl;
    uint32_t pl_idx, pl_m;
    uint32_t em_inst, em_tri;
    float em_u, em_v;
    float w_sum_em, w_em;
    uint32_t m_em, pad;
};
static_assert(sizeof(Reservoir) == 48, "reservoir layout");

__device__ __forceinline__ Reservoir res_init() {
    Reservoir r;
    r.w_sum_pl = 0.0f; r.w_pl = 0.0f; r.pl_idx = INVALID; r.pl_m = 0;
    r.em_inst = INVALID; r.em_tri = INVALID; r.em_u = 0.0f; r.em_v = 0.0f;
    r.w_sum_em = 0.0f; r.w_em = 0.0f; r.m_em = 0; r.pad = 0;
    return r;
}
__device__ __forceinline__ Reservoir res_load(const void* base, uint32_t i) {
    const float4* p = reinterpret_cast<const float4*>(base) + 3ull * i;
    Reservoir r;
    float4* q = reinterpret_cast<float4*>(&r);
    q[0] = p[0]; q[1] = p[1]; q[2] = p[2];
    return r;
}
__device__ __forceinline__ void res_store(void* base, uint32_t i, const Reservoir& r) {
    float4* p = reinterpret_cast<float4*>(base) + 3ull * i;
    const float4* q = reinterpret_cast<const float4*>(&r);
    p[0] = q[0]; p[1] = q[1]; p[2] = q[2];
}

// A shadow test of one pixel and frame is fixed by what its ray is aimed at:
// the origin (the pixel's biased surface point) is the same in every pass, so
// a point light with its distance variant, or an emissive sample (instance,
// triangle, barycentrics), determines the ray bit for bit.  Repeats of a test
// reuse it instead of tracing again: its known result, or its slot in the
// queue being recorded.
constexpr uint32_t MEMO_KNOWN = 0x100;  // answer code: MEMO_KNOWN | visibility, else a slot of the current queue
constexpr uint32_t MEMO_NONE = 0xFFFF;  // plan code of a test that was not made
constexpr int MEMO_PL = 4, MEMO_EM = 4;
// Tests already made for this pixel and frame, by what they aim at: the point
// light tested at its full distance, point lights tested at distance - 0.001,
// and emissive samples (instance, triangle, barycentric bits).
struct Memo {
    uint32_t pla_idx, pla_code;
    uint32_t n_pl, n_em;
    uint32_t pl_idx[MEMO_PL], pl_code[MEMO_PL];
    uint4 em_key[MEMO_EM];
    uint32_t em_code[MEMO_EM];
};
__device__ __forceinline__ void memo_clear(Memo& m) { m.pla_idx = INVALID; m.n_pl = 0; m.n_em = 0; }

// Per-pixel visibility context: records shadow rays into a queue, or replays
// their results, in call order.
struct Ctx {
    const SceneDev* S;
    uint32_t shadow_rays;   // rays recorded by this thread
    uint32_t reused;        // tests answered by an earlier identical test (counted when recording)
    float4* rays;           // recording
    const uint8_t* vis;     // replaying
    size_t base;            // the pixel: slot k is entry base + k * stride
    size_t stride;          // pixels of the view
    uint32_t k, cap;
    bool overflow;
    Memo* m;                // tests made so far (null: no reuse)
    uint32_t last;          // code of the last keyed test: MEMO_KNOWN | visibility or its slot
};

__device__ __forceinline__ void ctx_queue(Ctx& c, const RestirQueue& q, uint32_t pixel, bool record) {
    c.rays = record ? q.rays : nullptr;
    c.vis = record ? nullptr : q.vis;
    c.base = pixel;
    c.stride = q.pixels;
    c.k = 0;
    c.cap = q.per_pixel;
}

// marks the slots a recording pass left unused as empty (tmax < 0)
__device__ __forceinline__ void ctx_close(Ctx& c) {
    if (!c.rays) return;
    for (uint32_t k = c.k; k < c.cap; k++) c.rays[2 * (c.base + k * c.stride) + 1] = make_float4(0.0f, 0.0f, 0.0f, -1.0f);
}

// 1 when the segment is unoccluded (recording: always 1, the value is not used
// for anything the replay would see differently)
__device__ __forceinline__ float shadow_test(Ctx& c, V3 o, V3 d, float tmax) {
    if (c.k >= c.cap) { c.overflow = true; return 0.0f; }
    const size_t slot = c.base + (size_t)c.k++ * c.stride;
    if (c.rays) {
        c.shadow_rays++;
        c.rays[2 * slot] = make_float4(o.x, o.y, o.z, SHADOW_TMIN);
        c.rays[2 * slot + 1] = make_float4(d.x, d.y, d.z, tmax);
        return 1.0f;
    }
    return c.vis[slot] ? 1.0f : 0.0f;
}

// answer of an earlier test (recording: the result is not needed yet)
__device__ __forceinline__ float memo_answer(Ctx& c, uint32_t code) {
    if (c.rays) c.reused++;
    c.last = code;
    if (code & MEMO_KNOWN) return (code & 1u) ? 1.0f : 0.0f;
    return c.rays ? 1.0f : (c.vis[c.base + code * c.stride] ? 1.0f : 0.0f);
}

// shadow test toward point light idx at its full distance (minus == false) or at
// distance - 0.001, reusing an identical earlier test of this pixel
__device__ __forceinline__ float shadow_test_pl(Ctx& c, uint32_t idx, bool minus, V3 o, V3 d, float tmax) {
    Memo* m = c.m;
    if (m) {
        if (!minus && m->pla_idx == idx) return memo_answer(c, m->pla_code);
        if (minus)
            for (uint32_t j = 0; j < m->n_pl; j++)
                if (m->pl_idx[j] == idx) return memo_answer(c, m->pl_code[j]);
    }
    const uint32_t k = c.k;
    const float r = shadow_test(c, o, d, tmax);
    c.last = k;
    if (m && c.k == k + 1) {
        if (!minus) { m->pla_idx = idx; m->pla_code = k; }
        else if (m->n_pl < MEMO_PL) { m->pl_idx[m->n_pl] = idx; m->pl_code[m->n_pl] = k; m->n_pl++; }
    }
    return r;
}

// shadow test toward an emissive sample, reusing an identical earlier test of this pixel
__device__ __forceinline__ float shadow_test_em(Ctx& c, uint4 key, V3 o, V3 d, float tmax) {
    Memo* m = c.m;
    if (m)
        for (uint32_t j = 0; j < m->n_em; j++) {
            const uint4 e = m->em_key[j];
            if (e.x == key.x && e.y == key.y && e.z == key.z && e.w == key.w) return memo_answer(c, m->em_code[j]);
        }
    const uint32_t k = c.k;
    const float r = shadow_test(c, o, d, tmax);
    c.last = k;
    if (m && c.k == k + 1 && m->n_em < MEMO_EM) {
        m->em_key[m->n_em] = key;
        m->em_code[m->n_em] = k;
        m->n_em++;
    }
    return r;
}

__device__ __forceinline__ uint4 key_em(uint32_t inst, uint32_t tri, float u, float v) {
    return make_uint4(inst, tri, __float_as_uint(u), __float_as_uint(v));
}

// after a replay: tests still pointing at slots of the replayed queue get their results
__device__ __forceinline__ uint32_t resolve_code(const Ctx& c, uint32_t code) {
    return (code & MEMO_KNOWN) ? code : (MEMO_KNOWN | (c.vis[c.base + code * c.stride] ? 1u : 0u));
}
__device__ __forceinline__ void memo_resolve(Ctx& c) {
    Memo* m = c.m;
    if (!m || !c.vis) return;
    if (m->pla_idx != INVALID) m->pla_code = resolve_code(c, m->pla_code);
    for (uint32_t j = 0; j < m->n_pl; j++) m->pl_code[j] = resolve_code(c, m->pl_code[j]);
    for (uint32_t j = 0; j < m->n_em; j++) m->em_code[j] = resolve_code(c, m->em_code[j]);
}

// the initial pass's tests of pixel o (all answers known) for the spatial pass:
// 4 uint4 per pixel: (full-distance light, visibility bits, counts, -), the
// indices of up to 4 lights tested at distance - 0.001, and up to 2 emissive keys
__device__ __forceinline__ void memo_store(const Memo& m, const RestirView& R, uint32_t o) {
    const uint32_t npl = m.n_pl < 4u ? m.n_pl : 4u, nem = m.n_em < 2u ? m.n_em : 2u;
    uint32_t vis = (m.pla_idx != INVALID ? (m.pla_code & 1u) : 0u);
    uint4 pl = make_uint4(INVALID, INVALID, INVALID, INVALID);
    uint32_t* plw = &pl.x;
    for (uint32_t j = 0; j < npl; j++) { plw[j] = m.pl_idx[j]; vis |= (m.pl_code[j] & 1u) << (1 + j); }
    for (uint32_t j = 0; j < nem; j++) vis |= (m.em_code[j] & 1u) << (5 + j);
    uint4* dst = R.memo_keys + 4ull * o;
    dst[0] = make_uint4(m.pla_idx, vis, npl | (nem << 8), 0u);
    dst[1] = pl;
    if (nem > 0) dst[2] = m.em_key[0];
    if (nem > 1) dst[3] = m.em_key[1];
}
__device__ __forceinline__ void memo_load(Memo& m, const RestirView& R, uint32_t o) {
    const uint4* src = R.memo_keys + 4ull * o;
    const uint4 h = src[0];
    const uint32_t vis = h.y;
    m.pla_idx = h.x;
    m.pla_code = MEMO_KNOWN | (vis & 1u);
    m.n_pl = min(h.z & 0xFFu, (uint32_t)MEMO_PL);
    m.n_em = min((h.z >> 8) & 0xFFu, 2u);
    const uint4 pl = src[1];
    const uint32_t plw[4] = {pl.x, pl.y, pl.z, pl.w};
    for (uint32_t j = 0; j < m.n_pl; j++) { m.pl_idx[j] = plw[j]; m.pl_code[j] = MEMO_KNOWN | ((vis >> (1 + j)) & 1u); }
    for (uint32_t j = 0; j < m.n_em; j++) { m.em_key[j] = src[2 + j]; m.em_code[j] = MEMO_KNOWN | ((vis >> (5 + j)) & 1u); }
}

// visibility of a test answered by a plan code (a known result or a slot of the replayed queue)
__device__ __forceinline__ float plan_vis(const Ctx& c, uint32_t code) {
    if (code == MEMO_NONE) return 0.0f;   // (phase 2 only asks for tests phase 1 made)
    if (code & MEMO_KNOWN) return (code & 1u) ? 1.0f : 0.0f;
    if (code >= c.cap || !c.vis) return 0.0f;
    return c.vis[c.base + code * c.stride] ? 1.0f : 0.0f;
}

__device__ __forceinline__ void ctx_check(Ctx& c) {
    if (c.overflow && c.S->error_word) atomicOr(c.S->error_word, ERR_BAD_INDEX);
    c.overflow = false;
}

struct Shade { V3 ro, n, albedo, v, f0, biased; float rough, metal; };

__device__ __forceinline__ bool update_pl(Reservoir& r, uint32_t idx, float w, Pcg& rng) {
    r.pl_m++;
    float u = pcg_float(rng);
    r.w_sum_pl = r.w_sum_pl + w;
    if (r.w_sum_pl > 0.0f && u < w / r.w_sum_pl) { r.pl_idx = idx; return true; }
    return false;
}
__device__ __forceinline__ bool update_em(Reservoir& r, uint32_t inst, uint32_t tri, float bu, float bv, float w,
                                          Pcg& rng) {
    r.m_em++;
    float u = pcg_float(rng);
    r.w_sum_em = r.w_sum_em + w;
    if (r.w_sum_em > 0.0f && u < w / r.w_sum_em) {
        r.em_inst = inst; r.em_tri = tri; r.em_u = bu; r.em_v = bv;
        return true;
    }
    return false;
}

__device__ __forceinline__ void tri_point(const SceneDev& S, uint32_t inst, uint32_t tri, float bu, float bv, V3* p,
                                          V3* pn) {
    const InstShade& I = S.inst_shade[inst];
    const MeshInfo& M = S.meshes[I.mesh_id];
    const uint32_t* ix = S.indices + M.index_offset + 3ull * tri;
    uint32_t i0 = M.vertex_offset + ix[0], i1 = M.vertex_offset + ix[1], i2 = M.vertex_offset + ix[2];
    float bz = (1.0f - bu) - bv;
    V3 q0 = load3(S.positions + 3ull * i0), q1 = load3(S.positions + 3ull * i1), q2 = load3(S.positions + 3ull * i2);
    V3 q = add(add(mul(q0, bu), mul(q1, bv)), mul(q2, bz));
    V3 nn;
    if (M.has_normals)
        nn = add(add(mul(load3(S.normals + 3ull * i0), bu), mul(load3(S.normals + 3ull * i1), bv)),
                 mul(load3(S.normals + 3ull * i2), bz));
    else
        nn = cross(sub(q1, q0), sub(q2, q0));
    *p = xform_point(I.m, q);
    *pn = normalize(mat3_mul(I.nmat, nn));
}

__device__ __forceinline__ float tri_shadow(Ctx& c, uint32_t inst, uint32_t tri, float bu, float bv, V3 surface_pos) {
    V3 p, pn;
    tri_point(*c.S, inst, tri, bu, bv, &p, &pn);
    V3 target = add(p, mul(pn, 0.01f));
    float dist = length(sub(surface_pos, target));
    V3 dir = divs(sub(target, surface_pos), dist);
    return shadow_test_em(c, key_em(inst, tri, bu, bv), surface_pos, dir, dist);
}

// ComputeTriangleRadiance without the shadow test: emission of instance inst
// arriving from world point p at the shading point (no light-side cosine)
__device__ __forceinline__ V3 emitted_at(const SceneDev& S, uint32_t inst, V3 p, const Shade& sh) {
    V3 em = load3(S.materials[S.inst_shade[inst].material_id].albedo);
    V3 brdf = cook_torrance(brdf_terms(normalize(sub(p, sh.ro)), sh.v, sh.f0, sh.n, sh.rough, sh.metal));
    V3 dd = sub(sh.ro, p);
    float d2 = fabsf(dot(dd, dd));
    return v3(((em.x * sh.albedo.x) * brdf.x) / d2, ((em.y * sh.albedo.y) * brdf.y) / d2,
              ((em.z * sh.albedo.z) * brdf.z) / d2);
}

// The unshadowed radiance of sample (bu, bv) of the triangle and, when asked
// for, the triangle's world-space area (det(mat3) x object area), from one fetch
// of its vertices (the sample's normal is not needed: no shadow ray is aimed)
__device__ __forceinline__ V3 tri_candidate(const SceneDev& S, uint32_t inst, uint32_t tri, float bu, float bv,
                                         const Shade& sh, float* area) {
    const InstShade& I = S.inst_shade[inst];
    const MeshInfo& M = S.meshes[I.mesh_id];
    const uint32_t* ix = S.indices + M.index_offset + 3ull * tri;
    V3 p0 = load3(S.positions + 3ull * (M.vertex_offset + ix[0]));
    V3 p1 = load3(S.positions + 3ull * (M.vertex_offset + ix[1]));
    V3 p2 = load3(S.positions + 3ull * (M.vertex_offset + ix[2]));
    if (area) *area = (I.det3 * 0.5f) * length(cross(sub(p1, p0), sub(p1, p2)));
    float bz = (1.0f - bu) - bv;
    V3 q = add(add(mul(p0, bu), mul(p1, bv)), mul(p2, bz));
    return emitted_at(S, inst, xform_point(I.m, q), sh);
}

// tri_candidate for an initial RIS candidate, reading the emissive instance's record
__device__ __noinline__ V3 rec_candidate(const SceneDev& S, const EmissiveRec* E, uint32_t tri, float bu, float bv,
                                         const Shade& sh, float* area) {
    const float4* rp = reinterpret_cast<const float4*>(E);
    const float4 r0 = rp[0], r1 = rp[1], r2 = rp[2], r3 = rp[3], r4 = rp[4];
    const float m[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
    const uint32_t index_offset = __float_as_uint(r3.w), vertex_offset = __float_as_uint(r4.x);
    const uint32_t* ix = S.indices + index_offset + 3ull * tri;
    V3 p0 = load3(S.positions + 3ull * (vertex_offset + ix[0]));
    V3 p1 = load3(S.positions + 3ull * (vertex_offset + ix[1]));
    V3 p2 = load3(S.positions + 3ull * (vertex_offset + ix[2]));
    *area = (r3.x * 0.5f) * length(cross(sub(p1, p0), sub(p1, p2)));
    float bz = (1.0f - bu) - bv;
    V3 q = add(add(mul(p0, bu), mul(p1, bv)), mul(p2, bz));
    V3 p = xform_point(m, q);
    V3 em = v3(r4.y, r4.z, r4.w);
    V3 brdf = cook_torrance(brdf_terms(normalize(sub(p, sh.ro)), sh.v, sh.f0, sh.n, sh.rough, sh.metal));
    V3 dd = sub(sh.ro, p);
    float d2 = fabsf(dot(dd, dd));
    return v3(((em.x * sh.albedo.x) * brdf.x) / d2, ((em.y * sh.albedo.y) * brdf.y) / d2,
              ((em.z * sh.albedo.z) * brdf.z) / d2);
}

__device__ __forceinline__ V3 tri_radiance(Ctx& c, uint32_t inst, uint32_t tri, float bu, float bv, const Shade& sh,
                                        bool shadow, V3* unshadowed = nullptr) {
    const SceneDev& S = *c.S;
    V3 p, pn;
    tri_point(S, inst, tri, bu, bv, &p, &pn);
    V3 rad = emitted_at(S, inst, p, sh);
    if (unshadowed) *unshadowed = rad;
    if (shadow) {
        V3 target = add(p, mul(pn, 0.01f));
        float dist = length(sub(sh.biased, target));
        V3 dir = divs(sub(target, sh.biased), dist);
        rad = mul(rad, shadow_test_em(c, key_em(inst, tri, bu, bv), sh.biased, dir, dist));
    }
    return rad;
}

// Unshadowed target values of a pixel's combines, kept between the recording and
// the replaying run of a pass: slot j (the pixel's j-th combine) holds
// (|point-light radiance|, emissive radiance) at p[j * stride].  The recording run
// fills the slots; the replaying run reads them instead of evaluating the lights
// again and only applies the visibility it now knows.
struct ComboSlots {
    float4* p;
    size_t stride;
    uint32_t j, cap;
    bool fill, use;
};

__device__ __forceinline__ void combine(Ctx& c, Reservoir& cur, const Reservoir& nb, float& phat_pl, float& phat_em,
                                     const Shade& sh, Pcg& rng, ComboSlots& cs) {
    const SceneDev& S = *c.S;
    float4* slot = (cs.p && cs.j < cs.cap) ? cs.p + cs.j * cs.stride : nullptr;
    cs.j++;
    const bool use = cs.use && slot;
    float4 cv = use ? *slot : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    const V3 none = v3(0.0f, 0.0f, 0.0f);   // (a replayed test needs no ray)
    if (nb.pl_idx != INVALID) {
        float vis, len;
        if (use) {
            vis = shadow_test_pl(c, nb.pl_idx, true, none, none, 0.0f);
            len = cv.x;
        } else {
            const PointLightDev& L = S.point_lights[nb.pl_idx];
            V3 lp = load3(L.pos);
            float ld = length(sub(lp, sh.biased));
            vis = shadow_test_pl(c, nb.pl_idx, true, sh.biased, divs(sub(lp, sh.biased), ld), ld - 0.001f);
            len = length(calc_pointlight(L, sh.v, sh.f0, sh.ro, sh.n, sh.rough, sh.metal, sh.albedo));
            cv.x = len;
        }
        float p_hat = len * vis;
        float w = (p_hat * (float)nb.pl_m) * nb.w_pl;
        if (update_pl(cur, nb.pl_idx, w, rng)) phat_pl = p_hat;
    }
    if (nb.em_inst != INVALID) {
        V3 rad;
        if (use) {
            rad = mul(v3(cv.y, cv.z, cv.w),
                      shadow_test_em(c, key_em(nb.em_inst, nb.em_tri, nb.em_u, nb.em_v), none, none, 0.0f));
        } else {
            V3 un;
            rad = tri_radiance(c, nb.em_inst, nb.em_tri, nb.em_u, nb.em_v, sh, true, &un);
            cv.y = un.x; cv.z = un.y; cv.w = un.z;
        }
        float p_hat = length(rad);
        float w = (p_hat * nb.w_em) * (float)nb.m_em;
        if (update_em(cur, nb.em_inst, nb.em_tri, nb.em_u, nb.em_v, w, rng)) phat_em = p_hat;
    }
    if (cs.fill && slot) *slot = cv;
}

__device__ __forceinline__ Shade shade_of(const ViewParams& vw, V3 pos, V3 n, V3 albedo, float rough, float metal) {
    Shade sh;
    sh.ro = pos; sh.n = n; sh.albedo = albedo; sh.rough = rough; sh.metal = metal;
    V3 cam = load3(vw.pos);
    sh.v = normalize(sub(cam, pos));
    sh.f0 = f0_of(albedo, metal);
    float bias = 0.01f + fmax_(length(sub(cam, pos)) * 0.001f, 0.01f);
    sh.biased = add(pos, mul(n, bias));
    return sh;
}

__device__ __forceinline__ void flush_rays(uint32_t n, uint32_t* ctr) {
    for (int o = 16; o > 0; o >>= 1) n += __shfl_down_sync(0xFFFFFFFFu, n, o);
    if ((threadIdx.x & 31u) == 0 && n) atomicAdd(ctr, n);
}

// The reservoir passes run 8 resident blocks per SM (64 registers): their light
// and reservoir loads are latency bound and the extra warps outweigh the spills.
// Their helpers (visibility tests, combines, triangle radiance) are inlined: a call
// would keep the per-pixel context, memo and shading state it takes by reference
// in local memory (a kilobyte per thread, which L1 cannot hold for 32 warps).

// initial candidates (RayGen.rgen:296-357): resampled importance sampling of
// 32 point-light and 32 emissive-triangle candidates per surface pixel into the
// pixel's reservoir, with the candidates' target values and the random stream
// position after them (what k_restir_initial continues from).  A kernel of its
// own: it holds no visibility queue or reuse state, so the candidate loops keep
// their values in registers.
__global__ void __launch_bounds__(RBLK, 8) k_restir_ris(FrameParams F, uint32_t vi, RestirView R, RestirSettings rs) {
    const ViewDev& V = F.views[vi];
    const SceneDev& S = F.S;
    const uint32_t W = V.v.width, H = V.v.height, n = W * H;
    // surface pixels are gathered 32 at a time from each warp's pixels (per-warp ring)
    __shared__ uint32_t ring[RBLK / 32][64];
    // the point lights' target values of each thread's pixel (scenes of up to 16 lights)
    constexpr uint32_t RIS_PL_TABLE = 16;
    __shared__ float pl_table[RIS_PL_TABLE * RBLK];
    uint32_t* hq = ring[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t head = 0, cnt = 0;
    for (uint32_t base = blockIdx.x * RBLK + (threadIdx.x & ~31u);; base += gridDim.x * RBLK) {
        const bool more = base < n;
        if (more) {
            const uint32_t o = base + lane;
            const bool surf = o < n && R.g_pos[o].w == 1.0f;
            const unsigned sm = __ballot_sync(0xFFFFFFFFu, surf);
            if (surf) hq[(head + cnt + (uint32_t)__popc(sm & ((1u << lane) - 1u))) & 63u] = o;
            cnt += (uint32_t)__popc(sm);
            __syncwarp();
        }
        while (cnt >= 32u || (!more && cnt > 0u)) {
            const uint32_t take = cnt < 32u ? cnt : 32u;
            const bool have = lane < take;
            const uint32_t o = have ? hq[(head + lane) & 63u] : 0u;
            head = (head + take) & 63u;
            cnt -= take;
            __syncwarp();
            if (!have) continue;
            const float4 gp = R.g_pos[o], gn = R.g_normal[o], ga = R.g_albedo[o], gm = R.g_misc[o];
            const Shade sh = shade_of(V.v, v3(gp.x, gp.y, gp.z), v3(gn.x, gn.y, gn.z), v3(ga.x, ga.y, ga.z), ga.w, gm.x);
            Pcg rng = pcg_stream(V.pixel_offset + o, rs.frame_index, 0x80000001u, rs.seed);
            Reservoir Rr = res_init();
            float phat_pl = 0.0f, phat_em = 0.0f;
            const uint32_t npl = S.num_point_lights;
            if (npl > 0 && npl <= RIS_PL_TABLE && npl < rs.candidates) {
                // every light's target value once, then the candidates look theirs up (the
                // same values: the target is a function of the light and the surface)
                float* ph = pl_table + threadIdx.x;
                for (uint32_t l = 0; l < npl; l++)
                    ph[l * RBLK] = length(calc_pointlight(S.point_lights[l], sh.v, sh.f0, sh.ro, sh.n, sh.rough, sh.metal,
                                                          sh.albedo));
                for (uint32_t i = 0; i < rs.candidates; i++) {
                    uint32_t idx = (uint32_t)(pcg_float(rng) * (float)npl);
                    if (idx > npl - 1) idx = npl - 1;
                    const float p_hat = ph[idx * RBLK];
                    float w = p_hat / (1.0f / (float)npl);
                    if (update_pl(Rr, idx, w, rng)) phat_pl = p_hat;
                }
            } else if (npl > 0) {
                for (uint32_t i = 0; i < rs.candidates; i++) {
                    uint32_t idx = (uint32_t)(pcg_float(rng) * (float)npl);
                    if (idx > npl - 1) idx = npl - 1;
                    float p_hat = length(calc_pointlight(S.point_lights[idx], sh.v, sh.f0, sh.ro, sh.n, sh.rough, sh.metal,
                                                         sh.albedo));
                    float w = p_hat / (1.0f / (float)npl);
                    if (update_pl(Rr, idx, w, rng)) phat_pl = p_hat;
                }
            }
            const uint32_t nem = S.num_emissive_instances;
            if (nem > 0) {
                for (uint32_t i = 0; i < rs.candidates; i++) {
                    uint32_t k = (uint32_t)(pcg_float(rng) * (float)nem);
                    if (k > nem - 1) k = nem - 1;
                    const EmissiveRec* E = S.emissive_recs + k;
                    const uint32_t inst = E->inst, ntri = E->ntri;
                    uint32_t tri = (uint32_t)(pcg_float(rng) * (float)ntri);
                    if (tri > ntri - 1) tri = ntri - 1;
                    float bu = pcg_float(rng), bv = pcg_float(rng);
                    if (bu + bv >= 1.0f) { bu = 1.0f - bu; bv = 1.0f - bv; }
                    float area;
                    V3 rad = rec_candidate(S, E, tri, bu, bv, sh, &area);
                    float p_hat = length(rad);
                    float pdf = 1.0f / ((float)(nem * ntri) * area);
                    float w = p_hat / pdf;
                    if (update_em(Rr, inst, tri, bu, bv, w, rng)) phat_em = p_hat;
                }
            }
            res_store(R.temporal, o, Rr);
            R.ris[2ull * o] = make_float4(phat_pl, phat_em, 0.0f, 0.0f);
            R.ris[2ull * o + 1] =
                make_float4(__uint_as_float((uint32_t)rng.state), __uint_as_float((uint32_t)(rng.state >> 32)),
                            __uint_as_float((uint32_t)rng.inc), __uint_as_float((uint32_t)(rng.inc >> 32)));
        }
        if (!more) break;
    }
}

// WriteInitialReservoirs after the candidates of k_restir_ris: the visibility of
// the RIS samples, then temporal reuse; phase 0 records the visibility rays,
// phase 1 replays their results and writes the temporal reservoirs
template <int PHASE>
__global__ void __launch_bounds__(RBLK, 8) k_restir_initial(FrameParams F, uint32_t vi, RestirView R, RestirSettings rs,
                                                        RestirQueue q) {
    constexpr int phase = PHASE;
    const ViewDev& V = F.views[vi];
    const SceneDev& S = F.S;
    const uint32_t W = V.v.width, H = V.v.height, n = W * H;
    const bool record = phase == 0;
    Ctx c;
    c.S = &F.S; c.shadow_rays = 0; c.reused = 0; c.overflow = false; c.m = nullptr; c.last = MEMO_NONE;
    Memo memo;
    // background pixels end in a first pass over each warp's 32 pixels; surface
    // pixels wait in a per-warp ring and are processed 32 at a time
    __shared__ uint32_t ring[RBLK / 32][64];
    uint32_t* hq = ring[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t head = 0, cnt = 0;
    for (uint32_t base = blockIdx.x * RBLK + (threadIdx.x & ~31u);; base += gridDim.x * RBLK) {
        const bool more = base < n;
        if (more) {
            const uint32_t o = base + lane;
            bool surf = false;
            if (o < n) {
                surf = R.g_pos[o].w == 1.0f;
                if (!surf) {
                    ctx_queue(c, q, o, record);
                    if (record) ctx_close(c);
                    else res_store(R.temporal, o, res_init());
                }
            }
            const unsigned sm = __ballot_sync(0xFFFFFFFFu, surf);
            if (surf) hq[(head + cnt + (uint32_t)__popc(sm & ((1u << lane) - 1u))) & 63u] = o;
            cnt += (uint32_t)__popc(sm);
            __syncwarp();
        }
        while (cnt >= 32u || (!more && cnt > 0u)) {
            const uint32_t take = cnt < 32u ? cnt : 32u;
            const bool have = lane < take;
            const uint32_t o = have ? hq[(head + lane) & 63u] : 0u;
            head = (head + take) & 63u;
            cnt -= take;
            __syncwarp();
            if (!have) continue;
            uint32_t x = o % W, y = o / W;
            ctx_queue(c, q, o, record);
            memo_clear(memo);
            c.m = &memo;
            float4 gp = R.g_pos[o];
            float4 gn = R.g_normal[o], ga = R.g_albedo[o], gm = R.g_misc[o];
            V3 nrm = v3(gn.x, gn.y, gn.z);
            Shade sh = shade_of(V.v, v3(gp.x, gp.y, gp.z), nrm, v3(ga.x, ga.y, ga.z), ga.w, gm.x);
            // the RIS result of k_restir_ris: reservoir, target values and stream position
            Reservoir Rr = res_load(R.temporal, o);
            const float4 ra = R.ris[2ull * o], rb = R.ris[2ull * o + 1];
            const float phat_pl = ra.x, phat_em = ra.y;
            Pcg rng;
            rng.state = ((uint64_t)__float_as_uint(rb.y) << 32) | __float_as_uint(rb.x);
            rng.inc = ((uint64_t)__float_as_uint(rb.w) << 32) | __float_as_uint(rb.z);
            if (Rr.pl_idx != INVALID) {
                V3 lp = load3(S.point_lights[Rr.pl_idx].pos);
                float dist = length(sub(lp, sh.biased));
                float vis = shadow_test_pl(c, Rr.pl_idx, false, sh.biased, divs(sub(lp, sh.biased), dist), dist);
                Rr.w_pl = vis * ((Rr.w_sum_pl / (float)Rr.pl_m) / phat_pl);
            } else {
                Rr.w_pl = 0.0f;
            }
            if (Rr.em_inst != INVALID) {
                float vis = tri_shadow(c, Rr.em_inst, Rr.em_tri, Rr.em_u, Rr.em_v, sh.biased);
                Rr.w_em = vis * ((Rr.w_sum_em / (float)Rr.m_em) / phat_em);
            } else {
                Rr.w_em = 0.0f;
            }
            Reservoir out = Rr;
            if (R.history_valid && rs.temporal != 0 && V.v.prev_valid) {
                float hu = ((float)x + 0.5f) / (float)W + gm.y;
                float hv = ((float)y + 0.5f) / (float)H + gm.z;
                if (hu > 0.0f && hv > 0.0f && hu < 1.0f && hv < 1.0f) {
                    uint32_t hx = (uint32_t)(hu * (float)W), hy = (uint32_t)(hv * (float)H);
                    if (hx > W - 1) hx = W - 1;
                    if (hy > H - 1) hy = H - 1;
                    float4 pn = R.prev_normal[hy * W + hx];
                    if (dot(v3(pn.x, pn.y, pn.z), nrm) > 0.95f) {
                        Reservoir Hh = res_load(R.history, hy * W + hx);
                        // a history of an earlier scene: lights or instances that no longer exist are dropped
                        if (Hh.pl_idx != INVALID && Hh.pl_idx >= S.num_point_lights) Hh.pl_idx = INVALID;
                        if (Hh.em_inst != INVALID && Hh.em_inst >= S.num_instances) Hh.em_inst = INVALID;
                        float mcap = (float)rs.mcap;
                        if ((float)Hh.pl_m > mcap * (float)Rr.pl_m) {
                            Hh.w_sum_pl = Hh.w_sum_pl * ((mcap * (float)Rr.pl_m) / (float)Hh.pl_m);
                            Hh.pl_m = rs.mcap * Rr.pl_m;
                        }
                        if ((float)Hh.m_em > mcap * (float)Rr.m_em) {
                            Hh.w_sum_em = Hh.w_sum_em * ((mcap * (float)Rr.m_em) / (float)Hh.m_em);
                            Hh.m_em = rs.mcap * Rr.m_em;
                        }
                        Reservoir T = res_init();
                        float tp_pl = 0.0f, tp_em = 0.0f;
                        ComboSlots cs{R.combo + o, n, 0u, RESTIR_TEMPORAL_COMBOS, record, !record};
                        combine(c, T, Rr, tp_pl, tp_em, sh, rng, cs);
                        combine(c, T, Hh, tp_pl, tp_em, sh, rng, cs);
                        T.m_em = Hh.m_em + Rr.m_em;
                        T.pl_m = Hh.pl_m + Rr.pl_m;
                        T.w_em = tp_em > 0.0f ? (T.w_sum_em / (float)T.m_em) / tp_em : 0.0f;
                        T.w_pl = tp_pl > 0.0f ? (T.w_sum_pl / (float)T.pl_m) / tp_pl : 0.0f;
                        out = T;
                    }
                }
            }
            ctx_check(c);
            if (record) {
                ctx_close(c);
            } else {
                res_store(R.temporal, o, out);
                memo_resolve(c);
                memo_store(memo, R, o);
            }
        }
        if (!more) break;
    }
    flush_rays(c.shadow_rays, &F.counters[CNT_SHADOW_RAYS]);
    flush_rays(c.reused, &F.counters[CNT_SHADOW_REUSED]);
}

// ComputeAndWriteSpatialReservoirReuse + CalculateRadianceFromReservoirs + main
// phase 0: record q (sun ray, combine rays); phase 1: replay q, write the spatial
// reservoirs, record qs (final shading rays); phase 2: replay q's sun ray and qs,
// write radiance, the FP64 accumulator and the next frame's history normals.
template <int PHASE>
__global__ void __launch_bounds__(RBLK, 8) k_restir_spatial(FrameParams F, uint32_t vi, RestirView R, RestirSettings rs,
                                                        RestirQueue q, RestirQueue qs) {
    constexpr int phase = PHASE;
    const ViewDev& V = F.views[vi];
    const SceneDev& S = F.S;
    const uint32_t W = V.v.width, H = V.v.height, n = W * H;
    Ctx c;
    c.S = &F.S; c.shadow_rays = 0; c.reused = 0; c.overflow = false; c.m = nullptr; c.last = MEMO_NONE;
    Memo memo;
    // radiance, FP64 accumulation and the next frame's history normal of pixel o
    auto write_out = [&](uint32_t o, V3 colour, float4 hist_normal) {
        float4 r4 = make_float4(colour.x, colour.y, colour.z, 1.0f);
        if (V.radiance) V.radiance[o] = r4;
        if (F.accumulate && vi == 0) {
            double2 a0 = F.accum[2ull * o], a1 = F.accum[2ull * o + 1];
            a0.x += (double)r4.x; a0.y += (double)r4.y; a1.x += (double)r4.z; a1.y += 1.0;
            F.accum[2ull * o] = a0;
            F.accum[2ull * o + 1] = a1;
        }
        // this frame's normals become the next frame's history normals (the
        // initial pass of this frame has already consumed the previous ones)
        R.prev_normal[o] = hist_normal;
    };
    // background pixels end in a first pass over each warp's 32 pixels; surface
    // pixels wait in a per-warp ring and are processed 32 at a time
    __shared__ uint32_t ring[RBLK / 32][64];
    uint32_t* hq = ring[threadIdx.x >> 5];
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t head = 0, cnt = 0;
    for (uint32_t base = blockIdx.x * RBLK + (threadIdx.x & ~31u);; base += gridDim.x * RBLK) {
        const bool more = base < n;
        if (more) {
            const uint32_t o = base + lane;
            bool surf = false;
            if (o < n) {
                const float4 gp = R.g_pos[o];
                surf = gp.w == 1.0f;
                if (!surf) {
                    ctx_queue(c, q, o, phase == 0);
                    if (phase == 0) {
                        ctx_close(c);
                    } else if (phase == 1) {
                        res_store(R.spatial, o, res_init());
                        ctx_queue(c, qs, o, true);
                        ctx_close(c);
                    } else {
                        const float4 ga = R.g_albedo[o];
                        write_out(o, gp.w == 2.0f ? v3(ga.x, ga.y, ga.z) : v3(0.0f, 0.0f, 0.0f),
                                  make_float4(0.0f, 0.0f, 0.0f, 0.0f));
                    }
                }
            }
            const unsigned sm = __ballot_sync(0xFFFFFFFFu, surf);
            if (surf) hq[(head + cnt + (uint32_t)__popc(sm & ((1u << lane) - 1u))) & 63u] = o;
            cnt += (uint32_t)__popc(sm);
            __syncwarp();
        }
        while (cnt >= 32u || (!more && cnt > 0u)) {
            const uint32_t take = cnt < 32u ? cnt : 32u;
            const bool have = lane < take;
            const uint32_t o = have ? hq[(head + lane) & 63u] : 0u;
            head = (head + take) & 63u;
            cnt -= take;
            __syncwarp();
            if (!have) continue;
            uint32_t x = o % W, y = o / W;
            float4 gp = R.g_pos[o];
            float4 gn = R.g_normal[o], ga = R.g_albedo[o], gm = R.g_misc[o];
            ctx_queue(c, q, o, phase == 0);
            // the initial pass's tests are known; the combines add theirs (phases 0 and 1 alike)
            c.m = nullptr;
            if (phase < 2) {
                memo_load(memo, R, o);
                c.m = &memo;
            }
            V3 nrm = v3(gn.x, gn.y, gn.z);
            Shade sh = shade_of(V.v, v3(gp.x, gp.y, gp.z), nrm, v3(ga.x, ga.y, ga.z), ga.w, gm.x);
            V3 light = v3(0.0f, 0.0f, 0.0f);
            if (S.dir_light.enabled) {
                V3 cdl = calc_directional(load3(S.dir_light.dir), load3(S.dir_light.colour), sh.v, sh.f0, sh.n, sh.rough,
                                          sh.metal, sh.albedo);
                light = mul(cdl, shadow_test(c, sh.biased, load3(S.dir_light.dir), 1000.0f));
            }
            Reservoir Rr;
            if (phase < 2) {
                Pcg rng = pcg_stream(V.pixel_offset + o, rs.frame_index, 0x80000002u, rs.seed);
                Rr = res_init();
                float phat_pl = 0.0f, phat_em = 0.0f;
                Reservoir self = res_load(R.temporal, o);
                ComboSlots cs{R.combo + (size_t)RESTIR_TEMPORAL_COMBOS * n + o, n, 0u, 1u + (uint32_t)rs.spatial,
                              phase == 0, phase == 1};
                combine(c, Rr, self, phat_pl, phat_em, sh, rng, cs);
                Rr.m_em += self.m_em;
                Rr.pl_m += self.pl_m;
                for (int i = 0; i < rs.spatial; i++) {
                    int nx = -1, ny = -1;
                    for (int tries = 0; tries < 8; tries++) {
                        float ox = ((pcg_float(rng) - 0.5f) * 2.0f) * rs.radius;
                        float oy = ((pcg_float(rng) - 0.5f) * 2.0f) * rs.radius;
                        float fx = (float)x + ox, fy = (float)y + oy;
                        if (fx >= 0.0f && fy >= 0.0f && fx < (float)W && fy < (float)H) { nx = (int)fx; ny = (int)fy; break; }
                    }
                    if (nx < 0) continue;
                    uint32_t qi = (uint32_t)ny * W + (uint32_t)nx;
                    float4 qp = R.g_pos[qi];
                    float4 qn4 = R.g_normal[qi];
                    V3 qn = qp.w == 1.0f ? v3(qn4.x, qn4.y, qn4.z) : v3(0.0f, 0.0f, 0.0f);
                    if (dot(qn, nrm) < 0.95f) continue;
                    Reservoir Q = res_load(R.temporal, qi);
                    combine(c, Rr, Q, phat_pl, phat_em, sh, rng, cs);
                    Rr.m_em += Q.m_em;
                    Rr.pl_m += Q.pl_m;
                }
                Rr.w_em = phat_em > 0.0f ? (Rr.w_sum_em / phat_em) / (float)Rr.m_em : 0.0f;
                Rr.w_pl = phat_pl > 0.0f ? (Rr.w_sum_pl / phat_pl) / (float)Rr.pl_m : 0.0f;
                ctx_check(c);
                if (phase == 0) { ctx_close(c); continue; }
                res_store(R.spatial, o, Rr);
                memo_resolve(c);             // the combines' results are known now
                ctx_queue(c, qs, o, true);   // phase 1 records the final shading rays
            } else {
                Rr = res_load(R.spatial, o);
                ctx_queue(c, qs, o, false);
            }
            // phase 1 makes the final tests (reusing earlier ones) and writes how each is
            // answered; phase 2 reads the answers through that plan
            const uint32_t plan = phase == 2 ? R.plan[o] : 0u;
            uint32_t code_pl = MEMO_NONE, code_em = MEMO_NONE;
            V3 rad = v3(0.0f, 0.0f, 0.0f);
            if (S.num_point_lights > 0 && Rr.pl_idx != INVALID) {
                const PointLightDev& L = S.point_lights[Rr.pl_idx];
                V3 lp = load3(L.pos);
                float ld = length(sub(lp, sh.biased));
                V3 cpl = calc_pointlight(L, sh.v, sh.f0, sh.ro, sh.n, sh.rough, sh.metal, sh.albedo);
                float vis;
                if (phase == 1) {
                    vis = shadow_test_pl(c, Rr.pl_idx, false, sh.biased, divs(sub(lp, sh.biased), ld), ld);
                    code_pl = c.last;
                } else {
                    vis = plan_vis(c, plan & 0xFFFFu);
                }
                cpl = mul(cpl, vis);
                cpl = mul(cpl, Rr.w_pl);
                rad = add(rad, cpl);
            }
            if (S.num_emissive_instances > 0 && Rr.em_inst != INVALID) {
                V3 e;
                if (phase == 1) {
                    e = tri_radiance(c, Rr.em_inst, Rr.em_tri, Rr.em_u, Rr.em_v, sh, true);
                    code_em = c.last;
                } else {
                    e = mul(tri_candidate(S, Rr.em_inst, Rr.em_tri, Rr.em_u, Rr.em_v, sh, nullptr),
                            plan_vis(c, plan >> 16));
                }
                rad = add(rad, mul(e, Rr.w_em));
            }
            ctx_check(c);
            if (phase == 1) {
                R.plan[o] = (code_pl & 0xFFFFu) | (code_em << 16);
                ctx_close(c);
                continue;
            }
            V3 colour = add(light, rad);
            if (R.indirect) {   // main (:565-566): colour_sum = light + indirect (BounceDiffuse's role)
                const float4 ind = R.indirect[o];
                colour = add(colour, v3(ind.x, ind.y, ind.z));
            }
            write_out(o, colour, make_float4(gn.x, gn.y, gn.z, 0.0f));
        }
        if (!more) break;
    }
    flush_rays(c.shadow_rays, &F.counters[CNT_SHADOW_RAYS]);
    flush_rays(c.reused, &F.counters[CNT_SHADOW_REUSED]);
}

}  // namespace

cudaError_t launch_restir_stage(int stage, int phase, const FrameParams& F, uint32_t vi, const RestirView& R,
                                const RestirSettings& rs, const RestirQueue& q, const RestirQueue& qs, int grid,
                                cudaStream_t s) {
    // (one kernel per phase: each keeps only its own phase's paths)
    if (stage == 1 && phase < 0) k_restir_ris<<<grid, RBLK, 0, s>>>(F, vi, R, rs);
    else if (stage == 1 && phase == 0) k_restir_initial<0><<<grid, RBLK, 0, s>>>(F, vi, R, rs, q);
    else if (stage == 1 && phase == 1) k_restir_initial<1><<<grid, RBLK, 0, s>>>(F, vi, R, rs, q);
    else if (stage == 2 && phase == 0) k_restir_spatial<0><<<grid, RBLK, 0, s>>>(F, vi, R, rs, q, qs);
    else if (stage == 2 && phase == 1) k_restir_spatial<1><<<grid, RBLK, 0, s>>>(F, vi, R, rs, q, qs);
    else if (stage == 2 && phase == 2) k_restir_spatial<2><<<grid, RBLK, 0, s>>>(F, vi, R, rs, q, qs);
    else return cudaErrorInvalidValue;
    return cudaGetLastError();
}

}  // namespace snk
