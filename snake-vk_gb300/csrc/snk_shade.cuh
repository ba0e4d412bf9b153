// snk_shade.cuh -- surface interaction, camera rays and light sampling.
//
// Included only by translation units compiled with --fmad=false (see
// snk_device.cuh for the exactness contract).
//
// Reference (file:line in Snake-VK):
//   closest-hit attributes   Core/res/shaders/RayClosestHit.rchit:87-123
//   camera / depth -> world  Core/res/shaders/Util.glsl:1-13 (rays are generated
//                            directly from the view basis here)
//   motion vectors           Core/res/shaders/GBuffer.frag:41-43
//   directional light NEE    Core/res/shaders/RayClosestHit.rchit:127-136
#pragma once
#include "snk_device.cuh"

namespace snk {

// snk_view of include/snk_pt.h
struct ViewParams {
    float pos[3]; float tan_half_fov_y; float forward[3]; float aspect; float right[3]; uint32_t width;
    float up[3]; uint32_t height; float prev_pos[3]; float prev_tan_half_fov_y; float prev_forward[3];
    float prev_aspect; float prev_right[3]; uint32_t prev_valid; float prev_up[3]; uint32_t pad;
};
static_assert(sizeof(ViewParams) == 128, "snk_view layout");

// one view of a batched frame: camera, first global pixel, device outputs
struct ViewDev {
    ViewParams v;
    uint32_t pixel_offset;   // global index of the view's first pixel
    uint32_t pad[3];
    float4* radiance;
    float4* albedo;
    float4* normal;
    float4* position;
    float4* rma;
    float2* motion;
    float* depth;
    uint32_t* mat_flags;
    uint32_t* inst_id;
    uint32_t* prim_id;
    // ReSTIR surface records of the view (null unless the frame's first shading
    // pass writes them): position (w: 1 surface, 2 emissive, 0 miss), shading
    // normal, albedo (w: roughness), (metallic, motion.x, motion.y, 0)
    float4* rs_pos;
    float4* rs_normal;
    float4* rs_albedo;
    float4* rs_misc;
};

struct Surface {
    V3 pos, n, ng, p_obj;
    V3 albedo;
    float roughness, metallic, ao;
    uint32_t flags, inst, prim;
};

// The ReSTIR passes' record of a primary hit (RayGen.rgen:530-556 reads the same
// quantities from the G-buffer)
__device__ __forceinline__ void write_restir_surface(const ViewDev& V, uint32_t o, const Surface& s, float2 mo) {
    const float kind = (s.flags & MAT_EMISSIVE) ? 2.0f : 1.0f;
    V.rs_pos[o] = make_float4(s.pos.x, s.pos.y, s.pos.z, kind);
    V.rs_normal[o] = make_float4(s.n.x, s.n.y, s.n.z, 0.0f);
    V.rs_albedo[o] = make_float4(s.albedo.x, s.albedo.y, s.albedo.z, s.roughness);
    V.rs_misc[o] = make_float4(s.metallic, mo.x, mo.y, 0.0f);
}
__device__ __forceinline__ void write_restir_miss(const ViewDev& V, uint32_t o) {
    const float4 z = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    V.rs_pos[o] = z; V.rs_normal[o] = z; V.rs_albedo[o] = z; V.rs_misc[o] = z;
}

__device__ __forceinline__ Surface surface_at(const SceneDev& S, uint32_t inst, uint32_t prim, float b1, float b2,
                                              V3 ray_dir) {
    const InstShade& I = S.inst_shade[inst];
    const MeshInfo& M = S.meshes[I.mesh_id];
    const uint32_t* ix = S.indices + M.index_offset + 3ull * prim;
    uint32_t i0 = M.vertex_offset + ix[0], i1 = M.vertex_offset + ix[1], i2 = M.vertex_offset + ix[2];
    V3 p0 = load3(S.positions + 3ull * i0), p1 = load3(S.positions + 3ull * i1), p2 = load3(S.positions + 3ull * i2);
    float b0 = (1.0f - b1) - b2;
    V3 p = add(add(mul(p0, b0), mul(p1, b1)), mul(p2, b2));
    V3 ng_obj = cross(sub(p1, p0), sub(p2, p0));
    V3 nn;
    if (M.has_normals) {
        V3 n0 = load3(S.normals + 3ull * i0), n1 = load3(S.normals + 3ull * i1), n2 = load3(S.normals + 3ull * i2);
        nn = add(add(mul(n0, b0), mul(n1, b1)), mul(n2, b2));
    } else {
        nn = ng_obj;
    }
    Surface s;
    s.p_obj = p;
    s.pos = xform_point(I.m, p);
    s.n = normalize(mat3_mul(I.nmat, nn));
    s.ng = normalize(mat3_mul(I.nmat, ng_obj));
    V3 v = neg(ray_dir);
    if (dot(s.ng, v) < 0.0f) s.ng = neg(s.ng);
    if (dot(s.n, v) < 0.0f) s.n = neg(s.n);
    const MaterialDev& m = S.materials[I.material_id];
    s.albedo = load3(m.albedo);
    s.roughness = m.roughness; s.metallic = m.metallic; s.ao = m.ao; s.flags = m.flags;
    s.inst = inst; s.prim = prim;
    return s;
}

__device__ __forceinline__ float2 motion_of(const SceneDev& S, const ViewParams& vw, const Surface& s, uint32_t x,
                                            uint32_t y) {
    const InstShade& I = S.inst_shade[s.inst];
    V3 pp = xform_point(I.pm, s.p_obj);
    V3 rel = sub(pp, load3(vw.prev_pos));
    float z = dot(rel, load3(vw.prev_forward));
    float cu = ((float)x + 0.5f) / (float)vw.width;
    float cv = ((float)y + 0.5f) / (float)vw.height;
    if (!(z > 1e-6f)) return make_float2(0.0f, 0.0f);
    float xn = dot(rel, load3(vw.prev_right)) / (z * (vw.prev_tan_half_fov_y * vw.prev_aspect));
    float yn = dot(rel, load3(vw.prev_up)) / (z * vw.prev_tan_half_fov_y);
    float pu = (xn + 1.0f) * 0.5f;
    float pv = (1.0f - yn) * 0.5f;
    return make_float2(pu - cu, pv - cv);
}

__device__ __forceinline__ V3 camera_dir(const ViewParams& vw, uint32_t x, uint32_t y, float jx, float jy) {
    float fx = ((float)x + jx) / (float)vw.width;
    float fy = ((float)y + jy) / (float)vw.height;
    float sx = fx * 2.0f - 1.0f;
    float sy = 1.0f - fy * 2.0f;
    float px = sx * (vw.tan_half_fov_y * vw.aspect);
    float py = sy * vw.tan_half_fov_y;
    V3 d = v3((vw.forward[0] + vw.right[0] * px) + vw.up[0] * py,
              (vw.forward[1] + vw.right[1] * px) + vw.up[1] * py,
              (vw.forward[2] + vw.right[2] * px) + vw.up[2] * py);
    return normalize(d);
}

__device__ __forceinline__ uint32_t cdf_search(const float* cdf, uint32_t n, float u) {
    uint32_t lo = 0, hi = n - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (u < cdf[mid]) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// NEE toward one local light (sphere light or emissive triangle) chosen by
// power; returns false when the sample carries no contribution.
__device__ __forceinline__ bool sample_local(const SceneDev& S, const Surface& s, V3 v, V3 f0, V3 xb, float u_sel,
                                             float u1, float u2, V3* contrib, V3* sdir, float* stmax) {
    if (S.num_local_lights == 0) return false;
    uint32_t k = cdf_search(S.light_cdf, S.num_local_lights, u_sel);
    float pmf = S.light_pmf[k];
    if (!(pmf > 0.0f)) return false;
    const LocalLight& L = S.local_lights[k];
    V3 l;
    float scale, tmx;
    if (L.kind == 0) {
        V3 c = load3(L.p0);
        float r = L.p1[0];
        V3 dv = sub(c, xb);
        float dist2 = dot(dv, dv);
        float r2 = r * r;
        if (!(dist2 > r2)) return false;
        float dist = sqrtf(dist2);
        V3 w = divs(dv, dist);
        float sin2 = r2 / dist2;
        float cosmax = sqrtf(fmax_(0.0f, 1.0f - sin2));
        float one_minus = sin2 / (1.0f + cosmax);
        float cos_t = 1.0f - u1 * one_minus;
        float sin_t = sqrtf(fmax_(0.0f, 1.0f - cos_t * cos_t));
        float sp, cp;
        sincos2pi(u2, &sp, &cp);
        V3 t1, t2;
        onb(w, &t1, &t2);
        float a = sin_t * cp, b = sin_t * sp;
        l = v3((t1.x * a + t2.x * b) + w.x * cos_t, (t1.y * a + t2.y * b) + w.y * cos_t, (t1.z * a + t2.z * b) + w.z * cos_t);
        float bb = dot(dv, l);
        float disc = r2 - (dist2 - bb * bb);
        float th = bb - sqrtf(fmax_(disc, 0.0f));
        scale = ((2.0f * PI) * one_minus) / pmf;
        tmx = th * 0.999f;
    } else {
        float su = sqrtf(u1);
        float b0 = 1.0f - su;
        float b1 = u2 * su;
        float b2 = (1.0f - b0) - b1;
        V3 q = add(add(mul(load3(L.p0), b0), mul(load3(L.p1), b1)), mul(load3(L.p2), b2));
        V3 dv = sub(q, xb);
        float dist2 = dot(dv, dv);
        if (!(dist2 > 0.0f)) return false;
        float dist = sqrtf(dist2);
        l = divs(dv, dist);
        float cos_l = fabsf(dot(load3(L.n), l));
        if (!(cos_l > 0.0f)) return false;
        scale = (cos_l * L.L[3]) / (dist2 * pmf);
        tmx = dist * 0.999f;
    }
    Terms tm = brdf_terms(l, v, f0, s.n, s.roughness, s.metallic);
    V3 ct = cook_torrance(tm);
    V3 c = v3(((s.albedo.x * ct.x) * L.L[0]) * scale, ((s.albedo.y * ct.y) * L.L[1]) * scale,
              ((s.albedo.z * ct.z) * L.L[2]) * scale);
    if (!(maxc(c) > 0.0f)) return false;
    *contrib = c;
    *sdir = l;
    *stmax = tmx;
    return true;
}

// Continuation direction: with probability p_spec a GGX half-vector sample of
// the reference's DistributionGGX (LightBuffers.glsl:69-80, roughness^2 = alpha),
// otherwise cosine-weighted; weight = albedo * CookTorrance(l) / mixture pdf
// (the reference's BRDF with albedo on both terms, RayGen.rgen:273).
__device__ __forceinline__ bool sample_continuation(const Surface& s, V3 v, V3 f0, float u_lobe, float u1, float u2,
                                                    V3* wi, V3* weight, float* pdf_out) {
    const float p_spec = s.metallic > 0.5f ? 0.75f : 0.25f;
    V3 b1, b2;
    onb(s.n, &b1, &b2);
    float sp, cp;
    sincos2pi(u2, &sp, &cp);
    V3 l;
    if (u_lobe < p_spec) {
        float a = s.roughness * s.roughness;
        float a2 = a * a;
        float cos2 = (1.0f - u1) / (1.0f + (a2 - 1.0f) * u1);
        float ch = sqrtf(cos2);
        float sh = sqrtf(fmax_(0.0f, 1.0f - cos2));
        float hx = sh * cp, hy = sh * sp;
        V3 h = v3((b1.x * hx + b2.x * hy) + s.n.x * ch, (b1.y * hx + b2.y * hy) + s.n.y * ch,
                  (b1.z * hx + b2.z * hy) + s.n.z * ch);
        float vh2 = 2.0f * dot(v, h);
        l = sub(mul(h, vh2), v);
    } else {
        float r = sqrtf(u1);
        float lx = r * cp, ly = r * sp, lz = sqrtf(fmax_(0.0f, 1.0f - u1));
        l = v3((b1.x * lx + b2.x * ly) + s.n.x * lz, (b1.y * lx + b2.y * ly) + s.n.y * lz,
               (b1.z * lx + b2.z * ly) + s.n.z * lz);
    }
    if (!(dot(l, s.ng) > 0.0f)) return false;
    float ndl = dot(s.n, l);
    if (!(ndl > 0.0f)) return false;
    V3 vl = add(v, l);
    float vl2 = dot(vl, vl);
    V3 hh = vl2 > 0.0f ? divs(vl, sqrtf(vl2)) : s.n;
    float D = distribution_ggx(hh, s.n, s.roughness);
    float pdf_spec = (D * fmax_(dot(s.n, hh), 0.0f)) / (4.0f * fmax_(dot(v, hh), 1e-6f));
    float pdf = p_spec * pdf_spec + (1.0f - p_spec) * (ndl / PI);
    if (!(pdf > 0.0f)) return false;
    V3 ct = cook_torrance(brdf_terms(l, v, f0, s.n, s.roughness, s.metallic));
    *weight = v3((s.albedo.x * ct.x) / pdf, (s.albedo.y * ct.y) / pdf, (s.albedo.z * ct.z) / pdf);
    *wi = l;
    *pdf_out = pdf;
    return true;
}

// CalcPointlight (LightBuffers.glsl:147-157)
__device__ __forceinline__ V3 calc_pointlight(const PointLightDev& L, V3 v, V3 f0, V3 world_pos, V3 n, float roughness,
                                              float metallic, V3 albedo) {
    V3 lp = load3(L.pos);
    V3 ftl = sub(lp, world_pos);
    float distance = length(ftl);
    float atten = (L.atten_constant + L.atten_linear * distance) + L.atten_exp * (distance * distance);
    V3 brdf = cook_torrance(brdf_terms(normalize(ftl), v, f0, n, roughness, metallic));
    return v3(((brdf.x * albedo.x) * L.colour[0]) / atten, ((brdf.y * albedo.y) * L.colour[1]) / atten,
              ((brdf.z * albedo.z) * L.colour[2]) / atten);
}

// decode a path index into (view, x, y, sample, global pixel)
__device__ __forceinline__ uint32_t find_view(const ViewDev* views, uint32_t nviews, uint32_t gpix) {
    uint32_t v = 0;
    while (v + 1 < nviews && gpix >= views[v + 1].pixel_offset) v++;
    return v;
}

}  // namespace snk
