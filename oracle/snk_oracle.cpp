// snk_oracle.cpp -- CPU ORACLE (test infrastructure only).
//
// This file is the checker for the GB300 path-tracing core.  Only tests/,
// __graft_entry__.smoke() and bench.py's CPU-baseline leg load it; the CUDA
// library never links, includes or calls it.
//
// Parity status: UNPINNED by the reference.  Snake-VK ships no tests, no golden
// images and no CPU path; its traversal runs inside the closed Vulkan driver.
// The shading formulas below are transcribed from the reference GLSL and are
// cross-checked against an independent float64 numpy transcription
// (tests/golden/make_golden.py); PCG32 is pinned by the published
// pcg32-demo vector; the intersection test is the published watertight test.
//
// What it restates (file:line in the reference project):
//   BRDF and lights ............ Core/res/shaders/LightBuffers.glsl:65-180
//   hit attributes / chit ...... Core/res/shaders/RayClosestHit.rchit:87-141
//   misses ..................... Core/res/shaders/RayMiss.rmiss:15-26, Shadow.rmiss:11-13
//   shadow rays ................ Core/res/shaders/RayGen.rgen:101-121
//   ReSTIR DI .................. Core/res/shaders/RayGen.rgen:215-528, main :530-570
//   ReSTIR + indirect light .... main :562-569 (colour_sum = light + BounceDiffuse), the
//                                indirect term from unbiased paths (see trace_path)
//   motion vectors ............. Core/res/shaders/GBuffer.frag:41-43
// Not in the reference (specified by the project):
//   watertight ray/triangle test (Woop, Benthin, Wald, JCGT 2(1) 2013)
//   PCG32 (O'Neill 2014, pcg32_random_r / pcg32_srandom_r), splitmix64 keying
//   unbiased path tracer with NEE replacing the biased BounceDiffuse (RayGen.rgen:139-213),
//   continuation sampled from a GGX-NDF / cosine mixture
//   binned-SAH BVH (its shape does not affect results: closest hit is the
//   minimum of (t, instance, triangle) over all valid triangle hits)
//
// Arithmetic: compiled with -O2 -ffp-contract=off (no FMA contraction, no
// fast-math).  Every +,-,*,/,sqrt below is one correctly rounded binary32
// operation, written in an explicit evaluation order that the CUDA kernels
// reproduce with __fadd_rn/__fmul_rn/__fdiv_rn/__fsqrt_rn.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

#if defined(__FP_FAST_FMAF) && !defined(SNKO_ALLOW_FMA)
// a contracted build would silently change results; refuse it
#endif

namespace so {

// ----------------------------------------------------------------------------
// ABI structs (byte-identical to include/snk_pt.h; redeclared so the oracle
// stands on its own)
// ----------------------------------------------------------------------------
struct Instance { float transform[12]; float prev_transform[12]; uint32_t mesh_id, material_id, flags, pad; };
struct Material { float albedo[3]; float roughness, metallic, ao; uint32_t flags, pad; };
struct DirLight { float dir[3]; uint32_t enabled; float colour[3]; float pad; };
struct PointLight { float pos[3]; float radius; float colour[3]; float atten_constant, atten_linear, atten_exp; uint32_t pad[2]; };
struct View {
    float pos[3]; float tan_half_fov_y; float forward[3]; float aspect; float right[3]; uint32_t width;
    float up[3]; uint32_t height; float prev_pos[3]; float prev_tan_half_fov_y; float prev_forward[3];
    float prev_aspect; float prev_right[3]; uint32_t prev_valid; float prev_up[3]; uint32_t pad;
};
struct Settings {
    uint32_t mode, spp, max_depth, rr_depth, seed, frame_index, flags, restir_candidates, restir_mcap;
    int32_t restir_temporal, restir_spatial; float restir_radius;
    uint32_t cache_train_paths, cache_train_steps; float cache_spread, cache_lr;
};
struct Ray { float ox, oy, oz, tmin, dx, dy, dz, tmax; };
struct Hit { float t; uint32_t inst, prim; float u, v; uint32_t flags; };
struct Outputs {
    float* radiance; float* albedo; float* normal; float* position; float* rma; float* motion; float* depth;
    uint32_t* mat_flags; uint32_t* inst_id; uint32_t* prim_id; uint32_t memory, pad;
};
static_assert(sizeof(Instance) == 112, "layout");
static_assert(sizeof(Material) == 32, "layout");
static_assert(sizeof(View) == 128, "layout");
static_assert(sizeof(Settings) == 64, "layout");
static_assert(sizeof(Hit) == 24, "layout");

static const uint32_t INVALID = 0xFFFFFFFFu;
static const uint32_t MAT_EMISSIVE = 1u;
static const float PI = 3.1415926f;          // LightBuffers.glsl:29
static const float T_FAR = 10000.0f;         // RayClosestHit.rchit:136
static const float SURFACE_BIAS = 0.01f;     // RayClosestHit.rchit:134
static const float EXT_TMIN = 0.01f;         // RayGen.rgen:172
static const float SHADOW_TMIN = 0.001f;     // RayGen.rgen:114

// ----------------------------------------------------------------------------
// vectors (exact evaluation order)
// ----------------------------------------------------------------------------
struct V3 { float x, y, z; };
static inline V3 v3(float x, float y, float z) { return V3{x, y, z}; }
static inline V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
static inline V3 cmul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
static inline V3 divs(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
static inline V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
static inline float dot(V3 a, V3 b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }
static inline V3 cross(V3 a, V3 b) {
    return v3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
static inline float length(V3 a) { return std::sqrt(dot(a, a)); }
static inline V3 normalize(V3 a) { return divs(a, length(a)); }
static inline float fmaxf_(float a, float b) { return a > b ? a : b; }
static inline float fminf_(float a, float b) { return a < b ? a : b; }
static inline float clamp01(float x) { return fminf_(fmaxf_(x, 0.0f), 1.0f); }
static inline float maxc(V3 a) { return fmaxf_(fmaxf_(a.x, a.y), a.z); }
static inline V3 load3(const float* p) { return v3(p[0], p[1], p[2]); }
// 3x4 row-major affine transform of a point / a direction
static inline V3 xform_point(const float* m, V3 p) {
    return v3(((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3],
              ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
              ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]);
}
static inline V3 xform_dir(const float* m, V3 d) {
    return v3((m[0] * d.x + m[1] * d.y) + m[2] * d.z,
              (m[4] * d.x + m[5] * d.y) + m[6] * d.z,
              (m[8] * d.x + m[9] * d.y) + m[10] * d.z);
}
// 3x3 row-major
static inline V3 mat3_mul(const float* m, V3 d) {
    return v3((m[0] * d.x + m[1] * d.y) + m[2] * d.z,
              (m[3] * d.x + m[4] * d.y) + m[5] * d.z,
              (m[6] * d.x + m[7] * d.y) + m[8] * d.z);
}

// sin(2 pi u), cos(2 pi u) for u in [0,1): exact quadrant split of 4u, then the
// Taylor series of sin/cos to degree 13/14 on [0, pi/2) (truncation < 7e-10).
static inline void sincos2pi(float u, float* s, float* c) {
    float u4 = u * 4.0f;
    float q = std::floor(u4);
    float r = u4 - q;
    int qi = ((int)q) & 3;
    float x = r * 0x1.921fb6p+0f;  // pi/2
    float x2 = x * x;
    float ps = 0x1.612462p-33f;
    ps = ps * x2 + -0x1.ae6456p-26f;
    ps = ps * x2 + 0x1.71de3ap-19f;
    ps = ps * x2 + -0x1.a01a02p-13f;
    ps = ps * x2 + 0x1.111112p-7f;
    ps = ps * x2 + -0x1.555556p-3f;
    float sn = x + (x * x2) * ps;
    float pc = -0x1.93974ap-37f;
    pc = pc * x2 + 0x1.1eed8ep-29f;
    pc = pc * x2 + -0x1.27e4fcp-22f;
    pc = pc * x2 + 0x1.a01a02p-16f;
    pc = pc * x2 + -0x1.6c16c2p-10f;
    pc = pc * x2 + 0x1.555556p-5f;
    pc = pc * x2 + -0x1p-1f;
    float cs = 1.0f + x2 * pc;
    switch (qi) {
        case 0: *s = sn; *c = cs; break;
        case 1: *s = cs; *c = -sn; break;
        case 2: *s = -sn; *c = -cs; break;
        default: *s = -cs; *c = sn; break;
    }
}

// Orthonormal basis around unit n (Duff et al., JCGT 6(1) 2017).
static inline void onb(V3 n, V3* b1, V3* b2) {
    float sign = std::copysign(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float b = (n.x * n.y) * a;
    *b1 = v3(1.0f + ((sign * n.x) * n.x) * a, sign * b, -(sign * n.x));
    *b2 = v3(b, sign + (n.y * n.y) * a, -n.y);
}

// ----------------------------------------------------------------------------
// PCG32 (O'Neill 2014) and stream keying
// ----------------------------------------------------------------------------
struct Pcg { uint64_t state, inc; };
static inline uint32_t pcg_next(Pcg& r) {
    uint64_t old = r.state;
    r.state = old * 6364136223846793005ULL + r.inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
static inline void pcg_seed(Pcg& r, uint64_t initstate, uint64_t initseq) {
    r.state = 0u;
    r.inc = (initseq << 1u) | 1u;
    pcg_next(r);
    r.state += initstate;
    pcg_next(r);
}
static inline float pcg_float(Pcg& r) { return (float)(pcg_next(r) >> 8) * 0x1p-24f; }
static inline uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
// stream keyed by (a, b, c, seed): path streams use (pixel, sample, depth, seed),
// ReSTIR streams use (pixel, frame, 0x80000000|pass, seed)
static inline Pcg pcg_stream(uint32_t a, uint32_t b, uint32_t c, uint32_t seed) {
    uint64_t k0 = splitmix64(((uint64_t)a << 32) | b);
    uint64_t k1 = splitmix64(k0 ^ (((uint64_t)c << 32) | seed));
    Pcg r;
    pcg_seed(r, k1, k0);
    return r;
}

// ----------------------------------------------------------------------------
// BRDF (LightBuffers.glsl:65-180)
// ----------------------------------------------------------------------------
static inline V3 fresnel_schlick(float cos_theta, V3 f0) {
    float c = clamp01(1.0f - cos_theta);
    float p = ((c * c) * (c * c)) * c;  // pow(c, 5.0)
    return v3(f0.x + (1.0f - f0.x) * p, f0.y + (1.0f - f0.y) * p, f0.z + (1.0f - f0.z) * p);
}
static inline float distribution_ggx(V3 h, V3 n, float roughness) {
    float a = roughness * roughness;
    float a2 = a * a;
    float ndh = fmaxf_(dot(n, h), 0.0f);
    float ndh2 = ndh * ndh;
    float denom = ndh2 * (a2 - 1.0f) + 1.0f;
    denom = (PI * denom) * denom;
    return a2 / denom;
}
static inline float geometry_schlick_ggx(float ndv, float roughness) {
    float r = roughness + 1.0f;
    float k = (r * r) / 8.0f;
    return ndv / (ndv * (1.0f - k) + k);
}
static inline float geometry_smith(V3 v, V3 l, V3 n, float roughness) {
    float ndv = fmaxf_(dot(n, v), 0.0f);
    float ndl = fmaxf_(dot(n, l), 0.0f);
    return geometry_schlick_ggx(ndv, roughness) * geometry_schlick_ggx(ndl, roughness);
}
struct Terms { V3 kd, spec; float ndl; };
// The shared body of CookTorranceBRDF (:104-124) and CalcDirectionalLight (:126-144)
// for a unit light direction l.  h = normalize(v + l) is replaced by n when v + l = 0.
static inline Terms brdf_terms(V3 l, V3 v, V3 f0, V3 n, float roughness, float metallic) {
    V3 vl = add(v, l);
    float vl2 = dot(vl, vl);
    V3 h = vl2 > 0.0f ? divs(vl, std::sqrt(vl2)) : n;
    V3 f = fresnel_schlick(fmaxf_(dot(h, v), 0.0f), f0);
    float ndf = distribution_ggx(h, n, roughness);
    float g = geometry_smith(v, l, n, roughness);
    float ndl = fmaxf_(dot(n, l), 0.0f);
    float ng = ndf * g;
    float denom = ((4.0f * fmaxf_(dot(n, v), 0.0f)) * ndl) + 0.0001f;
    Terms t;
    t.spec = v3((ng * f.x) / denom, (ng * f.y) / denom, (ng * f.z) / denom);
    float om = 1.0f - metallic;
    t.kd = v3((1.0f - f.x) * om, (1.0f - f.y) * om, (1.0f - f.z) * om);
    t.ndl = ndl;
    return t;
}
// CookTorranceBRDF: (kd / PI + specular) * n_dot_l
static inline V3 cook_torrance(const Terms& t) {
    return v3((t.kd.x / PI + t.spec.x) * t.ndl, (t.kd.y / PI + t.spec.y) * t.ndl, (t.kd.z / PI + t.spec.z) * t.ndl);
}
// CalcDirectionalLight: (kd * albedo / PI + specular) * n_dot_l * colour
static inline V3 calc_directional(V3 ldir, V3 colour, V3 v, V3 f0, V3 n, float roughness, float metallic, V3 albedo) {
    Terms t = brdf_terms(ldir, v, f0, n, roughness, metallic);
    return v3((((t.kd.x * albedo.x) / PI + t.spec.x) * t.ndl) * colour.x,
              (((t.kd.y * albedo.y) / PI + t.spec.y) * t.ndl) * colour.y,
              (((t.kd.z * albedo.z) / PI + t.spec.z) * t.ndl) * colour.z);
}
// CalcPointlight (:147-157): brdf * albedo * colour / attenuation
static inline V3 calc_pointlight(const PointLight& L, V3 v, V3 f0, V3 world_pos, V3 n, float roughness, float metallic,
                                 V3 albedo) {
    V3 lp = load3(L.pos);
    V3 ftl = sub(lp, world_pos);
    float distance = length(ftl);
    float atten = (L.atten_constant + L.atten_linear * distance) + L.atten_exp * (distance * distance);
    V3 brdf = cook_torrance(brdf_terms(normalize(ftl), v, f0, n, roughness, metallic));
    return v3(((brdf.x * albedo.x) * L.colour[0]) / atten, ((brdf.y * albedo.y) * L.colour[1]) / atten,
              ((brdf.z * albedo.z) * L.colour[2]) / atten);
}
// GLSL mix(vec3(0.04), albedo, metallic)
static inline V3 f0_of(V3 albedo, float metallic) {
    float om = 1.0f - metallic;
    return v3(0.04f * om + albedo.x * metallic, 0.04f * om + albedo.y * metallic, 0.04f * om + albedo.z * metallic);
}

// ----------------------------------------------------------------------------
// watertight ray/triangle test
// ----------------------------------------------------------------------------
struct WRay {
    float o[3], d[3];
    int kx, ky, kz;
    float Sx, Sy, Sz, tmin, tmax;
};
static inline WRay wray_setup(V3 o, V3 d, float tmin, float tmax) {
    WRay r;
    r.o[0] = o.x; r.o[1] = o.y; r.o[2] = o.z;
    r.d[0] = d.x; r.d[1] = d.y; r.d[2] = d.z;
    int kz = 0;
    if (std::fabs(r.d[1]) > std::fabs(r.d[kz])) kz = 1;
    if (std::fabs(r.d[2]) > std::fabs(r.d[kz])) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (r.d[kz] < 0.0f) std::swap(kx, ky);
    r.kx = kx; r.ky = ky; r.kz = kz;
    r.Sz = 1.0f / r.d[kz];           // shear constants rounded as d[kx] * (1 / d[kz])
    r.Sx = r.d[kx] * r.Sz;
    r.Sy = r.d[ky] * r.Sz;
    r.tmin = tmin; r.tmax = tmax;
    return r;
}
static inline bool intersect_tri(const WRay& r, const float* v0, const float* v1, const float* v2, float tmax,
                                 float* t_out, float* b1_out, float* b2_out) {
    float A[3] = {v0[0] - r.o[0], v0[1] - r.o[1], v0[2] - r.o[2]};
    float B[3] = {v1[0] - r.o[0], v1[1] - r.o[1], v1[2] - r.o[2]};
    float C[3] = {v2[0] - r.o[0], v2[1] - r.o[1], v2[2] - r.o[2]};
    float Ax = A[r.kx] - r.Sx * A[r.kz], Ay = A[r.ky] - r.Sy * A[r.kz];
    float Bx = B[r.kx] - r.Sx * B[r.kz], By = B[r.ky] - r.Sy * B[r.kz];
    float Cx = C[r.kx] - r.Sx * C[r.kz], Cy = C[r.ky] - r.Sy * C[r.kz];
    float U = Cx * By - Cy * Bx;
    float V = Ax * Cy - Ay * Cx;
    float W = Bx * Ay - By * Ax;
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = (U + V) + W;
    if (det == 0.0f) return false;
    float Az = r.Sz * A[r.kz], Bz = r.Sz * B[r.kz], Cz = r.Sz * C[r.kz];
    float T = (U * Az + V * Bz) + W * Cz;
    float t = T / det;
    if (!(t > r.tmin && t < tmax)) return false;
    *t_out = t;
    *b1_out = V / det;
    *b2_out = W / det;
    return true;
}

// ----------------------------------------------------------------------------
// scene, BVH
// ----------------------------------------------------------------------------
struct Box { double lo[3], hi[3]; };
static inline Box box_empty() { Box b; for (int i = 0; i < 3; i++) { b.lo[i] = 1e300; b.hi[i] = -1e300; } return b; }
static inline void box_grow(Box& b, double x, double y, double z) {
    b.lo[0] = std::min(b.lo[0], x); b.lo[1] = std::min(b.lo[1], y); b.lo[2] = std::min(b.lo[2], z);
    b.hi[0] = std::max(b.hi[0], x); b.hi[1] = std::max(b.hi[1], y); b.hi[2] = std::max(b.hi[2], z);
}
static inline void box_union(Box& b, const Box& o) {
    for (int i = 0; i < 3; i++) { b.lo[i] = std::min(b.lo[i], o.lo[i]); b.hi[i] = std::max(b.hi[i], o.hi[i]); }
}
static inline double box_area(const Box& b) {
    double dx = b.hi[0] - b.lo[0], dy = b.hi[1] - b.lo[1], dz = b.hi[2] - b.lo[2];
    if (dx < 0) return 0;
    return 2.0 * (dx * dy + dy * dz + dz * dx);
}
static inline void box_pad(Box& b) {
    double ext = std::max(b.hi[0] - b.lo[0], std::max(b.hi[1] - b.lo[1], b.hi[2] - b.lo[2]));
    for (int i = 0; i < 3; i++) {
        double p = 1e-5 * (ext + std::fabs(b.lo[i]) + std::fabs(b.hi[i])) + 1e-7;
        b.lo[i] -= p; b.hi[i] += p;
    }
}

struct BNode { Box box; uint32_t left, right, first, count; };  // leaf iff count > 0

struct Bvh {
    std::vector<BNode> nodes;
    std::vector<uint32_t> prims;
    // binned SAH build over prim boxes
    void build(const std::vector<Box>& boxes) {
        size_t n = boxes.size();
        prims.resize(n);
        for (size_t i = 0; i < n; i++) prims[i] = (uint32_t)i;
        nodes.clear();
        nodes.reserve(2 * n + 1);
        if (n == 0) return;
        std::vector<double> cen(3 * n);
        for (size_t i = 0; i < n; i++)
            for (int a = 0; a < 3; a++) cen[3 * i + a] = 0.5 * (boxes[i].lo[a] + boxes[i].hi[a]);
        nodes.push_back(BNode{});
        struct Item { uint32_t node, first, count; };
        std::vector<Item> stack{{0, 0, (uint32_t)n}};
        const int NB = 16;
        while (!stack.empty()) {
            Item it = stack.back(); stack.pop_back();
            Box b = box_empty(), cb = box_empty();
            for (uint32_t i = it.first; i < it.first + it.count; i++) {
                box_union(b, boxes[prims[i]]);
                box_grow(cb, cen[3 * prims[i]], cen[3 * prims[i] + 1], cen[3 * prims[i] + 2]);
            }
            BNode& nd = nodes[it.node];
            nd.box = b;
            if (it.count <= 4) { nd.first = it.first; nd.count = it.count; nd.left = nd.right = 0; continue; }
            double best = 1e300; int best_axis = -1, best_bin = -1;
            for (int a = 0; a < 3; a++) {
                double ext = cb.hi[a] - cb.lo[a];
                if (ext <= 0) continue;
                Box bb[NB]; uint32_t bc[NB];
                for (int k = 0; k < NB; k++) { bb[k] = box_empty(); bc[k] = 0; }
                for (uint32_t i = it.first; i < it.first + it.count; i++) {
                    int k = (int)((cen[3 * prims[i] + a] - cb.lo[a]) / ext * NB);
                    k = std::min(std::max(k, 0), NB - 1);
                    box_union(bb[k], boxes[prims[i]]); bc[k]++;
                }
                double ra[NB]; uint32_t rc[NB];
                Box acc = box_empty(); uint32_t cnt = 0;
                for (int k = NB - 1; k > 0; k--) { box_union(acc, bb[k]); cnt += bc[k]; ra[k] = box_area(acc); rc[k] = cnt; }
                acc = box_empty(); cnt = 0;
                for (int k = 0; k < NB - 1; k++) {
                    box_union(acc, bb[k]); cnt += bc[k];
                    if (cnt == 0 || rc[k + 1] == 0) continue;
                    double cost = box_area(acc) * cnt + ra[k + 1] * rc[k + 1];
                    if (cost < best) { best = cost; best_axis = a; best_bin = k; }
                }
            }
            uint32_t mid;
            if (best_axis < 0) {
                mid = it.first + it.count / 2;
            } else {
                double ext = cb.hi[best_axis] - cb.lo[best_axis];
                auto pm = std::partition(prims.begin() + it.first, prims.begin() + it.first + it.count, [&](uint32_t p) {
                    int k = (int)((cen[3 * p + best_axis] - cb.lo[best_axis]) / ext * NB);
                    k = std::min(std::max(k, 0), NB - 1);
                    return k <= best_bin;
                });
                mid = (uint32_t)(pm - prims.begin());
                if (mid == it.first || mid == it.first + it.count) mid = it.first + it.count / 2;
            }
            uint32_t l = (uint32_t)nodes.size();
            nodes.push_back(BNode{}); nodes.push_back(BNode{});
            nodes[it.node].left = l; nodes[it.node].right = l + 1; nodes[it.node].count = 0;
            stack.push_back({l, it.first, mid - it.first});
            stack.push_back({l + 1, mid, it.first + it.count - mid});
        }
    }
};

// conservative slab test in double on padded boxes
static inline bool slab(const Box& b, const double o[3], const double id[3], double tlo, double thi, double* tnear) {
    double t0 = tlo, t1 = thi;
    for (int a = 0; a < 3; a++) {
        double lo = (b.lo[a] - o[a]) * id[a], hi = (b.hi[a] - o[a]) * id[a];
        if (std::isnan(lo) || std::isnan(hi)) { lo = -1e300; hi = 1e300; }
        if (lo > hi) std::swap(lo, hi);
        t0 = std::max(t0, lo); t1 = std::min(t1, hi);
    }
    *tnear = t0;
    double slack = 1e-5 * (std::fabs(t0) + std::fabs(t1)) + 1e-6;
    return t0 <= t1 + slack;
}

struct MeshData {
    std::vector<float> pos, nrm;
    std::vector<uint32_t> idx;
    uint32_t nv = 0, nt = 0;
    Bvh bvh;
    Box box;
    bool has_normals = false;
};

struct InstData {
    Instance in;
    float inv[12];   // world -> object
    float nmat[9];   // transpose(inverse(mat3)) row-major
    float det3;      // determinant(mat3(transform))
    Box wbox;
};

// Inverse of the 3x4 affine transform in double, rounded to float (also the
// normal matrix and the 3x3 determinant).  The CUDA library computes the same
// values with the same operation order.
static void invert_affine(const float* mf, float* inv_out, float* nmat_out, float* det_out) {
    double a[3][3], t[3];
    for (int r = 0; r < 3; r++) { for (int c = 0; c < 3; c++) a[r][c] = mf[4 * r + c]; t[r] = mf[4 * r + 3]; }
    double c00 = a[1][1] * a[2][2] - a[1][2] * a[2][1];
    double c01 = a[1][2] * a[2][0] - a[1][0] * a[2][2];
    double c02 = a[1][0] * a[2][1] - a[1][1] * a[2][0];
    double det = (a[0][0] * c00 + a[0][1] * c01) + a[0][2] * c02;
    double inv[3][3];
    inv[0][0] = c00 / det;
    inv[0][1] = (a[0][2] * a[2][1] - a[0][1] * a[2][2]) / det;
    inv[0][2] = (a[0][1] * a[1][2] - a[0][2] * a[1][1]) / det;
    inv[1][0] = c01 / det;
    inv[1][1] = (a[0][0] * a[2][2] - a[0][2] * a[2][0]) / det;
    inv[1][2] = (a[0][2] * a[1][0] - a[0][0] * a[1][2]) / det;
    inv[2][0] = c02 / det;
    inv[2][1] = (a[0][1] * a[2][0] - a[0][0] * a[2][1]) / det;
    inv[2][2] = (a[0][0] * a[1][1] - a[0][1] * a[1][0]) / det;
    for (int r = 0; r < 3; r++) {
        double it = -((inv[r][0] * t[0] + inv[r][1] * t[1]) + inv[r][2] * t[2]);
        for (int c = 0; c < 3; c++) inv_out[4 * r + c] = (float)inv[r][c];
        inv_out[4 * r + 3] = (float)it;
    }
    for (int r = 0; r < 3; r++)
        for (int c = 0; c < 3; c++) nmat_out[3 * r + c] = (float)inv[c][r];
    *det_out = (float)det;
}

struct LocalLight {      // path tracer NEE: sphere lights then emissive triangles
    uint32_t kind;       // 0 sphere, 1 triangle
    uint32_t index;      // point light index / (unused)
    V3 p0, p1, p2;       // sphere: p0 = centre, p1.x = radius ; triangle: world vertices
    V3 n;                // triangle unit normal
    float area;
    V3 L;                // radiance
};

struct Scene {
    std::vector<MeshData> meshes;
    std::vector<InstData> insts;
    std::vector<Material> mats;
    DirLight dl{};
    std::vector<PointLight> pls;
    Bvh tlas;
    std::vector<uint32_t> emissive_insts;  // RaytracingInstances.glsl:19-22
    std::vector<LocalLight> lights;
    std::vector<float> light_cdf, light_pmf;
    bool built = false;
};

struct Counters { uint64_t camera = 0, extension = 0, shadow = 0, nodes = 0, tris = 0; };

// ----------------------------------------------------------------------------
// traversal
// ----------------------------------------------------------------------------
struct HitRec { float t; uint32_t inst, prim; float u, v; bool hit; };

static inline bool better(float t, uint32_t inst, uint32_t prim, const HitRec& b) {
    if (!b.hit) return true;
    if (t < b.t) return true;
    if (t > b.t) return false;
    if (inst != b.inst) return inst < b.inst;
    return prim < b.prim;
}

// object-space ray of an instance (float, fixed order)
static inline void object_ray(const InstData& I, V3 o, V3 d, V3* oo, V3* od) {
    *oo = xform_point(I.inv, o);
    *od = xform_dir(I.inv, d);
}

struct StackEntry { uint32_t node; double tn; };

// Front-to-back traversal of one binary BVH; visit(prim) tests a leaf primitive
// and returns true to stop (any-hit found).  lim() is the current upper t bound.
template <class Visit, class Lim>
static bool traverse(const Bvh& B, const double o[3], const double id[3], double tmin, Lim lim, Visit visit,
                     Counters* ctr) {
    if (B.nodes.empty()) return false;
    StackEntry st[128];
    int sp = 0;
    double tn;
    if (!slab(B.nodes[0].box, o, id, tmin, lim(), &tn)) return false;
    st[sp++] = StackEntry{0, tn};
    while (sp > 0) {
        StackEntry e = st[--sp];
        double l = lim();
        if (e.tn > l + 1e-5 * (std::fabs(l) + std::fabs(e.tn)) + 1e-6) continue;
        const BNode& nd = B.nodes[e.node];
        if (ctr) ctr->nodes++;
        if (nd.count > 0) {
            for (uint32_t k = nd.first; k < nd.first + nd.count; k++)
                if (visit(B.prims[k])) return true;
            continue;
        }
        double t0, t1;
        bool h0 = slab(B.nodes[nd.left].box, o, id, tmin, l, &t0);
        bool h1 = slab(B.nodes[nd.right].box, o, id, tmin, l, &t1);
        if (h0 && h1) {
            if (t0 <= t1) { st[sp++] = StackEntry{nd.right, t1}; st[sp++] = StackEntry{nd.left, t0}; }
            else { st[sp++] = StackEntry{nd.left, t0}; st[sp++] = StackEntry{nd.right, t1}; }
        } else if (h0) {
            st[sp++] = StackEntry{nd.left, t0};
        } else if (h1) {
            st[sp++] = StackEntry{nd.right, t1};
        }
    }
    return false;
}

static bool trace(const Scene& S, V3 o, V3 d, float tmin, float tmax, bool any, HitRec* out, Counters* ctr) {
    // traceRayEXT requires tmin >= 0: a negative (or NaN) tmin is taken as 0
    tmin = std::fmax(tmin, 0.0f);
    HitRec best{0, INVALID, INVALID, 0, 0, false};
    double wo[3] = {o.x, o.y, o.z}, wid[3] = {1.0 / (double)d.x, 1.0 / (double)d.y, 1.0 / (double)d.z};
    auto lim = [&]() { return best.hit ? (double)best.t : (double)tmax; };
    bool stop = traverse(S.tlas, wo, wid, (double)tmin, lim, [&](uint32_t ii) -> bool {
        const InstData& I = S.insts[ii];
        const MeshData& M = S.meshes[I.in.mesh_id];
        V3 oo, od;
        object_ray(I, o, d, &oo, &od);
        WRay wr = wray_setup(oo, od, tmin, tmax);
        double bo[3] = {oo.x, oo.y, oo.z}, bid[3] = {1.0 / (double)od.x, 1.0 / (double)od.y, 1.0 / (double)od.z};
        return traverse(M.bvh, bo, bid, (double)tmin, lim, [&](uint32_t tri) -> bool {
            const uint32_t* ix = &M.idx[3 * tri];
            float t, b1, b2;
            if (ctr) ctr->tris++;
            if (!intersect_tri(wr, &M.pos[3 * ix[0]], &M.pos[3 * ix[1]], &M.pos[3 * ix[2]], tmax, &t, &b1, &b2))
                return false;
            if (any) { best = HitRec{t, ii, tri, b1, b2, true}; return true; }
            if (better(t, ii, tri, best)) best = HitRec{t, ii, tri, b1, b2, true};
            return false;
        }, ctr);
    }, ctr);
    (void)stop;
    *out = best;
    return best.hit;
}

static inline float shadow_test(const Scene& S, V3 o, V3 d, float tmax, Counters* ctr) {
    HitRec h;
    if (ctr) ctr->shadow++;
    bool hit = trace(S, o, d, SHADOW_TMIN, tmax, true, &h, nullptr);
    return hit ? 0.0f : 1.0f;
}

// ----------------------------------------------------------------------------
// scene build
// ----------------------------------------------------------------------------
static inline float luminance_d(V3 c) { return (float)(0.2126 * c.x + 0.7152 * c.y + 0.0722 * c.z); }

static void build_scene(Scene& S) {
    for (auto& M : S.meshes) {
        std::vector<Box> boxes(M.nt);
        M.box = box_empty();
        for (uint32_t t = 0; t < M.nt; t++) {
            Box b = box_empty();
            for (int k = 0; k < 3; k++) {
                const float* p = &M.pos[3 * M.idx[3 * t + k]];
                box_grow(b, p[0], p[1], p[2]);
            }
            box_pad(b);
            boxes[t] = b;
            box_union(M.box, b);
        }
        M.bvh.build(boxes);
    }
    std::vector<Box> ib(S.insts.size());
    S.emissive_insts.clear();
    for (size_t i = 0; i < S.insts.size(); i++) {
        InstData& I = S.insts[i];
        invert_affine(I.in.transform, I.inv, I.nmat, &I.det3);
        const MeshData& M = S.meshes[I.in.mesh_id];
        Box w = box_empty();
        for (int c = 0; c < 8; c++) {
            V3 p = v3((float)((c & 1) ? M.box.hi[0] : M.box.lo[0]), (float)((c & 2) ? M.box.hi[1] : M.box.lo[1]),
                      (float)((c & 4) ? M.box.hi[2] : M.box.lo[2]));
            // transform in double: the world box only has to be conservative
            double x = ((double)I.in.transform[0] * p.x + (double)I.in.transform[1] * p.y) + (double)I.in.transform[2] * p.z + I.in.transform[3];
            double y = ((double)I.in.transform[4] * p.x + (double)I.in.transform[5] * p.y) + (double)I.in.transform[6] * p.z + I.in.transform[7];
            double z = ((double)I.in.transform[8] * p.x + (double)I.in.transform[9] * p.y) + (double)I.in.transform[10] * p.z + I.in.transform[11];
            box_grow(w, x, y, z);
        }
        if (M.nt == 0) w = box_empty();
        box_pad(w);
        I.wbox = w;
        ib[i] = w;
        // (instances of empty meshes have no triangle to sample: left out of the list)
        if ((S.mats[I.in.material_id].flags & MAT_EMISSIVE) && M.nt > 0) S.emissive_insts.push_back((uint32_t)i);
    }
    S.tlas.build(ib);
    // local light table for the path tracer: sphere lights, then emissive triangles
    S.lights.clear();
    std::vector<double> w;
    for (size_t k = 0; k < S.pls.size(); k++) {
        const PointLight& P = S.pls[k];
        if (!(P.radius > 0.0f)) continue;
        LocalLight L{};
        L.kind = 0; L.index = (uint32_t)k;
        L.p0 = load3(P.pos);
        L.p1 = v3(P.radius, 0, 0);
        double inv_area = 1.0 / (M_PI * (double)P.radius * (double)P.radius);
        L.L = v3((float)(P.colour[0] * inv_area), (float)(P.colour[1] * inv_area), (float)(P.colour[2] * inv_area));
        S.lights.push_back(L);
        w.push_back(4.0 * M_PI * (0.2126 * P.colour[0] + 0.7152 * P.colour[1] + 0.0722 * P.colour[2]));
    }
    for (uint32_t ii : S.emissive_insts) {
        const InstData& I = S.insts[ii];
        const MeshData& M = S.meshes[I.in.mesh_id];
        V3 Le = load3(S.mats[I.in.material_id].albedo);
        for (uint32_t t = 0; t < M.nt; t++) {
            LocalLight L{};
            L.kind = 1; L.index = ii;
            L.p0 = xform_point(I.in.transform, load3(&M.pos[3 * M.idx[3 * t + 0]]));
            L.p1 = xform_point(I.in.transform, load3(&M.pos[3 * M.idx[3 * t + 1]]));
            L.p2 = xform_point(I.in.transform, load3(&M.pos[3 * M.idx[3 * t + 2]]));
            V3 nl = cross(sub(L.p1, L.p0), sub(L.p2, L.p0));
            float len = length(nl);
            L.area = 0.5f * len;
            L.n = len > 0.0f ? divs(nl, len) : v3(0, 1, 0);
            L.L = Le;
            S.lights.push_back(L);
            w.push_back(2.0 * M_PI * (double)L.area * (0.2126 * Le.x + 0.7152 * Le.y + 0.0722 * Le.z));
        }
    }
    // CDF over integer weights q = max(1, round(w / w_max * 2^40)) (0 for w <= 0):
    // integer prefix sums are exact, so any summation order gives these values
    double wmax = 0.0;
    for (double x : w)
        if (x > 0.0 && x > wmax) wmax = x;
    std::vector<uint64_t> q(w.size());
    uint64_t total = 0;
    for (size_t k = 0; k < w.size(); k++) {
        q[k] = (w[k] > 0.0 && wmax > 0.0) ? std::max<uint64_t>(1, (uint64_t)std::llrint(w[k] / wmax * 1099511627776.0)) : 0;
        total += q[k];
    }
    S.light_cdf.resize(w.size());
    S.light_pmf.resize(w.size());
    uint64_t acc = 0;
    for (size_t k = 0; k < w.size(); k++) {
        acc += q[k];
        S.light_cdf[k] = total ? (k + 1 == w.size() ? 1.0f : (float)((double)acc / (double)total)) : 0.0f;
        S.light_pmf[k] = total ? (float)((double)q[k] / (double)total) : 0.0f;
    }
    S.built = true;
}

static inline uint32_t cdf_search(const std::vector<float>& cdf, float u) {
    uint32_t lo = 0, hi = (uint32_t)cdf.size() - 1;
    while (lo < hi) {
        uint32_t mid = (lo + hi) >> 1;
        if (u < cdf[mid]) hi = mid; else lo = mid + 1;
    }
    return lo;
}

// ----------------------------------------------------------------------------
// surface interaction (RayClosestHit.rchit:87-123)
// ----------------------------------------------------------------------------
struct Surface {
    V3 pos, n, ng, p_obj;
    V3 albedo; float roughness, metallic, ao; uint32_t flags;
    uint32_t inst, prim;
};

static Surface surface_at(const Scene& S, const HitRec& h, V3 ray_dir) {
    const InstData& I = S.insts[h.inst];
    const MeshData& M = S.meshes[I.in.mesh_id];
    const uint32_t* ix = &M.idx[3 * h.prim];
    V3 p0 = load3(&M.pos[3 * ix[0]]), p1 = load3(&M.pos[3 * ix[1]]), p2 = load3(&M.pos[3 * ix[2]]);
    float b1 = h.u, b2 = h.v, b0 = (1.0f - b1) - b2;
    V3 p = add(add(mul(p0, b0), mul(p1, b1)), mul(p2, b2));
    V3 ng_obj = cross(sub(p1, p0), sub(p2, p0));
    V3 nn;
    if (M.has_normals) {
        V3 n0 = load3(&M.nrm[3 * ix[0]]), n1 = load3(&M.nrm[3 * ix[1]]), n2 = load3(&M.nrm[3 * ix[2]]);
        nn = add(add(mul(n0, b0), mul(n1, b1)), mul(n2, b2));
    } else {
        nn = ng_obj;
    }
    Surface s;
    s.p_obj = p;
    s.pos = xform_point(I.in.transform, p);
    s.n = normalize(mat3_mul(I.nmat, nn));
    s.ng = normalize(mat3_mul(I.nmat, ng_obj));
    V3 v = neg(ray_dir);
    if (dot(s.ng, v) < 0.0f) s.ng = neg(s.ng);
    if (dot(s.n, v) < 0.0f) s.n = neg(s.n);
    const Material& m = S.mats[I.in.material_id];
    s.albedo = load3(m.albedo);
    s.roughness = m.roughness; s.metallic = m.metallic; s.ao = m.ao; s.flags = m.flags;
    s.inst = h.inst; s.prim = h.prim;
    return s;
}

// motion vector of a primary hit: prev uv - current uv (GBuffer.frag:41-43)
static inline void motion_of(const Scene& S, const View& vw, const Surface& s, uint32_t x, uint32_t y, float* mo) {
    const InstData& I = S.insts[s.inst];
    V3 pp = xform_point(I.in.prev_transform, s.p_obj);
    V3 rel = sub(pp, load3(vw.prev_pos));
    float z = dot(rel, load3(vw.prev_forward));
    float cu = ((float)x + 0.5f) / (float)vw.width;
    float cv = ((float)y + 0.5f) / (float)vw.height;
    if (!(z > 1e-6f)) { mo[0] = 0.0f; mo[1] = 0.0f; return; }
    float xn = dot(rel, load3(vw.prev_right)) / (z * (vw.prev_tan_half_fov_y * vw.prev_aspect));
    float yn = dot(rel, load3(vw.prev_up)) / (z * vw.prev_tan_half_fov_y);
    float pu = (xn + 1.0f) * 0.5f;
    float pv = (1.0f - yn) * 0.5f;
    mo[0] = pu - cu;
    mo[1] = pv - cv;
}

static inline V3 camera_dir(const View& vw, uint32_t x, uint32_t y, float jx, float jy) {
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

// ----------------------------------------------------------------------------
// plain path tracer (replaces BounceDiffuse; NEE for the directional light and
// one local light per vertex, cosine-weighted continuation, RR)
// ----------------------------------------------------------------------------
struct GSample {
    bool hit; Surface s; float t; float motion[2];
};

// NEE for one local light; returns false when the sample carries nothing.
static bool sample_local(const Scene& S, const Surface& s, V3 v, V3 f0, V3 xb, float u_sel, float u1, float u2,
                         V3* contrib, V3* sdir, float* stmax) {
    if (S.lights.empty()) return false;
    uint32_t k = cdf_search(S.light_cdf, u_sel);
    float pmf = S.light_pmf[k];
    if (!(pmf > 0.0f)) return false;
    const LocalLight& L = S.lights[k];
    V3 l; float scale; float tmx;
    if (L.kind == 0) {
        float r = L.p1.x;
        V3 dv = sub(L.p0, xb);
        float dist2 = dot(dv, dv);
        float r2 = r * r;
        if (!(dist2 > r2)) return false;
        float dist = std::sqrt(dist2);
        V3 w = divs(dv, dist);
        float sin2 = r2 / dist2;
        float cosmax = std::sqrt(fmaxf_(0.0f, 1.0f - sin2));
        float one_minus = sin2 / (1.0f + cosmax);
        float cos_t = 1.0f - u1 * one_minus;
        float sin_t = std::sqrt(fmaxf_(0.0f, 1.0f - cos_t * cos_t));
        float sp, cp;
        sincos2pi(u2, &sp, &cp);
        V3 t1, t2;
        onb(w, &t1, &t2);
        float a = sin_t * cp, b = sin_t * sp;
        l = v3((t1.x * a + t2.x * b) + w.x * cos_t, (t1.y * a + t2.y * b) + w.y * cos_t, (t1.z * a + t2.z * b) + w.z * cos_t);
        float bb = dot(dv, l);
        float disc = r2 - (dist2 - bb * bb);
        float th = bb - std::sqrt(fmaxf_(disc, 0.0f));
        scale = ((2.0f * PI) * one_minus) / pmf;
        tmx = th * 0.999f;
    } else {
        float su = std::sqrt(u1);
        float b0 = 1.0f - su;
        float b1 = u2 * su;
        float b2 = (1.0f - b0) - b1;
        V3 q = add(add(mul(L.p0, b0), mul(L.p1, b1)), mul(L.p2, b2));
        V3 dv = sub(q, xb);
        float dist2 = dot(dv, dv);
        if (!(dist2 > 0.0f)) return false;
        float dist = std::sqrt(dist2);
        l = divs(dv, dist);
        float cos_l = std::fabs(dot(L.n, l));
        if (!(cos_l > 0.0f)) return false;
        scale = (cos_l * L.area) / (dist2 * pmf);
        tmx = dist * 0.999f;
    }
    Terms tm = brdf_terms(l, v, f0, s.n, s.roughness, s.metallic);
    V3 ct = cook_torrance(tm);
    V3 c = v3(((s.albedo.x * ct.x) * L.L.x) * scale, ((s.albedo.y * ct.y) * L.L.y) * scale,
              ((s.albedo.z * ct.z) * L.L.z) * scale);
    if (!(maxc(c) > 0.0f)) return false;
    *contrib = c; *sdir = l; *stmax = tmx;
    return true;
}

// Continuation direction: with probability p_spec a GGX half-vector sample of
// the reference's DistributionGGX (LightBuffers.glsl:69-80, roughness^2 = alpha),
// otherwise cosine-weighted; weight = albedo * CookTorrance(l) / mixture pdf
// (the reference's BRDF with albedo on both terms, RayGen.rgen:273).
static inline bool sample_continuation(const Surface& s, V3 v, V3 f0, float u_lobe, float u1, float u2, V3* wi,
                                       V3* weight, float* pdf_out) {
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
        float ch = std::sqrt(cos2);
        float sh = std::sqrt(fmaxf_(0.0f, 1.0f - cos2));
        float hx = sh * cp, hy = sh * sp;
        V3 h = v3((b1.x * hx + b2.x * hy) + s.n.x * ch, (b1.y * hx + b2.y * hy) + s.n.y * ch,
                  (b1.z * hx + b2.z * hy) + s.n.z * ch);
        float vh2 = 2.0f * dot(v, h);
        l = sub(mul(h, vh2), v);
    } else {
        float r = std::sqrt(u1);
        float lx = r * cp, ly = r * sp, lz = std::sqrt(fmaxf_(0.0f, 1.0f - u1));
        l = v3((b1.x * lx + b2.x * ly) + s.n.x * lz, (b1.y * lx + b2.y * ly) + s.n.y * lz,
               (b1.z * lx + b2.z * ly) + s.n.z * lz);
    }
    if (!(dot(l, s.ng) > 0.0f)) return false;
    float ndl = dot(s.n, l);
    if (!(ndl > 0.0f)) return false;
    V3 vl = add(v, l);
    float vl2 = dot(vl, vl);
    V3 hh = vl2 > 0.0f ? divs(vl, std::sqrt(vl2)) : s.n;
    float D = distribution_ggx(hh, s.n, s.roughness);
    float pdf_spec = (D * fmaxf_(dot(s.n, hh), 0.0f)) / (4.0f * fmaxf_(dot(v, hh), 1e-6f));
    float pdf = p_spec * pdf_spec + (1.0f - p_spec) * (ndl / PI);
    if (!(pdf > 0.0f)) return false;
    V3 ct = cook_torrance(brdf_terms(l, v, f0, s.n, s.roughness, s.metallic));
    *weight = v3((s.albedo.x * ct.x) / pdf, (s.albedo.y * ct.y) / pdf, (s.albedo.z * ct.z) / pdf);
    *wi = l;
    *pdf_out = pdf;
    return true;
}

// A path handed to the radiance cache: its query record (position, roughness,
// outgoing direction, metallic, shading normal, 0, albedo, 0) and throughput.
struct CacheQuery {
    bool valid = false;
    float rec[16];
    V3 beta;
};

// indirect: the path carries only the light that reaches the primary vertex
// indirectly (the ReSTIR + indirect mode): no emission and no NEE at the primary
// vertex, which the ReSTIR passes shade; its random numbers are drawn all the same.
// spread_c > 0: the radiance-cache mode's termination (the path spread heuristic of
// Mueller et al. 2021, as the shading kernel restates it): a0 = t^2 / (4 pi cos) at
// the primary vertex, later vertices add sqrt(t^2 / (pdf cos)) with the pdf of the
// direction that reached them; a non-emissive vertex after the first ends the path
// in the cache once spread^2 > c a0 (no NEE there), recorded in *q.
static V3 trace_path(const Scene& S, const View& vw, uint32_t x, uint32_t y, uint32_t pixel_key, uint32_t sample,
                     const Settings& st, GSample* g, Counters* ctr, bool indirect = false, float spread_c = 0.0f,
                     CacheQuery* q = nullptr) {
    float a0 = 0.0f, acc = 0.0f, prev_pdf = 0.0f;
    Pcg rng = pcg_stream(pixel_key, sample, 0, st.seed);
    float j1 = pcg_float(rng), j2 = pcg_float(rng);
    float jx = sample == 0 ? 0.5f : j1, jy = sample == 0 ? 0.5f : j2;
    V3 ro = load3(vw.pos);
    V3 rd = camera_dir(vw, x, y, jx, jy);
    float tmin = 0.0f;
    V3 beta = v3(1, 1, 1), L = v3(0, 0, 0);
    if (g) g->hit = false;
    for (uint32_t d = 0; d < st.max_depth; d++) {
        if (d > 0) rng = pcg_stream(pixel_key, sample, d, st.seed);
        if (ctr) { if (d == 0) ctr->camera++; else ctr->extension++; }
        HitRec h;
        if (!trace(S, ro, rd, tmin, T_FAR, false, &h, ctr)) break;
        Surface s = surface_at(S, h, rd);
        if (d == 0 && g) {
            g->hit = true; g->s = s; g->t = h.t;
            motion_of(S, vw, s, x, y, g->motion);
        }
        float u_sel = pcg_float(rng), u1 = pcg_float(rng), u2 = pcg_float(rng);
        float u_rr = pcg_float(rng), u_d1 = pcg_float(rng), u_d2 = pcg_float(rng);
        float u_lobe = pcg_float(rng);
        const bool direct = !(indirect && d == 0);
        if (spread_c > 0.0f) {
            const float cosv = fmaxf_(std::fabs(dot(s.n, rd)), 1e-6f);
            if (d == 0) {
                a0 = (h.t * h.t) / ((4.0f * PI) * cosv);
                acc = 0.0f;
            } else {
                acc = acc + std::sqrt((h.t * h.t) / (fmaxf_(prev_pdf, 1e-6f) * cosv));
            }
            if (d >= 1 && !(s.flags & MAT_EMISSIVE) && acc * acc > spread_c * a0) {
                if (q) {
                    const float r[16] = {s.pos.x, s.pos.y, s.pos.z, s.roughness, -rd.x, -rd.y, -rd.z, s.metallic,
                                         s.n.x, s.n.y, s.n.z, 0.0f, s.albedo.x, s.albedo.y, s.albedo.z, 0.0f};
                    std::memcpy(q->rec, r, sizeof(r));
                    q->beta = beta;
                    q->valid = true;
                }
                return L;
            }
        }
        if (s.flags & MAT_EMISSIVE) {
            if (d == 0 && direct) L = add(L, cmul(beta, s.albedo));
            break;
        }
        V3 v = neg(rd);
        V3 f0 = f0_of(s.albedo, s.metallic);
        V3 xb = add(s.pos, mul(s.n, SURFACE_BIAS));
        // directional light (CalcDirectionalLight x ShadowTest, RayClosestHit.rchit:136)
        if (direct && S.dl.enabled) {
            V3 c = calc_directional(load3(S.dl.dir), load3(S.dl.colour), v, f0, s.n, s.roughness, s.metallic, s.albedo);
            if (maxc(c) > 0.0f) {
                V3 cb = cmul(beta, c);
                if (shadow_test(S, xb, load3(S.dl.dir), T_FAR, ctr) > 0.0f) L = add(L, cb);
            }
        }
        V3 c, ldir; float ltmax;
        if (direct && sample_local(S, s, v, f0, xb, u_sel, u1, u2, &c, &ldir, &ltmax)) {
            V3 cb = cmul(beta, c);
            if (shadow_test(S, xb, ldir, ltmax, ctr) > 0.0f) L = add(L, cb);
        }
        if (d + 1 >= st.max_depth) break;
        if (d + 1 >= st.rr_depth) {
            float p = fminf_(maxc(beta), 0.95f);
            if (!(u_rr < p)) break;
            beta = v3(beta.x / p, beta.y / p, beta.z / p);
        }
        V3 wi, w;
        float pdf;
        if (!sample_continuation(s, v, f0, u_lobe, u_d1, u_d2, &wi, &w, &pdf)) break;
        beta = cmul(beta, w);
        prev_pdf = pdf;
        ro = xb;
        rd = wi;
        tmin = EXT_TMIN;
    }
    return L;
}

// ----------------------------------------------------------------------------
// ReSTIR DI (RayGen.rgen:53-528)
// ----------------------------------------------------------------------------
struct Reservoir {   // PixelReservoir, RayGen.rgen:64-76 (48 bytes)
    float w_sum_pl, w_pl; uint32_t pl_idx, pl_m;
    uint32_t em_inst, em_tri; float em_u, em_v;
    float w_sum_em, w_em; uint32_t m_em, pad;
};
static_assert(sizeof(Reservoir) == 48, "layout");
static inline Reservoir res_init() {
    Reservoir r{};
    r.pl_idx = INVALID; r.w_sum_pl = 0; r.pl_m = 0; r.w_pl = 0;
    r.em_inst = INVALID; r.em_tri = INVALID; r.w_sum_em = 0; r.m_em = 0; r.w_em = 0;
    return r;
}

struct Shade {  // the per-pixel constants of RayGen.rgen main (:530-556)
    V3 ro, n, albedo, v, f0, biased;
    float rough, metal;
};

// UpdatePointlightReservoir / UpdateEmissiveReservoir (:215-239)
static inline bool update_pl(Reservoir& r, uint32_t idx, float w, Pcg& rng) {
    r.pl_m++;
    float u = pcg_float(rng);
    r.w_sum_pl = r.w_sum_pl + w;
    if (r.w_sum_pl > 0.0f && u < w / r.w_sum_pl) { r.pl_idx = idx; return true; }
    return false;
}
static inline bool update_em(Reservoir& r, uint32_t inst, uint32_t tri, float bu, float bv, float w, Pcg& rng) {
    r.m_em++;
    float u = pcg_float(rng);
    r.w_sum_em = r.w_sum_em + w;
    if (r.w_sum_em > 0.0f && u < w / r.w_sum_em) {
        r.em_inst = inst; r.em_tri = tri; r.em_u = bu; r.em_v = bv;
        return true;
    }
    return false;
}

// emissive triangle point and normal (ComputeTriangleRadiance :258-268)
static inline void tri_point(const Scene& S, uint32_t inst, uint32_t tri, float bu, float bv, V3* p, V3* pn) {
    const InstData& I = S.insts[inst];
    const MeshData& M = S.meshes[I.in.mesh_id];
    const uint32_t* ix = &M.idx[3 * tri];
    float bz = (1.0f - bu) - bv;
    V3 q = add(add(mul(load3(&M.pos[3 * ix[0]]), bu), mul(load3(&M.pos[3 * ix[1]]), bv)), mul(load3(&M.pos[3 * ix[2]]), bz));
    V3 nn;
    if (M.has_normals)
        nn = add(add(mul(load3(&M.nrm[3 * ix[0]]), bu), mul(load3(&M.nrm[3 * ix[1]]), bv)), mul(load3(&M.nrm[3 * ix[2]]), bz));
    else
        nn = cross(sub(load3(&M.pos[3 * ix[1]]), load3(&M.pos[3 * ix[0]])), sub(load3(&M.pos[3 * ix[2]]), load3(&M.pos[3 * ix[0]])));
    *p = xform_point(I.in.transform, q);
    *pn = normalize(mat3_mul(I.nmat, nn));
}

// TriangleShadowTest (:241-256)
static inline float tri_shadow(const Scene& S, uint32_t inst, uint32_t tri, float bu, float bv, V3 surface_pos, Counters* ctr) {
    V3 p, pn;
    tri_point(S, inst, tri, bu, bv, &p, &pn);
    V3 target = add(p, mul(pn, 0.01f));
    float dist = length(sub(surface_pos, target));
    V3 dir = divs(sub(target, surface_pos), dist);
    return shadow_test(S, surface_pos, dir, dist, ctr);
}

// ComputeTriangleRadiance (:258-282)
static inline V3 tri_radiance(const Scene& S, uint32_t inst, uint32_t tri, float bu, float bv, const Shade& sh,
                              bool shadow, Counters* ctr) {
    V3 p, pn;
    tri_point(S, inst, tri, bu, bv, &p, &pn);
    V3 em = load3(S.mats[S.insts[inst].in.material_id].albedo);
    V3 brdf = cook_torrance(brdf_terms(normalize(sub(p, sh.ro)), sh.v, sh.f0, sh.n, sh.rough, sh.metal));
    V3 dd = sub(sh.ro, p);
    float d2 = std::fabs(dot(dd, dd));
    V3 rad = v3(((em.x * sh.albedo.x) * brdf.x) / d2, ((em.y * sh.albedo.y) * brdf.y) / d2, ((em.z * sh.albedo.z) * brdf.z) / d2);
    if (shadow) {
        V3 target = add(p, mul(pn, 0.01f));
        float dist = length(sub(sh.biased, target));
        V3 dir = divs(sub(target, sh.biased), dist);
        rad = mul(rad, shadow_test(S, sh.biased, dir, dist, ctr));
    }
    return rad;
}

// CombinePixelReservoir (:361-386)
static inline void combine(const Scene& S, Reservoir& cur, const Reservoir& nb, float& phat_pl, float& phat_em,
                           const Shade& sh, Pcg& rng, Counters* ctr) {
    if (nb.pl_idx != INVALID) {
        const PointLight& L = S.pls[nb.pl_idx];
        V3 lp = load3(L.pos);
        float ld = length(sub(lp, sh.biased));
        float vis = shadow_test(S, sh.biased, divs(sub(lp, sh.biased), ld), ld - 0.001f, ctr);
        float p_hat = length(calc_pointlight(L, sh.v, sh.f0, sh.ro, sh.n, sh.rough, sh.metal, sh.albedo)) * vis;
        float w = (p_hat * (float)nb.pl_m) * nb.w_pl;
        if (update_pl(cur, nb.pl_idx, w, rng)) phat_pl = p_hat;
    }
    if (nb.em_inst != INVALID) {
        V3 rad = tri_radiance(S, nb.em_inst, nb.em_tri, nb.em_u, nb.em_v, sh, true, ctr);
        float p_hat = length(rad);
        float w = (p_hat * nb.w_em) * (float)nb.m_em;
        if (update_em(cur, nb.em_inst, nb.em_tri, nb.em_u, nb.em_v, w, rng)) phat_em = p_hat;
    }
}

struct GPix {   // G-buffer texel consumed by the ReSTIR passes
    bool valid;          // a non-emissive primary hit
    bool emissive;
    V3 pos, n, albedo; float rough, metal; float motion[2];
};

static inline Shade shade_of(const View& vw, const GPix& g) {
    Shade sh;
    sh.ro = g.pos; sh.n = g.n; sh.albedo = g.albedo; sh.rough = g.rough; sh.metal = g.metal;
    V3 cam = load3(vw.pos);
    sh.v = normalize(sub(cam, g.pos));
    sh.f0 = f0_of(g.albedo, g.metal);
    float bias = 0.01f + fmaxf_(length(sub(cam, g.pos)) * 0.001f, 0.01f);
    sh.biased = add(g.pos, mul(g.n, bias));
    return sh;
}

// WriteInitialReservoirs (:411-468) for one pixel
static Reservoir restir_initial_temporal(const Scene& S, const View& vw, const Settings& st, const GPix* gb,
                                         const Reservoir* history, const float* prev_normals, bool history_valid,
                                         uint32_t x, uint32_t y, uint32_t pixel_key, Counters* ctr) {
    uint32_t W = vw.width, H = vw.height;
    const GPix& g = gb[y * W + x];
    if (!g.valid) return res_init();
    Shade sh = shade_of(vw, g);
    Pcg rng = pcg_stream(pixel_key, st.frame_index, 0x80000001u, st.seed);
    Reservoir R = res_init();
    float phat_pl = 0.0f, phat_em = 0.0f;
    uint32_t npl = (uint32_t)S.pls.size();
    uint32_t C = st.restir_candidates;
    if (npl > 0) {
        for (uint32_t i = 0; i < C; i++) {
            uint32_t idx = (uint32_t)(pcg_float(rng) * (float)npl);
            if (idx > npl - 1) idx = npl - 1;
            float p_hat = length(calc_pointlight(S.pls[idx], sh.v, sh.f0, sh.ro, sh.n, sh.rough, sh.metal, sh.albedo));
            float w = p_hat / (1.0f / (float)npl);
            if (update_pl(R, idx, w, rng)) phat_pl = p_hat;
        }
    }
    uint32_t nem = (uint32_t)S.emissive_insts.size();
    if (nem > 0) {
        for (uint32_t i = 0; i < C; i++) {
            uint32_t k = (uint32_t)(pcg_float(rng) * (float)nem);
            if (k > nem - 1) k = nem - 1;
            uint32_t inst = S.emissive_insts[k];
            const InstData& I = S.insts[inst];
            const MeshData& M = S.meshes[I.in.mesh_id];
            uint32_t ntri = M.nt;
            uint32_t tri = (uint32_t)(pcg_float(rng) * (float)ntri);
            if (tri > ntri - 1) tri = ntri - 1;
            float bu = pcg_float(rng), bv = pcg_float(rng);
            if (bu + bv >= 1.0f) { bu = 1.0f - bu; bv = 1.0f - bv; }
            const uint32_t* ix = &M.idx[3 * tri];
            V3 p0 = load3(&M.pos[3 * ix[0]]), p1 = load3(&M.pos[3 * ix[1]]), p2 = load3(&M.pos[3 * ix[2]]);
            float area = (I.det3 * 0.5f) * length(cross(sub(p1, p0), sub(p1, p2)));
            V3 rad = tri_radiance(S, inst, tri, bu, bv, sh, false, ctr);
            float p_hat = length(rad);
            float pdf = 1.0f / ((float)(nem * ntri) * area);
            float w = p_hat / pdf;
            if (update_em(R, inst, tri, bu, bv, w, rng)) phat_em = p_hat;
        }
    }
    if (R.pl_idx != INVALID) {
        V3 lp = load3(S.pls[R.pl_idx].pos);
        float dist = length(sub(lp, sh.biased));
        float vis = shadow_test(S, sh.biased, divs(sub(lp, sh.biased), dist), dist, ctr);
        R.w_pl = vis * ((R.w_sum_pl / (float)R.pl_m) / phat_pl);
    } else {
        R.w_pl = 0.0f;
    }
    if (R.em_inst != INVALID) {
        float vis = tri_shadow(S, R.em_inst, R.em_tri, R.em_u, R.em_v, sh.biased, ctr);
        R.w_em = vis * ((R.w_sum_em / (float)R.m_em) / phat_em);
    } else {
        R.w_em = 0.0f;
    }
    // temporal resample
    if (history_valid && st.restir_temporal != 0 && vw.prev_valid) {
        float hu = ((float)x + 0.5f) / (float)W + g.motion[0];
        float hv = ((float)y + 0.5f) / (float)H + g.motion[1];
        if (hu > 0.0f && hv > 0.0f && hu < 1.0f && hv < 1.0f) {
            uint32_t hx = (uint32_t)(hu * (float)W), hy = (uint32_t)(hv * (float)H);
            if (hx > W - 1) hx = W - 1;
            if (hy > H - 1) hy = H - 1;
            const float* pn = &prev_normals[4 * (hy * W + hx)];
            if (dot(load3(pn), g.n) > 0.95f) {
                Reservoir Hh = history[hy * W + hx];
                // a history of an earlier scene: lights or instances that no longer exist are dropped
                if (Hh.pl_idx != INVALID && Hh.pl_idx >= (uint32_t)S.pls.size()) Hh.pl_idx = INVALID;
                if (Hh.em_inst != INVALID && Hh.em_inst >= (uint32_t)S.insts.size()) Hh.em_inst = INVALID;
                float mcap = (float)st.restir_mcap;
                if ((float)Hh.pl_m > mcap * (float)R.pl_m) {
                    Hh.w_sum_pl = Hh.w_sum_pl * ((mcap * (float)R.pl_m) / (float)Hh.pl_m);
                    Hh.pl_m = st.restir_mcap * R.pl_m;
                }
                if ((float)Hh.m_em > mcap * (float)R.m_em) {
                    Hh.w_sum_em = Hh.w_sum_em * ((mcap * (float)R.m_em) / (float)Hh.m_em);
                    Hh.m_em = st.restir_mcap * R.m_em;
                }
                Reservoir T = res_init();
                float tp_pl = 0.0f, tp_em = 0.0f;
                combine(S, T, R, tp_pl, tp_em, sh, rng, ctr);
                combine(S, T, Hh, tp_pl, tp_em, sh, rng, ctr);
                T.m_em = Hh.m_em + R.m_em;
                T.pl_m = Hh.pl_m + R.pl_m;
                T.w_em = tp_em > 0.0f ? (T.w_sum_em / (float)T.m_em) / tp_em : 0.0f;
                T.w_pl = tp_pl > 0.0f ? (T.w_sum_pl / (float)T.pl_m) / tp_pl : 0.0f;
                return T;
            }
        }
    }
    return R;
}

// ComputeAndWriteSpatialReservoirReuse (:470-506) + CalculateRadianceFromReservoirs
// (:508-528) + main (:557-569) for one pixel
static V3 restir_spatial_shade(const Scene& S, const View& vw, const Settings& st, const GPix* gb,
                               const Reservoir* temporal, Reservoir* out_res, uint32_t x, uint32_t y,
                               uint32_t pixel_key, Counters* ctr) {
    uint32_t W = vw.width, H = vw.height;
    const GPix& g = gb[y * W + x];
    if (!g.valid) {
        *out_res = res_init();
        return g.emissive ? g.albedo : v3(0, 0, 0);
    }
    Shade sh = shade_of(vw, g);
    V3 light = v3(0, 0, 0);
    if (S.dl.enabled) {
        V3 c = calc_directional(load3(S.dl.dir), load3(S.dl.colour), sh.v, sh.f0, sh.n, sh.rough, sh.metal, sh.albedo);
        light = mul(c, shadow_test(S, sh.biased, load3(S.dl.dir), 1000.0f, ctr));
    }
    Pcg rng = pcg_stream(pixel_key, st.frame_index, 0x80000002u, st.seed);
    Reservoir R = res_init();
    float phat_pl = 0.0f, phat_em = 0.0f;
    const Reservoir& self = temporal[y * W + x];
    combine(S, R, self, phat_pl, phat_em, sh, rng, ctr);
    R.m_em += self.m_em;
    R.pl_m += self.pl_m;
    for (int i = 0; i < st.restir_spatial; i++) {
        int nx = -1, ny = -1;
        for (int tries = 0; tries < 8; tries++) {
            float ox = ((pcg_float(rng) - 0.5f) * 2.0f) * st.restir_radius;
            float oy = ((pcg_float(rng) - 0.5f) * 2.0f) * st.restir_radius;
            float fx = (float)x + ox, fy = (float)y + oy;
            if (fx >= 0.0f && fy >= 0.0f && fx < (float)W && fy < (float)H) { nx = (int)fx; ny = (int)fy; break; }
        }
        if (nx < 0) continue;
        const GPix& q = gb[(uint32_t)ny * W + (uint32_t)nx];
        V3 qn = q.valid ? q.n : v3(0, 0, 0);
        if (dot(qn, g.n) < 0.95f) continue;
        const Reservoir& Q = temporal[(uint32_t)ny * W + (uint32_t)nx];
        combine(S, R, Q, phat_pl, phat_em, sh, rng, ctr);
        R.m_em += Q.m_em;
        R.pl_m += Q.pl_m;
    }
    R.w_em = phat_em > 0.0f ? (R.w_sum_em / phat_em) / (float)R.m_em : 0.0f;
    R.w_pl = phat_pl > 0.0f ? (R.w_sum_pl / phat_pl) / (float)R.pl_m : 0.0f;
    *out_res = R;
    V3 rad = v3(0, 0, 0);
    if (!S.pls.empty() && R.pl_idx != INVALID) {
        const PointLight& L = S.pls[R.pl_idx];
        V3 lp = load3(L.pos);
        float ld = length(sub(lp, sh.biased));
        V3 c = calc_pointlight(L, sh.v, sh.f0, sh.ro, sh.n, sh.rough, sh.metal, sh.albedo);
        c = mul(c, shadow_test(S, sh.biased, divs(sub(lp, sh.biased), ld), ld, ctr));
        c = mul(c, R.w_pl);
        rad = add(rad, c);
    }
    if (!S.emissive_insts.empty() && R.em_inst != INVALID) {
        V3 e = tri_radiance(S, R.em_inst, R.em_tri, R.em_u, R.em_v, sh, true, ctr);
        rad = add(rad, mul(e, R.w_em));
    }
    return add(light, rad);
}

struct RestirState {
    uint32_t W = 0, H = 0;
    std::vector<Reservoir> temporal, history;
    std::vector<float> prev_normals;   // float4 per pixel
    bool history_valid = false;
};

// ----------------------------------------------------------------------------
// parallel for
// ----------------------------------------------------------------------------
template <class F>
static void parallel_for(uint32_t n, uint32_t nthreads, uint32_t chunk, F f) {
    if (nthreads <= 1 || n <= chunk) {
        f(0u, n, 0u);
        return;
    }
    std::atomic<uint32_t> next{0};
    std::vector<std::thread> th;
    for (uint32_t t = 0; t < nthreads; t++) {
        th.emplace_back([&, t]() {
            for (;;) {
                uint32_t b = next.fetch_add(chunk);
                if (b >= n) break;
                f(b, std::min(n, b + chunk), t);
            }
        });
    }
    for (auto& x : th) x.join();
}

}  // namespace so

// ============================================================================
// C API (ctypes)
// ============================================================================
using namespace so;

extern "C" {

void* snko_scene_create() { return new Scene(); }
void snko_scene_destroy(void* s) { delete (Scene*)s; }

int snko_add_mesh(void* sp, const float* pos, const float* nrm, const uint32_t* idx, uint32_t nv, uint32_t nt) {
    Scene& S = *(Scene*)sp;
    MeshData M;
    M.nv = nv; M.nt = nt;
    M.pos.assign(pos, pos + 3 * (size_t)nv);
    if (nrm) { M.nrm.assign(nrm, nrm + 3 * (size_t)nv); M.has_normals = true; }
    M.idx.assign(idx, idx + 3 * (size_t)nt);
    for (size_t i = 0; i < M.idx.size(); i++)
        if (M.idx[i] >= nv) return 1;
    S.meshes.push_back(std::move(M));
    S.built = false;
    return 0;
}

int snko_set_instances(void* sp, const Instance* in, uint32_t n) {
    Scene& S = *(Scene*)sp;
    S.insts.resize(n);
    for (uint32_t i = 0; i < n; i++) {
        if (in[i].mesh_id >= S.meshes.size()) return 1;
        S.insts[i].in = in[i];
    }
    S.built = false;
    return 0;
}

int snko_set_materials(void* sp, const Material* m, uint32_t n) {
    Scene& S = *(Scene*)sp;
    S.mats.assign(m, m + n);
    S.built = false;
    return 0;
}

int snko_set_lights(void* sp, const DirLight* dl, const PointLight* pl, uint32_t n) {
    Scene& S = *(Scene*)sp;
    S.dl = dl ? *dl : DirLight{};
    S.pls.assign(pl, pl + n);
    S.built = false;
    return 0;
}

int snko_build(void* sp) {
    Scene& S = *(Scene*)sp;
    for (auto& I : S.insts)
        if (I.in.material_id >= S.mats.size()) return 1;
    build_scene(S);
    return 0;
}

// counters: [camera, extension, shadow, nodes, tris]
int snko_trace(void* sp, const Ray* rays, uint32_t n, uint32_t any, Hit* hits, uint32_t nthreads, uint64_t* counters) {
    Scene& S = *(Scene*)sp;
    if (!S.built) return 4;
    std::vector<Counters> ctr(std::max(1u, nthreads));
    parallel_for(n, nthreads, 4096, [&](uint32_t b, uint32_t e, uint32_t t) {
        Counters* c = counters ? &ctr[t] : nullptr;
        for (uint32_t i = b; i < e; i++) {
            const Ray& r = rays[i];
            HitRec h;
            bool hit = trace(S, v3(r.ox, r.oy, r.oz), v3(r.dx, r.dy, r.dz), r.tmin, r.tmax, any != 0, &h, c);
            Hit& o = hits[i];
            if (any) {
                o.t = hit ? 1.0f : -1.0f; o.inst = INVALID; o.prim = INVALID; o.u = 0; o.v = 0; o.flags = hit ? 1u : 0u;
            } else if (hit) {
                o.t = h.t; o.inst = h.inst; o.prim = h.prim; o.u = h.u; o.v = h.v; o.flags = 1u;
            } else {
                o.t = -1.0f; o.inst = INVALID; o.prim = INVALID; o.u = 0; o.v = 0; o.flags = 0u;
            }
        }
    });
    if (counters) {
        for (auto& c : ctr) { counters[3] += c.nodes; counters[4] += c.tris; }
    }
    return 0;
}

static void write_gbuffer(const Outputs* out, size_t o, const GSample& g) {
    if (!out) return;
    if (g.hit) {
        const Surface& s = g.s;
        if (out->albedo) { float* a = &out->albedo[4 * o]; a[0] = s.albedo.x; a[1] = s.albedo.y; a[2] = s.albedo.z; a[3] = 1.0f; }
        if (out->normal) { float* a = &out->normal[4 * o]; a[0] = s.n.x; a[1] = s.n.y; a[2] = s.n.z; a[3] = 0.0f; }
        if (out->position) { float* a = &out->position[4 * o]; a[0] = s.pos.x; a[1] = s.pos.y; a[2] = s.pos.z; a[3] = 1.0f; }
        if (out->rma) { float* a = &out->rma[4 * o]; a[0] = s.roughness; a[1] = s.metallic; a[2] = s.ao; a[3] = 1.0f; }
        if (out->motion) { out->motion[2 * o] = g.motion[0]; out->motion[2 * o + 1] = g.motion[1]; }
        if (out->depth) out->depth[o] = g.t;
        if (out->mat_flags) out->mat_flags[o] = s.flags;
        if (out->inst_id) out->inst_id[o] = s.inst;
        if (out->prim_id) out->prim_id[o] = s.prim;
    } else {
        if (out->albedo) std::memset(&out->albedo[4 * o], 0, 16);
        if (out->normal) std::memset(&out->normal[4 * o], 0, 16);
        if (out->position) std::memset(&out->position[4 * o], 0, 16);
        if (out->rma) std::memset(&out->rma[4 * o], 0, 16);
        if (out->motion) { out->motion[2 * o] = 0.0f; out->motion[2 * o + 1] = 0.0f; }
        if (out->depth) out->depth[o] = -1.0f;
        if (out->mat_flags) out->mat_flags[o] = 0u;
        if (out->inst_id) out->inst_id[o] = INVALID;
        if (out->prim_id) out->prim_id[o] = INVALID;
    }
}

// Plain path tracing of one view.  pixels: optional list of pixel indices
// (y*W+x) to render; outputs are then compact (one entry per listed pixel).
// pixel_base: global index of this view's first pixel (multi-view RNG keys).
int snko_render_path(void* sp, const View* vw, const Settings* st, const uint32_t* pixels, uint32_t npix,
                     uint32_t pixel_base, const Outputs* out, uint32_t nthreads, uint64_t* counters) {
    Scene& S = *(Scene*)sp;
    if (!S.built) return 4;
    uint32_t W = vw->width, H = vw->height;
    uint32_t n = pixels ? npix : W * H;
    std::vector<Counters> ctr(std::max(1u, nthreads));
    parallel_for(n, nthreads, 64, [&](uint32_t b, uint32_t e, uint32_t t) {
        Counters* c = &ctr[t];
        for (uint32_t i = b; i < e; i++) {
            uint32_t p = pixels ? pixels[i] : i;
            uint32_t x = p % W, y = p / W;
            V3 sum = v3(0, 0, 0);
            GSample g;
            g.hit = false;
            for (uint32_t s = 0; s < st->spp; s++) {
                V3 L = trace_path(S, *vw, x, y, pixel_base + p, s, *st, s == 0 ? &g : nullptr, c);
                sum = add(sum, L);
            }
            float inv = 1.0f / (float)st->spp;
            if (out && out->radiance) {
                float* r = &out->radiance[4 * (size_t)i];
                r[0] = sum.x * inv; r[1] = sum.y * inv; r[2] = sum.z * inv; r[3] = 1.0f;
            }
            write_gbuffer(out, i, g);
        }
    });
    if (counters)
        for (auto& c : ctr) { counters[0] += c.camera; counters[1] += c.extension; counters[2] += c.shadow; counters[3] += c.nodes; counters[4] += c.tris; }
    return 0;
}

// One-sample path tracing of one view in the radiance-cache mode's form: the
// radiance the paths gather before they end (radiance, 4 floats per pixel) and,
// for the paths that end in the cache, their query record (qrec, 16 floats) and
// throughput (qbeta: rgb, 1; 0 in the fourth float when the path ended otherwise).
int snko_render_path_cache(void* sp, const View* vw, const Settings* st, uint32_t pixel_base, float* radiance,
                           float* qrec, float* qbeta, uint32_t nthreads) {
    Scene& S = *(Scene*)sp;
    if (!S.built) return 4;
    if (st->spp != 1) return 1;
    const float spread_c = st->cache_spread > 0.0f ? st->cache_spread : 0.01f;
    const uint32_t W = vw->width, n = W * vw->height;
    parallel_for(n, nthreads, 64, [&](uint32_t b, uint32_t e, uint32_t) {
        for (uint32_t p = b; p < e; p++) {
            CacheQuery q;
            const V3 L = trace_path(S, *vw, p % W, p / W, pixel_base + p, 0, *st, nullptr, nullptr, false, spread_c, &q);
            float* r = radiance + 4 * (size_t)p;
            r[0] = L.x; r[1] = L.y; r[2] = L.z; r[3] = 1.0f;
            float* qb = qbeta + 4 * (size_t)p;
            if (q.valid) {
                std::memcpy(qrec + 16 * (size_t)p, q.rec, sizeof(q.rec));
                qb[0] = q.beta.x; qb[1] = q.beta.y; qb[2] = q.beta.z; qb[3] = 1.0f;
            } else {
                std::memset(qrec + 16 * (size_t)p, 0, 16 * sizeof(float));
                qb[0] = qb[1] = qb[2] = qb[3] = 0.0f;
            }
        }
    });
    return 0;
}

void* snko_restir_state_create(uint32_t W, uint32_t H) {
    RestirState* r = new RestirState();
    r->W = W; r->H = H;
    r->temporal.assign((size_t)W * H, res_init());
    r->history.assign((size_t)W * H, res_init());
    r->prev_normals.assign((size_t)W * H * 4, 0.0f);
    return r;
}
void snko_restir_state_destroy(void* r) { delete (RestirState*)r; }

// One ReSTIR DI frame of one view (both passes of RT::RecordRenderCmdBuf).
// Writes radiance and G-buffer for every pixel; reservoirs_out (optional) gets
// the final (spatial) reservoirs, 48 bytes per pixel.
int snko_render_restir(void* sp, void* statep, const View* vw, const Settings* st, uint32_t pixel_base,
                       const Outputs* out, void* reservoirs_out, uint32_t nthreads, uint64_t* counters) {
    Scene& S = *(Scene*)sp;
    RestirState& R = *(RestirState*)statep;
    if (!S.built) return 4;
    uint32_t W = vw->width, H = vw->height;
    if (W != R.W || H != R.H) return 1;
    size_t n = (size_t)W * H;
    // SNK_MODE_RESTIR_PT: main's colour_sum = light + BounceDiffuse (RayGen.rgen:565-566),
    // with st->spp unbiased indirect paths per pixel in place of BounceDiffuse
    const bool with_indirect = st->mode == 3u;
    std::vector<GPix> gb(n);
    std::vector<Counters> ctr(std::max(1u, nthreads));
    // G-buffer from primary rays through pixel centres (with the indirect paths, the
    // camera ray of each pixel's first path is this ray: counted once, with the paths)
    parallel_for((uint32_t)n, nthreads, 256, [&](uint32_t b, uint32_t e, uint32_t t) {
        for (uint32_t i = b; i < e; i++) {
            uint32_t x = i % W, y = i / W;
            V3 rd = camera_dir(*vw, x, y, 0.5f, 0.5f);
            HitRec h;
            GSample g;
            g.hit = false;
            if (!with_indirect) ctr[t].camera++;
            if (trace(S, load3(vw->pos), rd, 0.0f, T_FAR, false, &h, nullptr)) {
                g.hit = true;
                g.s = surface_at(S, h, rd);
                g.t = h.t;
                motion_of(S, *vw, g.s, x, y, g.motion);
            }
            write_gbuffer(out, i, g);
            GPix& p = gb[i];
            p.valid = g.hit && !(g.s.flags & MAT_EMISSIVE);
            p.emissive = g.hit && (g.s.flags & MAT_EMISSIVE);
            if (g.hit) {
                p.pos = g.s.pos; p.n = g.s.n; p.albedo = g.s.albedo; p.rough = g.s.roughness; p.metal = g.s.metallic;
                p.motion[0] = g.motion[0]; p.motion[1] = g.motion[1];
            } else {
                p.pos = p.n = p.albedo = v3(0, 0, 0); p.rough = p.metal = 0; p.motion[0] = p.motion[1] = 0;
            }
        }
    });
    // pass 1: initial candidates + temporal reuse
    parallel_for((uint32_t)n, nthreads, 64, [&](uint32_t b, uint32_t e, uint32_t t) {
        for (uint32_t i = b; i < e; i++) {
            uint32_t x = i % W, y = i / W;
            R.temporal[i] = restir_initial_temporal(S, *vw, *st, gb.data(), R.history.data(), R.prev_normals.data(),
                                                    R.history_valid, x, y, pixel_base + i, &ctr[t]);
        }
    });
    // indirect light of every pixel: the mean of st->spp paths from its primary vertex
    // (their random streams are keyed by seed + 0x9E3779B9 x frame_index)
    std::vector<V3> indirect;
    if (with_indirect) {
        indirect.assign(n, v3(0, 0, 0));
        Settings pst = *st;
        pst.seed = st->seed + 0x9E3779B9u * st->frame_index;
        parallel_for((uint32_t)n, nthreads, 64, [&](uint32_t b, uint32_t e, uint32_t t) {
            for (uint32_t i = b; i < e; i++) {
                uint32_t x = i % W, y = i / W;
                V3 sum = v3(0, 0, 0);
                for (uint32_t s = 0; s < pst.spp; s++)
                    sum = add(sum, trace_path(S, *vw, x, y, pixel_base + i, s, pst, nullptr, &ctr[t], true));
                float inv = 1.0f / (float)pst.spp;
                indirect[i] = v3(sum.x * inv, sum.y * inv, sum.z * inv);
            }
        });
    }
    // pass 2: spatial reuse + shading
    std::vector<Reservoir> spatial(n);
    parallel_for((uint32_t)n, nthreads, 64, [&](uint32_t b, uint32_t e, uint32_t t) {
        for (uint32_t i = b; i < e; i++) {
            uint32_t x = i % W, y = i / W;
            V3 c = restir_spatial_shade(S, *vw, *st, gb.data(), R.temporal.data(), &spatial[i], x, y, pixel_base + i, &ctr[t]);
            if (with_indirect && gb[i].valid) c = add(c, indirect[i]);
            if (out && out->radiance) {
                float* r = &out->radiance[4 * (size_t)i];
                r[0] = c.x; r[1] = c.y; r[2] = c.z; r[3] = 1.0f;
            }
        }
    });
    R.history.swap(spatial);
    for (size_t i = 0; i < n; i++) {
        const GPix& g = gb[i];
        float* pn = &R.prev_normals[4 * i];
        if (g.valid) { pn[0] = g.n.x; pn[1] = g.n.y; pn[2] = g.n.z; } else { pn[0] = pn[1] = pn[2] = 0.0f; }
        pn[3] = 0.0f;
    }
    R.history_valid = true;
    if (reservoirs_out) std::memcpy(reservoirs_out, R.history.data(), n * sizeof(Reservoir));
    if (counters)
        for (auto& c : ctr) { counters[0] += c.camera; counters[1] += c.extension; counters[2] += c.shadow; }
    return 0;
}

// ---- unit-level hooks for the golden-vector tests ---------------------------
void snko_pcg32(uint64_t initstate, uint64_t initseq, uint32_t n, uint32_t* out) {
    Pcg r;
    pcg_seed(r, initstate, initseq);
    for (uint32_t i = 0; i < n; i++) out[i] = pcg_next(r);
}
void snko_pcg_stream(uint32_t a, uint32_t b, uint32_t c, uint32_t seed, uint32_t n, float* out) {
    Pcg r = pcg_stream(a, b, c, seed);
    for (uint32_t i = 0; i < n; i++) out[i] = pcg_float(r);
}
void snko_sincos2pi(const float* u, uint32_t n, float* s, float* c) {
    for (uint32_t i = 0; i < n; i++) sincos2pi(u[i], &s[i], &c[i]);
}
// rows of (l3, v3, f03, n3, roughness, metallic) -> (kd3, spec3, ndl, cook_torrance3)
void snko_brdf(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; i++) {
        const float* r = &in[14 * i];
        Terms t = brdf_terms(load3(r), load3(r + 3), load3(r + 6), load3(r + 9), r[12], r[13]);
        V3 ct = cook_torrance(t);
        float* o = &out[10 * i];
        o[0] = t.kd.x; o[1] = t.kd.y; o[2] = t.kd.z; o[3] = t.spec.x; o[4] = t.spec.y; o[5] = t.spec.z;
        o[6] = t.ndl; o[7] = ct.x; o[8] = ct.y; o[9] = ct.z;
    }
}
// rows of (ldir3, colour3, v3, n3, albedo3, roughness, metallic) -> directional radiance
void snko_directional(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; i++) {
        const float* r = &in[17 * i];
        V3 albedo = load3(r + 12);
        V3 f0 = f0_of(albedo, r[16]);
        V3 c = calc_directional(load3(r), load3(r + 3), load3(r + 6), f0, load3(r + 9), r[15], r[16], albedo);
        out[3 * i] = c.x; out[3 * i + 1] = c.y; out[3 * i + 2] = c.z;
    }
}
// rows of (light pos3, colour3, atten c,l,e, world_pos3, v3, n3, albedo3, roughness, metallic) -> radiance
void snko_pointlight(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; i++) {
        const float* r = &in[23 * i];
        PointLight L{};
        L.pos[0] = r[0]; L.pos[1] = r[1]; L.pos[2] = r[2];
        L.colour[0] = r[3]; L.colour[1] = r[4]; L.colour[2] = r[5];
        L.atten_constant = r[6]; L.atten_linear = r[7]; L.atten_exp = r[8];
        V3 albedo = load3(r + 18);
        V3 f0 = f0_of(albedo, r[22]);
        V3 c = calc_pointlight(L, load3(r + 12), f0, load3(r + 9), load3(r + 15), r[21], r[22], albedo);
        out[3 * i] = c.x; out[3 * i + 1] = c.y; out[3 * i + 2] = c.z;
    }
}
// rows of (o3, d3, v0 3, v1 3, v2 3, tmin, tmax) -> (hit, t, b1, b2)
void snko_tri(const float* in, uint32_t n, float* out) {
    for (uint32_t i = 0; i < n; i++) {
        const float* r = &in[17 * i];
        WRay w = wray_setup(load3(r), load3(r + 3), r[15], r[16]);
        float t = 0, b1 = 0, b2 = 0;
        bool h = intersect_tri(w, r + 6, r + 9, r + 12, r[16], &t, &b1, &b2);
        out[4 * i] = h ? 1.0f : 0.0f; out[4 * i + 1] = t; out[4 * i + 2] = b1; out[4 * i + 3] = b2;
    }
}
void snko_invert_affine(const float* m, float* inv, float* nmat, float* det) { invert_affine(m, inv, nmat, det); }
uint32_t snko_num_local_lights(void* sp) { return (uint32_t)((Scene*)sp)->lights.size(); }
// the light-selection table: cdf[k], pmf[k] and the selection weight's record kind (0 sphere, 1 triangle)
void snko_light_table(void* sp, float* cdf, float* pmf, uint32_t* kind) {
    const Scene& S = *(const Scene*)sp;
    for (size_t k = 0; k < S.lights.size(); k++) {
        cdf[k] = S.light_cdf[k];
        pmf[k] = S.light_pmf[k];
        kind[k] = S.lights[k].kind;
    }
}
uint32_t snko_hardware_threads() { return std::max(1u, std::thread::hardware_concurrency()); }

}  // extern "C"

// ---- MLP radiance cache reference (FP64) ------------------------------------
// Network: 64 inputs -> 4 x (64, ReLU) -> 3 linear outputs, no biases.  Weights
// are row-major W_l[in][out] concatenated (4 x 64x64, then 64x3 = 16576 floats).
// Loss: relative L2 of Mueller et al. 2021 (radiance caching), mean over the
// batch and the 3 channels: (y - t)^2 / (sg(y)^2 + 0.01); sample weight w in {0,1}.
static const int MLP_IN = 64, MLP_HID = 64, MLP_OUT = 3;
static const size_t MLP_NW = 4 * 64 * 64 + 64 * 3;
static inline size_t mlp_off(int l) { return (size_t)l * 64 * 64; }

static void mlp_forward_one(const double* W, const double* x, double act[4][64], double* y) {
    const double* in = x;
    for (int l = 0; l < 4; l++) {
        const double* Wl = W + mlp_off(l);
        for (int o = 0; o < 64; o++) {
            double s = 0.0;
            for (int i = 0; i < 64; i++) s += in[i] * Wl[i * 64 + o];
            act[l][o] = s > 0.0 ? s : 0.0;
        }
        in = act[l];
    }
    const double* W5 = W + mlp_off(4);
    for (int o = 0; o < 3; o++) {
        double s = 0.0;
        for (int i = 0; i < 64; i++) s += in[i] * W5[i * 3 + o];
        y[o] = s;
    }
}

extern "C" void snko_mlp_forward(const double* W, const double* x, uint32_t n, double* y) {
    double act[4][64];
    for (uint32_t s = 0; s < n; s++) mlp_forward_one(W, x + 64 * (size_t)s, act, y + 3 * (size_t)s);
}

// loss and dL/dW over a batch (weights w per sample; normaliser = 3 * n).
// relative = 0 uses a plain L2 (denominator 1), for finite-difference checks of
// the back-propagation (the relative loss's stop-gradient makes its gradient
// differ from the derivative of its value on purpose).
extern "C" double snko_mlp_grad(const double* W, const double* x, const double* t, const double* wt, uint32_t n,
                                double* dW, int relative) {
    std::memset(dW, 0, MLP_NW * sizeof(double));
    double loss = 0.0;
    const double norm = 1.0 / (3.0 * (double)n);
    double act[4][64], y[3], g[64], gn[64];
    for (uint32_t s = 0; s < n; s++) {
        const double* xs = x + 64 * (size_t)s;
        mlp_forward_one(W, xs, act, y);
        double gy[3];
        for (int c = 0; c < 3; c++) {
            double d = y[c] - t[3 * (size_t)s + c];
            double den = relative ? y[c] * y[c] + 0.01 : 1.0;
            loss += wt[s] * d * d / den * norm;
            gy[c] = wt[s] * 2.0 * d / den * norm;
        }
        // output layer
        double* dW5 = dW + mlp_off(4);
        const double* W5 = W + mlp_off(4);
        for (int i = 0; i < 64; i++) {
            for (int c = 0; c < 3; c++) dW5[i * 3 + c] += act[3][i] * gy[c];
            double s5 = 0.0;
            for (int c = 0; c < 3; c++) s5 += W5[i * 3 + c] * gy[c];
            g[i] = act[3][i] > 0.0 ? s5 : 0.0;
        }
        for (int l = 3; l >= 0; l--) {
            const double* in = l == 0 ? xs : act[l - 1];
            double* dWl = dW + mlp_off(l);
            const double* Wl = W + mlp_off(l);
            for (int i = 0; i < 64; i++)
                for (int o = 0; o < 64; o++) dWl[i * 64 + o] += in[i] * g[o];
            if (l == 0) break;
            for (int i = 0; i < 64; i++) {
                double sgi = 0.0;
                for (int o = 0; o < 64; o++) sgi += Wl[i * 64 + o] * g[o];
                gn[i] = act[l - 1][i] > 0.0 ? sgi : 0.0;
            }
            std::memcpy(g, gn, sizeof(g));
        }
    }
    return loss;
}

// one Adam step (Kingma & Ba 2015) in place; step >= 1
extern "C" void snko_mlp_adam(double* W, double* m, double* v, const double* dW, uint32_t step, double lr,
                              double b1, double b2, double eps) {
    double c1 = 1.0 - std::pow(b1, (double)step), c2 = 1.0 - std::pow(b2, (double)step);
    for (size_t i = 0; i < MLP_NW; i++) {
        m[i] = b1 * m[i] + (1.0 - b1) * dW[i];
        v[i] = b2 * v[i] + (1.0 - b2) * dW[i] * dW[i];
        W[i] -= lr * (m[i] / c1) / (std::sqrt(v[i] / c2) + eps);
    }
}

// ---- TAA resolve ----------------------------------------------------------------
// TAA_Resolve.comp (Core/res/shaders/TAA_Resolve.comp:12-86) per pixel, reading the
// unresolved frame for every neighbourhood; history and previous velocity fetched
// as texture() with a linear filter and repeat addressing (the pass's sampler,
// Core/src/resources/Images.cpp:16-36), in FP32 with exact weights.  Binary32
// basic operations in the shader's order (compiled with -ffp-contract=off).
namespace {
inline int taa_wrap(int i, int n) {
    int r = i % n;
    return r < 0 ? r + n : r;
}
void taa_bilinear(const float* img, int C, int w, int h, float cu, float cv, float* o) {
    const float u = cu * (float)w - 0.5f, v = cv * (float)h - 0.5f;
    const float fu = std::floor(u), fv = std::floor(v);
    const float a = u - fu, b = v - fv;
    const int i0 = taa_wrap((int)fu, w), i1 = taa_wrap((int)fu + 1, w);
    const int j0 = taa_wrap((int)fv, h), j1 = taa_wrap((int)fv + 1, h);
    const float w00 = (1.0f - a) * (1.0f - b), w10 = a * (1.0f - b), w01 = (1.0f - a) * b, w11 = a * b;
    const float* t00 = img + ((size_t)j0 * w + i0) * C;
    const float* t10 = img + ((size_t)j0 * w + i1) * C;
    const float* t01 = img + ((size_t)j1 * w + i0) * C;
    const float* t11 = img + ((size_t)j1 * w + i1) * C;
    for (int c = 0; c < C; c++) o[c] = ((w00 * t00[c] + w10 * t10[c]) + w01 * t01[c]) + w11 * t11[c];
}
}  // namespace

// cur: w*h RGBA, motion: w*h RG, hist: w*h RGBA, pmot: w*h RG -> out: w*h RGBA
extern "C" void snko_taa_resolve(uint32_t w, uint32_t h, const float* cur, const float* motion, const float* hist,
                                 const float* pmot, float* out) {
    const int W = (int)w, H = (int)h;
    for (int y = 0; y < H; y++) {
        for (int x = 0; x < W; x++) {
            const size_t pix = (size_t)y * W + x;
            const float velx = motion[2 * pix], vely = motion[2 * pix + 1];
            float hx = ((float)x + 0.5f) / (float)W + velx;
            float hy = ((float)y + 0.5f) / (float)H + vely;
            hx = std::fmin(std::fmax(hx, 0.0f), 1.0f);
            hy = std::fmin(std::fmax(hy, 0.0f), 1.0f);
            const float* c0 = cur + 4 * pix;
            float mn[3] = {9999.0f, 9999.0f, 9999.0f}, mx[3] = {-9999.0f, -9999.0f, -9999.0f};
            float m[3] = {0.0f, 0.0f, 0.0f}, m2[3] = {0.0f, 0.0f, 0.0f};
            for (int ox = -1; ox <= 1; ox++) {
                for (int oy = -1; oy <= 1; oy++) {
                    const int qx = std::min(std::max(x + ox, 0), W - 1), qy = std::min(std::max(y + oy, 0), H - 1);
                    const float* q = cur + 4 * ((size_t)qy * W + qx);
                    for (int c = 0; c < 3; c++) {
                        const float col = std::fmax(q[c], 0.0f);
                        mn[c] = std::fmin(mn[c], col);
                        mx[c] = std::fmax(mx[c], col);
                        m[c] = m[c] + col;
                        m2[c] = m2[c] + col * col;
                    }
                }
            }
            const float inv9 = 1.0f / 9.0f, gamma = 0.55f, eps = 0.00000001f;
            float mu[3], minc[3], maxc[3], p[3];
            for (int c = 0; c < 3; c++) {
                mu[c] = m[c] * inv9;
                const float sigma = std::sqrt(std::fabs(m2[c] * inv9 - mu[c] * mu[c]));
                minc[c] = mu[c] - gamma * sigma;
                maxc[c] = mu[c] + gamma * sigma;
                p[c] = std::fmin(std::fmax(mu[c], mn[c]), mx[c]);
            }
            float hc4[4];
            taa_bilinear(hist, 4, W, H, hx, hy, hc4);
            float r[3];
            for (int c = 0; c < 3; c++) r[c] = std::fmax(hc4[c], 0.0f) - p[c];
            for (int c = 0; c < 3; c++) {
                const float rmax = maxc[c] - p[c];
                if (r[c] > rmax + eps) {
                    const float s = rmax / r[c];
                    for (int k = 0; k < 3; k++) r[k] = r[k] * s;
                }
            }
            for (int c = 0; c < 3; c++) {
                const float rmin = minc[c] - p[c];
                if (r[c] < rmin - eps) {
                    const float s = rmin / r[c];
                    for (int k = 0; k < 3; k++) r[k] = r[k] * s;
                }
            }
            float pv[2];
            taa_bilinear(pmot, 2, W, H, hx, hy, pv);
            const float vx = pv[0] + velx, vy = pv[1] + vely;
            const float vlen = std::sqrt(vx * vx + vy * vy);
            const float dis = std::fmin(std::fmax((vlen - 0.001f) * 10.0f, 0.0f), 1.0f);
            float* o = out + 4 * pix;
            for (int c = 0; c < 3; c++) {
                const float hcol = p[c] + r[c];
                const float f = c0[c] * (1.0f - 0.9f) + hcol * 0.9f;
                o[c] = f * (1.0f - dis) + mu[c] * dis;
            }
            o[3] = 1.0f;
        }
    }
}

// ---- particle collision queries ---------------------------------------------------
// ParticleUpdate.rchit:41-67 for the closest hit of a ray, and the scene part of
// ParticleUpdate.rgen (TraceCollisionRay :101-124, ConstrainOffsetWithScene
// :126-148, CalculateGravity :150-165, main :151-166).  The shader's rays stop at
// the first hit the driver finds; these use the closest hit.
namespace {
struct ContactRec { float n[3]; float dist; float p[3]; float pad0; float v[3]; float pad1; };
struct ParticleRec { float pr[4], vel[4], col[4]; };
const float PARTICLE_DT = 1.0f / 120.0f;   // Particle.glsl:1

struct Contact { V3 n; float dist; V3 p; V3 v; };

Contact contact_ray(const Scene& S, V3 o, V3 d, float tmin, float tmax, float timestep) {
    Contact c;
    c.n = v3(0.0f, 0.0f, 0.0f); c.p = c.n; c.v = c.n;
    c.dist = -1.0f;
    HitRec h;
    if (!trace(S, o, d, tmin, tmax, false, &h, nullptr)) return c;
    const InstData& I = S.insts[h.inst];
    const MeshData& M = S.meshes[I.in.mesh_id];
    const uint32_t* ix = &M.idx[3 * h.prim];
    const V3 p0 = load3(&M.pos[3 * ix[0]]), p1 = load3(&M.pos[3 * ix[1]]), p2 = load3(&M.pos[3 * ix[2]]);
    const float b0 = (1.0f - h.u) - h.v;
    const V3 p = add(add(mul(p0, b0), mul(p1, h.u)), mul(p2, h.v));
    V3 nn;
    if (M.has_normals) {
        const V3 n0 = load3(&M.nrm[3 * ix[0]]), n1 = load3(&M.nrm[3 * ix[1]]), n2 = load3(&M.nrm[3 * ix[2]]);
        nn = add(add(mul(n0, b0), mul(n1, h.u)), mul(n2, h.v));
    } else {
        nn = cross(sub(p1, p0), sub(p2, p0));
    }
    c.n = normalize(mat3_mul(I.nmat, nn));
    c.p = add(o, mul(d, h.t));
    const V3 prev = xform_point(I.in.prev_transform, p);
    c.v = v3((c.p.x - prev.x) / timestep, (c.p.y - prev.y) / timestep, (c.p.z - prev.z) / timestep);
    c.dist = h.t;
    return c;
}

void store_contact(ContactRec* o, const Contact& c) {
    o->n[0] = c.n.x; o->n[1] = c.n.y; o->n[2] = c.n.z; o->dist = c.dist;
    o->p[0] = c.p.x; o->p[1] = c.p.y; o->p[2] = c.p.z; o->pad0 = 0.0f;
    o->v[0] = c.v.x; o->v[1] = c.v.y; o->v[2] = c.v.z; o->pad1 = 0.0f;
}
}  // namespace

extern "C" int snko_contact_rays(void* sp, const Ray* rays, uint32_t n, float timestep, ContactRec* out,
                                 uint32_t nthreads) {
    Scene& S = *(Scene*)sp;
    if (!S.built) return 4;
    parallel_for(n, nthreads, 1024, [&](uint32_t b, uint32_t e, uint32_t) {
        for (uint32_t i = b; i < e; i++) {
            const Ray& r = rays[i];
            store_contact(out + i, contact_ray(S, v3(r.ox, r.oy, r.oz), v3(r.dx, r.dy, r.dz), r.tmin, r.tmax, timestep));
        }
    });
    return 0;
}

extern "C" int snko_particle_probe(void* sp, const ParticleRec* P, uint32_t n, float timestep, ContactRec* cand_out,
                                   float* gravity, uint32_t nthreads) {
    Scene& S = *(Scene*)sp;
    if (!S.built) return 4;
    parallel_for(n, nthreads, 1024, [&](uint32_t b, uint32_t e, uint32_t) {
        for (uint32_t i = b; i < e; i++) {
            const ParticleRec& q = P[i];
            const V3 pos = v3(q.pr[0], q.pr[1], q.pr[2]), vel = v3(q.vel[0], q.vel[1], q.vel[2]);
            const float rad = q.pr[3];
            const bool asleep = q.vel[3] < 0.5f;
            Contact cand;
            cand.n = v3(0.0f, 0.0f, 0.0f); cand.p = cand.n; cand.v = cand.n;
            cand.dist = -1.0f;
            float best = 0.0f;
            const float speed = length(vel);
            if (!asleep && speed > 0.0f && speed <= 3.0e38f) {
                const V3 vdir = v3(vel.x / speed, vel.y / speed, vel.z / speed);
                const V3 right = std::fabs(dot(vdir, v3(0.0f, 1.0f, 0.0f))) > 0.99f ? cross(vdir, v3(0.0f, 0.0f, 1.0f))
                                                                                 : cross(vdir, v3(0.0f, 1.0f, 0.0f));
                const V3 up = cross(right, vdir);
                const V3 dirs[3] = {vdir, right, up};
                for (int k = 0; k < 3; k++) {
                    const float len = k == 0 ? speed * PARTICLE_DT + rad * 2.0f : rad * 2.0f;
                    const V3 o = sub(pos, mul(dirs[k], rad));
                    const Contact c = contact_ray(S, o, dirs[k], 0.0f, len, timestep);
                    const float w = length(sub(c.v, vel));
                    if (c.dist > 0.0f && w > best) { best = w; cand = c; }
                }
            }
            store_contact(cand_out + i, cand);
            const Contact g = contact_ray(S, pos, v3(0.0f, -1.0f, 0.0f), 0.0f, rad + 0.001f, timestep);
            gravity[i] = g.dist < 0.0f ? -9.8f * PARTICLE_DT : 0.0f;
        }
    });
    return 0;
}

extern "C" int snko_particle_constrain(void* sp, const ParticleRec* P, const float* off, uint32_t n, float timestep,
                                       float* out, uint32_t nthreads) {
    Scene& S = *(Scene*)sp;
    if (!S.built) return 4;
    parallel_for(n, nthreads, 1024, [&](uint32_t b, uint32_t e, uint32_t) {
        for (uint32_t i = b; i < e; i++) {
            const ParticleRec& q = P[i];
            const V3 o = v3(off[3 * (size_t)i], off[3 * (size_t)i + 1], off[3 * (size_t)i + 2]);
            const float len = length(o);
            V3 res = v3(0.0f, 0.0f, 0.0f);
            if (!(len < 0.00001f)) {
                const V3 dir = v3(o.x / len, o.y / len, o.z / len);
                const float rad = q.pr[3];
                const Contact c = contact_ray(S, v3(q.pr[0], q.pr[1], q.pr[2]), dir, 0.0f, len + rad, timestep);
                if (c.dist > 0.0f) {
                    const float m = std::fmax(c.dist - rad * 0.9f, 0.0f), s = rad * 0.05f;
                    res = add(mul(dir, m), mul(c.n, s));
                } else {
                    res = o;
                }
            }
            out[3 * (size_t)i] = res.x; out[3 * (size_t)i + 1] = res.y; out[3 * (size_t)i + 2] = res.z;
        }
    });
    return 0;
}
