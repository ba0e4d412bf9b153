// snk_device.cuh -- device-side math, random streams, BRDF and intersection.
//
// Exactness contract: every translation unit that includes this header for
// shading is compiled with --fmad=false and the default -prec-div/-prec-sqrt,
// so each float +,-,*,/,sqrt written below is one correctly rounded binary32
// operation evaluated in the written (left-to-right) order.  The same
// expressions evaluated on any IEEE-754 host give the same bits, which is what
// makes per-ray hits and per-pixel radiance reproducible across devices.
//
// Reference functions (file:line in Snake-VK):
//   FresnelSchlick, DistributionGGX, GeometrySchlickGGX, GeometrySmith,
//   CookTorranceBRDF, CalcDirectionalLight, CalcPointlight
//                                   Core/res/shaders/LightBuffers.glsl:65-157
//   PI = 3.1415926                  Core/res/shaders/LightBuffers.glsl:29
//   hit attribute interpolation     Core/res/shaders/RayClosestHit.rchit:88-111
// Published methods:
//   watertight ray/triangle test    Woop, Benthin, Wald, JCGT 2(1), 2013
//   PCG32 (XSH-RR 64/32)            O'Neill, "PCG: A Family of ... RNGs", 2014
//   splitmix64                      Steele, Lea, Flood, OOPSLA 2014
//   orthonormal basis               Duff et al., JCGT 6(1), 2017
#pragma once
#include <cstdint>

#ifdef __CUDACC__
#define SNK_HD __host__ __device__ __forceinline__
#else
#define SNK_HD inline
#endif

namespace snk {

constexpr uint32_t INVALID = 0xFFFFFFFFu;
constexpr uint32_t MAT_EMISSIVE = 1u;
constexpr float PI = 3.1415926f;          // LightBuffers.glsl:29
constexpr float T_FAR = 10000.0f;         // RayClosestHit.rchit:136 (shadow tmax)
constexpr float SURFACE_BIAS = 0.01f;     // RayClosestHit.rchit:134
constexpr float EXT_TMIN = 0.01f;         // RayGen.rgen:172
constexpr float SHADOW_TMIN = 0.001f;     // RayGen.rgen:114

// --------------------------------------------------------------------------
// vectors
// --------------------------------------------------------------------------
struct V3 { float x, y, z; };
SNK_HD V3 v3(float x, float y, float z) { V3 r; r.x = x; r.y = y; r.z = z; return r; }
SNK_HD V3 add(V3 a, V3 b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
SNK_HD V3 sub(V3 a, V3 b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
SNK_HD V3 mul(V3 a, float s) { return v3(a.x * s, a.y * s, a.z * s); }
SNK_HD V3 cmul(V3 a, V3 b) { return v3(a.x * b.x, a.y * b.y, a.z * b.z); }
SNK_HD V3 divs(V3 a, float s) { return v3(a.x / s, a.y / s, a.z / s); }
SNK_HD V3 neg(V3 a) { return v3(-a.x, -a.y, -a.z); }
SNK_HD float dot(V3 a, V3 b) { return ((a.x * b.x) + (a.y * b.y)) + (a.z * b.z); }
SNK_HD V3 cross(V3 a, V3 b) {
    return v3((a.y * b.z) - (a.z * b.y), (a.z * b.x) - (a.x * b.z), (a.x * b.y) - (a.y * b.x));
}
SNK_HD float length(V3 a) { return sqrtf(dot(a, a)); }
SNK_HD V3 normalize(V3 a) { return divs(a, length(a)); }
SNK_HD float fmax_(float a, float b) { return a > b ? a : b; }
SNK_HD float fmin_(float a, float b) { return a < b ? a : b; }
SNK_HD float clamp01(float x) { return fmin_(fmax_(x, 0.0f), 1.0f); }
SNK_HD float maxc(V3 a) { return fmax_(fmax_(a.x, a.y), a.z); }
SNK_HD V3 load3(const float* p) { return v3(p[0], p[1], p[2]); }
// row-major 3x4 affine transform of a point / direction
SNK_HD V3 xform_point(const float* m, V3 p) {
    return v3(((m[0] * p.x + m[1] * p.y) + m[2] * p.z) + m[3],
              ((m[4] * p.x + m[5] * p.y) + m[6] * p.z) + m[7],
              ((m[8] * p.x + m[9] * p.y) + m[10] * p.z) + m[11]);
}
SNK_HD V3 xform_dir(const float* m, V3 d) {
    return v3((m[0] * d.x + m[1] * d.y) + m[2] * d.z,
              (m[4] * d.x + m[5] * d.y) + m[6] * d.z,
              (m[8] * d.x + m[9] * d.y) + m[10] * d.z);
}
SNK_HD V3 mat3_mul(const float* m, V3 d) {
    return v3((m[0] * d.x + m[1] * d.y) + m[2] * d.z,
              (m[3] * d.x + m[4] * d.y) + m[5] * d.z,
              (m[6] * d.x + m[7] * d.y) + m[8] * d.z);
}

// sin(2 pi u), cos(2 pi u) for u in [0,1): exact quadrant split of 4u, then the
// Taylor series of sin/cos to degree 13/14 in x = r*pi/2 (truncation < 7e-10).
SNK_HD void sincos2pi(float u, float* s, float* c) {
    float u4 = u * 4.0f;
    float q = floorf(u4);
    float r = u4 - q;
    int qi = ((int)q) & 3;
    float x = r * 0x1.921fb6p+0f;
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
    if (qi == 0) { *s = sn; *c = cs; }
    else if (qi == 1) { *s = cs; *c = -sn; }
    else if (qi == 2) { *s = -sn; *c = -cs; }
    else { *s = -cs; *c = sn; }
}

SNK_HD void onb(V3 n, V3* b1, V3* b2) {
    float sign = copysignf(1.0f, n.z);
    float a = -1.0f / (sign + n.z);
    float b = (n.x * n.y) * a;
    *b1 = v3(1.0f + ((sign * n.x) * n.x) * a, sign * b, -(sign * n.x));
    *b2 = v3(b, sign + (n.y * n.y) * a, -n.y);
}

// --------------------------------------------------------------------------
// PCG32 random streams
// --------------------------------------------------------------------------
struct Pcg { uint64_t state, inc; };
SNK_HD uint32_t pcg_next(Pcg& r) {
    uint64_t old = r.state;
    r.state = old * 6364136223846793005ULL + r.inc;
    uint32_t xs = (uint32_t)(((old >> 18u) ^ old) >> 27u);
    uint32_t rot = (uint32_t)(old >> 59u);
    return (xs >> rot) | (xs << ((32u - rot) & 31u));
}
SNK_HD void pcg_seed(Pcg& r, uint64_t initstate, uint64_t initseq) {
    r.state = 0u;
    r.inc = (initseq << 1u) | 1u;
    pcg_next(r);
    r.state += initstate;
    pcg_next(r);
}
SNK_HD float pcg_float(Pcg& r) { return (float)(pcg_next(r) >> 8) * 0x1p-24f; }
SNK_HD uint64_t splitmix64(uint64_t x) {
    uint64_t z = x + 0x9E3779B97F4A7C15ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}
// streams keyed by (pixel, sample, depth, seed) for paths and by
// (pixel, frame, 0x80000000 | pass, seed) for the ReSTIR passes
SNK_HD Pcg pcg_stream(uint32_t a, uint32_t b, uint32_t c, uint32_t seed) {
    uint64_t k0 = splitmix64(((uint64_t)a << 32) | b);
    uint64_t k1 = splitmix64(k0 ^ (((uint64_t)c << 32) | seed));
    Pcg r;
    pcg_seed(r, k1, k0);
    return r;
}

// --------------------------------------------------------------------------
// BRDF (LightBuffers.glsl:65-157)
// --------------------------------------------------------------------------
SNK_HD V3 fresnel_schlick(float cos_theta, V3 f0) {
    float c = clamp01(1.0f - cos_theta);
    float p = ((c * c) * (c * c)) * c;
    return v3(f0.x + (1.0f - f0.x) * p, f0.y + (1.0f - f0.y) * p, f0.z + (1.0f - f0.z) * p);
}
SNK_HD float distribution_ggx(V3 h, V3 n, float roughness) {
    float a = roughness * roughness;
    float a2 = a * a;
    float ndh = fmax_(dot(n, h), 0.0f);
    float ndh2 = ndh * ndh;
    float denom = ndh2 * (a2 - 1.0f) + 1.0f;
    denom = (PI * denom) * denom;
    return a2 / denom;
}
SNK_HD float geometry_schlick_ggx(float ndv, float roughness) {
    float r = roughness + 1.0f;
    float k = (r * r) / 8.0f;
    return ndv / (ndv * (1.0f - k) + k);
}
SNK_HD float geometry_smith(V3 v, V3 l, V3 n, float roughness) {
    float ndv = fmax_(dot(n, v), 0.0f);
    float ndl = fmax_(dot(n, l), 0.0f);
    return geometry_schlick_ggx(ndv, roughness) * geometry_schlick_ggx(ndl, roughness);
}
struct Terms { V3 kd, spec; float ndl; };
// shared body of CookTorranceBRDF and CalcDirectionalLight for a unit light direction
SNK_HD Terms brdf_terms(V3 l, V3 v, V3 f0, V3 n, float roughness, float metallic) {
    V3 vl = add(v, l);
    float vl2 = dot(vl, vl);
    V3 h = vl2 > 0.0f ? divs(vl, sqrtf(vl2)) : n;
    V3 f = fresnel_schlick(fmax_(dot(h, v), 0.0f), f0);
    float ndf = distribution_ggx(h, n, roughness);
    float g = geometry_smith(v, l, n, roughness);
    float ndl = fmax_(dot(n, l), 0.0f);
    float ng = ndf * g;
    float denom = ((4.0f * fmax_(dot(n, v), 0.0f)) * ndl) + 0.0001f;
    Terms t;
    t.spec = v3((ng * f.x) / denom, (ng * f.y) / denom, (ng * f.z) / denom);
    float om = 1.0f - metallic;
    t.kd = v3((1.0f - f.x) * om, (1.0f - f.y) * om, (1.0f - f.z) * om);
    t.ndl = ndl;
    return t;
}
SNK_HD V3 cook_torrance(const Terms& t) {
    return v3((t.kd.x / PI + t.spec.x) * t.ndl, (t.kd.y / PI + t.spec.y) * t.ndl, (t.kd.z / PI + t.spec.z) * t.ndl);
}
SNK_HD V3 calc_directional(V3 ldir, V3 colour, V3 v, V3 f0, V3 n, float roughness, float metallic, V3 albedo) {
    Terms t = brdf_terms(ldir, v, f0, n, roughness, metallic);
    return v3((((t.kd.x * albedo.x) / PI + t.spec.x) * t.ndl) * colour.x,
              (((t.kd.y * albedo.y) / PI + t.spec.y) * t.ndl) * colour.y,
              (((t.kd.z * albedo.z) / PI + t.spec.z) * t.ndl) * colour.z);
}
SNK_HD V3 f0_of(V3 albedo, float metallic) {
    float om = 1.0f - metallic;
    return v3(0.04f * om + albedo.x * metallic, 0.04f * om + albedo.y * metallic, 0.04f * om + albedo.z * metallic);
}

// --------------------------------------------------------------------------
// device scene records
// --------------------------------------------------------------------------
// 8-wide compressed BVH node (80 bytes = 5 x 16 B), the compressed wide node of
// Ylitie, Karras, Laine (HPG 2017): child boxes quantised to 8 bits per plane
// relative to origin p with per-axis power-of-two scales 2^(e-127).
//   w0: p.x p.y p.z | e.x e.y e.z imask (bytes)
//   w1: child_base  | prim_base | meta[0..3] | meta[4..7]
//   w2: qlo_x[8] qlo_y[8]   w3: qlo_z[8] qhi_x[8]   w4: qhi_y[8] qhi_z[8]
// meta: 0 = empty slot; META_INTERNAL = internal child (also bit s of imask);
// leaf = (count << 5) | offset: count 1..LEAF_MAX_LIMIT primitives at
// prim_base + offset, offset + count <= 32.  Internal children are stored
// contiguously from child_base in slot order.
constexpr uint32_t META_INTERNAL = 0x1Fu;   // count 0: never a leaf
constexpr uint32_t LEAF_MAX_LIMIT = 4;       // 8 leaves x 4 primitives = the 32 primitive hit bits
struct alignas(16) WideNode {
    float px, py, pz;
    uint8_t ex, ey, ez, imask;
    uint32_t child_base, prim_base;
    uint8_t meta[8];
    uint8_t qlo[3][8];
    uint8_t qhi[3][8];
};
static_assert(sizeof(WideNode) == 80, "wide node is 80 bytes");

// triangle record: object-space vertices; v0.w holds the triangle index bits
struct alignas(16) TriRecord { float v0[4], v1[4], v2[4]; };
static_assert(sizeof(TriRecord) == 48, "triangle record is 48 bytes");

// instance record for traversal: world->object 3x4 and the BLAS root
struct alignas(16) InstTrace {
    float inv[12];
    uint32_t blas_root, mesh_id, material_id, pad;
};
static_assert(sizeof(InstTrace) == 64, "instance trace record is 64 bytes");

// instance record for shading
struct InstShade {
    float m[12];        // object -> world
    float pm[12];       // previous frame object -> world
    float nmat[9];      // transpose(inverse(mat3(m)))
    float det3;         // determinant(mat3(m))
    uint32_t mesh_id, material_id;
};

struct MeshInfo {
    uint32_t vertex_offset, index_offset, num_triangles, has_normals;
    uint32_t blas_root, pad0, pad1, pad2;
    float lo[4], hi[4];   // object-space bounds (padded)
};

struct MaterialDev { float albedo[3]; float roughness, metallic, ao; uint32_t flags, pad; };
struct PointLightDev { float pos[3]; float radius; float colour[3]; float atten_constant, atten_linear, atten_exp; uint32_t pad[2]; };

struct LocalLight {     // path-tracer NEE table: sphere lights, then emissive triangles
    uint32_t kind, index, pad0, pad1;
    float p0[4], p1[4], p2[4];   // sphere: p0 = centre, p1[0] = radius; triangle: world vertices
    float n[4];                  // triangle unit normal
    float L[4];                  // radiance (w = area)
};

// per emissive instance (ReSTIR candidate sampling): copies of what one candidate
// reads from the instance, mesh and material records, so a candidate costs one
// record fetch before its triangle's indices
struct alignas(16) EmissiveRec {
    float m[12];                 // object -> world (the instance's transform)
    float det3;                  // determinant(mat3(m))
    uint32_t inst, ntri, index_offset;
    uint32_t vertex_offset;
    float albedo[3];             // emitted radiance (the material's albedo)
};
static_assert(sizeof(EmissiveRec) == 80, "emissive record is 80 bytes");

struct DirLightDev { float dir[3]; uint32_t enabled; float colour[3]; float pad; };

// Traversal bounds: the default number of traversal units (node groups and
// primitives) a ray may take, and the capacity of its stack (STACK_SH entries in
// shared memory, the rest in a local array).  A context may lower both
// (snk_tuning.max_traversal_steps / stack_limit); a ray that reaches either
// bound stops and sets a bit in the scene's error word.
constexpr uint32_t MAX_TRAVERSAL_STEPS = 1u << 16;
constexpr int STACK_SH = 8;
// rows of a traversal kernel's shared array per thread: the STACK_SH stack
// entries, then five rows that keep the world ray (origin, direction,
// reciprocal direction and octant) while it is traced
constexpr int TRACE_SH_ROWS = STACK_SH + 5;
constexpr int STACK_MAX = 64;

// device pointers of the whole scene, passed by value to kernels
struct SceneDev {
    const WideNode* blas_nodes;
    const TriRecord* tris;
    const WideNode* tlas_nodes;
    const uint32_t* tlas_prims;
    uint32_t tlas_root;       // INVALID when the scene is empty
    uint32_t num_instances;
    const InstTrace* inst_trace;
    const InstShade* inst_shade;
    const MeshInfo* meshes;
    const float* positions;
    const float* normals;
    const uint32_t* indices;
    const MaterialDev* materials;
    const PointLightDev* point_lights;
    uint32_t num_point_lights;
    uint32_t num_emissive_instances;
    const uint32_t* emissive_instances;
    const EmissiveRec* emissive_recs;   // one per entry of emissive_instances
    const LocalLight* local_lights;
    const float* light_cdf;
    const float* light_pmf;
    uint32_t num_local_lights;
    uint32_t single_leaf;       // non-zero when every leaf of both levels holds one primitive
    DirLightDev dir_light;
    unsigned int* error_word;   // device status: 0 ok, else SNK_ERR_LIMIT info
    uint32_t num_blas_nodes, num_tris, num_tlas_nodes, num_tlas_prims;   // bounds checked by traversal
    uint32_t max_steps;         // traversal units per ray (1..MAX_TRAVERSAL_STEPS)
    int stack_max;              // stack entries per ray (1..STACK_MAX)
};

// --------------------------------------------------------------------------
// watertight ray/triangle test
// --------------------------------------------------------------------------
// The per-ray set-up: the axis permutation packed as kx | ky << 2 | kz << 4 (k) and
// the shear constants; the ray origin is passed to the test separately.
struct WRay {
    uint32_t k;
    float Sx, Sy, Sz;
};
SNK_HD WRay wray_setup(V3 dv) {
    WRay r;
    float d[3] = {dv.x, dv.y, dv.z};
    int kz = 0;
    if (fabsf(d[1]) > fabsf(d[0])) kz = 1;
    if (fabsf(d[2]) > fabsf(kz == 1 ? d[1] : d[0])) kz = 2;
    int kx = kz + 1; if (kx == 3) kx = 0;
    int ky = kx + 1; if (ky == 3) ky = 0;
    if (d[kz] < 0.0f) { int t = kx; kx = ky; ky = t; }
    r.k = (uint32_t)kx | ((uint32_t)ky << 2) | ((uint32_t)kz << 4);
    float dx = kx == 0 ? d[0] : (kx == 1 ? d[1] : d[2]);
    float dy = ky == 0 ? d[0] : (ky == 1 ? d[1] : d[2]);
    float dz = kz == 0 ? d[0] : (kz == 1 ? d[1] : d[2]);
    // one division: the shear constants are dx / dz and dy / dz rounded as
    // dx * (1 / dz) (any per-ray constants keep the test watertight; the CPU
    // oracle rounds them the same way)
#ifdef __CUDA_ARCH__
    r.Sz = __fdiv_rn(1.0f, dz);
    r.Sx = __fmul_rn(dx, r.Sz);
    r.Sy = __fmul_rn(dy, r.Sz);
#else
    r.Sz = 1.0f / dz;
    r.Sx = dx * r.Sz;
    r.Sy = dy * r.Sz;
#endif
    return r;
}
SNK_HD float sel3(const float* a, int k) { return k == 0 ? a[0] : (k == 1 ? a[1] : a[2]); }
// Returns true for a hit with tmin < t < tmax; exact binary32 arithmetic via
// _rn intrinsics on the device (so the result does not depend on --fmad).
SNK_HD bool intersect_tri(const WRay& r, V3 org, const float* v0, const float* v1, const float* v2, float tmin,
                          float tmax, float* t_out, float* b1_out, float* b2_out) {
#ifdef __CUDA_ARCH__
#define SNK_SUB __fsub_rn
#define SNK_MUL __fmul_rn
#define SNK_ADD __fadd_rn
#define SNK_DIV __fdiv_rn
#else
#define SNK_SUB(a, b) ((a) - (b))
#define SNK_MUL(a, b) ((a) * (b))
#define SNK_ADD(a, b) ((a) + (b))
#define SNK_DIV(a, b) ((a) / (b))
#endif
    float A[3] = {SNK_SUB(v0[0], org.x), SNK_SUB(v0[1], org.y), SNK_SUB(v0[2], org.z)};
    float B[3] = {SNK_SUB(v1[0], org.x), SNK_SUB(v1[1], org.y), SNK_SUB(v1[2], org.z)};
    float C[3] = {SNK_SUB(v2[0], org.x), SNK_SUB(v2[1], org.y), SNK_SUB(v2[2], org.z)};
    const int kx = (int)(r.k & 3u), ky = (int)((r.k >> 2) & 3u), kz = (int)(r.k >> 4);
    float Akx = sel3(A, kx), Aky = sel3(A, ky), Akz = sel3(A, kz);
    float Bkx = sel3(B, kx), Bky = sel3(B, ky), Bkz = sel3(B, kz);
    float Ckx = sel3(C, kx), Cky = sel3(C, ky), Ckz = sel3(C, kz);
    float Ax = SNK_SUB(Akx, SNK_MUL(r.Sx, Akz)), Ay = SNK_SUB(Aky, SNK_MUL(r.Sy, Akz));
    float Bx = SNK_SUB(Bkx, SNK_MUL(r.Sx, Bkz)), By = SNK_SUB(Bky, SNK_MUL(r.Sy, Bkz));
    float Cx = SNK_SUB(Ckx, SNK_MUL(r.Sx, Ckz)), Cy = SNK_SUB(Cky, SNK_MUL(r.Sy, Ckz));
    float U = SNK_SUB(SNK_MUL(Cx, By), SNK_MUL(Cy, Bx));
    float V = SNK_SUB(SNK_MUL(Ax, Cy), SNK_MUL(Ay, Cx));
    float W = SNK_SUB(SNK_MUL(Bx, Ay), SNK_MUL(By, Ax));
    if (U == 0.0f || V == 0.0f || W == 0.0f) {
#ifdef __CUDA_ARCH__
        U = __double2float_rn(__dsub_rn(__dmul_rn((double)Cx, (double)By), __dmul_rn((double)Cy, (double)Bx)));
        V = __double2float_rn(__dsub_rn(__dmul_rn((double)Ax, (double)Cy), __dmul_rn((double)Ay, (double)Cx)));
        W = __double2float_rn(__dsub_rn(__dmul_rn((double)Bx, (double)Ay), __dmul_rn((double)By, (double)Ax)));
#else
        U = (float)((double)Cx * (double)By - (double)Cy * (double)Bx);
        V = (float)((double)Ax * (double)Cy - (double)Ay * (double)Cx);
        W = (float)((double)Bx * (double)Ay - (double)By * (double)Ax);
#endif
    }
    if ((U < 0.0f || V < 0.0f || W < 0.0f) && (U > 0.0f || V > 0.0f || W > 0.0f)) return false;
    float det = SNK_ADD(SNK_ADD(U, V), W);
    if (det == 0.0f) return false;
    float Az = SNK_MUL(r.Sz, Akz), Bz = SNK_MUL(r.Sz, Bkz), Cz = SNK_MUL(r.Sz, Ckz);
    float T = SNK_ADD(SNK_ADD(SNK_MUL(U, Az), SNK_MUL(V, Bz)), SNK_MUL(W, Cz));
    float t = SNK_DIV(T, det);
    if (!(t > tmin && t < tmax)) return false;
    *t_out = t;
    *b1_out = SNK_DIV(V, det);
    *b2_out = SNK_DIV(W, det);
    return true;
#undef SNK_SUB
#undef SNK_MUL
#undef SNK_ADD
#undef SNK_DIV
}

// object-space ray of an instance, exact order (xform with the float inverse)
SNK_HD V3 xform_point_rn(const float* m, V3 p) {
#ifdef __CUDA_ARCH__
    return v3(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[0], p.x), __fmul_rn(m[1], p.y)), __fmul_rn(m[2], p.z)), m[3]),
              __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[4], p.x), __fmul_rn(m[5], p.y)), __fmul_rn(m[6], p.z)), m[7]),
              __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(m[8], p.x), __fmul_rn(m[9], p.y)), __fmul_rn(m[10], p.z)), m[11]));
#else
    return xform_point(m, p);
#endif
}
SNK_HD V3 xform_dir_rn(const float* m, V3 d) {
#ifdef __CUDA_ARCH__
    return v3(__fadd_rn(__fadd_rn(__fmul_rn(m[0], d.x), __fmul_rn(m[1], d.y)), __fmul_rn(m[2], d.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m[4], d.x), __fmul_rn(m[5], d.y)), __fmul_rn(m[6], d.z)),
              __fadd_rn(__fadd_rn(__fmul_rn(m[8], d.x), __fmul_rn(m[9], d.y)), __fmul_rn(m[10], d.z)));
#else
    return xform_dir(m, d);
#endif
}

}  // namespace snk
