// particles.cu -- scene collision queries of the particle update pass.
// Compiled with --fmad=false (exact binary32 operation order, as the oracle).
//
// Reference: Core/res/shaders/ParticleUpdate.rgen
//   TraceCollisionRay ......... :101-124 (from the particle's back, speed-weighted choice)
//   ConstrainOffsetWithScene .. :126-148
//   CalculateGravity .......... :150-165
//   main (scene part) ......... :151-166
// and ParticleUpdate.rchit:41-67 (contact normal / position / velocity).
// Every query is a closest-hit trace (the shader asks for the first hit found);
// one thread per particle or ray, each traces with the shared traversal core.
#include "snk_frame.h"
#include "snk_trace.cuh"
#include "snk_shade.cuh"
#include "snk_particles.h"

namespace snk {
namespace {

constexpr int PBLK = 128;
constexpr float PARTICLE_DT = 1.0f / 120.0f;   // Particle.glsl:1

struct Contact {
    V3 n;
    float dist;
    V3 p;
    V3 v;
};

__device__ __forceinline__ void store(ContactOut* out, const Contact& c) {
    ContactOut o;
    o.n[0] = c.n.x; o.n[1] = c.n.y; o.n[2] = c.n.z; o.dist = c.dist;
    o.p[0] = c.p.x; o.p[1] = c.p.y; o.p[2] = c.p.z; o.pad0 = 0.0f;
    o.v[0] = c.v.x; o.v[1] = c.v.y; o.v[2] = c.v.z; o.pad1 = 0.0f;
    *out = o;
}

// traceRayEXT + ParticleUpdate.rchit
__device__ __noinline__ Contact contact_ray(const SceneDev& S, V3 o, V3 d, float tmin, float tmax, float timestep,
                                            uint2* sh) {
    Contact c;
    c.n = v3(0.0f, 0.0f, 0.0f); c.p = c.n; c.v = c.n;
    c.dist = -1.0f;
    TraceResult r;
    if (!trace_scene<false, false>(S, o, d, tmin, tmax, r, sh, threadIdx.x, PBLK, nullptr)) return c;
    const InstShade& I = S.inst_shade[r.inst];
    const MeshInfo& M = S.meshes[I.mesh_id];
    const uint32_t* ix = S.indices + M.index_offset + 3ull * r.prim;
    const uint32_t i0 = M.vertex_offset + ix[0], i1 = M.vertex_offset + ix[1], i2 = M.vertex_offset + ix[2];
    const V3 p0 = load3(S.positions + 3ull * i0), p1 = load3(S.positions + 3ull * i1), p2 = load3(S.positions + 3ull * i2);
    const float b0 = (1.0f - r.u) - r.v;
    const V3 p = add(add(mul(p0, b0), mul(p1, r.u)), mul(p2, r.v));
    V3 nn;
    if (M.has_normals) {
        const V3 n0 = load3(S.normals + 3ull * i0), n1 = load3(S.normals + 3ull * i1), n2 = load3(S.normals + 3ull * i2);
        nn = add(add(mul(n0, b0), mul(n1, r.u)), mul(n2, r.v));
    } else {
        nn = cross(sub(p1, p0), sub(p2, p0));
    }
    c.n = normalize(mat3_mul(I.nmat, nn));
    c.p = add(o, mul(d, r.t));
    const V3 prev = xform_point(I.pm, p);
    c.v = v3((c.p.x - prev.x) / timestep, (c.p.y - prev.y) / timestep, (c.p.z - prev.z) / timestep);
    c.dist = r.t;
    return c;
}

__global__ void __launch_bounds__(PBLK) k_contact_rays(SceneDev S, const float4* __restrict__ rays, uint32_t n,
                                                       float timestep, ContactOut* out) {
    __shared__ uint2 sh[TRACE_SH_ROWS * PBLK];
    for (uint32_t i = blockIdx.x * PBLK + threadIdx.x; i < n; i += gridDim.x * PBLK) {
        const float4 a = rays[2ull * i], b = rays[2ull * i + 1];
        store(out + i, contact_ray(S, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), a.w, b.w, timestep, sh));
    }
}

__global__ void __launch_bounds__(PBLK) k_particle_probe(SceneDev S, const ParticleDev* __restrict__ P, uint32_t n,
                                                         float timestep, ContactOut* cand_out, float* gravity) {
    __shared__ uint2 sh[TRACE_SH_ROWS * PBLK];
    for (uint32_t i = blockIdx.x * PBLK + threadIdx.x; i < n; i += gridDim.x * PBLK) {
        const ParticleDev q = P[i];
        const V3 pos = v3(q.pr.x, q.pr.y, q.pr.z), vel = v3(q.vel.x, q.vel.y, q.vel.z);
        const float rad = q.pr.w;
        const bool asleep = q.vel.w < 0.5f;   // IsParticleAsleep
        Contact cand;
        cand.n = v3(0.0f, 0.0f, 0.0f); cand.p = cand.n; cand.v = cand.n;
        cand.dist = -1.0f;
        float best = 0.0f;
        const float speed = length(vel);
        if (!asleep && speed > 0.0f && speed <= 3.0e38f) {
            const V3 vdir = v3(vel.x / speed, vel.y / speed, vel.z / speed);
            const V3 right = fabsf(dot(vdir, v3(0.0f, 1.0f, 0.0f))) > 0.99f ? cross(vdir, v3(0.0f, 0.0f, 1.0f))
                                                                          : cross(vdir, v3(0.0f, 1.0f, 0.0f));
            const V3 up = cross(right, vdir);
            const V3 dirs[3] = {vdir, right, up};
            for (int k = 0; k < 3; k++) {
                const float len = k == 0 ? speed * PARTICLE_DT + rad * 2.0f : rad * 2.0f;
                const V3 o = sub(pos, mul(dirs[k], rad));
                const Contact c = contact_ray(S, o, dirs[k], 0.0f, len, timestep, sh);
                const float w = length(sub(c.v, vel));
                if (c.dist > 0.0f && w > best) { best = w; cand = c; }
            }
        }
        store(cand_out + i, cand);
        const Contact g = contact_ray(S, pos, v3(0.0f, -1.0f, 0.0f), 0.0f, rad + 0.001f, timestep, sh);
        gravity[i] = g.dist < 0.0f ? -9.8f * PARTICLE_DT : 0.0f;
    }
}

__global__ void __launch_bounds__(PBLK) k_particle_constrain(SceneDev S, const ParticleDev* __restrict__ P,
                                                             const float* __restrict__ off, uint32_t n, float timestep,
                                                             float* out) {
    __shared__ uint2 sh[TRACE_SH_ROWS * PBLK];
    for (uint32_t i = blockIdx.x * PBLK + threadIdx.x; i < n; i += gridDim.x * PBLK) {
        const ParticleDev q = P[i];
        const V3 o = v3(off[3ull * i], off[3ull * i + 1], off[3ull * i + 2]);
        const float len = length(o);
        V3 res = v3(0.0f, 0.0f, 0.0f);
        if (!(len < 0.00001f)) {
            const V3 dir = v3(o.x / len, o.y / len, o.z / len);
            const float rad = q.pr.w;
            const Contact c = contact_ray(S, v3(q.pr.x, q.pr.y, q.pr.z), dir, 0.0f, len + rad, timestep, sh);
            if (c.dist > 0.0f) {
                const float m = fmaxf(c.dist - rad * 0.9f, 0.0f), s = rad * 0.05f;
                res = add(mul(dir, m), mul(c.n, s));
            } else {
                res = o;
            }
        }
        out[3ull * i] = res.x; out[3ull * i + 1] = res.y; out[3ull * i + 2] = res.z;
    }
}

inline int pgrid(uint32_t n, int max_blocks) {
    const uint32_t g = (n + PBLK - 1) / PBLK;
    return (int)(g < (uint32_t)max_blocks ? (g ? g : 1u) : (uint32_t)max_blocks);
}

}  // namespace

cudaError_t launch_contact_rays(const SceneDev& S, const float4* rays, uint32_t n, float timestep, ContactOut* out,
                                int max_blocks, cudaStream_t s) {
    k_contact_rays<<<pgrid(n, max_blocks), PBLK, 0, s>>>(S, rays, n, timestep, out);
    return cudaGetLastError();
}

cudaError_t launch_particle_probe(const SceneDev& S, const ParticleDev* p, uint32_t n, float timestep,
                                  ContactOut* cand, float* gravity, int max_blocks, cudaStream_t s) {
    k_particle_probe<<<pgrid(n, max_blocks), PBLK, 0, s>>>(S, p, n, timestep, cand, gravity);
    return cudaGetLastError();
}

cudaError_t launch_particle_constrain(const SceneDev& S, const ParticleDev* p, const float* off, uint32_t n,
                                      float timestep, float* out, int max_blocks, cudaStream_t s) {
    k_particle_constrain<<<pgrid(n, max_blocks), PBLK, 0, s>>>(S, p, off, n, timestep, out);
    return cudaGetLastError();
}

}  // namespace snk
