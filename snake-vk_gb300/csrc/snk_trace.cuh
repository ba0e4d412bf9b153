// snk_trace.cuh -- two-level traversal of 8-wide compressed BVHs.
//
// Replaces traceRayEXT (Core/res/shaders/RayGen.rgen:101-121, 164-176, 195-207;
// RayClosestHit.rchit:64-84), which runs on the driver's RT-core traversal in
// the reference.  Semantics (BVH independent, so every device and the CPU
// oracle agree bit for bit):
//   closest hit = the minimum of (t, instance, triangle) over all triangles
//                 with tmin < t < tmax under the watertight test;
//   any hit     = whether such a triangle exists.
// Box tests are only required to be conservative: child boxes are quantised
// outwards and accepted with a relative slack of 1e-5 in t.
//
// Traversal scheme (Ylitie, Karras, Laine, HPG 2017): the current node group
// is (child_base, hit bits of internal children << 24 | imask) and the current
// primitive group is (prim_base, 24 primitive hit bits).  Groups are kept on a
// short per-thread stack in shared memory ([entry][thread] layout, conflict
// free) that spills to local memory.  Children are visited in the order of the
// slot index xor the ray octant, which the builder makes approximately
// front-to-back.  Leaves of the instance BVH hold instance ids: on reaching one
// the ray is transformed into object space and the BLAS root is entered; when
// the stack unwinds to the entry depth, the world ray is restored.
#pragma once
#include "snk_device.cuh"

namespace snk {

constexpr int STACK_SH = 8;           // shared-memory entries per thread
constexpr int STACK_MAX = 64;         // total entries (shared + local spill)
constexpr uint32_t MAX_TRAVERSAL_STEPS = 1u << 16;   // node groups popped per ray

// device error word bits
constexpr unsigned ERR_STACK_OVERFLOW = 1u;
constexpr unsigned ERR_STEP_LIMIT = 2u;
constexpr unsigned ERR_BAD_INDEX = 4u;    // a node/primitive/instance index outside its array

struct NodeRay {
    float ox, oy, oz;
    float idx, idy, idz;
    uint32_t oct;   // bit i set when direction component i is negative
};

__device__ __forceinline__ float safe_rcp(float d) {
    return 1.0f / (fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d));
}

__device__ __forceinline__ NodeRay make_node_ray(V3 o, V3 d) {
    NodeRay r;
    r.ox = o.x; r.oy = o.y; r.oz = o.z;
    r.idx = safe_rcp(d.x); r.idy = safe_rcp(d.y); r.idz = safe_rcp(d.z);
    r.oct = (d.x < 0.0f ? 1u : 0u) | (d.y < 0.0f ? 2u : 0u) | (d.z < 0.0f ? 4u : 0u);
    return r;
}

__device__ __forceinline__ float byte_f(uint32_t w, uint32_t k) { return (float)((w >> (8u * k)) & 0xFFu); }

// Tests the 8 children of node idx.  ngroup <- (child_base, internal hits << 24 | imask)
// with internal hit bits at position (slot ^ oct); tgroup <- (prim_base, primitive hits).
__device__ __forceinline__ void intersect_node(const WideNode* __restrict__ nodes, uint32_t idx, const NodeRay& r,
                                               float tmin, float tmax, uint2& ngroup, uint2& tgroup) {
    const float4* np = reinterpret_cast<const float4*>(nodes + idx);
    float4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    uint32_t e = __float_as_uint(w0.w);
    float sx = __uint_as_float((e & 0xFFu) << 23);
    float sy = __uint_as_float(((e >> 8) & 0xFFu) << 23);
    float sz = __uint_as_float(((e >> 16) & 0xFFu) << 23);
    uint32_t imask = e >> 24;
    float ax = sx * r.idx, ay = sy * r.idy, az = sz * r.idz;
    float bx = (w0.x - r.ox) * r.idx, by = (w0.y - r.oy) * r.idy, bz = (w0.z - r.oz) * r.idz;
    uint32_t meta_lo = __float_as_uint(w1.z), meta_hi = __float_as_uint(w1.w);
    uint32_t qlx[2] = {__float_as_uint(w2.x), __float_as_uint(w2.y)};
    uint32_t qly[2] = {__float_as_uint(w2.z), __float_as_uint(w2.w)};
    uint32_t qlz[2] = {__float_as_uint(w3.x), __float_as_uint(w3.y)};
    uint32_t qhx[2] = {__float_as_uint(w3.z), __float_as_uint(w3.w)};
    uint32_t qhy[2] = {__float_as_uint(w4.x), __float_as_uint(w4.y)};
    uint32_t qhz[2] = {__float_as_uint(w4.z), __float_as_uint(w4.w)};
    uint32_t hit_int = 0, hit_prim = 0;
#pragma unroll
    for (int s = 0; s < 8; s++) {
        uint32_t meta = ((s < 4 ? meta_lo : meta_hi) >> (8 * (s & 3))) & 0xFFu;
        if (meta == 0) continue;
        const int h = s >> 2, k = s & 3;
        float tx0 = __fmaf_rn(byte_f(qlx[h], k), ax, bx), tx1 = __fmaf_rn(byte_f(qhx[h], k), ax, bx);
        float ty0 = __fmaf_rn(byte_f(qly[h], k), ay, by), ty1 = __fmaf_rn(byte_f(qhy[h], k), ay, by);
        float tz0 = __fmaf_rn(byte_f(qlz[h], k), az, bz), tz1 = __fmaf_rn(byte_f(qhz[h], k), az, bz);
        float tn = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), tmin));
        float tf = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
        float slack = (fabsf(tn) + fabsf(tf)) * 1e-5f + 1e-7f;
        if (tn <= tf + slack) {
            if (meta & 0x80u) {
                hit_int |= 1u << ((uint32_t)s ^ r.oct);
            } else {
                uint32_t cnt = (meta >> 5) & 3u, off = meta & 31u;
                hit_prim |= ((1u << cnt) - 1u) << off;
            }
        }
    }
    ngroup = make_uint2(__float_as_uint(w1.x), (hit_int << 24) | imask);
    tgroup = make_uint2(__float_as_uint(w1.y), hit_prim);
}

struct TraceResult { float t, u, v; uint32_t inst, prim; bool hit; };

struct TraceCounters { unsigned long long nodes, tris; };

// Short stack: entries [0, STACK_SH) live in shared memory at sh[k * nthreads + tid],
// deeper entries in a local array.
struct ShortStack {
    uint2* sh;
    uint32_t tid, nthreads;
    int sp;
    uint2 spill[STACK_MAX - STACK_SH];
    __device__ __forceinline__ bool push(uint2 v) {
        if (sp < STACK_SH) sh[sp * nthreads + tid] = v;
        else if (sp < STACK_MAX) spill[sp - STACK_SH] = v;
        else return false;
        sp++;
        return true;
    }
    __device__ __forceinline__ uint2 pop() {
        sp--;
        return sp < STACK_SH ? sh[sp * nthreads + tid] : spill[sp - STACK_SH];
    }
};

template <bool ANY, bool COUNT>
__device__ __forceinline__ bool trace_scene(const SceneDev& S, V3 o, V3 d, float tmin, float tmax, TraceResult& res,
                                         uint2* sh_stack, uint32_t tid, uint32_t nthreads, TraceCounters* ctr) {
    res.hit = false;
    res.t = -1.0f; res.u = 0.0f; res.v = 0.0f; res.inst = INVALID; res.prim = INVALID;
    if (S.tlas_root == INVALID) return false;
    const NodeRay wr = make_node_ray(o, d);
    NodeRay cr = wr;
    WRay tri_ray;
    float best_t = tmax;
    bool found = false;
    uint32_t best_inst = INVALID, best_prim = INVALID;
    float best_u = 0.0f, best_v = 0.0f;
    int level = 0, blas_sp = 0;
    uint32_t cur_inst = 0;
    ShortStack st;
    st.sh = sh_stack; st.tid = tid; st.nthreads = nthreads; st.sp = 0;
    uint2 ngroup = make_uint2(S.tlas_root, (1u << (24 + cr.oct)) | 1u);
    uint32_t steps = 0;
    unsigned err = 0;
    while (true) {
        if (++steps > MAX_TRAVERSAL_STEPS) { err |= ERR_STEP_LIMIT; break; }
        uint2 tgroup = make_uint2(0u, 0u);
        if (ngroup.y > 0x00FFFFFFu) {
            uint32_t k = __ffs(ngroup.y >> 24) - 1;
            ngroup.y &= ~(1u << (24 + k));
            uint32_t slot = k ^ cr.oct;
            uint32_t child = ngroup.x + __popc(ngroup.y & ((1u << slot) - 1u) & 0xFFu);
            if (ngroup.y > 0x00FFFFFFu) {
                if (!st.push(ngroup)) { err |= ERR_STACK_OVERFLOW; break; }
            }
            if (COUNT) ctr->nodes++;
            if (child >= (level ? S.num_blas_nodes : S.num_tlas_nodes)) { err |= ERR_BAD_INDEX; break; }
            intersect_node(level ? S.blas_nodes : S.tlas_nodes, child, cr, tmin, best_t, ngroup, tgroup);
        } else {
            tgroup = ngroup;
            ngroup = make_uint2(0u, 0u);
        }
        while (tgroup.y != 0u) {
            uint32_t k = __ffs(tgroup.y) - 1;
            tgroup.y &= tgroup.y - 1u;
            uint32_t pidx = tgroup.x + k;
            if (level == 0) {
                if (pidx >= S.num_tlas_prims) { err |= ERR_BAD_INDEX; break; }
                uint32_t inst = __ldg(&S.tlas_prims[pidx]);
                if (inst >= S.num_instances) { err |= ERR_BAD_INDEX; break; }
                if (tgroup.y != 0u && !st.push(tgroup)) { err |= ERR_STACK_OVERFLOW; break; }
                if (ngroup.y > 0x00FFFFFFu && !st.push(ngroup)) { err |= ERR_STACK_OVERFLOW; break; }
                const float4* ip = reinterpret_cast<const float4*>(S.inst_trace + inst);
                float4 r0 = __ldg(ip), r1 = __ldg(ip + 1), r2 = __ldg(ip + 2), r3 = __ldg(ip + 3);
                float inv[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
                V3 oo = xform_point_rn(inv, o);
                V3 od = xform_dir_rn(inv, d);
                cr = make_node_ray(oo, od);
                tri_ray = wray_setup(oo, od);
                blas_sp = st.sp;
                level = 1;
                cur_inst = inst;
                ngroup = make_uint2(__float_as_uint(r3.x), (1u << (24 + cr.oct)) | 1u);
                tgroup.y = 0u;
                break;
            } else {
                if (pidx >= S.num_tris) { err |= ERR_BAD_INDEX; break; }
                if (COUNT) ctr->tris++;
                const float4* tp = reinterpret_cast<const float4*>(S.tris + pidx);
                float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                float va[3] = {a.x, a.y, a.z}, vb[3] = {b.x, b.y, b.z}, vc[3] = {c.x, c.y, c.z};
                float t, b1, b2;
                if (intersect_tri(tri_ray, va, vb, vc, tmin, tmax, &t, &b1, &b2)) {
                    uint32_t prim = __float_as_uint(a.w);
                    if (ANY) {
                        found = true; best_t = t; best_inst = cur_inst; best_prim = prim; best_u = b1; best_v = b2;
                        goto done;
                    }
                    bool better = !found || t < best_t ||
                                  (t == best_t && (cur_inst < best_inst || (cur_inst == best_inst && prim < best_prim)));
                    if (better) {
                        found = true; best_t = t; best_inst = cur_inst; best_prim = prim; best_u = b1; best_v = b2;
                    }
                }
            }
        }
        if (err) break;
        if (ngroup.y > 0x00FFFFFFu) continue;
        if (level == 1 && st.sp == blas_sp) { level = 0; cr = wr; }
        if (st.sp == 0) break;
        ngroup = st.pop();
    }
done:
    if (err) {
        if (S.error_word) atomicOr(S.error_word, err);
        return false;
    }
    if (found) {
        res.hit = true; res.t = best_t; res.inst = best_inst; res.prim = best_prim; res.u = best_u; res.v = best_v;
    }
    return found;
}

}  // namespace snk
