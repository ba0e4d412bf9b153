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
// outwards and accepted with a slack of BOX_SLACK_ULPS units in the last place
// of the exit distance.  tmin below 0 (or NaN) is taken as 0, as traceRayEXT
// requires tmin >= 0; entry distances are then never negative.
//
// Traversal scheme (Ylitie, Karras, Laine, HPG 2017): the current node group
// is (child_base, hit bits of internal children << 24 | imask) and the current
// primitive group is (prim_base, 32 primitive hit bits).  Groups are kept on a
// short per-thread stack in shared memory ([entry][thread] layout, conflict
// free) that spills to local memory; primitive groups carry PRIM_GROUP in the
// base word there.  Closest-hit rays visit children in the order of the slot
// index xor the ray octant, which the builder makes approximately front to back;
// any-hit rays visit them in slot order.  Leaves of the instance BVH hold instance ids: on reaching one
// the ray is transformed into object space and the BLAS root is entered; when
// the stack unwinds to the entry depth, the world ray is restored.  Coherent rays
// (the camera rays of large views) can instead be traced 32 at a time by a whole
// warp (PacketTraverser, below), with the same results.
#pragma once
#include "snk_device.cuh"

namespace snk {

constexpr uint32_t PRIM_GROUP = 0x80000000u;         // stack tag of a primitive group (bases are < 2^31)
// A child box is accepted when bits(t_enter) <= bits(t_exit) + BOX_SLACK_ULPS as
// signed integers.  With t_enter >= tmin >= 0 this orders like the floats, and
// the slack (>= 2^-19 of t_exit) covers the 2-ulp reciprocal of the direction and
// the final rounding of each plane distance (about 6 ulps of t in all); a
// negative t_exit (box behind the origin) compares below every t_enter.  The
// absolute rounding of the plane offsets is covered by the per-axis widening.
constexpr int BOX_SLACK_ULPS = 32;

// device error word bits
constexpr unsigned ERR_STACK_OVERFLOW = 1u;
constexpr unsigned ERR_STEP_LIMIT = 2u;
constexpr unsigned ERR_BAD_INDEX = 4u;    // a node/primitive/instance index outside its array

struct NodeRay {
    float ox, oy, oz;
    float idx, idy, idz;
    uint32_t oct;   // bit i set when direction component i is negative
};

// Reciprocal for box tests only (they need to be conservative, not exact): the
// fast approximate division is within 2 ulp, inside BOX_SLACK_ULPS.
__device__ __forceinline__ float safe_rcp(float d) {
    return __fdividef(1.0f, fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d));
}

__device__ __forceinline__ NodeRay make_node_ray(V3 o, V3 d) {
    NodeRay r;
    r.ox = o.x; r.oy = o.y; r.oz = o.z;
    r.idx = safe_rcp(d.x); r.idy = safe_rcp(d.y); r.idz = safe_rcp(d.z);
    // sign bits (not d < 0): -0.0 has a negative reciprocal and must enter through the high plane
    r.oct = (__float_as_uint(d.x) >> 31) | ((__float_as_uint(d.y) >> 31) << 1) | ((__float_as_uint(d.z) >> 31) << 2);
    return r;
}

// Three-input maximum / minimum (one instruction on sm_100 and later; NaN inputs
// are ignored, as with fmaxf / fminf).
__device__ __forceinline__ float max3f(float a, float b, float c) {
    float d;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
__device__ __forceinline__ float min3f(float a, float b, float c) {
    float d;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
    return d;
}
// ((1 << len) - 1) << pos in one instruction
__device__ __forceinline__ uint32_t bit_mask(uint32_t pos, uint32_t len) {
    uint32_t d;
    asm("bmsk.clamp.b32 %0, %1, %2;" : "=r"(d) : "r"(pos), "r"(len));
    return d;
}

// Byte k of w as 1 + q 2^-15 (bits 8..15 of the mantissa of 1.0f): one byte permute.
__device__ __forceinline__ float byte_m(uint32_t w, uint32_t k) {
    return __uint_as_float(__byte_perm(w, 0x3F800000u, 0x7604u | (k << 4)));
}

// Box tests of the 8 children of a node (words w0, w2, w3, w4) against ray r on
// [tmin, tmax]: bit s of the result is set when the box of slot s is hit.
// Near/far planes are swapped once per node by the ray octant; each plane costs a
// byte permute and half a packed FMA, and an integer compare with BOX_SLACK_ULPS of slack
// (on top of the per-axis widening below) keeps the test conservative.
__device__ __forceinline__ uint32_t box_hits(const float4& w0, const float4& w2, const float4& w3, const float4& w4,
                                             const NodeRay& r, float tmin, float tmax) {
    const uint32_t e = __float_as_uint(w0.w);
    // per axis A = 2^15 x (grid step) / d, B = (p - o) / d - A rounded once; a plane
    // byte q decodes as x = 1 + q 2^-15 (one byte permute), so t = fma(x, A, B).
    // B's rounding (at most |A| 2^-24) is covered with room to spare by moving the
    // near planes down and the far planes up by |A| 2^-21 (1/64 of a grid step).
    const float ax = __uint_as_float(((e & 0xFFu) + 15u) << 23) * r.idx;
    const float ay = __uint_as_float((((e >> 8) & 0xFFu) + 15u) << 23) * r.idy;
    const float az = __uint_as_float((((e >> 16) & 0xFFu) + 15u) << 23) * r.idz;
    const float bx = __fmaf_rn(w0.x - r.ox, r.idx, -ax), by = __fmaf_rn(w0.y - r.oy, r.idy, -ay),
                bz = __fmaf_rn(w0.z - r.oz, r.idz, -az);
    const float mx = fabsf(ax) * 4.76837158e-7f, my = fabsf(ay) * 4.76837158e-7f, mz = fabsf(az) * 4.76837158e-7f;
    const float bnx = bx - mx, bfx = bx + mx, bny = by - my, bfy = by + my, bnz = bz - mz, bfz = bz + mz;
    const bool sx = r.oct & 1u, sy = r.oct & 2u, sz = r.oct & 4u;
    uint32_t lx0 = __float_as_uint(w2.x), lx1 = __float_as_uint(w2.y), ly0 = __float_as_uint(w2.z),
             ly1 = __float_as_uint(w2.w), lz0 = __float_as_uint(w3.x), lz1 = __float_as_uint(w3.y),
             hx0 = __float_as_uint(w3.z), hx1 = __float_as_uint(w3.w), hy0 = __float_as_uint(w4.x),
             hy1 = __float_as_uint(w4.y), hz0 = __float_as_uint(w4.z), hz1 = __float_as_uint(w4.w);
    // near / far plane words per axis (a negative direction enters through the high plane)
    uint32_t nx[2] = {sx ? hx0 : lx0, sx ? hx1 : lx1}, fx[2] = {sx ? lx0 : hx0, sx ? lx1 : hx1};
    uint32_t ny[2] = {sy ? hy0 : ly0, sy ? hy1 : ly1}, fy[2] = {sy ? ly0 : hy0, sy ? ly1 : hy1};
    uint32_t nz[2] = {sz ? hz0 : lz0, sz ? hz1 : lz1}, fz[2] = {sz ? lz0 : hz0, sz ? lz1 : hz1};
    uint32_t hits = 0;   // bit s: the box of slot s is hit
    // children s and s + 1 in one packed FMA per plane (sm_100 and later: two
    // binary32 FMAs per instruction, each rounded as fmaf)
    const float2 AX = make_float2(ax, ax), AY = make_float2(ay, ay), AZ = make_float2(az, az);
    const float2 BNX = make_float2(bnx, bnx), BNY = make_float2(bny, bny), BNZ = make_float2(bnz, bnz);
    const float2 BFX = make_float2(bfx, bfx), BFY = make_float2(bfy, bfy), BFZ = make_float2(bfz, bfz);
#pragma unroll
    for (int s = 0; s < 8; s += 2) {
        const int h = s >> 2, k = s & 3;
        const float2 tnx = __ffma2_rn(make_float2(byte_m(nx[h], k), byte_m(nx[h], k + 1)), AX, BNX);
        const float2 tny = __ffma2_rn(make_float2(byte_m(ny[h], k), byte_m(ny[h], k + 1)), AY, BNY);
        const float2 tnz = __ffma2_rn(make_float2(byte_m(nz[h], k), byte_m(nz[h], k + 1)), AZ, BNZ);
        const float2 tfx = __ffma2_rn(make_float2(byte_m(fx[h], k), byte_m(fx[h], k + 1)), AX, BFX);
        const float2 tfy = __ffma2_rn(make_float2(byte_m(fy[h], k), byte_m(fy[h], k + 1)), AY, BFY);
        const float2 tfz = __ffma2_rn(make_float2(byte_m(fz[h], k), byte_m(fz[h], k + 1)), AZ, BFZ);
        const float tn0 = max3f(tnx.x, tny.x, fmaxf(tnz.x, tmin)), tn1 = max3f(tnx.y, tny.y, fmaxf(tnz.y, tmin));
        const float tf0 = min3f(tfx.x, tfy.x, fminf(tfz.x, tmax)), tf1 = min3f(tfx.y, tfy.y, fminf(tfz.y, tmax));
        hits |= (__float_as_int(tn0) <= __float_as_int(tf0) + BOX_SLACK_ULPS) ? (1u << s) : 0u;
        hits |= (__float_as_int(tn1) <= __float_as_int(tf1) + BOX_SLACK_ULPS) ? (2u << s) : 0u;
    }
    return hits;
}

// Leaf slots of a single-primitive-leaf node (meta count bits 1: bit 5 of each
// byte), gathered from the four bytes of each meta word by one multiply.
__device__ __forceinline__ uint32_t leaf_slots(uint32_t meta0, uint32_t meta1) {
    const uint32_t l0 = (meta0 >> 5) & 0x01010101u, l1 = (meta1 >> 5) & 0x01010101u;
    return ((l0 * 0x10204080u) >> 28) | (((l1 * 0x10204080u) >> 28) << 4);
}

// Child bits in visiting order for octant oct: bit s moves to s ^ oct (three
// conditional swaps).
__device__ __forceinline__ uint32_t visit_order(uint32_t x, uint32_t oct) {
    x = (oct & 1u) ? (((x & 0x55u) << 1) | ((x >> 1) & 0x55u)) : x;
    x = (oct & 2u) ? (((x & 0x33u) << 2) | ((x >> 2) & 0x33u)) : x;
    x = (oct & 4u) ? (((x & 0x0Fu) << 4) | ((x >> 4) & 0x0Fu)) : x;
    return x;
}

// Tests the 8 children of node idx.  ngroup <- (child_base, internal hits << 24 | imask)
// with internal hit bit of slot s at position s ^ oct (ORDERED) or s; tgroup <- (prim_base,
// primitive hits).  The internal-child bits are moved into visiting order with three
// conditional swaps (bit s -> s ^ oct) when the order matters (closest hit; an any-hit
// ray stops at whichever occluder it meets first and skips the swaps), and only the
// hit leaf slots are expanded into primitive bits.
template <bool ORDERED, bool SINGLE>
__device__ __forceinline__ void intersect_node(const WideNode* __restrict__ nodes, uint32_t idx, const NodeRay& r,
                                               float tmin, float tmax, uint2& ngroup, uint2& tgroup) {
    const float4* np = reinterpret_cast<const float4*>(nodes + idx);
    float4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3), w4 = __ldg(np + 4);
    const uint32_t imask = __float_as_uint(w0.w) >> 24;
    const uint32_t meta0 = __float_as_uint(w1.z), meta1 = __float_as_uint(w1.w);
    const uint32_t hits = box_hits(w0, w2, w3, w4, r, tmin, tmax);
    // internal children (imask bits) in visiting order: bit s moves to s ^ oct
    uint32_t x = hits & imask;
    if (ORDERED) x = visit_order(x, r.oct);
    ngroup = make_uint2(__float_as_uint(w1.x), (x << 24) | imask);
    if constexpr (SINGLE) {
        // every leaf holds one primitive, stored in slot order; primitive groups are
        // (prim_base, hit leaf slots << 24 | leaf slots), like node groups
        const uint32_t leafmask = leaf_slots(meta0, meta1);
        tgroup = make_uint2(__float_as_uint(w1.y), ((hits & leafmask) << 24) | leafmask);
    } else {
        // leaf children: (count << 5) | offset -> primitive bits; an empty slot (meta 0) adds none
        uint32_t leaves = hits & ~imask, hit_prim = 0;
        while (leaves) {
            const uint32_t s = __ffs(leaves) - 1;
            leaves &= leaves - 1u;
            const uint32_t m = __byte_perm(meta0, meta1, s) & 0xFFu;
            hit_prim |= bit_mask(m & 31u, m >> 5);
        }
        tgroup = make_uint2(__float_as_uint(w1.y), hit_prim);
    }
}

struct TraceResult { float t, u, v; uint32_t inst, prim; bool hit; };

struct TraceCounters { unsigned long long nodes, tris; };

// Short stack: entries [0, STACK_SH) live in shared memory at sh[k * nthreads + tid],
// deeper entries in a local array; at most lim (<= STACK_MAX) entries.  Rows
// STACK_SH .. STACK_SH + 4 of sh (TRACE_SH_ROWS rows in all) keep the world ray.
struct ShortStack {
    uint2* sh;
    uint2* spill;   // STACK_MAX - STACK_SH entries (a local array of the caller)
    uint32_t tid, nthreads;
    int sp, lim;
    __device__ __forceinline__ bool push(uint2 v) {
        if (sp >= lim) return false;
        if (sp < STACK_SH) sh[sp * nthreads + tid] = v;
        else spill[sp - STACK_SH] = v;
        sp++;
        return true;
    }
    __device__ __forceinline__ uint2 pop() {
        sp--;
        return sp < STACK_SH ? sh[sp * nthreads + tid] : spill[sp - STACK_SH];
    }
};

// Resumable traversal state of one ray.  The work is split into single units so
// a warp can vote each iteration which kind of unit its lanes execute together:
//   node_step()  intersect one internal child of the current node group
//   prim_step()  test one primitive of the current primitive group (a triangle,
//                or at the instance level: enter that instance's BLAS)
//   settle()     pop the stack until there is work again, leaving the BLAS
//                when its part of the stack is used up; true when finished
// SINGLE: every leaf of both levels holds one primitive (SceneDev::single_leaf);
// primitive groups are then (prim_base, hit leaf slots << 24 | leaf slots).  The
// general form (primitive offset bits from the meta bytes) is valid for any tree.
template <bool ANY, bool COUNT, bool SINGLE = false>
struct Traverser {
    static constexpr bool ORD = !ANY;   // visit children front to back (closest hit only)
    static constexpr uint32_t PTHR = SINGLE ? 0x00FFFFFFu : 0u;   // a primitive group is pending above this
    float tmin, tmax;    // (the world-space ray itself is kept in shared memory: save_world)
    NodeRay cr;          // ray of the current level (world or object space)
    WRay tr;             // object-space watertight set-up (in a BLAS, once k != INVALID)
    float best_t, best_u, best_v;
    uint32_t best_inst, best_prim;
    uint2 ngroup, tgroup;
    int level, blas_sp;
    uint32_t cur_inst, steps;
    unsigned err;
    bool done;
    ShortStack st;

    __device__ __forceinline__ void init(const SceneDev& S, V3 o_, V3 d_, float tmin_, float tmax_, uint2* sh,
                                         uint2* spill, uint32_t tid, uint32_t nthreads) {
        tmin = fmaxf(tmin_, 0.0f); tmax = tmax_;
        cr = make_node_ray(o_, d_);
        best_t = tmax; best_u = 0.0f; best_v = 0.0f; best_inst = INVALID; best_prim = INVALID;
        level = 0; blas_sp = 0; cur_inst = 0; steps = 0; err = 0; done = false;
        st.sh = sh; st.spill = spill; st.tid = tid; st.nthreads = nthreads; st.sp = 0;
        st.lim = S.stack_max < STACK_MAX ? S.stack_max : STACK_MAX;
        save_world(d_);
        ngroup = S.tlas_root == INVALID ? make_uint2(0u, 0u) : make_uint2(S.tlas_root, (1u << (24 + (ORD ? cr.oct : 0u))) | 1u);
        tgroup = make_uint2(0u, 0u);
    }

    __device__ __forceinline__ bool has_node() const { return ngroup.y > 0x00FFFFFFu; }
    __device__ __forceinline__ bool has_prim() const { return tgroup.y > PTHR; }

    __device__ __forceinline__ void fail(unsigned e) { err |= e; done = true; }

    // the world ray (origin, direction) and its node-test set-up, kept in shared
    // memory rows STACK_SH .. STACK_SH + 4 of this thread: read when the ray enters an
    // instance and when it leaves one
    __device__ __forceinline__ uint2& row(int k) const { return st.sh[(STACK_SH + k) * st.nthreads + st.tid]; }
    __device__ __forceinline__ void save_world(V3 d) {
        row(0) = make_uint2(__float_as_uint(cr.idx), __float_as_uint(cr.idy));
        row(1) = make_uint2(__float_as_uint(cr.idz), cr.oct);
        row(2) = make_uint2(__float_as_uint(cr.ox), __float_as_uint(cr.oy));
        row(3) = make_uint2(__float_as_uint(cr.oz), __float_as_uint(d.x));
        row(4) = make_uint2(__float_as_uint(d.y), __float_as_uint(d.z));
    }
    __device__ __forceinline__ void restore_world() {
        const uint2 a = row(0), b = row(1), c = row(2), e = row(3);
        cr.ox = __uint_as_float(c.x); cr.oy = __uint_as_float(c.y); cr.oz = __uint_as_float(e.x);
        cr.idx = __uint_as_float(a.x); cr.idy = __uint_as_float(a.y); cr.idz = __uint_as_float(b.x);
        cr.oct = b.y;
    }
    __device__ __forceinline__ void world_ray(V3& o, V3& d) const {
        const uint2 c = row(2), e = row(3), f = row(4);
        o = v3(__uint_as_float(c.x), __uint_as_float(c.y), __uint_as_float(e.x));
        d = v3(__uint_as_float(e.y), __uint_as_float(f.x), __uint_as_float(f.y));
    }

    // Pops until a node or primitive group is pending; sets done when the ray is finished.
    __device__ __forceinline__ void settle() {
        while (!done && !has_node() && !has_prim()) {
            if (level == 1 && st.sp == blas_sp) { level = 0; restore_world(); }
            if (st.sp == 0) { done = true; return; }
            uint2 g = st.pop();
            if (g.x & PRIM_GROUP) tgroup = make_uint2(g.x & ~PRIM_GROUP, g.y);
            else ngroup = g;
        }
    }

    __device__ __forceinline__ void node_step(const SceneDev& S, TraceCounters* ctr) {
        if (++steps > S.max_steps) { fail(ERR_STEP_LIMIT); return; }
        // a pending primitive group is postponed onto the stack
        if (has_prim()) {
            if (!st.push(make_uint2(tgroup.x | PRIM_GROUP, tgroup.y))) { fail(ERR_STACK_OVERFLOW); return; }
            tgroup = make_uint2(0u, 0u);
        }
        uint32_t k = __ffs(ngroup.y >> 24) - 1;
        ngroup.y &= ~(1u << (24 + k));
        uint32_t slot = ORD ? k ^ cr.oct : k;
        uint32_t child = ngroup.x + __popc(ngroup.y & ((1u << slot) - 1u) & 0xFFu);
        if (has_node()) {
            if (!st.push(ngroup)) { fail(ERR_STACK_OVERFLOW); return; }
        }
        if (COUNT) ctr->nodes++;
        if (child >= (level ? S.num_blas_nodes : S.num_tlas_nodes)) { fail(ERR_BAD_INDEX); return; }
        intersect_node<ORD, SINGLE>(level ? S.blas_nodes : S.tlas_nodes, child, cr, tmin, best_t, ngroup, tgroup);
    }

    __device__ __forceinline__ void prim_step(const SceneDev& S, TraceCounters* ctr) {
        if (++steps > S.max_steps) { fail(ERR_STEP_LIMIT); return; }
        uint32_t pidx;
        if constexpr (SINGLE) {   // the primitive's rank among the node's leaf slots
            const uint32_t k = __ffs(tgroup.y >> 24) - 1;
            tgroup.y &= ~(1u << (24 + k));
            pidx = tgroup.x + __popc(tgroup.y & ((1u << k) - 1u));
        } else {
            const uint32_t k = __ffs(tgroup.y) - 1;
            tgroup.y &= tgroup.y - 1u;
            pidx = tgroup.x + k;
        }
        if (level == 0) {
            if (pidx >= S.num_tlas_prims) { fail(ERR_BAD_INDEX); return; }
            uint32_t inst = __ldg(&S.tlas_prims[pidx]);
            if (inst >= S.num_instances) { fail(ERR_BAD_INDEX); return; }
            if (has_prim()) {
                if (!st.push(make_uint2(tgroup.x | PRIM_GROUP, tgroup.y))) { fail(ERR_STACK_OVERFLOW); return; }
            }
            if (has_node()) {
                if (!st.push(ngroup)) { fail(ERR_STACK_OVERFLOW); return; }
            }
            const float4* ip = reinterpret_cast<const float4*>(S.inst_trace + inst);
            float4 r0 = __ldg(ip), r1 = __ldg(ip + 1), r2 = __ldg(ip + 2);
            uint32_t root = __ldg(reinterpret_cast<const uint32_t*>(ip + 3));
            float inv[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
            V3 o, d;
            world_ray(o, d);
            V3 oo = xform_point_rn(inv, o);
            V3 od = xform_dir_rn(inv, d);
            cr = make_node_ray(oo, od);
            // the watertight set-up waits for the instance's first triangle test (many
            // instances are left without one); until then its shear slots hold the direction
            tr.k = INVALID; tr.Sx = od.x; tr.Sy = od.y; tr.Sz = od.z;
            blas_sp = st.sp;
            level = 1;
            cur_inst = inst;
            ngroup = make_uint2(root, (1u << (24 + (ORD ? cr.oct : 0u))) | 1u);
            tgroup = make_uint2(0u, 0u);
        } else {
            if (pidx >= S.num_tris) { fail(ERR_BAD_INDEX); return; }
            if (COUNT) ctr->tris++;
            if (tr.k == INVALID) tr = wray_setup(v3(tr.Sx, tr.Sy, tr.Sz));
            const float4* tp = reinterpret_cast<const float4*>(S.tris + pidx);
            float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
            float va[3] = {a.x, a.y, a.z}, vb[3] = {b.x, b.y, b.z}, vc[3] = {c.x, c.y, c.z};
            float t, b1, b2;
            if (intersect_tri(tr, v3(cr.ox, cr.oy, cr.oz), va, vb, vc, tmin, tmax, &t, &b1, &b2)) {
                uint32_t prim = __float_as_uint(a.w);
                bool better = best_inst == INVALID || t < best_t ||
                              (t == best_t && (cur_inst < best_inst || (cur_inst == best_inst && prim < best_prim)));
                if (ANY || better) {
                    best_t = t; best_inst = cur_inst; best_prim = prim; best_u = b1; best_v = b2;
                }
                if (ANY) done = true;
            }
        }
    }

    // Result once done; traversal errors are reported through the scene's
    // error word and read as a miss.
    __device__ __forceinline__ bool finish(const SceneDev& S, TraceResult& res) {
        res.hit = false;
        res.t = -1.0f; res.u = 0.0f; res.v = 0.0f; res.inst = INVALID; res.prim = INVALID;
        if (err) {
            if (S.error_word) atomicOr(S.error_word, err);
            return false;
        }
        if (best_inst != INVALID) {
            res.hit = true; res.t = best_t; res.inst = best_inst; res.prim = best_prim; res.u = best_u; res.v = best_v;
        }
        return res.hit;
    }
};

// ---- warp packets ------------------------------------------------------------
// Traversal of up to 32 coherent rays (one per lane) by the whole warp together,
// for queues whose neighbouring entries are neighbouring pixels (camera rays).
// Node groups and instance groups are uniform over the warp and carry the mask of
// the lanes whose rays hit one of their boxes: every node is tested by all lanes
// against their own rays (lanes outside the mask count no hits), and the children
// hit by any lane form the next group, visited in the order of the octant of the
// group's first lane.  A mesh node's hit triangles stay per lane and are tested
// before anything else, each lane its own, in as many rounds as the lane with the
// most.  Hits equal the per-ray traversal's: boxes only cull, and the closest hit
// is the minimum over the tested triangles in the same (t, instance, triangle)
// order.  The group stack is one array of PSTACK entries (base, bits, lane mask)
// per warp in shared memory; every lane writes the same values, so each lane
// reads back what it wrote itself.  Each lane's world ray and its node-test
// set-up wait in shared-memory rows while the lane's ray is in an instance.  For
// single-primitive-leaf trees only.  A packet that runs past its stack or past
// 32x the per-ray step cap reports the same error bits as a ray would (all its
// rays then miss).
constexpr int PSTACK = 2 * STACK_MAX;

template <bool ANY, int NT>
struct PacketTraverser {
    static constexpr bool ORD = !ANY;
    static constexpr uint32_t FULL = 0xFFFFFFFFu;
    // per lane
    float tmin, tmax;
    uint2* rows;             // this thread's 5 shared-memory rows (stride NT): the world ray and its set-up
    NodeRay cr;              // node-test set-up of the current level's ray
    WRay tr;                 // object-space watertight set-up (in a mesh, once k != INVALID)
    float best_t, best_u, best_v;
    uint32_t best_inst, best_prim;
    uint32_t tbits;          // hit leaf slots of the current mesh node this lane still has to test
    // uniform over the warp
    uint4* stk;
    uint2 ngroup, tgroup;    // node group; instance group (leaves of the instance BVH)
    uint32_t nmask, tmask, live, lane_bit;
    uint32_t tri_base, tri_leaves;   // prim_base and leaf slots of the mesh node tbits refers to
    uint32_t woct, coct;     // visiting octant of the world level and of the current level
    int level, sp, blas_sp;
    uint32_t cur_inst, steps, step_limit;
    unsigned err;

    __device__ __forceinline__ uint2& row(int k) const { return rows[k * NT]; }
    __device__ __forceinline__ void restore_world() {
        const uint2 a = row(0), b = row(1), c = row(2), e = row(3);
        cr.ox = __uint_as_float(c.x); cr.oy = __uint_as_float(c.y); cr.oz = __uint_as_float(e.x);
        cr.idx = __uint_as_float(a.x); cr.idy = __uint_as_float(a.y); cr.idz = __uint_as_float(b.x);
        cr.oct = b.y;
    }

    __device__ __forceinline__ void init(const SceneDev& S, V3 o, V3 d, float tmin_, float tmax_, bool active,
                                         uint4* stack, uint2* world_rows) {
        tmin = fmaxf(tmin_, 0.0f); tmax = tmax_;
        cr = make_node_ray(o, d);
        rows = world_rows;
        row(0) = make_uint2(__float_as_uint(cr.idx), __float_as_uint(cr.idy));
        row(1) = make_uint2(__float_as_uint(cr.idz), cr.oct);
        row(2) = make_uint2(__float_as_uint(o.x), __float_as_uint(o.y));
        row(3) = make_uint2(__float_as_uint(o.z), __float_as_uint(d.x));
        row(4) = make_uint2(__float_as_uint(d.y), __float_as_uint(d.z));
        tr.k = INVALID; tr.Sx = 0.0f; tr.Sy = 0.0f; tr.Sz = 0.0f;
        best_t = tmax; best_u = 0.0f; best_v = 0.0f; best_inst = INVALID; best_prim = INVALID;
        tbits = 0;
        stk = stack;
        lane_bit = 1u << (threadIdx.x & 31u);
        live = __ballot_sync(FULL, active);
        woct = live ? __shfl_sync(FULL, cr.oct, __ffs(live) - 1) : 0u;
        coct = woct;
        level = 0; sp = 0; blas_sp = 0; cur_inst = 0; steps = 0; err = 0; tri_base = 0; tri_leaves = 0;
        step_limit = S.max_steps < 0x07FFFFFFu ? 32u * S.max_steps : 0xFFFFFFFFu;
        ngroup = (S.tlas_root == INVALID || !live) ? make_uint2(0u, 0u)
                                                   : make_uint2(S.tlas_root, (1u << (24 + (ORD ? woct : 0u))) | 1u);
        nmask = live;
        tgroup = make_uint2(0u, 0u);
        tmask = 0;
    }

    __device__ __forceinline__ bool push(uint32_t x, uint32_t y, uint32_t mask) {
        if (sp >= PSTACK) { err |= ERR_STACK_OVERFLOW; return false; }
        stk[sp++] = make_uint4(x, y, mask, 0u);
        return true;
    }

    // one internal child of the node group, tested by every lane
    __device__ __forceinline__ void node_step(const SceneDev& S) {
        const uint32_t k = __ffs(ngroup.y >> 24) - 1;
        ngroup.y &= ~(1u << (24 + k));
        const uint32_t m = nmask & live;
        if (m == 0) { ngroup.y &= 0x00FFFFFFu; return; }   // the group's rays are all finished
        const uint32_t slot = ORD ? k ^ coct : k;
        const uint32_t child = ngroup.x + __popc(ngroup.y & ((1u << slot) - 1u) & 0xFFu);
        if (tgroup.y > 0x00FFFFFFu) {
            if (!push(tgroup.x | PRIM_GROUP, tgroup.y, tmask)) return;
            tgroup = make_uint2(0u, 0u);
        }
        if (ngroup.y > 0x00FFFFFFu && !push(ngroup.x, ngroup.y, nmask)) return;
        if (child >= (level ? S.num_blas_nodes : S.num_tlas_nodes)) { err |= ERR_BAD_INDEX; return; }
        const float4* np = reinterpret_cast<const float4*>((level ? S.blas_nodes : S.tlas_nodes) + child);
        const float4 w0 = __ldg(np + 0), w1 = __ldg(np + 1), w2 = __ldg(np + 2), w3 = __ldg(np + 3),
                     w4 = __ldg(np + 4);
        uint32_t hits = box_hits(w0, w2, w3, w4, cr, tmin, best_t);
        if (!(m & lane_bit)) hits = 0;
        const uint32_t imask = __float_as_uint(w0.w) >> 24;
        const uint32_t leaves = leaf_slots(__float_as_uint(w1.z), __float_as_uint(w1.w));
        const uint32_t hi = hits & imask, hl = hits & leaves;
        const uint32_t ui = __reduce_or_sync(FULL, hi);
        nmask = __ballot_sync(FULL, hi != 0u);
        ngroup = make_uint2(__float_as_uint(w1.x), ((ORD ? visit_order(ui, coct) : ui) << 24) | imask);
        if (level == 0) {
            const uint32_t ul = __reduce_or_sync(FULL, hl);
            tmask = __ballot_sync(FULL, hl != 0u);
            tgroup = make_uint2(__float_as_uint(w1.y), (ul << 24) | leaves);
        } else {
            tbits = hl;
            tri_base = __float_as_uint(w1.y);
            tri_leaves = leaves;
        }
    }

    // enter the next instance of the instance group (the lanes that hit its leaf box)
    __device__ __forceinline__ void inst_step(const SceneDev& S) {
        const uint32_t k = __ffs(tgroup.y >> 24) - 1;
        tgroup.y &= ~(1u << (24 + k));
        const uint32_t m = tmask & live;
        if (m == 0) { tgroup.y &= 0x00FFFFFFu; return; }
        const uint32_t pidx = tgroup.x + __popc(tgroup.y & ((1u << k) - 1u));
        if (pidx >= S.num_tlas_prims) { err |= ERR_BAD_INDEX; return; }
        const uint32_t inst = __ldg(&S.tlas_prims[pidx]);
        if (inst >= S.num_instances) { err |= ERR_BAD_INDEX; return; }
        if (tgroup.y > 0x00FFFFFFu && !push(tgroup.x | PRIM_GROUP, tgroup.y, tmask)) return;
        if (ngroup.y > 0x00FFFFFFu && !push(ngroup.x, ngroup.y, nmask)) return;
        const float4* ip = reinterpret_cast<const float4*>(S.inst_trace + inst);
        const float4 r0 = __ldg(ip), r1 = __ldg(ip + 1), r2 = __ldg(ip + 2);
        const uint32_t root = __ldg(reinterpret_cast<const uint32_t*>(ip + 3));
        if (m & lane_bit) {
            const float inv[12] = {r0.x, r0.y, r0.z, r0.w, r1.x, r1.y, r1.z, r1.w, r2.x, r2.y, r2.z, r2.w};
            const uint2 c = row(2), e = row(3), f = row(4);
            const V3 wo = v3(__uint_as_float(c.x), __uint_as_float(c.y), __uint_as_float(e.x));
            const V3 wd = v3(__uint_as_float(e.y), __uint_as_float(f.x), __uint_as_float(f.y));
            const V3 oo = xform_point_rn(inv, wo);
            const V3 od = xform_dir_rn(inv, wd);
            cr = make_node_ray(oo, od);
            // (the watertight set-up waits for the instance's first triangle test)
            tr.k = INVALID; tr.Sx = od.x; tr.Sy = od.y; tr.Sz = od.z;
        }
        coct = __shfl_sync(FULL, cr.oct, __ffs(m) - 1);
        blas_sp = sp;
        level = 1;
        cur_inst = inst;
        ngroup = make_uint2(root, (1u << (24 + (ORD ? coct : 0u))) | 1u);
        nmask = m;
        tgroup = make_uint2(0u, 0u);
        tmask = 0;
    }

    // every lane with a hit leaf slot left tests its next triangle
    __device__ __forceinline__ void tri_step(const SceneDev& S) {
        bool found = false;
        unsigned e = 0;
        if (tbits) {
            const uint32_t k = __ffs(tbits) - 1;
            tbits &= tbits - 1u;
            const uint32_t pidx = tri_base + __popc(tri_leaves & ((1u << k) - 1u));
            if (pidx >= S.num_tris) {
                e = ERR_BAD_INDEX;
            } else {
                if (tr.k == INVALID) tr = wray_setup(v3(tr.Sx, tr.Sy, tr.Sz));
                const float4* tp = reinterpret_cast<const float4*>(S.tris + pidx);
                const float4 a = __ldg(tp), b = __ldg(tp + 1), c = __ldg(tp + 2);
                const float va[3] = {a.x, a.y, a.z}, vb[3] = {b.x, b.y, b.z}, vc[3] = {c.x, c.y, c.z};
                float t, b1, b2;
                if (intersect_tri(tr, v3(cr.ox, cr.oy, cr.oz), va, vb, vc, tmin, tmax, &t, &b1, &b2)) {
                    const uint32_t prim = __float_as_uint(a.w);
                    const bool better = best_inst == INVALID || t < best_t ||
                                        (t == best_t && (cur_inst < best_inst || (cur_inst == best_inst && prim < best_prim)));
                    if (ANY || better) {
                        best_t = t; best_inst = cur_inst; best_prim = prim; best_u = b1; best_v = b2;
                    }
                    found = true;
                }
            }
        }
        err |= __reduce_or_sync(FULL, e);
        if (ANY) {
            const uint32_t f = __ballot_sync(FULL, found);
            live &= ~f;
            if (f & lane_bit) tbits = 0;
        }
    }

    __device__ __forceinline__ void run(const SceneDev& S) {
        for (;;) {
            if (err || live == 0) return;
            if (++steps > step_limit) { err |= ERR_STEP_LIMIT; return; }
            if (level == 1 && __any_sync(FULL, tbits != 0u)) { tri_step(S); continue; }
            if (tgroup.y > 0x00FFFFFFu) { inst_step(S); continue; }
            if (ngroup.y > 0x00FFFFFFu) { node_step(S); continue; }
            if (level == 1 && sp == blas_sp) { level = 0; restore_world(); coct = woct; }
            if (sp == 0) return;
            const uint4 g = stk[--sp];
            if (g.x & PRIM_GROUP) { tgroup = make_uint2(g.x & ~PRIM_GROUP, g.y); tmask = g.z; }
            else { ngroup = make_uint2(g.x, g.y); nmask = g.z; }
        }
    }

    // this lane's result; an error of the packet is reported once and read as a miss
    __device__ __forceinline__ bool finish(const SceneDev& S, TraceResult& res) {
        res.hit = false;
        res.t = -1.0f; res.u = 0.0f; res.v = 0.0f; res.inst = INVALID; res.prim = INVALID;
        if (err) {
            if (S.error_word && (threadIdx.x & 31u) == 0) atomicOr(S.error_word, err);
            return false;
        }
        if (best_inst != INVALID) {
            res.hit = true; res.t = best_t; res.inst = best_inst; res.prim = best_prim; res.u = best_u; res.v = best_v;
        }
        return res.hit;
    }
};

// Traces one ray to completion by itself (for kernels that trace inline, e.g.
// the ReSTIR passes): primitives first, then nodes.
template <bool ANY, bool COUNT>
__device__ __forceinline__ bool trace_scene(const SceneDev& S, V3 o, V3 d, float tmin, float tmax, TraceResult& res,
                                            uint2* sh_stack, uint32_t tid, uint32_t nthreads, TraceCounters* ctr) {
    Traverser<ANY, COUNT> tv;
    uint2 spill[STACK_MAX - STACK_SH];
    tv.init(S, o, d, tmin, tmax, sh_stack, spill, tid, nthreads);
    for (;;) {
        tv.settle();
        if (tv.done) break;
        if (tv.has_prim()) tv.prim_step(S, ctr);
        else tv.node_step(S, ctr);
    }
    return tv.finish(S, res);
}

}  // namespace snk
