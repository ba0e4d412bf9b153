// trace_kernels.cu -- persistent traversal kernels of the wavefront.
//
// One lane traces one ray.  Warps are persistent (the grid is a fixed multiple
// of the SM count and the number of rays is read on the device, which keeps the
// frame capturable in a CUDA graph).  Each warp takes chunks of CHUNK rays from
// a global counter and, between traversal steps, hands a new ray to every lane
// whose ray has finished, so lanes do not idle until the warp's longest ray ends
// (Aila & Laine, HPG 2009, persistent threads with ray replacement).  The short
// traversal stack of every lane lives in shared memory (STACK_SH entries) with a
// local spill.
#include "snk_frame.h"
#include "snk_trace.cuh"
#include "snk_shade.cuh"

namespace snk {
namespace {

constexpr int TBLK = 128;

struct Knobs {
    uint32_t chunk;
    int refill_idle;
    uint32_t prim_bias;
    __device__ __forceinline__ explicit Knobs(const TraceTuning& t)
        : chunk(t.chunk ? t.chunk : 64u), refill_idle(t.refill_idle ? (int)t.refill_idle : 4),
          prim_bias(t.prim_bias ? t.prim_bias : 4u) {}
};

// One warp-voted traversal step: every active lane first pops until it has work
// (or finishes); then the warp runs either a node step in the lanes that have an
// internal child pending or a primitive step in the lanes that have a primitive
// pending, whichever more lanes want.  Returns true for a lane whose ray finished.
template <class TV>
__device__ __forceinline__ bool warp_step(TV& tv, bool active, const SceneDev& S, TraceCounters* ctr,
                                          uint32_t prim_bias) {
    if (active) tv.settle();
    const bool live = active && !tv.done;
    const unsigned want_prim = __ballot_sync(0xFFFFFFFFu, live && tv.has_prim());
    const unsigned want_node = __ballot_sync(0xFFFFFFFFu, live && tv.has_node());
    const bool prims = 4u * (uint32_t)__popc(want_prim) >= prim_bias * (uint32_t)__popc(want_node);
    const uint32_t lane = threadIdx.x & 31u;
    if (prims) {
        if ((want_prim >> lane) & 1u) tv.prim_step(S, ctr);
    } else {
        if ((want_node >> lane) & 1u) tv.node_step(S, ctr);
    }
    return active && tv.done;
}

template <bool COUNT>
__device__ __forceinline__ void flush_counts(const TraceCounters& c, unsigned long long* out) {
    if (!COUNT || !out) return;
    unsigned long long a = c.nodes, b = c.tris;
    for (int o = 16; o > 0; o >>= 1) {
        a += __shfl_down_sync(0xFFFFFFFFu, a, o);
        b += __shfl_down_sync(0xFFFFFFFFu, b, o);
    }
    if ((threadIdx.x & 31u) == 0) { atomicAdd(&out[0], a); atomicAdd(&out[1], b); }
}

// Warp-uniform source of ray indices: a local chunk refilled from `work`.
struct RayFeed {
    uint32_t next, end;
    bool exhausted;
    __device__ __forceinline__ void init() { next = 0; end = 0; exhausted = false; }
    // Assigns new indices to the idle lanes (mask `idle`); returns this lane's index
    // or INVALID.  Must be called by the whole warp.
    __device__ __forceinline__ uint32_t refill(unsigned idle, uint32_t lane, uint32_t* work, uint32_t n,
                                               uint32_t chunk) {
        if (next >= end && !exhausted) {
            uint32_t b = 0;
            if (lane == 0) b = atomicAdd(work, chunk);
            b = __shfl_sync(0xFFFFFFFFu, b, 0);
            if (b >= n) {
                exhausted = true;
            } else {
                next = b;
                end = min(b + chunk, n);
            }
        }
        uint32_t mine = INVALID;
        if (next < end) {
            uint32_t i = next + __popc(idle & ((1u << lane) - 1u));
            if (((idle >> lane) & 1u) && i < end) mine = i;
            next = min(next + (uint32_t)__popc(idle), end);
        }
        return mine;
    }
    __device__ __forceinline__ bool done() const { return exhausted && next >= end; }
};

// closest hit of the rays queued for segment d
template <bool COUNT, int MINB, bool SINGLE>
__global__ void __launch_bounds__(TBLK, MINB) k_trace_closest(FrameParams F, uint32_t d) {
    const Knobs kn(F.tune);
    __shared__ uint2 sh_stack[TRACE_SH_ROWS * TBLK];
    const uint32_t n = F.counters[CNT_QUEUE + d];
    const float4* rays = F.rays[d & 1u];
    uint32_t* work = &F.counters[CNT_WORK_TRACE + d];
    const uint32_t lane = threadIdx.x & 31u;
    TraceCounters ctr{0ull, 0ull};
    Traverser<false, COUNT, SINGLE> tv;
    uint2 spill[STACK_MAX - STACK_SH];
    RayFeed feed;
    feed.init();
    bool active = false;
    uint32_t ri = 0;
    for (;;) {
        unsigned act = __ballot_sync(0xFFFFFFFFu, active);
        if (__popc(~act) >= kn.refill_idle && !feed.done()) {
            uint32_t i = feed.refill(~act, lane, work, n, kn.chunk);
            if (i != INVALID) {
                float4 a = __ldg(rays + 2ull * i), b = __ldg(rays + 2ull * i + 1);
                tv.init(F.S, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), a.w, b.w, sh_stack, spill, threadIdx.x, TBLK);
                ri = i;
                active = true;
            }
            act = __ballot_sync(0xFFFFFFFFu, active);
        }
        if (act == 0) {
            if (feed.done()) break;
            continue;
        }
        if (warp_step(tv, active, F.S, &ctr, kn.prim_bias)) {
            TraceResult r;
            tv.finish(F.S, r);
            HitDev h;
            h.t = r.t; h.inst = r.inst; h.prim = r.prim; h.u = r.u; h.v = r.v; h.flags = r.hit ? 1u : 0u;
            uint2* dst = reinterpret_cast<uint2*>(F.hits + ri);
            const uint2* src = reinterpret_cast<const uint2*>(&h);
            dst[0] = src[0]; dst[1] = src[1]; dst[2] = src[2];
            active = false;
        }
    }
    flush_counts<COUNT>(ctr, F.trav_counters);
}

// closest hits of segment d's rays in warp packets of 32 consecutive queue entries
// (the camera segment: the 32 pixels of one 8 x 4 tile per warp)
template <int MINB>
__global__ void __launch_bounds__(TBLK, MINB) k_trace_packet(FrameParams F, uint32_t d) {
    __shared__ uint4 sh_pstack[(TBLK / 32) * PSTACK];
    __shared__ uint2 sh_world[5 * TBLK];
    const uint32_t n = F.counters[CNT_QUEUE + d];
    const float4* rays = F.rays[d & 1u];
    uint32_t* work = &F.counters[CNT_WORK_TRACE + d];
    const uint32_t lane = threadIdx.x & 31u;
    uint4* stack = sh_pstack + (threadIdx.x >> 5) * PSTACK;
    for (;;) {
        uint32_t b = 0;
        if (lane == 0) b = atomicAdd(work, 32u);
        b = __shfl_sync(0xFFFFFFFFu, b, 0);
        if (b >= n) break;
        const uint32_t i = b + lane;
        const bool active = i < n;
        float4 a = make_float4(0.0f, 0.0f, 0.0f, 0.0f), c = a;
        if (active) { a = __ldg(rays + 2ull * i); c = __ldg(rays + 2ull * i + 1); }
        PacketTraverser<false, TBLK> tv;
        tv.init(F.S, v3(a.x, a.y, a.z), v3(c.x, c.y, c.z), a.w, c.w, active, stack, sh_world + threadIdx.x);
        tv.run(F.S);
        TraceResult r;
        tv.finish(F.S, r);
        if (active) {
            HitDev h;
            h.t = r.t; h.inst = r.inst; h.prim = r.prim; h.u = r.u; h.v = r.v; h.flags = r.hit ? 1u : 0u;
            uint2* dst = reinterpret_cast<uint2*>(F.hits + i);
            const uint2* src = reinterpret_cast<const uint2*>(&h);
            dst[0] = src[0]; dst[1] = src[1]; dst[2] = src[2];
        }
    }
}

// shadow rays of segment d: the compacted queue's n0 directional-light rays, then
// its n1 local-light rays (from n_paths on).  A ray's origin w holds its
// contribution entry (shadow_entry); the visibility goes to that contribution's w
// component, and k_accum_shadow adds the visible contributions in entry order
// (the same order as the CPU oracle, so sums are bit-identical).
template <bool COUNT, int MINB, bool SINGLE>
__global__ void __launch_bounds__(TBLK, MINB) k_trace_shadow(FrameParams F, uint32_t d) {
    const Knobs kn(F.tune_any);
    __shared__ uint2 sh_stack[TRACE_SH_ROWS * TBLK];
    const uint32_t n0 = F.counters[CNT_SHADOW_Q + 2 * d], n = n0 + F.counters[CNT_SHADOW_Q + 2 * d + 1];
    uint32_t* work = &F.counters[CNT_WORK_SHADOW + d];
    const uint32_t lane = threadIdx.x & 31u;
    TraceCounters ctr{0ull, 0ull};
    Traverser<true, COUNT, SINGLE> tv;
    uint2 spill[STACK_MAX - STACK_SH];
    RayFeed feed;
    feed.init();
    bool active = false;
    uint32_t ri = 0;
    for (;;) {
        unsigned act = __ballot_sync(0xFFFFFFFFu, active);
        if (__popc(~act) >= kn.refill_idle && !feed.done()) {
            uint32_t j = feed.refill(~act, lane, work, n, kn.chunk);
            if (j != INVALID) {
                const size_t e = j < n0 ? (size_t)j : (size_t)F.n_paths + (j - n0);
                const float4* sr = F.shadow_rays + 2 * e;
                const float4 a = __ldg(sr), b = __ldg(sr + 1);
                tv.init(F.S, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), SHADOW_TMIN, b.w, sh_stack, spill, threadIdx.x, TBLK);
                ri = __float_as_uint(a.w);
                active = true;
            }
            act = __ballot_sync(0xFFFFFFFFu, active);
        }
        if (act == 0) {
            if (feed.done()) break;
            continue;
        }
        if (warp_step(tv, active, F.S, &ctr, kn.prim_bias)) {
            TraceResult r;
            bool occ = tv.finish(F.S, r);
            F.shadow_contrib[ri].w = occ ? 0.0f : 1.0f;
            active = false;
        }
    }
    flush_counts<COUNT>(ctr, F.trav_counters ? F.trav_counters + 2 : nullptr);
}

// adds the visible shadow-ray contributions of segment d to the path radiance
__global__ void __launch_bounds__(256) k_accum_shadow(FrameParams F, uint32_t d) {
    const uint32_t n = F.counters[CNT_QUEUE + d];
    const uint32_t* pids = F.path_ids[d & 1u];
    for (uint32_t i = blockIdx.x * 256 + threadIdx.x; i < n; i += gridDim.x * 256) {
        float4 c0 = F.shadow_contrib[shadow_entry(F, i, 0)], c1 = F.shadow_contrib[shadow_entry(F, i, 1)];
        const bool add = c0.w != 0.0f || c1.w != 0.0f;
        uint32_t p = 0;
        bool fin = false;   // (early resolve) the path ends in this segment
        if (F.early_resolve) {
            const uint32_t raw = pids[i];
            p = raw & 0x7FFFFFFFu;
            fin = (raw >> 31) != 0u;
        } else {
            if (!add) continue;
            p = pids[i];
        }
        if (!add && !fin) continue;
        float4 l = F.L[p];
        if (c0.w != 0.0f) l = make_float4(l.x + c0.x, l.y + c0.y, l.z + c0.z, 0.0f);
        if (c1.w != 0.0f) l = make_float4(l.x + c1.x, l.y + c1.y, l.z + c1.z, 0.0f);
        if (fin) {   // the pixel's outputs, as the resolve pass writes them for one sample
            const uint32_t vi = find_view(F.views, F.nviews, p);   // (one sample: path p is pixel p)
            const ViewDev& V = F.views[vi];
            const uint32_t o = p - V.pixel_offset;
            const float4 r = make_float4(l.x, l.y, l.z, 1.0f);
            if (V.radiance) V.radiance[o] = r;
            if (vi == 0 && frame_accumulate(F)) {
                double2 a0 = F.accum[2ull * o], a1 = F.accum[2ull * o + 1];
                a0.x += (double)r.x; a0.y += (double)r.y; a1.x += (double)r.z; a1.y += 1.0;
                F.accum[2ull * o] = a0;
                F.accum[2ull * o + 1] = a1;
            }
            continue;
        }
        F.L[p] = l;
        if (F.cache && p >= F.n_render) {   // radiance gathered at this vertex of a training path
            const uint32_t slot = (p - F.n_render) * TRAIN_V + (d < TRAIN_V - 1 ? d : TRAIN_V - 1);
            float4 v = F.train_L[slot];
            if (c0.w != 0.0f) v = make_float4(v.x + c0.x, v.y + c0.y, v.z + c0.z, 0.0f);
            if (c1.w != 0.0f) v = make_float4(v.x + c1.x, v.y + c1.y, v.z + c1.z, 0.0f);
            F.train_L[slot] = v;
        }
    }
}

// Ray feed over a queue with empty entries (tmax < 0): the warp takes 32 entries
// at a time from the work counter, keeps the real ones in a per-warp ring in
// shared memory and hands only those to its idle lanes, so an empty entry costs
// one 4-byte load instead of a lane's turn.
struct FilteredFeed {
    RayFeed raw;
    uint32_t head, cnt;   // the ring's pending entries (warp-uniform)
    __device__ __forceinline__ void init() { raw.init(); head = 0; cnt = 0; }
    __device__ __forceinline__ uint32_t refill(unsigned idle, uint32_t lane, uint32_t* work, uint32_t n, uint32_t chunk,
                                               const float4* rays, uint32_t* ring) {
        const uint32_t nidle = (uint32_t)__popc(idle), lt = (1u << lane) - 1u;
        while (cnt < nidle && !raw.done()) {   // (cnt < 32 here, so the ring of 64 never overflows)
            const uint32_t e = raw.refill(0xFFFFFFFFu, lane, work, n, chunk);
            const bool real = e != INVALID && __ldg(reinterpret_cast<const float*>(rays + 2ull * e + 1) + 3) >= 0.0f;
            const unsigned rm = __ballot_sync(0xFFFFFFFFu, real);
            if (real) ring[(head + cnt + (uint32_t)__popc(rm & lt)) & 63u] = e;
            cnt += (uint32_t)__popc(rm);
            __syncwarp();
        }
        uint32_t mine = INVALID;
        const uint32_t r = (uint32_t)__popc(idle & lt);
        if (((idle >> lane) & 1u) && r < cnt) mine = ring[(head + r) & 63u];
        const uint32_t take = nidle < cnt ? nidle : cnt;
        head = (head + take) & 63u;
        cnt -= take;
        __syncwarp();
        return mine;
    }
    __device__ __forceinline__ bool done() const { return raw.done() && cnt == 0; }
};

// visibility of a queue of segments: vis[i] = 1 when nothing is hit in (tmin, tmax),
// 0 when something is; entries with tmax < 0 are empty (skipped, vis[i] not written:
// the passes never read the result of a slot they did not record).
// The ReSTIR passes queue their visibility rays here instead of tracing inline.
template <int MINB, bool SINGLE>
__global__ void __launch_bounds__(TBLK, MINB) k_trace_visibility(SceneDev S, const float4* __restrict__ rays,
                                                                 uint32_t n, uint8_t* vis, uint32_t* work,
                                                                 TraceTuning tune) {
    const Knobs kn(tune);
    __shared__ uint2 sh_stack[TRACE_SH_ROWS * TBLK];
    __shared__ uint32_t ring[TBLK / 32][64];
    const uint32_t lane = threadIdx.x & 31u;
    Traverser<true, false, SINGLE> tv;
    uint2 spill[STACK_MAX - STACK_SH];
    FilteredFeed feed;
    feed.init();
    bool active = false;
    uint32_t ri = 0;
    for (;;) {
        unsigned act = __ballot_sync(0xFFFFFFFFu, active);
        if (__popc(~act) >= kn.refill_idle && !feed.done()) {
            uint32_t i = feed.refill(~act, lane, work, n, kn.chunk, rays, ring[threadIdx.x >> 5]);
            if (i != INVALID) {
                const float4 a = __ldg(rays + 2ull * i), b = __ldg(rays + 2ull * i + 1);
                tv.init(S, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), a.w, b.w, sh_stack, spill, threadIdx.x, TBLK);
                ri = i;
                active = true;
            }
            act = __ballot_sync(0xFFFFFFFFu, active);
        }
        if (act == 0) {
            if (feed.done()) break;
            continue;
        }
        if (warp_step(tv, active, S, nullptr, kn.prim_bias)) {
            TraceResult r;
            vis[ri] = tv.finish(S, r) ? 0u : 1u;
            active = false;
        }
    }
}

// generic trace of an array of rays (the snk_pt_trace_rays test hook)
template <bool ANY, bool SINGLE>
__global__ void __launch_bounds__(TBLK, 6) k_trace_rays(SceneDev S, const float4* __restrict__ rays, uint32_t n,
                                                     HitDev* hits, uint32_t* work, TraceTuning tune) {
    const Knobs kn(tune);
    __shared__ uint2 sh_stack[TRACE_SH_ROWS * TBLK];
    const uint32_t lane = threadIdx.x & 31u;
    Traverser<ANY, false, SINGLE> tv;
    uint2 spill[STACK_MAX - STACK_SH];
    RayFeed feed;
    feed.init();
    bool active = false;
    uint32_t ri = 0;
    for (;;) {
        unsigned act = __ballot_sync(0xFFFFFFFFu, active);
        if (__popc(~act) >= kn.refill_idle && !feed.done()) {
            uint32_t i = feed.refill(~act, lane, work, n, kn.chunk);
            if (i != INVALID) {
                float4 a = __ldg(rays + 2ull * i), b = __ldg(rays + 2ull * i + 1);
                tv.init(S, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), a.w, b.w, sh_stack, spill, threadIdx.x, TBLK);
                ri = i;
                active = true;
            }
            act = __ballot_sync(0xFFFFFFFFu, active);
        }
        if (act == 0) {
            if (feed.done()) break;
            continue;
        }
        if (warp_step(tv, active, S, nullptr, kn.prim_bias)) {
            TraceResult r;
            bool hit = tv.finish(S, r);
            HitDev h;
            if (ANY) {
                h.t = hit ? 1.0f : -1.0f; h.inst = INVALID; h.prim = INVALID; h.u = 0.0f; h.v = 0.0f;
                h.flags = hit ? 1u : 0u;
            } else {
                h.t = r.t; h.inst = r.inst; h.prim = r.prim; h.u = r.u; h.v = r.v; h.flags = hit ? 1u : 0u;
            }
            hits[ri] = h;
            active = false;
        }
    }
}

}  // namespace

// register budget variants: 0 -> at most 85 registers (6 blocks of 128 per SM),
// 1 -> 64 registers (8 blocks), 2 -> unconstrained (4 blocks); each in the
// single-primitive-leaf form when the scene's trees allow it
template <bool COUNT, bool SINGLE>
void launch_closest_variant(const FrameParams& F, uint32_t depth, int grid, cudaStream_t s) {
    if (F.tune.variant == 1) k_trace_closest<COUNT, 8, SINGLE><<<grid, TBLK, 0, s>>>(F, depth);
    else if (F.tune.variant == 2) k_trace_closest<COUNT, 4, SINGLE><<<grid, TBLK, 0, s>>>(F, depth);
    else k_trace_closest<COUNT, 6, SINGLE><<<grid, TBLK, 0, s>>>(F, depth);
}
template <bool COUNT, bool SINGLE>
void launch_shadow_variant(const FrameParams& F, uint32_t depth, int grid, cudaStream_t s) {
    if (F.tune_any.variant == 1) k_trace_shadow<COUNT, 8, SINGLE><<<grid, TBLK, 0, s>>>(F, depth);
    else if (F.tune_any.variant == 2) k_trace_shadow<COUNT, 4, SINGLE><<<grid, TBLK, 0, s>>>(F, depth);
    else k_trace_shadow<COUNT, 6, SINGLE><<<grid, TBLK, 0, s>>>(F, depth);
}

cudaError_t launch_trace_closest(const FrameParams& F, uint32_t depth, int grid, bool count, cudaStream_t s) {
    const bool single = F.S.single_leaf != 0u;
    // camera rays (segment 0) in warp packets when the frame allows them
    // (FrameParams::packet_primary; a counting launch always traces ray by ray)
    if (depth == 0 && F.packet_primary && !count) {
        k_trace_packet<6><<<grid, TBLK, 0, s>>>(F, depth);
        return cudaGetLastError();
    }
    if (count) single ? launch_closest_variant<true, true>(F, depth, grid, s) : launch_closest_variant<true, false>(F, depth, grid, s);
    else single ? launch_closest_variant<false, true>(F, depth, grid, s) : launch_closest_variant<false, false>(F, depth, grid, s);
    return cudaGetLastError();
}

cudaError_t launch_trace_shadow(const FrameParams& F, uint32_t depth, int grid, bool count, cudaStream_t s) {
    const bool single = F.S.single_leaf != 0u;
    if (count) single ? launch_shadow_variant<true, true>(F, depth, grid, s) : launch_shadow_variant<true, false>(F, depth, grid, s);
    else single ? launch_shadow_variant<false, true>(F, depth, grid, s) : launch_shadow_variant<false, false>(F, depth, grid, s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    k_accum_shadow<<<grid / 2 > 0 ? grid / 2 : 1, 256, 0, s>>>(F, depth);
    return cudaGetLastError();
}

cudaError_t launch_trace_visibility(const SceneDev& S, const float4* rays, uint32_t n, uint8_t* vis, uint32_t* work,
                                    int grid, const TraceTuning& tune, cudaStream_t s) {
    if (S.single_leaf) {
        if (tune.variant == 1) k_trace_visibility<8, true><<<grid, TBLK, 0, s>>>(S, rays, n, vis, work, tune);
        else if (tune.variant == 2) k_trace_visibility<4, true><<<grid, TBLK, 0, s>>>(S, rays, n, vis, work, tune);
        else k_trace_visibility<6, true><<<grid, TBLK, 0, s>>>(S, rays, n, vis, work, tune);
    } else {
        if (tune.variant == 1) k_trace_visibility<8, false><<<grid, TBLK, 0, s>>>(S, rays, n, vis, work, tune);
        else if (tune.variant == 2) k_trace_visibility<4, false><<<grid, TBLK, 0, s>>>(S, rays, n, vis, work, tune);
        else k_trace_visibility<6, false><<<grid, TBLK, 0, s>>>(S, rays, n, vis, work, tune);
    }
    return cudaGetLastError();
}

cudaError_t launch_trace_rays(const SceneDev& S, const float4* rays, uint32_t n, HitDev* hits, bool any,
                              uint32_t* work, int grid, const TraceTuning& tune, cudaStream_t s) {
    if (S.single_leaf) {
        if (any) k_trace_rays<true, true><<<grid, TBLK, 0, s>>>(S, rays, n, hits, work, tune);
        else k_trace_rays<false, true><<<grid, TBLK, 0, s>>>(S, rays, n, hits, work, tune);
    } else {
        if (any) k_trace_rays<true, false><<<grid, TBLK, 0, s>>>(S, rays, n, hits, work, tune);
        else k_trace_rays<false, false><<<grid, TBLK, 0, s>>>(S, rays, n, hits, work, tune);
    }
    return cudaGetLastError();
}

}  // namespace snk
