// trace_kernels.cu -- persistent traversal kernels of the wavefront.
//
// One thread traces one ray; warps fetch 32 rays at a time from a global work
// counter (persistent threads, Aila & Laine, HPG 2009), so the grid is a fixed
// multiple of the SM count and the number of rays is read on the device (which
// keeps the frame capturable in a CUDA graph).  The short traversal stack of
// every thread lives in shared memory (STACK_SH entries) with a local spill.
#include "snk_frame.h"
#include "snk_trace.cuh"

namespace snk {
namespace {

constexpr int TBLK = 128;

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

// closest hit of the rays queued for segment d
template <bool COUNT>
__global__ void __launch_bounds__(TBLK) k_trace_closest(FrameParams F, uint32_t d) {
    __shared__ uint2 sh_stack[STACK_SH * TBLK];
    const uint32_t n = F.counters[CNT_QUEUE + d];
    const float4* rays = F.rays[d & 1u];
    uint32_t* work = &F.counters[CNT_WORK_TRACE + d];
    const uint32_t lane = threadIdx.x & 31u;
    TraceCounters ctr{0ull, 0ull};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        uint32_t i = base + lane;
        if (i < n) {
            float4 a = __ldg(rays + 2ull * i), b = __ldg(rays + 2ull * i + 1);
            TraceResult r;
            trace_scene<false, COUNT>(F.S, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), a.w, b.w, r, sh_stack, threadIdx.x,
                                      TBLK, &ctr);
            HitDev h;
            h.t = r.t; h.inst = r.inst; h.prim = r.prim; h.u = r.u; h.v = r.v; h.flags = r.hit ? 1u : 0u;
            uint2* dst = reinterpret_cast<uint2*>(F.hits + i);
            const uint2* src = reinterpret_cast<const uint2*>(&h);
            dst[0] = src[0]; dst[1] = src[1]; dst[2] = src[2];
        }
    }
    flush_counts<COUNT>(ctr, F.trav_counters);
}

// shadow rays of segment d: up to two per queue slot (directional light, local
// light), traced in that order; an unoccluded one adds its contribution to the
// path radiance (the same order as the CPU oracle, so sums are bit-identical)
template <bool COUNT>
__global__ void __launch_bounds__(TBLK) k_trace_shadow(FrameParams F, uint32_t d) {
    __shared__ uint2 sh_stack[STACK_SH * TBLK];
    const uint32_t n = F.counters[CNT_QUEUE + d];
    const uint32_t* pids = F.path_ids[d & 1u];
    uint32_t* work = &F.counters[CNT_WORK_SHADOW + d];
    const uint32_t lane = threadIdx.x & 31u;
    TraceCounters ctr{0ull, 0ull};
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        uint32_t i = base + lane;
        if (i < n) {
            uint32_t p = pids[i];
            for (int k = 0; k < 2; k++) {
                const float4* sr = F.shadow_rays + 4ull * i + 2 * k;
                float4 b = sr[1];
                if (b.w < 0.0f) continue;
                float4 a = sr[0];
                TraceResult r;
                bool occ = trace_scene<true, COUNT>(F.S, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), a.w, b.w, r, sh_stack,
                                                    threadIdx.x, TBLK, &ctr);
                if (!occ) {
                    float4 c = F.shadow_contrib[2ull * i + k];
                    float4 l = F.L[p];
                    F.L[p] = make_float4(l.x + c.x, l.y + c.y, l.z + c.z, 0.0f);
                }
            }
        }
    }
    flush_counts<COUNT>(ctr, F.trav_counters ? F.trav_counters + 2 : nullptr);
}

// generic trace of an array of rays (the snk_pt_trace_rays test hook)
template <bool ANY>
__global__ void __launch_bounds__(TBLK) k_trace_rays(SceneDev S, const float4* __restrict__ rays, uint32_t n,
                                                     HitDev* hits, uint32_t* work) {
    __shared__ uint2 sh_stack[STACK_SH * TBLK];
    const uint32_t lane = threadIdx.x & 31u;
    for (;;) {
        uint32_t base = 0;
        if (lane == 0) base = atomicAdd(work, 32u);
        base = __shfl_sync(0xFFFFFFFFu, base, 0);
        if (base >= n) break;
        uint32_t i = base + lane;
        if (i < n) {
            float4 a = __ldg(rays + 2ull * i), b = __ldg(rays + 2ull * i + 1);
            TraceResult r;
            bool hit = trace_scene<ANY, false>(S, v3(a.x, a.y, a.z), v3(b.x, b.y, b.z), a.w, b.w, r, sh_stack,
                                               threadIdx.x, TBLK, nullptr);
            HitDev h;
            if (ANY) {
                h.t = hit ? 1.0f : -1.0f; h.inst = INVALID; h.prim = INVALID; h.u = 0.0f; h.v = 0.0f;
                h.flags = hit ? 1u : 0u;
            } else {
                h.t = r.t; h.inst = r.inst; h.prim = r.prim; h.u = r.u; h.v = r.v; h.flags = hit ? 1u : 0u;
            }
            hits[i] = h;
        }
    }
}

}  // namespace

cudaError_t launch_trace_closest(const FrameParams& F, uint32_t depth, int grid, bool count, cudaStream_t s) {
    if (count) k_trace_closest<true><<<grid, TBLK, 0, s>>>(F, depth);
    else k_trace_closest<false><<<grid, TBLK, 0, s>>>(F, depth);
    return cudaGetLastError();
}

cudaError_t launch_trace_shadow(const FrameParams& F, uint32_t depth, int grid, bool count, cudaStream_t s) {
    if (count) k_trace_shadow<true><<<grid, TBLK, 0, s>>>(F, depth);
    else k_trace_shadow<false><<<grid, TBLK, 0, s>>>(F, depth);
    return cudaGetLastError();
}

cudaError_t launch_trace_rays(const SceneDev& S, const float4* rays, uint32_t n, HitDev* hits, bool any,
                              uint32_t* work, int grid, cudaStream_t s) {
    if (any) k_trace_rays<true><<<grid, TBLK, 0, s>>>(S, rays, n, hits, work);
    else k_trace_rays<false><<<grid, TBLK, 0, s>>>(S, rays, n, hits, work);
    return cudaGetLastError();
}

}  // namespace snk
