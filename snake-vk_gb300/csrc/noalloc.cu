// noalloc.cu -- snk_pt_render_noalloc: the wavefront path tracer for one small
// view, running entirely in a fixed scratch area that the library reserves in
// this file instead of allocating device memory per call.
//
// Who needs it: callers that may not call cudaMalloc/cudaFree (or let a library
// do so) while rendering -- an engine whose frame loop hands every device byte
// out of its own allocator and budget, or code that runs inside a frame where
// the implicit device-wide synchronisation of cudaMalloc/cudaFree would stall
// other work.  Such a caller builds the scene once (building allocates), then
// renders small views (thumbnails, material previews, probes) with this entry
// point, which allocates nothing.
//
// Scratch: g_noalloc_scratch below, NOALLOC_MAX_PATHS (65536) paths of 224 bytes
// plus a 4 KiB header: 14,684,160 bytes.  Every GPU that loads the library holds
// this array until the process exits.  All calls share it and it keeps the last
// call's contents; the frame counters and work counters are cleared at the start
// of every call.  Calls whose GPU work overlaps (other streams, other contexts on
// the same device) race on the array, so callers serialise them.
//
// Set-up: host code cannot use the array's name as a device address; the first
// call on each device looks the address up with cudaGetSymbolAddress (with that
// device current) and caches it.  That first call should come before any stream
// capture begins.  The cached address belongs to the device's current primary
// context: a caller that resets the device (cudaDeviceReset) unloads the module,
// and the address must not be used after that.
//
// Launch settings: the context's traversal knobs and grids (snk_pt_set_tuning,
// snk_pt_autotune) apply here as in snk_pt_render.  The view descriptor is
// written into the scratch header by a one-warp kernel from its by-value
// argument, so no host memory is read by the stream after the call returns.
#include <cstring>
#include <mutex>
#include <string>

#include "../../include/snk_pt.h"
#include "snk_frame.h"

namespace snk {
namespace {

constexpr uint32_t NOALLOC_MAX_PATHS = SNK_NOALLOC_MAX_PATHS;
constexpr size_t NOALLOC_HEADER = 4096;
// per path: rays 2 x 32, path ids 2 x 4, hit 24, beta 16, radiance 16, shadow rays 64, shadow contributions 32
constexpr size_t NOALLOC_PATH_BYTES = 224;
constexpr size_t NOALLOC_BYTES = NOALLOC_HEADER + (size_t)NOALLOC_MAX_PATHS * NOALLOC_PATH_BYTES;

static __device__ __align__(256) unsigned char g_noalloc_scratch[NOALLOC_BYTES];

constexpr int MAX_DEVICES = 64;
std::mutex g_scratch_mu;
unsigned char* g_scratch_addr[MAX_DEVICES] = {};

// Copies the view descriptor (a kernel parameter) into the scratch header.
__global__ void k_put_view(ViewDev* dst, ViewDev v) {
    static_assert(sizeof(ViewDev) % 4 == 0, "view descriptor is whole words");
    const uint32_t* src = reinterpret_cast<const uint32_t*>(&v);
    uint32_t* out = reinterpret_cast<uint32_t*>(dst);
    for (uint32_t i = threadIdx.x; i < sizeof(ViewDev) / 4; i += blockDim.x) out[i] = src[i];
}

// Device address of g_noalloc_scratch on `device` (which must be current).
cudaError_t scratch_address(int device, unsigned char** out) {
    if (device < 0 || device >= MAX_DEVICES) return cudaErrorInvalidDevice;
    std::lock_guard<std::mutex> lock(g_scratch_mu);
    if (!g_scratch_addr[device]) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return e;
        g_scratch_addr[device] = static_cast<unsigned char*>(p);
    }
    *out = g_scratch_addr[device];
    return cudaSuccess;
}

}  // namespace
}  // namespace snk

using namespace snk;

extern "C" int snk_pt_render_noalloc(snk_pt_ctx* ctx, const snk_view* view, const snk_render_settings* settings,
                                     const snk_view_outputs* outputs) {
    if (!ctx) return SNK_ERR_INVALID_ARG;
    if (!view || !settings || !outputs)
        return ctx_fail(ctx, SNK_ERR_INVALID_ARG, "render_noalloc: null view, settings or outputs");
    const snk_render_settings& rs = *settings;
    if (outputs->memory != SNK_MEM_DEVICE)
        return ctx_fail(ctx, SNK_ERR_INVALID_ARG, "render_noalloc: outputs must be device memory");
    if (rs.mode != SNK_MODE_PATH)
        return ctx_fail(ctx, SNK_ERR_UNSUPPORTED, "render_noalloc: only SNK_MODE_PATH is supported");
    if (rs.flags & (SNK_RENDER_ACCUMULATE_F64 | SNK_RENDER_RESET_ACCUM | SNK_RENDER_PROFILE | SNK_RENDER_USE_GRAPH))
        return ctx_fail(ctx, SNK_ERR_UNSUPPORTED, "render_noalloc: accumulate, profile and graph flags need allocations");
    if (rs.spp == 0 || rs.max_depth == 0 || rs.max_depth > MAX_DEPTH)
        return ctx_fail(ctx, SNK_ERR_INVALID_ARG, "render_noalloc: spp must be >= 1 and 1 <= max_depth <= 16");
    if (view->width == 0 || view->height == 0)
        return ctx_fail(ctx, SNK_ERR_INVALID_ARG, "render_noalloc: empty view");
    const uint64_t n_pixels = (uint64_t)view->width * view->height;
    const uint64_t n_paths = n_pixels * rs.spp;
    if (n_paths > NOALLOC_MAX_PATHS)
        return ctx_fail(ctx, SNK_ERR_INVALID_ARG,
                        "render_noalloc: width x height x spp exceeds the 65536-path scratch (SNK_NOALLOC_MAX_PATHS)");
    CtxView cv;
    if (!ctx_view(ctx, &cv)) return SNK_ERR_INVALID_ARG;
    if (!cv.built)
        return ctx_fail(ctx, SNK_ERR_STATE, "render_noalloc: scene changed since the last snk_pt_build (building allocates)");
    if (cudaSetDevice(cv.device) != cudaSuccess) return ctx_fail(ctx, SNK_ERR_CUDA, "render_noalloc: cudaSetDevice");
    unsigned char* base = nullptr;
    cudaError_t e = scratch_address(cv.device, &base);
    if (e != cudaSuccess)
        return ctx_fail(ctx, SNK_ERR_CUDA, (std::string("render_noalloc: cudaGetSymbolAddress: ") + cudaGetErrorString(e)).c_str());

    // header: counters (at 0), traversal counters (32 B at 512), the view descriptor (at 1024)
    const size_t P = NOALLOC_MAX_PATHS;
    static_assert(CNT_TOTAL * sizeof(uint32_t) <= 512, "frame counters fit the header");
    uint32_t* counters = reinterpret_cast<uint32_t*>(base);
    unsigned long long* trav = reinterpret_cast<unsigned long long*>(base + 512);
    ViewDev* dview = reinterpret_cast<ViewDev*>(base + 1024);
    static_assert(1024 + sizeof(ViewDev) <= NOALLOC_HEADER, "view descriptor fits the header");
    unsigned char* q = base + NOALLOC_HEADER;
    auto take = [&](size_t bytes) { unsigned char* r = q; q += bytes; return r; };

    FrameParams F;
    std::memset(&F, 0, sizeof(F));
    F.rays[0] = reinterpret_cast<float4*>(take(32 * P));
    F.rays[1] = reinterpret_cast<float4*>(take(32 * P));
    F.shadow_rays = reinterpret_cast<float4*>(take(64 * P));
    F.shadow_contrib = reinterpret_cast<float4*>(take(32 * P));
    F.beta = reinterpret_cast<float4*>(take(16 * P));
    F.L = reinterpret_cast<float4*>(take(16 * P));
    F.hits = reinterpret_cast<HitDev*>(take(24 * P));
    F.path_ids[0] = reinterpret_cast<uint32_t*>(take(4 * P));
    F.path_ids[1] = reinterpret_cast<uint32_t*>(take(4 * P));

    ViewDev vd;
    std::memset(&vd, 0, sizeof(vd));
    std::memcpy(&vd.v, view, sizeof(ViewParams));
    vd.pixel_offset = 0;
    vd.radiance = reinterpret_cast<float4*>(outputs->radiance);
    vd.albedo = reinterpret_cast<float4*>(outputs->albedo);
    vd.normal = reinterpret_cast<float4*>(outputs->normal);
    vd.position = reinterpret_cast<float4*>(outputs->position);
    vd.rma = reinterpret_cast<float4*>(outputs->rma);
    vd.motion = reinterpret_cast<float2*>(outputs->motion);
    vd.depth = outputs->depth;
    vd.mat_flags = outputs->mat_flags;
    vd.inst_id = outputs->inst_id;
    vd.prim_id = outputs->prim_id;

    cudaStream_t st = cv.stream;
    const bool count_nodes = (rs.flags & SNK_RENDER_COUNT_NODES) != 0;
    k_put_view<<<1, 32, 0, st>>>(dview, vd);
    if (cudaGetLastError() != cudaSuccess ||
        cudaMemsetAsync(counters, 0, CNT_TOTAL * sizeof(uint32_t), st) != cudaSuccess ||
        cudaMemsetAsync(trav, 0, 4 * sizeof(unsigned long long), st) != cudaSuccess)
        return ctx_fail(ctx, SNK_ERR_CUDA, "render_noalloc: scratch set-up");

    F.S = cv.scene;
    F.views = dview;
    F.nviews = 1;
    F.spp = rs.spp;
    F.max_depth = rs.max_depth;
    F.rr_depth = rs.rr_depth;
    F.seed = rs.seed;
    F.n_paths = (uint32_t)n_paths;
    F.n_pixels = (uint32_t)n_pixels;
    F.counters = counters;
    F.trav_counters = count_nodes ? trav : nullptr;
    F.tune = cv.tune;
    F.tune_any = cv.tune_any;

    e = launch_generate(F, cv.shade_grid, st);
    for (uint32_t d = 0; d < rs.max_depth && e == cudaSuccess; d++) {
        e = launch_trace_closest(F, d, cv.trace_grid, count_nodes, st);
        if (e == cudaSuccess) e = launch_shade(F, d, cv.shade_grid, st);
        if (e == cudaSuccess) e = launch_trace_shadow(F, d, cv.any_grid, count_nodes, st);
    }
    if (e == cudaSuccess) e = launch_resolve(F, cv.shade_grid, st);
    if (e != cudaSuccess)
        return ctx_fail(ctx, SNK_ERR_CUDA, (std::string("render_noalloc: launch: ") + cudaGetErrorString(e)).c_str());
    // counters for snk_pt_get_stats (pinned host buffers owned by the context)
    if (cudaMemcpyAsync(cv.h_counters, counters, CNT_TOTAL * sizeof(uint32_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(cv.h_trav, trav, 4 * sizeof(unsigned long long), cudaMemcpyDeviceToHost, st) != cudaSuccess)
        return ctx_fail(ctx, SNK_ERR_CUDA, "render_noalloc: counter copies");
    ctx_note_render(ctx, SNK_MODE_PATH, rs.max_depth, n_paths, n_pixels, count_nodes);
    return SNK_OK;
}
