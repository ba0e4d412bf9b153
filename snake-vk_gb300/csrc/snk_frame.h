// snk_frame.h -- wavefront frame state shared by the kernel translation units.
#pragma once
#include <cuda_runtime.h>

#include "snk_shade.cuh"

namespace snk {

constexpr uint32_t MAX_DEPTH = 16;
constexpr uint32_t MAX_VIEWS = 64;

// counters (uint32) of one frame, zeroed at frame start
constexpr uint64_t PACKET_MIN_PIXELS = 1280ull * 720ull;   // smallest view traced in warp packets
// camera-ray tile of one warp packet (16 x 2 and 4 x 8 tiles were slower at 1080p)
constexpr uint32_t PACKET_TILE_W = 8, PACKET_TILE_H = 4;
constexpr uint32_t CNT_QUEUE = 0;         // [d]: rays queued for segment d
constexpr uint32_t CNT_WORK_TRACE = 16;   // [d]: work fetch of the closest-hit pass of segment d
constexpr uint32_t CNT_WORK_SHADOW = 32;  // [d]: work fetch of the shadow pass of segment d
constexpr uint32_t CNT_SHADOW_RAYS = 48;  // valid shadow rays
constexpr uint32_t CNT_CACHE_QUERIES = 49; // paths terminated into the radiance cache
constexpr uint32_t CNT_SHADOW_REUSED = 50;  // ReSTIR visibility tests answered by an identical earlier test
constexpr uint32_t CNT_SHADOW_Q = 64;     // [2d + k]: shadow rays of light kind k queued by segment d
constexpr uint32_t CNT_TOTAL = 96;
constexpr uint32_t TRAIN_V = 4;           // recorded vertices per cache training path

struct HitDev { float t; uint32_t inst, prim; float u, v; uint32_t flags; };
static_assert(sizeof(HitDev) == 24, "hit layout");

// traversal knobs (zero = default), chosen by snk_pt_set_tuning / the autotuner
struct TraceTuning {
    uint32_t chunk;        // rays a warp takes per global fetch (default 64)
    uint32_t refill_idle;  // refill a warp when at least this many lanes are idle (default 4)
    uint32_t prim_bias;    // primitive step when 4 * n_prim >= prim_bias * n_node (default 4)
    uint32_t variant;      // registers: 0 <= 85 (6 blocks / SM), 1 <= 64 (8 blocks), 2 unconstrained
};

struct FrameParams {
    SceneDev S;
    const ViewDev* views;
    uint32_t nviews;
    uint32_t spp, max_depth, rr_depth, seed;
    uint32_t n_paths;        // sum over views of width * height * spp
    uint32_t n_pixels;       // sum over views of width * height
    uint32_t accumulate;     // add view 0's radiance into accum
    float4* rays[2];         // 2 float4 per ray: (origin, tmin), (direction, tmax)
    uint32_t* path_ids[2];
    HitDev* hits;
    float4* beta;            // per path
    float4* L;               // per path radiance
    float4* shadow_rays;     // compacted shadow-ray queue of a segment, 2 float4 per ray: (origin, bits of its
                             // contribution entry), (direction, tmax); directional-light rays from 0,
                             // local-light rays from n_paths (counts in CNT_SHADOW_Q)
    float4* shadow_contrib;  // 1 per shadow entry (shadow_entry): contribution, w = visibility (0: none)
    uint32_t* counters;
    unsigned long long* trav_counters;   // closest: [0] nodes [1] triangles; shadow: [2] [3]
    double2* accum;          // FP64 accumulator of view 0 (2 double2 per pixel)
    TraceTuning tune;        // closest-hit traversal knobs
    TraceTuning tune_any;    // any-hit (shadow ray) traversal knobs
    // radiance cache mode: paths [0, n_render) render pixels, [n_render, n_paths) train
    uint32_t cache, n_render, n_train, frame;
    float spread_c;
    float2* spread;          // per path: (a0, accumulated spread)
    float4* qrec;            // 4 float4 per cache query (record), path id in qrec[3].w
    float4* qbeta;           // throughput of each query
    float4* train_rec;       // n_train * TRAIN_V records (4 float4)
    float4* train_beta;      // n_train * TRAIN_V (throughput, valid)
    float4* train_L;         // n_train * TRAIN_V radiance gathered at each vertex
    float4* samples;         // n_train * TRAIN_V training samples (5 float4)
    // ReSTIR + path-traced indirect mode: the primary vertex does no NEE and adds no
    // emission (ReSTIR DI shades it); its continuation starts the indirect paths, and
    // the resolve writes each pixel's mean into indirect_out (global pixel order)
    // instead of the views' radiance outputs
    uint32_t indirect;
    float4* indirect_out;
    // one sample per pixel and no cache or indirect mode: a path's radiance is final
    // once the segment it ends in has added its shadow-ray contributions, so
    // k_shade marks the queue entries whose path ends (bit 31 of the path id) and
    // k_accum_shadow writes those pixels' outputs; no resolve pass follows
    uint32_t early_resolve;
    // every view's sides are multiples of the tile's and it has at least
    // PACKET_MIN_PIXELS pixels (neighbouring pixels of smaller images are too far
    // apart in the scene for a packet's rays to share their nodes), both trees have
    // single-primitive leaves, the traversal bounds are the defaults (their limits
    // are per ray) and the frame does not count traversal work: the camera rays are
    // queued in PACKET_TILE_W x PACKET_TILE_H pixel tiles and traced in warp packets
    uint32_t packet_primary;
    // per-frame values in device memory (seed, frame, accumulate), read by the kernels
    // instead of the fields above when set, so that a captured frame replays for new
    // values of them
    const uint32_t* dyn;
};

__device__ __forceinline__ uint32_t frame_seed(const FrameParams& F) { return F.dyn ? __ldg(F.dyn) : F.seed; }
__device__ __forceinline__ uint32_t frame_index(const FrameParams& F) { return F.dyn ? __ldg(F.dyn + 1) : F.frame; }
__device__ __forceinline__ uint32_t frame_accumulate(const FrameParams& F) {
    return F.dyn ? __ldg(F.dyn + 2) : F.accumulate;
}

// The contribution of shadow ray k (0: directional light, 1: local light) of queue
// slot i is entry k * n_paths + i.  The rays themselves are compacted: each kind's
// rays that carry a contribution are appended to that kind's part of the queue,
// so the traversal kernel takes only real rays, the directional-light rays
// together (one direction, neighbouring origins), then the local-light rays.
__host__ __device__ __forceinline__ size_t shadow_entry(const FrameParams& F, uint32_t i, uint32_t k) {
    return (size_t)k * F.n_paths + i;
}

// launch helpers (defined in pt_kernels.cu / trace_kernels.cu / restir.cu)
cudaError_t launch_generate(const FrameParams& F, int grid, cudaStream_t s);
cudaError_t launch_shade(const FrameParams& F, uint32_t depth, int grid, cudaStream_t s);
cudaError_t launch_resolve(const FrameParams& F, int grid, cudaStream_t s);
cudaError_t launch_make_samples(const FrameParams& F, int grid, cudaStream_t s);
cudaError_t launch_trace_closest(const FrameParams& F, uint32_t depth, int grid, bool count, cudaStream_t s);
cudaError_t launch_trace_shadow(const FrameParams& F, uint32_t depth, int grid, bool count, cudaStream_t s);
cudaError_t launch_trace_rays(const SceneDev& S, const float4* rays, uint32_t n, HitDev* hits, bool any,
                              uint32_t* work_counter, int grid, const TraceTuning& tune, cudaStream_t s);
// vis[i] = 1 when segment i (origin, tmin | direction, tmax) is unoccluded, 0 when it
// is not; an empty entry (tmax < 0) is skipped and its vis[i] left as it was
cudaError_t launch_trace_visibility(const SceneDev& S, const float4* rays, uint32_t n, uint8_t* vis,
                                    uint32_t* work_counter, int grid, const TraceTuning& tune, cudaStream_t s);

// ReSTIR DI state of one view
struct RestirView {
    float4* g_pos;      // world position, w: 1 = valid non-emissive hit, 2 = emissive hit, 0 = miss
    float4* g_normal;   // shading normal
    float4* g_albedo;   // albedo, w = roughness
    float4* g_misc;     // metallic, motion.x, motion.y
    float4* prev_normal;
    void* temporal;     // reservoirs (48 bytes per pixel)
    void* history;      // final reservoirs of the previous frame
    void* spatial;      // final reservoirs of this frame
    float4* ris;        // 2 per pixel: the initial pass's RIS state between its two runs
    uint4* memo_keys;   // 4 per pixel: the initial pass's visibility tests and their results
    uint32_t* plan;     // per pixel: how the final shading's two tests are answered (codes, 16 bits each)
    float4* combo;      // unshadowed combine targets, slot-major (slot * pixels + pixel): the temporal
                        // pass's RESTIR_TEMPORAL_COMBOS slots, then the spatial pass's 1 + spatial
    const float4* indirect;   // per pixel of the view: path-traced indirect light added to the
                              // shaded surface pixels (null: direct light only)
    uint32_t history_valid;
};

constexpr uint32_t RESTIR_TEMPORAL_COMBOS = 2;   // current + history reservoir

struct RestirSettings {
    uint32_t frame_index, seed, candidates, mcap;
    int32_t temporal, spatial;
    float radius;
    uint32_t pad;
};

// Visibility rays of a ReSTIR pass: `per_pixel` slots for each of the view's
// `pixels` pixels, slot-major: slot k of pixel p is entry k * pixels + p, whose
// ray is 2 float4 (origin, tmin | direction, tmax) at rays[2 * entry].  Slot k
// of neighbouring pixels is written, traced and read together.  A pass either
// records its rays into `rays` or replays their results from `vis`.
struct RestirQueue {
    float4* rays;
    const uint8_t* vis;
    uint32_t per_pixel;
    uint32_t pixels;
};
// slots per pixel of the passes
constexpr uint32_t RESTIR_INITIAL_SLOTS = 6;   // 2 visibility + 2 x 2 temporal combine
__host__ __device__ constexpr uint32_t restir_spatial_slots(int spatial) {
    return 1u + 2u * (1u + (uint32_t)(spatial > 0 ? spatial : 0));   // sun + 2 x (self + neighbours)
}
constexpr uint32_t RESTIR_SHADE_SLOTS = 2;

// (the G-buffer and surface records come from the wavefront's first shading pass)
// stage 1: initial RIS + temporal reuse: phase 0 records q's rays, phase 1 replays them
// stage 2: spatial reuse + shading: phase 0 records q's rays; phase 1 replays q,
//          writes the spatial reservoirs and records qs's (final shading) rays;
//          phase 2 replays the sun ray of q and qs, writes the frame's outputs
cudaError_t launch_restir_stage(int stage, int phase, const FrameParams& F, uint32_t view_index, const RestirView& R,
                                const RestirSettings& rs, const RestirQueue& q, const RestirQueue& qs, int grid,
                                cudaStream_t s);

// Read-only view of a context (defined in api.cu) for entry points that live in
// other translation units.
struct CtxView {
    int device;
    cudaStream_t stream;
    int num_sms;
    bool built;                 // scene uploaded and built, nothing pending
    SceneDev scene;
    uint32_t* h_counters;       // pinned host copy of the frame counters (CNT_TOTAL)
    unsigned long long* h_trav; // pinned host copy of the traversal counters (4)
    TraceTuning tune, tune_any; // the context's traversal knobs (closest hit, any hit)
    int trace_grid, any_grid, shade_grid;   // the context's launch grids
};

}  // namespace snk

struct snk_pt_ctx;
namespace snk {
bool ctx_view(snk_pt_ctx* ctx, CtxView* out);
int ctx_fail(snk_pt_ctx* ctx, int code, const char* msg);
void ctx_note_render(snk_pt_ctx* ctx, uint32_t mode, uint32_t depth, uint64_t paths, uint64_t pixels, bool counted);
}  // namespace snk
