/*
 * snk_pt.h -- C ABI of the GB300 path-tracing core.
 *
 * This library replaces the ray-traced render pass of Snake-VK:
 *   class RT                         Core/headers/rendering/Raytracing.h:11-31
 *   RT::Init                         Core/src/rendering/Raytracing.cpp:269-278
 *   RT::RecordRenderCmdBuf           Core/src/rendering/Raytracing.cpp:227-267
 *   descriptor table (bindings 0-21) Core/src/rendering/Raytracing.cpp:72-93
 * together with the scene -> GPU buffer systems that feed that pass
 * (Core/src/scene/RaytracingBufferSystem.cpp, LightBufferSystem.cpp,
 * TransformBufferSystem.h, SceneInfoBufferSystem.cpp,
 * Core/src/assets/ResourceBufferManagers.cpp, Core/src/rendering/MeshBufferManager.cpp)
 * and the driver's acceleration structures (Core/src/resources/TLAS.cpp).
 *
 * Conventions
 *  - Every entry point returns an int status: SNK_OK (0) or an SNK_ERR_* code.
 *    snk_pt_get_last_error() returns the message of the last failure on a context.
 *    (The reference asserts and exits instead, Core/headers/util/util.h:14-31.)
 *  - Scene data (meshes, instances, materials, lights) is passed in HOST memory
 *    and copied; the context owns every device copy, the BVHs and the queues.
 *  - Ray/hit buffers and frame outputs are caller-owned; their memory space is
 *    given per call (SNK_MEM_DEVICE or SNK_MEM_HOST).  Host outputs are written
 *    with device->host copies on the context's stream and the call synchronises.
 *  - One context is used by one host thread at a time.  All GPU work is issued on
 *    the context's stream (snk_pt_set_stream; default: a stream the context creates).
 *  - No globals: two contexts never share state.
 */
#ifndef SNK_PT_H
#define SNK_PT_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SNK_PT_ABI_VERSION 2u

/* status codes */
#define SNK_OK                 0
#define SNK_ERR_INVALID_ARG    1
#define SNK_ERR_CUDA           2
#define SNK_ERR_OUT_OF_MEMORY  3
#define SNK_ERR_STATE          4  /* e.g. render before build */
#define SNK_ERR_LIMIT          5  /* a device-side bound was hit (stack depth, iteration cap) */
#define SNK_ERR_UNSUPPORTED    6

/* memory spaces of caller buffers */
#define SNK_MEM_DEVICE 0u
#define SNK_MEM_HOST   1u

/* material flags (TexMatBuffers.glsl:3, MAT_FLAG_EMISSIVE) */
#define SNK_MAT_EMISSIVE 1u

/* invalid index in hits / id outputs (TexMatBuffers.glsl:1, INVALID_GLOBAL_INDEX) */
#define SNK_INVALID_INDEX 0xFFFFFFFFu

/* render modes */
#define SNK_MODE_PATH        0u  /* plain unbiased wavefront path tracing with NEE */
#define SNK_MODE_RESTIR_DI   1u  /* the reference's two-pass ReSTIR DI (RayGen.rgen:411-570) */
#define SNK_MODE_PATH_CACHE  2u  /* path tracing with the online-trained MLP radiance cache */
#define SNK_MODE_RESTIR_PT   3u  /* the reference's whole pass-2 output (RayGen.rgen:530-570): ReSTIR DI at
                                    the primary vertex plus path-traced indirect light from it -- spp
                                    unbiased paths of max_depth segments per pixel (NEE from the second
                                    vertex on, roulette from rr_depth) in place of the biased BounceDiffuse
                                    (:139-213); the paths' streams are keyed by seed + 0x9E3779B9 x
                                    frame_index */

/* render flags */
#define SNK_RENDER_ACCUMULATE_F64  1u  /* add this frame's radiance into the FP64 accumulator */
#define SNK_RENDER_RESET_ACCUM     2u  /* zero the FP64 accumulator first */
#define SNK_RENDER_COUNT_NODES     4u  /* count traversal node visits / triangle tests (slower) */
#define SNK_RENDER_USE_GRAPH       8u  /* replay the frame's kernels from a captured CUDA graph */
#define SNK_RENDER_PROFILE        16u  /* time every kernel launch with CUDA events (stage_ms) */

/* stages reported in snk_pt_stats.stage_ms / stage_launches */
#define SNK_STAGE_GENERATE        0
#define SNK_STAGE_TRACE_CLOSEST   1
#define SNK_STAGE_SHADE           2
#define SNK_STAGE_TRACE_SHADOW    3
#define SNK_STAGE_RESOLVE         4
#define SNK_STAGE_RESTIR_GBUFFER  5  /* (no longer used: the ReSTIR G-buffer is the wavefront's first segment) */
#define SNK_STAGE_RESTIR_INITIAL  6
#define SNK_STAGE_RESTIR_SPATIAL  7
#define SNK_STAGE_CACHE_INFER     8
#define SNK_STAGE_CACHE_SAMPLES   9
#define SNK_STAGE_CACHE_TRAIN    10
#define SNK_STAGE_TRACE_ANY      11  /* stage_ms only: time during which a path-tracing traversal kernel
                                        runs (the union of the closest-hit and shadow launches' spans,
                                        which overlap on two streams) */
#define SNK_NUM_STAGES           12

/* trace flags */
#define SNK_TRACE_ANY_HIT 1u

typedef struct snk_pt_ctx snk_pt_ctx;

typedef struct snk_pt_config {
    int32_t  device;        /* CUDA device ordinal */
    uint32_t flags;         /* reserved, 0 */
    void*    stream;        /* cudaStream_t to issue work on, or NULL to create one */
    uint64_t reserved[4];
} snk_pt_config;

/* One mesh (a submesh in the reference: MeshBufferManager.cpp:49-70).
 * positions/normals: num_vertices x 3 floats; indices: num_triangles x 3 u32.
 * normals may be NULL (flat geometric normals are used). */
typedef struct snk_mesh {
    const float*    positions;
    const float*    normals;
    const uint32_t* indices;
    uint32_t        num_vertices;
    uint32_t        num_triangles;
} snk_mesh;

/* One instance of one mesh (InstanceData, RaytracingInstances.glsl:7-13, plus the
 * current/previous transforms of Transforms.glsl:9-10 and the TLAS instance of
 * TLAS.cpp:188-200).  transform: row-major 3x4 object->world. 112 bytes. */
typedef struct snk_instance {
    float    transform[12];
    float    prev_transform[12];
    uint32_t mesh_id;
    uint32_t material_id;
    uint32_t flags;         /* reserved, 0 */
    uint32_t pad;
} snk_instance;

/* Material (TexMatBuffers.glsl:5-20 without texture indices).  For emissive
 * materials albedo is the emitted radiance (RayClosestHit.rchit:119-122). 32 bytes. */
typedef struct snk_material {
    float    albedo[3];
    float    roughness;
    float    metallic;
    float    ao;
    uint32_t flags;         /* SNK_MAT_EMISSIVE */
    uint32_t pad;
} snk_material;

/* Directional light (LightBuffers.glsl:1-5): dir points towards the light. 32 bytes. */
typedef struct snk_directional_light {
    float    dir[3];
    uint32_t enabled;
    float    colour[3];
    float    pad;
} snk_directional_light;

/* Point light (LightBuffers.glsl:7-15).  colour is the radiant intensity.  With
 * radius > 0 the path tracer treats it as a sphere light of that radius with
 * radiance colour / (pi radius^2); ReSTIR DI evaluates it as the reference's
 * attenuated point light.  48 bytes. */
typedef struct snk_point_light {
    float    pos[3];
    float    radius;
    float    colour[3];
    float    atten_constant;
    float    atten_linear;
    float    atten_exp;
    uint32_t pad[2];
} snk_point_light;

/* Pinhole camera for one view plus its previous-frame pose (for motion vectors).
 * Replaces CommonUBO / CommonUBO_PrevFrame (CommonUBO.glsl:1-27).  forward, right,
 * up: orthonormal world-space basis; rows of the image go from +up (row 0) to -up.
 * 128 bytes. */
typedef struct snk_view {
    float    pos[3];
    float    tan_half_fov_y;
    float    forward[3];
    float    aspect;
    float    right[3];
    uint32_t width;
    float    up[3];
    uint32_t height;
    float    prev_pos[3];
    float    prev_tan_half_fov_y;
    float    prev_forward[3];
    float    prev_aspect;
    float    prev_right[3];
    uint32_t prev_valid;    /* 0: history invalid (CommonUBO.prev_frame_invalid) */
    float    prev_up[3];
    uint32_t pad;
} snk_view;

/* Per-frame settings.  restir_* mirror RtSettings (Raytracing.h:13-16) and the
 * compile-time LIGHT_RIS_ITERS / M_CAP of RayGen.rgen:95-97.  64 bytes. */
typedef struct snk_render_settings {
    uint32_t mode;               /* SNK_MODE_* */
    uint32_t spp;                /* samples per pixel (path modes) */
    uint32_t max_depth;          /* path segments per sample */
    uint32_t rr_depth;           /* russian roulette from this segment on */
    uint32_t seed;
    uint32_t frame_index;        /* keys the per-frame random streams */
    uint32_t flags;              /* SNK_RENDER_* */
    uint32_t restir_candidates;  /* initial RIS candidates per light kind (32) */
    uint32_t restir_mcap;        /* temporal M cap (20) */
    int32_t  restir_temporal;    /* num_temporal_resamples (0 disables temporal reuse) */
    int32_t  restir_spatial;     /* num_spatial_resamples */
    float    restir_radius;      /* spatial radius in pixels (30) */
    uint32_t cache_train_paths;  /* SNK_MODE_PATH_CACHE: training paths per frame (0: 16384) */
    uint32_t cache_train_steps;  /* Adam steps per frame over the 4 x paths samples (0: 4) */
    float    cache_spread;       /* path-spread threshold c for cache termination (0: 0.01) */
    float    cache_lr;           /* Adam learning rate (0: 1e-2; < 0: no update) */
} snk_render_settings;

/* Outputs of one view (RaytracingResources, RenderCommon.h:6-35, plus img_output).
 * Every pointer may be NULL (not written).  Layouts are row-major width x height:
 *   radiance  float4 (rgb, 1)        albedo    float4 (rgb, 1)
 *   normal    float4 (xyz, 0)        position  float4 (world xyz, 1)
 *   rma       float4 (roughness, metallic, ao, 1)
 *   motion    float2 (prev uv - current uv, CalcVelocity GBuffer.frag:41-43)
 *   depth     float  (hit distance along the primary ray, -1 on a miss)
 *   mat_flags u32, inst_id u32, prim_id u32 (SNK_INVALID_INDEX on a miss) */
typedef struct snk_view_outputs {
    float*    radiance;
    float*    albedo;
    float*    normal;
    float*    position;
    float*    rma;
    float*    motion;
    float*    depth;
    uint32_t* mat_flags;
    uint32_t* inst_id;
    uint32_t* prim_id;
    uint32_t  memory;            /* SNK_MEM_DEVICE or SNK_MEM_HOST */
    uint32_t  pad;
} snk_view_outputs;

/* A ray: origin, tmin, direction, tmax (32 bytes).  Hits have tmin < t < tmax; a
 * negative (or NaN) tmin is taken as 0, as traceRayEXT requires tmin >= 0. */
typedef struct snk_ray {
    float ox, oy, oz, tmin;
    float dx, dy, dz, tmax;
} snk_ray;

/* A hit (24 bytes): t (-1 on a miss), instance, triangle index within the mesh,
 * barycentrics of vertices 1 and 2 (hitAttributeEXT, RayClosestHit.rchit:88),
 * flags bit 0 = hit.  Any-hit queries fill t = 1 / -1 and flags only. */
typedef struct snk_hit {
    float    t;
    uint32_t inst;
    uint32_t prim;
    float    u;
    float    v;
    uint32_t flags;
} snk_hit;

typedef struct snk_pt_stats {
    uint64_t rays_camera;        /* primary rays of the last render */
    uint64_t rays_extension;     /* closest-hit continuation rays */
    uint64_t rays_shadow;        /* any-hit rays */
    uint64_t node_visits;        /* closest-hit rays, only with SNK_RENDER_COUNT_NODES */
    uint64_t triangle_tests;     /* closest-hit rays, only with SNK_RENDER_COUNT_NODES */
    uint64_t shadow_node_visits; /* shadow rays, only with SNK_RENDER_COUNT_NODES */
    uint64_t shadow_triangle_tests;
    uint64_t wide_nodes;         /* 8-wide BVH nodes (all BLAS + TLAS) */
    uint64_t triangles;          /* unique triangles stored */
    uint64_t instances;
    double   blas_sah_cost;      /* SAH cost of the BLASes (surface-area weighted) */
    double   last_render_ms;     /* device time of the last render (CUDA events) */
    uint32_t device_error;       /* last device error word (0 = none) */
    uint32_t instance_bvh_refits; /* instance BVH updates done by refit since create */
    double   stage_ms[12];       /* device time per stage of the last render (SNK_RENDER_PROFILE) */
    uint64_t stage_launches[12]; /* kernel launches per stage of the last render */
    uint64_t cache_queries;      /* paths terminated into the radiance cache */
    uint64_t cache_samples;      /* training samples of the last frame */
    uint64_t shadow_tests_reused; /* ReSTIR modes: visibility tests answered by an identical
                                     earlier test of the same pixel and frame (not traced; they are
                                     not counted in rays_shadow) */
    uint64_t graph_launches;     /* SNK_RENDER_USE_GRAPH frames launched as a CUDA graph since create */
    uint64_t graph_captures;     /* of those, frames captured anew (the others replayed the last
                                    capture: same views, sizes, settings and scene buffers) */
} snk_pt_stats;

/* Launch knobs of the wavefront (0 = default).  The reference has no equivalent:
 * its dispatch shape is fixed by traceRaysKHR(W, H, 1) (Raytracing.cpp:253,260). */
typedef struct snk_tuning {
    uint32_t trace_blocks_per_sm;   /* persistent traversal grid = SMs x this (16) */
    uint32_t shade_blocks_per_sm;   /* generate / shade / resolve grid = SMs x this (8) */
    uint32_t ray_chunk;             /* rays a warp takes per global work fetch (64) */
    uint32_t refill_idle;           /* hand new rays to a warp when this many lanes idle (4) */
    uint32_t prim_bias;             /* warp runs a primitive step if 4*n_prim >= bias*n_node (4) */
    uint32_t trace_variant;         /* registers: 0 <= 85 (6 blocks/SM), 1 <= 64, 2 unconstrained */
    uint32_t bvh_treelet_passes;    /* treelet restructuring passes of later mesh BVH builds (3);
                                       SNK_TREELET_PASSES_NONE builds the plain LBVH */
    uint32_t tlas_treelet_passes;   /* the same for the per-frame instance BVH (0: with
                                       single-instance leaves the clustered tree gains ~1 % of
                                       trace time from a pass that costs more per rebuild); up to
                                       1024 instances it is built in one launch by locally-ordered
                                       clustering, and the passes refine that tree */
    uint32_t tlas_refit_interval;   /* 0: rebuild the instance BVH on every instance update (as
                                       TlasSystem::BuildTlas, TlasSystem.cpp:16-20); k >= 1:
                                       refit it (same topology, new boxes) when only transforms
                                       or materials changed, with a full rebuild every k-th
                                       update (any number of instances) */
    uint32_t bvh_leaf_max;          /* primitives per leaf of later mesh BVH builds, 1..4 (1) */
    uint32_t tlas_leaf_max;         /* instances per leaf of the instance BVH, 1..4 (1) */
    uint32_t bvh_leaf_pack;         /* largest mesh-BVH subtree a full node keeps as one leaf
                                       (bvh_leaf_max..4; default bvh_leaf_max) */
    uint32_t max_traversal_steps;   /* traversal units (node groups and primitives) one ray may take;
                                       a ray that needs more stops and the next synchronising call
                                       returns SNK_ERR_LIMIT (0: 65536) */
    uint32_t stack_limit;           /* traversal stack entries per ray, 1..64; a deeper stack stops
                                       the ray with SNK_ERR_LIMIT (0: 64) */
    uint32_t shadow_blocks_per_sm;  /* any-hit traversal (shadow and ReSTIR visibility rays): grid =
                                       SMs x this (0: trace_blocks_per_sm) */
    uint32_t shadow_ray_chunk;      /* any-hit traversal: rays per work fetch (0: ray_chunk) */
    uint32_t shadow_refill_idle;    /* any-hit traversal: refill threshold (0: refill_idle) */
    uint32_t shadow_prim_bias;      /* any-hit traversal: primitive-step bias (0: prim_bias) */
    uint32_t shadow_variant;        /* any-hit traversal registers: 0 as trace_variant, k + 1 variant k */
    uint32_t bvh_collapse;          /* how BVH builds (later mesh BVHs, every instance BVH) pick each
                                       8-wide node's children from the binary tree: 0 the least-SAH
                                       choice (dynamic programming over the tree), 1 greedily opening
                                       the largest child */
} snk_tuning;

#define SNK_TREELET_PASSES_NONE 0xFFFFFFFFu

/* ---- lifetime ---------------------------------------------------------------- */
int snk_pt_abi_version(uint32_t* version);
/* RT::Init (Raytracing.cpp:269-278) */
int snk_pt_create(const snk_pt_config* config, snk_pt_ctx** out_ctx);
int snk_pt_destroy(snk_pt_ctx* ctx);
int snk_pt_set_stream(snk_pt_ctx* ctx, void* stream);
int snk_pt_get_last_error(const snk_pt_ctx* ctx, char* buf, size_t len);
int snk_pt_get_stats(const snk_pt_ctx* ctx, snk_pt_stats* out);

/* ---- scene ------------------------------------------------------------------- */
/* MeshBufferManager::LoadMeshFromData + BLAS::GenerateFromMeshData
 * (MeshBufferManager.cpp:22-88, TLAS.cpp:109-186): replaces all meshes. */
int snk_pt_upload_meshes(snk_pt_ctx* ctx, const snk_mesh* meshes, uint32_t num_meshes);
/* RaytracingInstanceBufferSystem::UpdateInstanceBuffer / UpdateEmissiveIdxBuffer,
 * TransformBufferSystem::UpdateTransformBuffer (RaytracingBufferSystem.cpp:69-130,
 * TransformBufferSystem.h:92-122). */
int snk_pt_set_instances(snk_pt_ctx* ctx, const snk_instance* instances, uint32_t num_instances);
/* GlobalMaterialBufferManager::UpdateMaterialUBO (ResourceBufferManagers.cpp:64-101) */
int snk_pt_set_materials(snk_pt_ctx* ctx, const snk_material* materials, uint32_t num_materials);
/* LightBufferSystem::UpdateLightSSBO (LightBufferSystem.cpp:65-108) */
int snk_pt_set_lights(snk_pt_ctx* ctx, const snk_directional_light* dir_light,
                      const snk_point_light* point_lights, uint32_t num_point_lights);
/* BLAS builds for new meshes (GPU LBVH -> 8-wide) and the per-frame instance
 * BVH rebuild of TlasSystem::BuildTlas (TlasSystem.cpp:27-49).  The instance,
 * emissive-light and light-selection tables are derived on the device from the
 * records given to snk_pt_set_instances; tables whose inputs did not change
 * since the last build are kept. */
int snk_pt_build(snk_pt_ctx* ctx);

/* ---- render ------------------------------------------------------------------ */
/* RT::RecordRenderCmdBuf (Raytracing.cpp:227-267): renders num_views views in
 * one batched launch sequence and writes each view's outputs.  Returns after the
 * work is enqueued (device outputs) or after host outputs are written. */
int snk_pt_render(snk_pt_ctx* ctx, const snk_view* views, uint32_t num_views,
                  const snk_render_settings* settings, const snk_view_outputs* outputs);

/* Launch knobs of this context (snk_tuning; zero fields mean the defaults). */
int snk_pt_set_tuning(snk_pt_ctx* ctx, const snk_tuning* tuning);
int snk_pt_get_tuning(const snk_pt_ctx* ctx, snk_tuning* tuning);
/* Autotuner: times frames_per_trial renders of the given views/settings for each
 * candidate knob value (coordinate descent, two passes), keeps the fastest
 * setting in the context and returns it.  Outputs are not written. */
int snk_pt_autotune(snk_pt_ctx* ctx, const snk_view* views, uint32_t num_views, const snk_render_settings* settings,
                    uint32_t frames_per_trial, snk_tuning* best);

/* Waits for the context's stream and reports device-side errors (a traversal
 * bound that was hit) of the work issued so far.  The reference has no
 * equivalent; its submissions are fenced by the frame loop (VkRenderer.h:49-50). */
int snk_pt_synchronize(snk_pt_ctx* ctx);

/* Test hook for per-ray parity: closest hit (flags 0) or any hit (SNK_TRACE_ANY_HIT)
 * of n rays against the built scene (traceRayEXT, RayGen.rgen:101-121,164-176). */
int snk_pt_trace_rays(snk_pt_ctx* ctx, const snk_ray* rays, uint32_t n, snk_hit* hits,
                      uint32_t flags, uint32_t memory);

/* No counterpart in the reference.  Plain path tracing (SNK_MODE_PATH) of one
 * view with no device allocation, for callers that must not allocate while they
 * render: an engine whose frame loop owns every device byte through its own
 * allocator, or code where the device-wide synchronisation that cudaMalloc and
 * cudaFree can cause would stall other work.  The scene must already be built
 * (building allocates).  All wavefront scratch lives in one fixed array of
 * 14,684,160 bytes that every GPU loading the library keeps until exit, so
 * width * height * spp may not exceed SNK_NOALLOC_MAX_PATHS (larger views are
 * rejected with SNK_ERR_INVALID_ARG).  Outputs must be device memory; the
 * accumulate, profile and graph flags are rejected.  The first call on a device
 * looks up the array's device address, so make it before any stream capture;
 * the address is kept for the life of the process and does not survive a
 * device reset (cudaDeviceReset).  The context's launch knobs (snk_pt_set_tuning)
 * apply.  Calls share the array: calls whose GPU work overlaps race. */
#define SNK_NOALLOC_MAX_PATHS 65536u
int snk_pt_render_noalloc(snk_pt_ctx* ctx, const snk_view* view, const snk_render_settings* settings,
                          const snk_view_outputs* outputs);

/* ---- MLP radiance cache (no counterpart in the reference) ------------------------
 * 64 encoded inputs -> 4 x 64 ReLU -> RGB, no biases; SNK_CACHE_NUM_WEIGHTS FP32
 * master weights, row-major W_l[in][out], layers concatenated (4 x 64x64, 64x3).
 * A query/sample record is 16 floats: position xyz, roughness, outgoing direction
 * xyz, metallic, shading normal xyz, 0, albedo xyz, 0.  A training sample appends
 * 4 floats: target radiance rgb and a weight (0 or 1). */
#define SNK_CACHE_NUM_WEIGHTS 16576u
/* He-uniform initialisation from a PCG32 stream, Adam state cleared. */
int snk_pt_cache_reset(snk_pt_ctx* ctx, uint32_t seed);
int snk_pt_cache_set_weights(snk_pt_ctx* ctx, const float* weights, uint32_t n);
int snk_pt_cache_get_weights(snk_pt_ctx* ctx, float* weights, uint32_t n);
/* positions are normalised to this box (default: the built scene's bounds) */
int snk_pt_cache_set_bounds(snk_pt_ctx* ctx, const float lo[3], const float hi[3]);
/* the 64 input features of n records, as the network consumes them (BF16 values) */
int snk_pt_cache_encode(snk_pt_ctx* ctx, const float* records, uint32_t n, float* features, uint32_t memory);
/* network outputs (n x 3) for n records */
int snk_pt_cache_infer(snk_pt_ctx* ctx, const float* records, uint32_t n, float* out, uint32_t memory);
/* one training step on n samples (20 floats each): relative-L2 loss, gradient
 * summed over the batch, Adam (lr; lr = 0 computes the gradient only).
 * grad (SNK_CACHE_NUM_WEIGHTS floats, host) and loss may be NULL. */
int snk_pt_cache_train(snk_pt_ctx* ctx, const float* samples, uint32_t n, float lr, float* grad, float* loss,
                       uint32_t memory);

/* Quality guard of the radiance cache: frames over a relMSE budget fall back to
 * plain path tracing.  With a guard set, every check_every-th SNK_MODE_PATH_CACHE
 * frame (from the second on) is preceded by a probe: view 0 at 1/probe_scale
 * resolution, probe_spp samples per pixel, rendered with the cache (no training
 * step) and plainly; their relMSE over block x block pixel means
 * (snk_cache_guard_relmse) above relmse_budget makes the following cache frames
 * render plainly -- no path ends in the cache, so the image is the plain tracer's
 * bit for bit, while the frame's training paths keep training the network -- until
 * a later probe passes.  The probe synchronises.  32 bytes. */
typedef struct snk_cache_guard {
    float    relmse_budget;   /* (0.05) */
    uint32_t check_every;     /* cache frames per probe; 0 turns the guard off */
    uint32_t probe_scale;     /* probe resolution divisor (4) */
    uint32_t probe_spp;       /* (16) */
    uint32_t block;           /* pixel block side of the relMSE (4) */
    uint32_t pad[3];
} snk_cache_guard;
typedef struct snk_cache_guard_state {
    uint64_t frames;          /* cache frames rendered since the guard was set */
    uint64_t probes;
    uint64_t fallback_frames; /* of the frames, those rendered plainly */
    double   last_probe_relmse;  /* -1 before the first probe */
    uint32_t fallback;        /* 1 while the last probe was over budget */
    uint32_t pad;
} snk_cache_guard_state;
/* sets (or, with NULL / check_every 0, removes) the guard; resets its state */
int snk_pt_cache_set_guard(snk_pt_ctx* ctx, const snk_cache_guard* guard);
int snk_pt_cache_get_guard_state(const snk_pt_ctx* ctx, snk_cache_guard_state* state);
/* the guard's error measure of two RGBA32F host images of width x height:
 * mean over the block x block pixel means and 3 channels of (c - p)^2 / (p^2 + 0.01)
 * (block clamped to [1, min(width, height)]; pixels past the last whole block are left out) */
int snk_cache_guard_relmse(const float* cached, const float* plain, uint32_t width, uint32_t height, uint32_t block,
                           double* relmse);

/* FP64 converged-image accumulator of view 0: copies the running mean (samples
 * accumulated so far) as float4 into out (memory space as given). */
int snk_pt_read_accumulator(snk_pt_ctx* ctx, float* out, uint32_t memory, uint64_t* num_frames);

/* ---- particle collision queries -----------------------------------------------------
 * The scene queries of the particle update pass (ParticleUpdate.rgen, run by
 * ParticleSystem, Core/src/scene/ParticleSystem.cpp:60-62): rays whose closest
 * hit returns the contact of ParticleUpdate.rchit:41-67 -- interpolated vertex
 * normal through the instance's normal matrix, contact point origin + t*dir, and
 * contact velocity (contact point - previous-frame transform of the hit point) /
 * timestep.  The shader's rays use TerminateOnFirstHit, whose chosen hit depends
 * on the driver's traversal order; these queries return the closest hit. */
typedef struct snk_particle {         /* Particle, Core/res/shaders/Particle.glsl:3-7 */
    float position_radius[4];
    float velocity[4];                /* w: 1 awake, 0 asleep */
    float colour[4];
} snk_particle;
typedef struct snk_contact {          /* RayPayload, ParticleUpdate.rgen:5-10 */
    float normal[3];
    float distance;                   /* hit t; -1 when nothing was hit */
    float position[3];
    float pad0;
    float velocity[3];
    float pad1;
} snk_contact;
/* traceRayEXT + ParticleUpdate.rchit for each ray (closest hit in (tmin, tmax)) */
int snk_pt_contact_rays(snk_pt_ctx* ctx, const snk_ray* rays, uint32_t n, float timestep, snk_contact* out,
                        uint32_t memory);
/* Per particle, the scene part of ParticleUpdate.rgen main (:151-166): for an awake
 * particle with non-zero speed the three TraceCollisionRay probes (:101-124; velocity
 * direction, then the unnormalised right and up vectors, from the particle's back,
 * lengths speed*DT + 2r and 2r) keeping the hit with the largest relative speed,
 * and CalculateGravity (:150-165, DT = 1/120): gravity_dv[i] = -9.8*DT when the
 * downward ray of length r + 0.001 hits nothing, else 0. */
int snk_pt_particle_probe(snk_pt_ctx* ctx, const snk_particle* particles, uint32_t n, float timestep,
                          snk_contact* candidate, float* gravity_dv, uint32_t memory);
/* ConstrainOffsetWithScene (:126-148) of offsets (n x 3 floats) -> out (n x 3). */
int snk_pt_particle_constrain(snk_pt_ctx* ctx, const snk_particle* particles, const float* offsets, uint32_t n,
                              float timestep, float* out, uint32_t memory);

/* ---- .meshdata assets ------------------------------------------------------------
 * Reader of the reference's binary mesh asset: AssetLoader::DeserializeMeshData
 * (Core/src/assets/AssetLoader.cpp:166-211) of files written by
 * SerializeMeshDataBinary (:146-164) through ByteSerializer
 * (Core/headers/util/ByteSerializer.h:18-112).  Layout, little-endian, 64-bit
 * byte counts: u64 uuid; name (u64 count + bytes); submeshes (u64 count + 20-byte
 * records below); u32 num_vertices; u32 num_indices; positions, normals, tangents
 * (u64 count + 12-byte vec3 each); tex_coords (u64 count + 8-byte vec2 each);
 * indices (u64 count + u32 each); material UUIDs and texture UUIDs (u64 count +
 * u64 each).  Every count is checked against the remaining bytes, and the vertex
 * arrays against num_vertices / num_indices (the reference asserts only the
 * former): a malformed file is SNK_ERR_INVALID_ARG with a message, never a read
 * out of bounds.  Trailing bytes are ignored, as in the reference. */
typedef struct snk_meshdata snk_meshdata;
typedef struct snk_submesh {          /* Submesh, Core/headers/assets/MeshData.h:11-17 */
    uint32_t num_indices, num_vertices, base_vertex, base_index, material_index;
} snk_submesh;
typedef struct snk_meshdata_info {    /* views into the loaded asset (valid until free) */
    uint64_t           uuid;
    const char*        name;
    uint64_t           name_len;
    uint32_t           num_submeshes, num_vertices, num_indices, num_materials, num_textures, pad;
    const snk_submesh* submeshes;
    const float*       positions;     /* num_vertices x 3 */
    const float*       normals;       /* num_vertices x 3 */
    const float*       tangents;      /* num_vertices x 3 */
    const float*       tex_coords;    /* num_vertices x 2 */
    const uint32_t*    indices;       /* num_indices */
    const uint64_t*    materials;     /* material asset UUIDs (submesh material_index selects one) */
    const uint64_t*    textures;      /* texture asset UUIDs */
} snk_meshdata_info;
/* copies what it needs out of bytes; err (may be NULL) receives the reason of a failure */
int snk_meshdata_load(const void* bytes, size_t size, snk_meshdata** out, char* err, size_t err_len);
int snk_meshdata_get_info(const snk_meshdata* md, snk_meshdata_info* info);
/* One submesh as an snk_mesh for snk_pt_upload_meshes (one BLAS per submesh, as
 * BLAS::GenerateFromMeshData, Core/src/resources/TLAS.cpp:109-186): positions and
 * normals from base_vertex, indices from base_index (local to the submesh). */
int snk_meshdata_submesh(const snk_meshdata* md, uint32_t index, snk_mesh* out);
int snk_meshdata_free(snk_meshdata* md);

/* ---- TAA resolve ---------------------------------------------------------------
 * TAA_ResolvePass (Core/src/renderpasses/TAA_ResolvePass.cpp:6-56) running
 * TAA_Resolve.comp (Core/res/shaders/TAA_Resolve.comp:12-86): 3x3 neighbourhood
 * mean/variance box (gamma 0.55), history fetched bilinearly at the motion-
 * reprojected coordinate (repeat addressing, as the pass's sampler) and clipped
 * to the box, 0.9 history blend, velocity-based disocclusion towards the mean.
 * The object owns the history and previous-motion images (the pass's
 * m_history_image / m_prev_frame_velocity_image) and updates them after each
 * resolve, as the pass's two blits do.  radiance: RGBA32F, motion: RG32F (the
 * render pass's outputs), out: RGBA32F, width x height, row-major; out may equal
 * radiance (resolved in place, as the pass does).  The first resolve after create
 * or reset takes the current frame as its history. */
typedef struct snk_taa snk_taa;
int snk_taa_create(int32_t device, void* stream, uint32_t width, uint32_t height, snk_taa** out);
int snk_taa_destroy(snk_taa* taa);
int snk_taa_reset(snk_taa* taa);
int snk_taa_resolve(snk_taa* taa, const float* radiance, const float* motion, float* out, uint32_t memory);
int snk_taa_get_last_error(const snk_taa* taa, char* buf, size_t len);

#ifdef __cplusplus
}
#endif

#endif /* SNK_PT_H */
