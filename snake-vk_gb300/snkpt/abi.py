"""numpy dtypes mirroring the structs of ``include/snk_pt.h`` byte for byte.

The same buffers are handed to the CUDA library (``libsnkpt.so``) and, in the
tests, to the CPU oracle, so both sides read identical bits.
"""
import numpy as np

INSTANCE_DTYPE = np.dtype([
    ("transform", "<f4", (12,)),
    ("prev_transform", "<f4", (12,)),
    ("mesh_id", "<u4"),
    ("material_id", "<u4"),
    ("flags", "<u4"),
    ("pad", "<u4"),
])
assert INSTANCE_DTYPE.itemsize == 112

MATERIAL_DTYPE = np.dtype([
    ("albedo", "<f4", (3,)),
    ("roughness", "<f4"),
    ("metallic", "<f4"),
    ("ao", "<f4"),
    ("flags", "<u4"),
    ("pad", "<u4"),
])
assert MATERIAL_DTYPE.itemsize == 32

DIR_LIGHT_DTYPE = np.dtype([
    ("dir", "<f4", (3,)),
    ("enabled", "<u4"),
    ("colour", "<f4", (3,)),
    ("pad", "<f4"),
])
assert DIR_LIGHT_DTYPE.itemsize == 32

POINT_LIGHT_DTYPE = np.dtype([
    ("pos", "<f4", (3,)),
    ("radius", "<f4"),
    ("colour", "<f4", (3,)),
    ("atten_constant", "<f4"),
    ("atten_linear", "<f4"),
    ("atten_exp", "<f4"),
    ("pad", "<u4", (2,)),
])
assert POINT_LIGHT_DTYPE.itemsize == 48

VIEW_DTYPE = np.dtype([
    ("pos", "<f4", (3,)), ("tan_half_fov_y", "<f4"),
    ("forward", "<f4", (3,)), ("aspect", "<f4"),
    ("right", "<f4", (3,)), ("width", "<u4"),
    ("up", "<f4", (3,)), ("height", "<u4"),
    ("prev_pos", "<f4", (3,)), ("prev_tan_half_fov_y", "<f4"),
    ("prev_forward", "<f4", (3,)), ("prev_aspect", "<f4"),
    ("prev_right", "<f4", (3,)), ("prev_valid", "<u4"),
    ("prev_up", "<f4", (3,)), ("pad", "<u4"),
])
assert VIEW_DTYPE.itemsize == 128

SETTINGS_DTYPE = np.dtype([
    ("mode", "<u4"), ("spp", "<u4"), ("max_depth", "<u4"), ("rr_depth", "<u4"),
    ("seed", "<u4"), ("frame_index", "<u4"), ("flags", "<u4"), ("restir_candidates", "<u4"),
    ("restir_mcap", "<u4"), ("restir_temporal", "<i4"), ("restir_spatial", "<i4"),
    ("restir_radius", "<f4"), ("cache_train_paths", "<u4"), ("cache_train_steps", "<u4"),
    ("cache_spread", "<f4"), ("cache_lr", "<f4"),
])
assert SETTINGS_DTYPE.itemsize == 64

RAY_DTYPE = np.dtype([("o", "<f4", (3,)), ("tmin", "<f4"), ("d", "<f4", (3,)), ("tmax", "<f4")])
assert RAY_DTYPE.itemsize == 32

HIT_DTYPE = np.dtype([("t", "<f4"), ("inst", "<u4"), ("prim", "<u4"), ("u", "<f4"), ("v", "<f4"),
                      ("flags", "<u4")])
assert HIT_DTYPE.itemsize == 24

# snk_particle (Particle.glsl:3-7) and snk_contact (ParticleUpdate.rgen:5-10)
PARTICLE_DTYPE = np.dtype([("position_radius", "<f4", (4,)), ("velocity", "<f4", (4,)), ("colour", "<f4", (4,))])
assert PARTICLE_DTYPE.itemsize == 48
CONTACT_DTYPE = np.dtype([("normal", "<f4", (3,)), ("distance", "<f4"), ("position", "<f4", (3,)), ("pad0", "<f4"),
                          ("velocity", "<f4", (3,)), ("pad1", "<f4")])
assert CONTACT_DTYPE.itemsize == 48

STATS_DTYPE = np.dtype([
    ("rays_camera", "<u8"), ("rays_extension", "<u8"), ("rays_shadow", "<u8"),
    ("node_visits", "<u8"), ("triangle_tests", "<u8"), ("shadow_node_visits", "<u8"),
    ("shadow_triangle_tests", "<u8"), ("wide_nodes", "<u8"),
    ("triangles", "<u8"), ("instances", "<u8"), ("blas_sah_cost", "<f8"),
    ("last_render_ms", "<f8"), ("device_error", "<u4"), ("instance_bvh_refits", "<u4"),
    ("stage_ms", "<f8", (12,)), ("stage_launches", "<u8", (12,)), ("cache_queries", "<u8"),
    ("cache_samples", "<u8"), ("shadow_tests_reused", "<u8"), ("graph_launches", "<u8"), ("graph_captures", "<u8"),
])
assert STATS_DTYPE.itemsize == 336
STAGES = ("generate", "trace_closest", "shade", "trace_shadow", "resolve", "restir_gbuffer", "restir_initial",
          "restir_spatial", "cache_infer", "cache_samples", "cache_train", "trace_any")

OK, ERR_INVALID_ARG, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_STATE, ERR_LIMIT, ERR_UNSUPPORTED = 0, 1, 2, 3, 4, 5, 6
MODE_PATH, MODE_RESTIR_DI, MODE_PATH_CACHE, MODE_RESTIR_PT = 0, 1, 2, 3
RENDER_ACCUMULATE_F64, RENDER_RESET_ACCUM, RENDER_COUNT_NODES, RENDER_USE_GRAPH, RENDER_PROFILE = 1, 2, 4, 8, 16
TRACE_ANY_HIT = 1
MEM_DEVICE, MEM_HOST = 0, 1
MAT_EMISSIVE = 1
INVALID_INDEX = 0xFFFFFFFF


def settings(mode=MODE_PATH, spp=1, max_depth=4, rr_depth=3, seed=1, frame_index=0, flags=0,
             restir_candidates=32, restir_mcap=20, restir_temporal=1, restir_spatial=5,
             restir_radius=30.0, cache_train_paths=0, cache_train_steps=0, cache_spread=0.0,
             cache_lr=0.0) -> np.ndarray:
    s = np.zeros((), SETTINGS_DTYPE)
    s["mode"], s["spp"], s["max_depth"], s["rr_depth"] = mode, spp, max_depth, rr_depth
    s["seed"], s["frame_index"], s["flags"] = seed, frame_index, flags
    s["restir_candidates"], s["restir_mcap"] = restir_candidates, restir_mcap
    s["restir_temporal"], s["restir_spatial"], s["restir_radius"] = restir_temporal, restir_spatial, restir_radius
    s["cache_train_paths"], s["cache_train_steps"] = cache_train_paths, cache_train_steps
    s["cache_spread"], s["cache_lr"] = cache_spread, cache_lr
    return s
