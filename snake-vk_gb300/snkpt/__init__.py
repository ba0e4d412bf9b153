"""snkpt -- Python host side of the GB300 path-tracing core.

Thin ctypes binding of ``libsnkpt.so`` (the C ABI of ``include/snk_pt.h``)
plus :class:`RT`, which mirrors the reference's render-pass class
(``Core/headers/rendering/Raytracing.h:11-31``: ``RT::Init``,
``RT::RecordRenderCmdBuf``, ``RT::RtSettings``).

There is no fallback: if the CUDA library is missing or no GPU is present the
calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import abi

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libsnkpt.so")

EXPORTS = [
    "snk_pt_abi_version", "snk_pt_create", "snk_pt_destroy", "snk_pt_set_stream", "snk_pt_get_last_error",
    "snk_pt_get_stats", "snk_pt_upload_meshes", "snk_pt_set_instances", "snk_pt_set_materials",
    "snk_pt_set_lights", "snk_pt_build", "snk_pt_render", "snk_pt_synchronize", "snk_pt_trace_rays",
    "snk_pt_read_accumulator", "snk_pt_render_noalloc", "snk_pt_set_tuning", "snk_pt_get_tuning",
    "snk_pt_autotune", "snk_pt_cache_reset", "snk_pt_cache_set_weights", "snk_pt_cache_get_weights",
    "snk_pt_cache_set_bounds", "snk_pt_cache_encode", "snk_pt_cache_infer", "snk_pt_cache_train",
    "snk_taa_create", "snk_taa_destroy", "snk_taa_reset", "snk_taa_resolve", "snk_taa_get_last_error",
    "snk_meshdata_load", "snk_meshdata_get_info", "snk_meshdata_submesh", "snk_meshdata_free",
    "snk_pt_contact_rays", "snk_pt_particle_probe", "snk_pt_particle_constrain",
    "snk_pt_cache_set_guard", "snk_pt_cache_get_guard_state", "snk_cache_guard_relmse",
]


class SnkError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"snk_pt error {code}: {msg}")
        self.code = code


class Mesh(C.Structure):
    _fields_ = [("positions", C.c_void_p), ("normals", C.c_void_p), ("indices", C.c_void_p),
                ("num_vertices", C.c_uint32), ("num_triangles", C.c_uint32)]


class Config(C.Structure):
    _fields_ = [("device", C.c_int32), ("flags", C.c_uint32), ("stream", C.c_void_p), ("reserved", C.c_uint64 * 4)]


class Tuning(C.Structure):
    """snk_tuning: launch knobs of the wavefront (0 = default)."""
    _fields_ = [("trace_blocks_per_sm", C.c_uint32), ("shade_blocks_per_sm", C.c_uint32),
                ("ray_chunk", C.c_uint32), ("refill_idle", C.c_uint32), ("prim_bias", C.c_uint32),
                ("trace_variant", C.c_uint32), ("bvh_treelet_passes", C.c_uint32), ("tlas_treelet_passes", C.c_uint32),
                ("tlas_refit_interval", C.c_uint32), ("bvh_leaf_max", C.c_uint32), ("tlas_leaf_max", C.c_uint32),
                ("bvh_leaf_pack", C.c_uint32), ("max_traversal_steps", C.c_uint32), ("stack_limit", C.c_uint32),
                ("shadow_blocks_per_sm", C.c_uint32), ("shadow_ray_chunk", C.c_uint32),
                ("shadow_refill_idle", C.c_uint32), ("shadow_prim_bias", C.c_uint32), ("shadow_variant", C.c_uint32),
                ("bvh_collapse", C.c_uint32)]
    KNOBS = ("trace_blocks_per_sm", "shade_blocks_per_sm", "ray_chunk", "refill_idle", "prim_bias", "trace_variant",
             "bvh_treelet_passes", "tlas_treelet_passes", "tlas_refit_interval", "bvh_leaf_max", "tlas_leaf_max",
             "bvh_leaf_pack", "max_traversal_steps", "stack_limit", "shadow_blocks_per_sm", "shadow_ray_chunk",
             "shadow_refill_idle", "shadow_prim_bias", "shadow_variant", "bvh_collapse")

    def as_dict(self) -> dict:
        return {k: int(getattr(self, k)) for k in self.KNOBS}

    @classmethod
    def from_dict(cls, d: dict) -> "Tuning":
        t = cls()
        for k in cls.KNOBS:
            setattr(t, k, int(d.get(k, 0)))
        return t


class CacheGuard(C.Structure):
    """snk_cache_guard: the radiance cache's quality guard (check_every 0: off)."""
    _fields_ = [("relmse_budget", C.c_float), ("check_every", C.c_uint32), ("probe_scale", C.c_uint32),
                ("probe_spp", C.c_uint32), ("block", C.c_uint32), ("pad", C.c_uint32 * 3)]


class CacheGuardState(C.Structure):
    _fields_ = [("frames", C.c_uint64), ("probes", C.c_uint64), ("fallback_frames", C.c_uint64),
                ("last_probe_relmse", C.c_double), ("fallback", C.c_uint32), ("pad", C.c_uint32)]


class ViewOutputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("radiance", "albedo", "normal", "position", "rma", "motion", "depth",
                                          "mat_flags", "inst_id", "prim_id")] + \
               [("memory", C.c_uint32), ("pad", C.c_uint32)]


OUTPUT_NAMES = ("radiance", "albedo", "normal", "position", "rma", "motion", "depth", "mat_flags", "inst_id", "prim_id")
OUTPUT_SHAPES = {"radiance": 4, "albedo": 4, "normal": 4, "position": 4, "rma": 4, "motion": 2, "depth": 1,
                 "mat_flags": 1, "inst_id": 1, "prim_id": 1}
OUTPUT_DTYPES = {"radiance": np.float32, "albedo": np.float32, "normal": np.float32, "position": np.float32,
                 "rma": np.float32, "motion": np.float32, "depth": np.float32, "mat_flags": np.uint32,
                 "inst_id": np.uint32, "prim_id": np.uint32}

TREELET_PASSES_NONE = 0xFFFFFFFF
NOALLOC_MAX_PATHS = 65536   # SNK_NOALLOC_MAX_PATHS
CACHE_NUM_WEIGHTS = 16576   # SNK_CACHE_NUM_WEIGHTS

_lib = None


def lib():
    """Load libsnkpt.so (raises when it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with __graft_entry__.build()")
        L = C.CDLL(LIB_PATH)
        vp, u32 = C.c_void_p, C.c_uint32
        for name in EXPORTS:
            getattr(L, name).restype = C.c_int
        L.snk_pt_abi_version.argtypes = [C.POINTER(C.c_uint32)]
        L.snk_pt_create.argtypes = [C.POINTER(Config), C.POINTER(vp)]
        L.snk_pt_destroy.argtypes = [vp]
        L.snk_pt_set_stream.argtypes = [vp, vp]
        L.snk_pt_get_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.snk_pt_get_stats.argtypes = [vp, vp]
        L.snk_pt_upload_meshes.argtypes = [vp, vp, u32]
        L.snk_pt_set_instances.argtypes = [vp, vp, u32]
        L.snk_pt_set_materials.argtypes = [vp, vp, u32]
        L.snk_pt_set_lights.argtypes = [vp, vp, vp, u32]
        L.snk_pt_build.argtypes = [vp]
        L.snk_pt_render.argtypes = [vp, vp, u32, vp, vp]
        L.snk_pt_synchronize.argtypes = [vp]
        L.snk_pt_trace_rays.argtypes = [vp, vp, u32, vp, u32, u32]
        L.snk_pt_read_accumulator.argtypes = [vp, vp, u32, C.POINTER(C.c_uint64)]
        L.snk_pt_render_noalloc.argtypes = [vp, vp, vp, vp]
        L.snk_pt_set_tuning.argtypes = [vp, C.POINTER(Tuning)]
        L.snk_pt_get_tuning.argtypes = [vp, C.POINTER(Tuning)]
        L.snk_pt_autotune.argtypes = [vp, vp, u32, vp, u32, C.POINTER(Tuning)]
        L.snk_pt_cache_reset.argtypes = [vp, u32]
        L.snk_pt_cache_set_weights.argtypes = [vp, vp, u32]
        L.snk_pt_cache_get_weights.argtypes = [vp, vp, u32]
        L.snk_pt_cache_set_bounds.argtypes = [vp, vp, vp]
        L.snk_pt_cache_encode.argtypes = [vp, vp, u32, vp, u32]
        L.snk_pt_cache_infer.argtypes = [vp, vp, u32, vp, u32]
        L.snk_pt_cache_train.argtypes = [vp, vp, u32, C.c_float, vp, C.POINTER(C.c_float), u32]
        L.snk_taa_create.argtypes = [C.c_int32, vp, u32, u32, C.POINTER(vp)]
        L.snk_taa_destroy.argtypes = [vp]
        L.snk_taa_reset.argtypes = [vp]
        L.snk_taa_resolve.argtypes = [vp, vp, vp, vp, u32]
        L.snk_taa_get_last_error.argtypes = [vp, C.c_char_p, C.c_size_t]
        L.snk_meshdata_load.argtypes = [vp, C.c_size_t, C.POINTER(vp), C.c_char_p, C.c_size_t]
        L.snk_meshdata_get_info.argtypes = [vp, vp]
        L.snk_meshdata_submesh.argtypes = [vp, u32, C.POINTER(Mesh)]
        L.snk_meshdata_free.argtypes = [vp]
        L.snk_pt_contact_rays.argtypes = [vp, vp, u32, C.c_float, vp, u32]
        L.snk_pt_particle_probe.argtypes = [vp, vp, u32, C.c_float, vp, vp, u32]
        L.snk_pt_particle_constrain.argtypes = [vp, vp, vp, u32, C.c_float, vp, u32]
        L.snk_pt_cache_set_guard.argtypes = [vp, C.POINTER(CacheGuard)]
        L.snk_pt_cache_get_guard_state.argtypes = [vp, C.POINTER(CacheGuardState)]
        L.snk_cache_guard_relmse.argtypes = [vp, vp, u32, u32, u32, C.POINTER(C.c_double)]
        _lib = L
    return _lib


def _ptr(a) -> int | None:
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


def _is_device(a) -> bool:
    return hasattr(a, "is_cuda") and a.is_cuda


def check_device_outputs(outputs: dict, width: int, height: int, device: int):
    """Raises ValueError unless every given output is a contiguous torch CUDA
    tensor on `device` with the element type of its snk_view_outputs slot and
    room for width * height pixels (the sizes of alloc_outputs)."""
    n = width * height
    for k, b in outputs.items():
        if k not in OUTPUT_SHAPES:
            raise ValueError(f"unknown output {k!r}")
        if b is None:
            continue
        if not _is_device(b):
            raise ValueError(f"output {k!r} must be a torch CUDA tensor (device memory)")
        if b.device.index != device:
            raise ValueError(f"output {k!r} is on cuda:{b.device.index}, the context renders on cuda:{device}")
        if not b.is_contiguous():
            raise ValueError(f"output {k!r} must be contiguous")
        import torch
        want = (torch.float32,) if OUTPUT_DTYPES[k] == np.float32 else (torch.int32, torch.uint32)
        if b.dtype not in want:
            raise ValueError(f"output {k!r} must have dtype {want[0]}, not {b.dtype}")
        if b.numel() < n * OUTPUT_SHAPES[k]:
            raise ValueError(f"output {k!r} holds {b.numel()} elements, the view needs {n * OUTPUT_SHAPES[k]}")


class PathTracer:
    """One library context (``snk_pt_ctx``): scene, acceleration structures, frame state."""

    def __init__(self, device: int = 0, stream=None):
        L = lib()
        cfg = Config()
        cfg.device = device
        cfg.stream = None if stream is None else int(getattr(stream, "cuda_stream", stream))
        h = C.c_void_p()
        rc = L.snk_pt_create(C.byref(cfg), C.byref(h))
        if rc != 0:
            raise SnkError(rc, "snk_pt_create failed (no usable CUDA device?)")
        self._h = h
        self.device = device
        self._keep = []

    def close(self):
        if getattr(self, "_h", None):
            lib().snk_pt_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc: int):
        if rc != 0:
            buf = C.create_string_buffer(1024)
            lib().snk_pt_get_last_error(self._h, buf, 1024)
            raise SnkError(rc, buf.value.decode(errors="replace"))

    # ---- scene ---------------------------------------------------------------
    def set_stream(self, stream):
        self._check(lib().snk_pt_set_stream(self._h, None if stream is None else int(getattr(stream, "cuda_stream", stream))))

    def upload_meshes(self, meshes):
        arr = (Mesh * max(1, len(meshes)))()
        keep = []
        for i, m in enumerate(meshes):
            p = np.ascontiguousarray(m.positions, np.float32)
            n = None if m.normals is None else np.ascontiguousarray(m.normals, np.float32)
            ix = np.ascontiguousarray(m.indices, np.uint32)
            keep += [p, n, ix]
            arr[i] = Mesh(p.ctypes.data, None if n is None else n.ctypes.data, ix.ctypes.data, p.shape[0], ix.shape[0])
        self._check(lib().snk_pt_upload_meshes(self._h, arr, len(meshes)))

    def set_instances(self, instances: np.ndarray):
        a = np.ascontiguousarray(instances, abi.INSTANCE_DTYPE)
        self._check(lib().snk_pt_set_instances(self._h, a.ctypes.data, len(a)))

    def set_materials(self, materials: np.ndarray):
        a = np.ascontiguousarray(materials, abi.MATERIAL_DTYPE)
        self._check(lib().snk_pt_set_materials(self._h, a.ctypes.data, len(a)))

    def set_lights(self, dir_light, point_lights):
        dl = np.ascontiguousarray(np.asarray(dir_light, abi.DIR_LIGHT_DTYPE).reshape(1))
        pl = np.ascontiguousarray(point_lights, abi.POINT_LIGHT_DTYPE)
        self._check(lib().snk_pt_set_lights(self._h, dl.ctypes.data, pl.ctypes.data if len(pl) else None, len(pl)))

    def build(self):
        self._check(lib().snk_pt_build(self._h))

    def load_scene(self, scene):
        self.upload_meshes(scene.meshes)
        self.set_materials(scene.materials)
        self.set_lights(scene.dir_light, scene.point_lights)
        self.set_instances(scene.instances)
        self.build()

    # ---- frames ----------------------------------------------------------------
    def render(self, views, settings, outputs):
        """views: list of abi.VIEW_DTYPE; outputs: list (one per view) of dicts name -> buffer.
        Buffers are either all torch CUDA tensors (device outputs) or all numpy arrays (host)."""
        v = np.ascontiguousarray(np.array([np.asarray(x, abi.VIEW_DTYPE) for x in views], abi.VIEW_DTYPE))
        st = np.ascontiguousarray(np.asarray(settings, abi.SETTINGS_DTYPE).reshape(1))
        outs = (ViewOutputs * len(views))()
        if any(_is_device(b) for o in outputs for b in o.values() if b is not None):
            import torch
            torch.cuda.current_stream().synchronize()   # buffers were filled on torch's stream
        for i, o in enumerate(outputs):
            dev = any(_is_device(b) for b in o.values() if b is not None)
            for k in OUTPUT_NAMES:
                b = o.get(k)
                setattr(outs[i], k, None if b is None else _ptr(b))
            outs[i].memory = abi.MEM_DEVICE if dev else abi.MEM_HOST
        self._check(lib().snk_pt_render(self._h, v.ctypes.data, len(views), st.ctypes.data, outs))

    def render_noalloc(self, view, settings, outputs: dict):
        """Path-traced render of one small view through snk_pt_render_noalloc: no
        device allocation; outputs must be contiguous torch CUDA tensors on this
        context's device with the dtype and size of alloc_outputs (checked here:
        the library writes through the pointers as device memory); at most
        NOALLOC_MAX_PATHS = width * height * spp paths."""
        v = np.ascontiguousarray(np.asarray(view, abi.VIEW_DTYPE).reshape(1))
        st = np.ascontiguousarray(np.asarray(settings, abi.SETTINGS_DTYPE).reshape(1))
        check_device_outputs(outputs, int(v["width"][0]), int(v["height"][0]), self.device)
        o = ViewOutputs()
        for k in OUTPUT_NAMES:
            b = outputs.get(k)
            setattr(o, k, None if b is None else _ptr(b))
        o.memory = abi.MEM_DEVICE
        import torch
        torch.cuda.current_stream().synchronize()
        self._check(lib().snk_pt_render_noalloc(self._h, v.ctypes.data, st.ctypes.data, C.byref(o)))

    def synchronize(self):
        self._check(lib().snk_pt_synchronize(self._h))

    # ---- MLP radiance cache --------------------------------------------------------
    def cache_reset(self, seed: int = 1):
        self._check(lib().snk_pt_cache_reset(self._h, seed))

    def cache_set_weights(self, w):
        w = np.ascontiguousarray(w, np.float32)
        self._check(lib().snk_pt_cache_set_weights(self._h, w.ctypes.data, w.size))

    def cache_get_weights(self):
        w = np.zeros(CACHE_NUM_WEIGHTS, np.float32)
        self._check(lib().snk_pt_cache_get_weights(self._h, w.ctypes.data, w.size))
        return w

    def cache_set_bounds(self, lo, hi):
        lo = np.ascontiguousarray(lo, np.float32)
        hi = np.ascontiguousarray(hi, np.float32)
        self._check(lib().snk_pt_cache_set_bounds(self._h, lo.ctypes.data, hi.ctypes.data))

    def cache_encode(self, records):
        r = np.ascontiguousarray(records, np.float32).reshape(-1, 16)
        out = np.zeros((r.shape[0], 64), np.float32)
        self._check(lib().snk_pt_cache_encode(self._h, r.ctypes.data, r.shape[0], out.ctypes.data, abi.MEM_HOST))
        return out

    def cache_infer(self, records):
        r = np.ascontiguousarray(records, np.float32).reshape(-1, 16)
        out = np.zeros((r.shape[0], 3), np.float32)
        self._check(lib().snk_pt_cache_infer(self._h, r.ctypes.data, r.shape[0], out.ctypes.data, abi.MEM_HOST))
        return out

    def cache_train(self, samples, lr: float = 1e-2, want_grad: bool = False):
        """One training step on host samples (n x 20 floats); returns (loss, grad or None)."""
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 20)
        grad = np.zeros(CACHE_NUM_WEIGHTS, np.float32) if want_grad else None
        loss = C.c_float()
        self._check(lib().snk_pt_cache_train(self._h, s.ctypes.data, s.shape[0], lr,
                                             None if grad is None else grad.ctypes.data, C.byref(loss), abi.MEM_HOST))
        return loss.value, grad

    def set_cache_guard(self, relmse_budget: float = 0.05, check_every: int = 10, probe_scale: int = 4,
                        probe_spp: int = 16, block: int = 4):
        """Quality guard of the cache (snk_pt_cache_set_guard); check_every=0 removes it."""
        g = CacheGuard()
        g.relmse_budget, g.check_every, g.probe_scale = relmse_budget, check_every, probe_scale
        g.probe_spp, g.block = probe_spp, block
        self._check(lib().snk_pt_cache_set_guard(self._h, C.byref(g)))

    def cache_guard_state(self) -> dict:
        s = CacheGuardState()
        self._check(lib().snk_pt_cache_get_guard_state(self._h, C.byref(s)))
        return {"frames": s.frames, "probes": s.probes, "fallback_frames": s.fallback_frames,
                "last_probe_relmse": s.last_probe_relmse, "fallback": bool(s.fallback)}

    # ---- launch knobs ------------------------------------------------------------
    def set_tuning(self, tuning: "Tuning | dict"):
        t = tuning if isinstance(tuning, Tuning) else Tuning.from_dict(tuning)
        self._check(lib().snk_pt_set_tuning(self._h, C.byref(t)))

    def get_tuning(self) -> dict:
        t = Tuning()
        self._check(lib().snk_pt_get_tuning(self._h, C.byref(t)))
        return t.as_dict()

    def autotune(self, views, settings, frames_per_trial: int = 3, cache: str | None = None, key: str = "") -> dict:
        """Coordinate-descent search of the launch knobs on this workload (the
        library's snk_pt_autotune).  With ``cache`` (a JSON file) a result stored
        under (device name, key) is reused instead of searching again."""
        import json
        dev_key = None
        if cache:
            import torch
            dev_key = f"{torch.cuda.get_device_name()}|{key}"
            if os.path.exists(cache):
                try:
                    stored = json.load(open(cache)).get(dev_key)
                except ValueError:
                    stored = None
                if stored:
                    self.set_tuning(stored)
                    return stored
        v = np.ascontiguousarray(np.array([np.asarray(x, abi.VIEW_DTYPE) for x in views], abi.VIEW_DTYPE))
        st = np.ascontiguousarray(np.asarray(settings, abi.SETTINGS_DTYPE).reshape(1))
        best = Tuning()
        self._check(lib().snk_pt_autotune(self._h, v.ctypes.data, len(views), st.ctypes.data, frames_per_trial,
                                          C.byref(best)))
        result = best.as_dict()
        if cache:
            data = {}
            if os.path.exists(cache):
                try:
                    data = json.load(open(cache))
                except ValueError:
                    data = {}
            data[dev_key] = result
            os.makedirs(os.path.dirname(os.path.abspath(cache)), exist_ok=True)
            with open(cache, "w") as f:
                json.dump(data, f, indent=1, sort_keys=True)
        return result

    def trace_rays(self, rays, any_hit: bool = False):
        """rays: numpy abi.RAY_DTYPE array (host) or a torch CUDA tensor of shape (n, 8) float32."""
        flags = abi.TRACE_ANY_HIT if any_hit else 0
        if _is_device(rays):
            import torch
            n = rays.shape[0]
            hits = torch.empty((n, 6), dtype=torch.int32, device=rays.device)
            torch.cuda.synchronize(rays.device)
            self._check(lib().snk_pt_trace_rays(self._h, rays.data_ptr(), n, hits.data_ptr(), flags, abi.MEM_DEVICE))
            return hits
        r = np.ascontiguousarray(rays, abi.RAY_DTYPE)
        hits = np.zeros(len(r), abi.HIT_DTYPE)
        self._check(lib().snk_pt_trace_rays(self._h, r.ctypes.data, len(r), hits.ctypes.data, flags, abi.MEM_HOST))
        return hits

    # ---- particle collision queries (ParticleUpdate.rgen / .rchit) -------------------
    def contact_rays(self, rays, timestep: float):
        """Closest-hit contacts (abi.CONTACT_DTYPE) of host rays (abi.RAY_DTYPE)."""
        r = np.ascontiguousarray(rays, abi.RAY_DTYPE)
        out = np.zeros(len(r), abi.CONTACT_DTYPE)
        self._check(lib().snk_pt_contact_rays(self._h, r.ctypes.data, len(r), timestep, out.ctypes.data,
                                              abi.MEM_HOST))
        return out

    def particle_probe(self, particles, timestep: float):
        """(candidate contact, gravity velocity change) per particle; host or CUDA buffers."""
        if _is_device(particles):
            import torch
            n = particles.shape[0]
            cand = torch.empty((n, 12), dtype=torch.float32, device=particles.device)
            grav = torch.empty(n, dtype=torch.float32, device=particles.device)
            torch.cuda.synchronize(particles.device)
            self._check(lib().snk_pt_particle_probe(self._h, particles.data_ptr(), n, timestep, cand.data_ptr(),
                                                    grav.data_ptr(), abi.MEM_DEVICE))
            return cand, grav
        p = np.ascontiguousarray(particles, abi.PARTICLE_DTYPE)
        cand = np.zeros(len(p), abi.CONTACT_DTYPE)
        grav = np.zeros(len(p), np.float32)
        self._check(lib().snk_pt_particle_probe(self._h, p.ctypes.data, len(p), timestep, cand.ctypes.data,
                                                grav.ctypes.data, abi.MEM_HOST))
        return cand, grav

    def particle_constrain(self, particles, offsets, timestep: float):
        p = np.ascontiguousarray(particles, abi.PARTICLE_DTYPE)
        off = np.ascontiguousarray(offsets, np.float32).reshape(len(p), 3)
        out = np.zeros_like(off)
        self._check(lib().snk_pt_particle_constrain(self._h, p.ctypes.data, off.ctypes.data, len(p), timestep,
                                                    out.ctypes.data, abi.MEM_HOST))
        return out

    def stats(self) -> dict:
        s = np.zeros(1, abi.STATS_DTYPE)
        self._check(lib().snk_pt_get_stats(self._h, s.ctypes.data))
        d = dict(zip(abi.STATS_DTYPE.names, s[0].tolist()))   # (one conversion of the whole record)
        d["stage_ms"] = dict(zip(abi.STAGES, np.asarray(d["stage_ms"]).tolist()))
        d["stage_launches"] = dict(zip(abi.STAGES, np.asarray(d["stage_launches"]).tolist()))
        return d

    def read_accumulator(self, width: int, height: int):
        out = np.zeros((height * width, 4), np.float32)
        nf = C.c_uint64()
        self._check(lib().snk_pt_read_accumulator(self._h, out.ctypes.data, abi.MEM_HOST, C.byref(nf)))
        return out, nf.value


def alloc_outputs(width: int, height: int, device=None, names=OUTPUT_NAMES) -> dict:
    """Output buffers of one view: torch CUDA tensors when ``device`` is given, else numpy."""
    n = width * height
    out = {}
    for k in names:
        c = OUTPUT_SHAPES[k]
        shape = (n, c) if c > 1 else (n,)
        if device is not None:
            import torch
            dt = torch.float32 if OUTPUT_DTYPES[k] == np.float32 else torch.int32
            out[k] = torch.zeros(shape, dtype=dt, device=device)
        else:
            out[k] = np.zeros(shape, OUTPUT_DTYPES[k])
    return out


class TaaResolve:
    """TAA_ResolvePass mirror (snk_taa_*): owns the history and previous-motion
    images of one view and resolves a frame's radiance with its motion vectors.
    Buffers: radiance (W*H, 4) float32, motion (W*H, 2) float32, either numpy
    arrays (host) or torch CUDA tensors (device, on the resolver's stream)."""

    def __init__(self, width: int, height: int, device: int = 0, stream=None):
        self.width, self.height = int(width), int(height)
        h = C.c_void_p()
        s = None if stream is None else int(getattr(stream, "cuda_stream", stream))
        rc = lib().snk_taa_create(device, s, self.width, self.height, C.byref(h))
        if rc != 0:
            raise SnkError(rc, "snk_taa_create failed")
        self._h = h

    def __del__(self):
        h = getattr(self, "_h", None)
        if h:
            lib().snk_taa_destroy(h)
            self._h = None

    def _check(self, rc: int):
        if rc != 0:
            buf = C.create_string_buffer(512)
            lib().snk_taa_get_last_error(self._h, buf, 512)
            raise SnkError(rc, buf.value.decode(errors="replace"))

    def reset(self):
        self._check(lib().snk_taa_reset(self._h))

    def resolve(self, radiance, motion, out=None):
        """Resolves into `out` (default: a new array/tensor; may be `radiance`
        itself for the in-place form of the reference pass)."""
        dev = _is_device(radiance)
        if dev != _is_device(motion):
            raise ValueError("radiance and motion must both be host arrays or both device tensors")
        if dev:
            import torch
            if out is None:
                out = torch.empty_like(radiance)
            torch.cuda.current_stream().synchronize()
            self._check(lib().snk_taa_resolve(self._h, _ptr(radiance), _ptr(motion), _ptr(out), abi.MEM_DEVICE))
        else:
            radiance = np.ascontiguousarray(radiance, np.float32)
            motion = np.ascontiguousarray(motion, np.float32)
            if out is None:
                out = np.empty_like(radiance)
            self._check(lib().snk_taa_resolve(self._h, radiance.ctypes.data, motion.ctypes.data, out.ctypes.data,
                                              abi.MEM_HOST))
        return out


class RT:
    """Mirror of the reference's ``SNAKE::RT`` (Core/headers/rendering/Raytracing.h:11-31).

    ``init(scene)`` corresponds to ``RT::Init`` (descriptor table + pipeline;
    here: upload + BVH builds), ``record_render(views, outputs, settings)`` to
    ``RT::RecordRenderCmdBuf`` (the two-pass ReSTIR dispatch, or the wavefront
    path tracer), and :class:`RT.RtSettings` to ``RT::RtSettings`` (defaults
    temporal 1, spatial 3, ``Raytracing.h:13-16``).
    """

    class RtSettings:
        def __init__(self, num_temporal_resamples: int = 1, num_spatial_resamples: int = 3):
            self.num_temporal_resamples = num_temporal_resamples
            self.num_spatial_resamples = num_spatial_resamples

    def __init__(self, device: int = 0, stream=None):
        self.tracer = PathTracer(device, stream)
        self.frame_index = 0

    def init(self, scene):
        if scene is None or not len(scene.meshes):
            raise SnkError(abi.ERR_STATE, "RT::Init: scene has no meshes")
        self.tracer.load_scene(scene)

    def record_render(self, views, outputs, settings: "RT.RtSettings | None" = None, mode=abi.MODE_RESTIR_PT,
                      **overrides):
        """The pass's output: by default ReSTIR DI plus path-traced indirect light
        (main, RayGen.rgen:530-570); mode=abi.MODE_RESTIR_DI gives the direct light alone."""
        s = settings or RT.RtSettings()
        st = abi.settings(mode=mode, frame_index=self.frame_index, restir_temporal=s.num_temporal_resamples,
                          restir_spatial=s.num_spatial_resamples, **overrides)
        self.tracer.render(views, st, outputs)
        self.frame_index += 1
