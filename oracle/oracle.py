"""ctypes wrapper of the CPU oracle (test infrastructure only).

The oracle is the checker of the CUDA path tracer: ``tests/``,
``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg use it; the
library under ``snake-vk_gb300/`` never does.  Parity is UNPINNED by the
reference (Snake-VK has no tests, golden images or CPU path); see the header
of ``snk_oracle.cpp`` for what the oracle restates and how it is pinned.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "libsnk_oracle.so")
SRC = os.path.join(HERE, "snk_oracle.cpp")

_ROOT = os.path.dirname(HERE)
_PKG = os.path.join(_ROOT, "snake-vk_gb300")
if _PKG not in sys.path:
    sys.path.insert(0, _PKG)
from snkpt import abi  # noqa: E402

GCC_FLAGS = ["-std=c++17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-shared", "-pthread"]


def build(force: bool = False) -> str:
    """Compile the oracle with g++ (no FMA contraction)."""
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(SRC):
        tmp = LIB + ".tmp"
        subprocess.check_call(["g++", *GCC_FLAGS, "-o", tmp, SRC])
        os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(LIB)
        vp, u32, u64p = C.c_void_p, C.c_uint32, C.POINTER(C.c_uint64)
        L.snko_scene_create.restype = vp
        L.snko_scene_destroy.argtypes = [vp]
        L.snko_add_mesh.argtypes = [vp, vp, vp, vp, u32, u32]
        L.snko_set_instances.argtypes = [vp, vp, u32]
        L.snko_set_materials.argtypes = [vp, vp, u32]
        L.snko_set_lights.argtypes = [vp, vp, vp, u32]
        L.snko_build.argtypes = [vp]
        L.snko_trace.argtypes = [vp, vp, u32, u32, vp, u32, u64p]
        L.snko_render_path.argtypes = [vp, vp, vp, vp, u32, u32, vp, u32, u64p]
        L.snko_render_path_cache.argtypes = [vp, vp, vp, u32, vp, vp, vp, u32]
        L.snko_restir_state_create.restype = vp
        L.snko_restir_state_create.argtypes = [u32, u32]
        L.snko_restir_state_destroy.argtypes = [vp]
        L.snko_render_restir.argtypes = [vp, vp, vp, vp, u32, vp, vp, u32, u64p]
        L.snko_pcg32.argtypes = [C.c_uint64, C.c_uint64, u32, vp]
        L.snko_pcg_stream.argtypes = [u32, u32, u32, u32, u32, vp]
        L.snko_sincos2pi.argtypes = [vp, u32, vp, vp]
        L.snko_brdf.argtypes = [vp, u32, vp]
        L.snko_directional.argtypes = [vp, u32, vp]
        L.snko_pointlight.argtypes = [vp, u32, vp]
        L.snko_tri.argtypes = [vp, u32, vp]
        L.snko_invert_affine.argtypes = [vp, vp, vp, vp]
        L.snko_num_local_lights.argtypes = [vp]
        L.snko_num_local_lights.restype = u32
        L.snko_light_table.argtypes = [vp, vp, vp, vp]
        L.snko_hardware_threads.restype = u32
        L.snko_mlp_forward.argtypes = [vp, vp, u32, vp]
        L.snko_mlp_grad.argtypes = [vp, vp, vp, vp, u32, vp, C.c_int]
        L.snko_mlp_grad.restype = C.c_double
        L.snko_taa_resolve.argtypes = [u32, u32, vp, vp, vp, vp, vp]
        L.snko_contact_rays.argtypes = [vp, vp, u32, C.c_float, vp, u32]
        L.snko_particle_probe.argtypes = [vp, vp, u32, C.c_float, vp, vp, u32]
        L.snko_particle_constrain.argtypes = [vp, vp, vp, u32, C.c_float, vp, u32]
        L.snko_mlp_adam.argtypes = [vp, vp, vp, vp, u32, C.c_double, C.c_double, C.c_double, C.c_double]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


class Outputs(C.Structure):
    _fields_ = [(n, C.c_void_p) for n in ("radiance", "albedo", "normal", "position", "rma", "motion", "depth",
                                          "mat_flags", "inst_id", "prim_id")] + [("memory", C.c_uint32), ("pad", C.c_uint32)]


def alloc_outputs(n: int) -> dict:
    return {
        "radiance": np.zeros((n, 4), np.float32), "albedo": np.zeros((n, 4), np.float32),
        "normal": np.zeros((n, 4), np.float32), "position": np.zeros((n, 4), np.float32),
        "rma": np.zeros((n, 4), np.float32), "motion": np.zeros((n, 2), np.float32),
        "depth": np.zeros(n, np.float32), "mat_flags": np.zeros(n, np.uint32),
        "inst_id": np.zeros(n, np.uint32), "prim_id": np.zeros(n, np.uint32),
    }


def _outputs_struct(d: dict) -> Outputs:
    o = Outputs()
    for k, v in d.items():
        setattr(o, k, v.ctypes.data)
    o.memory = 1
    return o


def threads() -> int:
    return int(lib().snko_hardware_threads())


class OracleScene:
    """A scene loaded into the oracle (same arrays as the CUDA library receives)."""

    def __init__(self, scene):
        L = lib()
        self._h = L.snko_scene_create()
        self._keep = []
        for m in scene.meshes:
            pos = np.ascontiguousarray(m.positions, np.float32)
            nrm = None if m.normals is None else np.ascontiguousarray(m.normals, np.float32)
            idx = np.ascontiguousarray(m.indices, np.uint32)
            self._keep += [pos, nrm, idx]
            assert L.snko_add_mesh(self._h, _p(pos), _p(nrm), _p(idx), pos.shape[0], idx.shape[0]) == 0
        inst = np.ascontiguousarray(scene.instances)
        mats = np.ascontiguousarray(scene.materials)
        assert L.snko_set_instances(self._h, _p(inst), len(inst)) == 0
        assert L.snko_set_materials(self._h, _p(mats), len(mats)) == 0
        dl = np.ascontiguousarray(scene.dir_light).reshape(1)
        pl = np.ascontiguousarray(scene.point_lights)
        assert L.snko_set_lights(self._h, _p(dl), _p(pl) if len(pl) else None, len(pl)) == 0
        assert L.snko_build(self._h) == 0

    def __del__(self):
        try:
            lib().snko_scene_destroy(self._h)
        except Exception:
            pass

    def set_instances(self, instances):
        """Replaces the instance list and rebuilds (as snk_pt_set_instances + snk_pt_build)."""
        inst = np.ascontiguousarray(instances)
        self._keep.append(inst)
        assert lib().snko_set_instances(self._h, _p(inst), len(inst)) == 0
        assert lib().snko_build(self._h) == 0

    def num_local_lights(self) -> int:
        return int(lib().snko_num_local_lights(self._h))

    def light_table(self):
        """(cdf, pmf, kind) of the path tracer's light-selection table."""
        n = self.num_local_lights()
        cdf, pmf, kind = np.zeros(n, np.float32), np.zeros(n, np.float32), np.zeros(n, np.uint32)
        lib().snko_light_table(self._h, cdf.ctypes.data, pmf.ctypes.data, kind.ctypes.data)
        return cdf, pmf, kind

    def trace(self, rays: np.ndarray, any_hit: bool = False, nthreads: int | None = None, counters=None):
        rays = np.ascontiguousarray(rays, abi.RAY_DTYPE)
        hits = np.zeros(len(rays), abi.HIT_DTYPE)
        ctr = np.zeros(5, np.uint64) if counters is None else counters
        rc = lib().snko_trace(self._h, _p(rays), len(rays), 1 if any_hit else 0, _p(hits),
                              nthreads or threads(), ctr.ctypes.data_as(C.POINTER(C.c_uint64)))
        assert rc == 0, rc
        return hits

    def contact_rays(self, rays, timestep: float, nthreads: int | None = None):
        rays = np.ascontiguousarray(rays, abi.RAY_DTYPE)
        out = np.zeros(len(rays), abi.CONTACT_DTYPE)
        rc = lib().snko_contact_rays(self._h, _p(rays), len(rays), timestep, _p(out), nthreads or threads())
        assert rc == 0, rc
        return out

    def particle_probe(self, particles, timestep: float, nthreads: int | None = None):
        p = np.ascontiguousarray(particles, abi.PARTICLE_DTYPE)
        cand = np.zeros(len(p), abi.CONTACT_DTYPE)
        grav = np.zeros(len(p), np.float32)
        rc = lib().snko_particle_probe(self._h, _p(p), len(p), timestep, _p(cand), _p(grav), nthreads or threads())
        assert rc == 0, rc
        return cand, grav

    def particle_constrain(self, particles, offsets, timestep: float, nthreads: int | None = None):
        p = np.ascontiguousarray(particles, abi.PARTICLE_DTYPE)
        off = np.ascontiguousarray(offsets, np.float32).reshape(len(p), 3)
        out = np.zeros_like(off)
        rc = lib().snko_particle_constrain(self._h, _p(p), _p(off), len(p), timestep, _p(out), nthreads or threads())
        assert rc == 0, rc
        return out

    def render_path(self, view, settings, pixels=None, pixel_base: int = 0, nthreads: int | None = None,
                    counters=None) -> dict:
        view = np.ascontiguousarray(np.asarray(view, abi.VIEW_DTYPE).reshape(1))
        st = np.ascontiguousarray(np.asarray(settings, abi.SETTINGS_DTYPE).reshape(1))
        n = int(view["width"][0] * view["height"][0]) if pixels is None else len(pixels)
        px = None if pixels is None else np.ascontiguousarray(pixels, np.uint32)
        out = alloc_outputs(n)
        os_ = _outputs_struct(out)
        ctr = np.zeros(5, np.uint64) if counters is None else counters
        rc = lib().snko_render_path(self._h, _p(view), _p(st), _p(px), 0 if px is None else len(px), pixel_base,
                                    C.byref(os_), nthreads or threads(), ctr.ctypes.data_as(C.POINTER(C.c_uint64)))
        assert rc == 0, rc
        return out


    def render_path_cache(self, view, settings, pixel_base: int = 0, nthreads: int | None = None) -> dict:
        """One-sample paths with the radiance-cache mode's termination (settings'
        cache_spread, 0 = 0.01): the radiance gathered before each path ends, and
        the query record (16 floats) and throughput (rgb, 1) of each path that ends
        in the cache (zeros otherwise)."""
        view = np.ascontiguousarray(np.asarray(view, abi.VIEW_DTYPE).reshape(1))
        st = np.ascontiguousarray(np.asarray(settings, abi.SETTINGS_DTYPE).reshape(1))
        n = int(view["width"][0] * view["height"][0])
        rad = np.zeros((n, 4), np.float32)
        qrec = np.zeros((n, 16), np.float32)
        qbeta = np.zeros((n, 4), np.float32)
        rc = lib().snko_render_path_cache(self._h, _p(view), _p(st), pixel_base, rad.ctypes.data, qrec.ctypes.data,
                                          qbeta.ctypes.data, nthreads or threads())
        assert rc == 0, rc
        return {"radiance": rad, "qrec": qrec, "qbeta": qbeta}


class OracleRestir:
    """ReSTIR DI state of one view (reservoir halves + previous normals)."""

    RES_DTYPE = np.dtype([("w_sum_pl", "<f4"), ("w_pl", "<f4"), ("pl_idx", "<u4"), ("pl_m", "<u4"),
                          ("em_inst", "<u4"), ("em_tri", "<u4"), ("em_u", "<f4"), ("em_v", "<f4"),
                          ("w_sum_em", "<f4"), ("w_em", "<f4"), ("m_em", "<u4"), ("pad", "<u4")])

    def __init__(self, scene: OracleScene, width: int, height: int):
        self.scene = scene
        self.w, self.h = width, height
        self._h = lib().snko_restir_state_create(width, height)

    def __del__(self):
        try:
            lib().snko_restir_state_destroy(self._h)
        except Exception:
            pass

    def frame(self, view, settings, pixel_base: int = 0, nthreads: int | None = None, counters=None):
        view = np.ascontiguousarray(np.asarray(view, abi.VIEW_DTYPE).reshape(1))
        st = np.ascontiguousarray(np.asarray(settings, abi.SETTINGS_DTYPE).reshape(1))
        n = self.w * self.h
        out = alloc_outputs(n)
        res = np.zeros(n, self.RES_DTYPE)
        os_ = _outputs_struct(out)
        ctr = np.zeros(5, np.uint64) if counters is None else counters
        rc = lib().snko_render_restir(self.scene._h, self._h, _p(view), _p(st), pixel_base, C.byref(os_), _p(res),
                                      nthreads or threads(), ctr.ctypes.data_as(C.POINTER(C.c_uint64)))
        assert rc == 0, rc
        return out, res


# ---- unit hooks ---------------------------------------------------------------

def pcg32(initstate: int, initseq: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().snko_pcg32(initstate, initseq, n, _p(out))
    return out


def pcg_stream(a, b, c, seed, n) -> np.ndarray:
    out = np.zeros(n, np.float32)
    lib().snko_pcg_stream(a, b, c, seed, n, _p(out))
    return out


def sincos2pi(u: np.ndarray):
    u = np.ascontiguousarray(u, np.float32)
    s = np.zeros_like(u)
    c = np.zeros_like(u)
    lib().snko_sincos2pi(_p(u), len(u), _p(s), _p(c))
    return s, c


def brdf(rows: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, np.float32)
    out = np.zeros((rows.shape[0], 10), np.float32)
    lib().snko_brdf(_p(rows), rows.shape[0], _p(out))
    return out


def directional(rows: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, np.float32)
    out = np.zeros((rows.shape[0], 3), np.float32)
    lib().snko_directional(_p(rows), rows.shape[0], _p(out))
    return out


def pointlight(rows: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, np.float32)
    out = np.zeros((rows.shape[0], 3), np.float32)
    lib().snko_pointlight(_p(rows), rows.shape[0], _p(out))
    return out


def tri(rows: np.ndarray) -> np.ndarray:
    rows = np.ascontiguousarray(rows, np.float32)
    out = np.zeros((rows.shape[0], 4), np.float32)
    lib().snko_tri(_p(rows), rows.shape[0], _p(out))
    return out


def invert_affine(m: np.ndarray):
    m = np.ascontiguousarray(m, np.float32).reshape(12)
    inv = np.zeros(12, np.float32)
    nm = np.zeros(9, np.float32)
    det = np.zeros(1, np.float32)
    lib().snko_invert_affine(_p(m), _p(inv), _p(nm), _p(det))
    return inv, nm, float(det[0])


# ---- MLP radiance cache reference (FP64) -------------------------------------------
MLP_NW = 4 * 64 * 64 + 64 * 3


def mlp_forward(W, x):
    W = np.ascontiguousarray(W, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    y = np.zeros((x.shape[0], 3))
    lib().snko_mlp_forward(_p(W), _p(x), x.shape[0], _p(y))
    return y


def mlp_grad(W, x, t, w=None, relative=True):
    """(loss, dL/dW) of the relative-L2 loss over the batch (FP64); relative=False: plain L2."""
    W = np.ascontiguousarray(W, np.float64)
    x = np.ascontiguousarray(x, np.float64)
    t = np.ascontiguousarray(t, np.float64)
    w = np.ones(x.shape[0]) if w is None else np.ascontiguousarray(w, np.float64)
    dW = np.zeros(MLP_NW)
    loss = lib().snko_mlp_grad(_p(W), _p(x), _p(t), _p(w), x.shape[0], _p(dW), 1 if relative else 0)
    return loss, dW


def mlp_adam(W, m, v, dW, step, lr=1e-2, b1=0.9, b2=0.99, eps=1e-8):
    """One Adam step in place on float64 arrays."""
    for a in (W, m, v):
        assert a.dtype == np.float64 and a.flags.c_contiguous
    dW = np.ascontiguousarray(dW, np.float64)
    lib().snko_mlp_adam(_p(W), _p(m), _p(v), _p(dW), step, lr, b1, b2, eps)


class OracleTaa:
    """TAA_ResolvePass on the CPU: history and previous motion images, the first
    resolve takes the current frame as its history (as snk_taa_resolve)."""

    def __init__(self, width: int, height: int):
        self.w, self.h = int(width), int(height)
        self.hist = None
        self.pmot = None

    def reset(self):
        self.hist = None
        self.pmot = None

    def resolve(self, radiance, motion):
        cur = np.ascontiguousarray(radiance, np.float32).reshape(self.h * self.w, 4)
        mot = np.ascontiguousarray(motion, np.float32).reshape(self.h * self.w, 2)
        if self.hist is None:
            self.hist, self.pmot = cur.copy(), mot.copy()
        out = np.empty_like(cur)
        lib().snko_taa_resolve(self.w, self.h, _p(cur), _p(mot), _p(self.hist), _p(self.pmot), _p(out))
        self.hist, self.pmot = out.copy(), mot.copy()
        return out
