#!/usr/bin/env python3
"""Benchmark of the GB300 path-tracing core on the 1080p headline workload.

Workload (one step = one frame of the render pass): the two-level scene of 200
icosphere-3 instances over a 256x256 ground grid (1 directional + 16 sphere
lights), 1920x1080, 1 sample per pixel, 4 path segments, russian roulette from
segment 3: plain wavefront path tracing with next-event estimation.  The metric
is Mrays/s = (camera + extension + shadow rays) / device time.

  value  device-resident inputs, CUDA events on the library's stream around each
         frame; L2 flushed (256 MiB memset, untimed) between frames
  e2e    the same frames through the C ABI with host buffers: per frame every
         instance moves, the instance table goes host->device (instance records,
         light tables and instance BVH rebuilt, as the reference's
         TlasSystem::BuildTlas does every frame) and the HDR radiance image comes
         back device->host; wall clock around the frames
  roofline  the dominant kernel's algorithmic bytes per launch / its average
         launch time (events on the launching stream), against measured HBM peak
  cpu_baseline  the CPU oracle (multithreaded C++) on this host's cores, one
         full 1080p frame

--impl reference runs the reference arm: the reference renders through Vulkan
ray tracing, which cannot run here, so the arm times the CPU oracle (the
transcription of the reference shaders) on all host cores, each step a
1/8-row sample of the same frame.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for p in (os.path.join(ROOT, "snake-vk_gb300"), os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "Mrays/s at 1080p"
UNIT = "Mrays/s"
WORKLOAD = ("config 1: 200 icosphere-3 instances (1280 tris) + 256x256 ground (131072 tris), 1 directional + "
            "16 sphere lights, 1920x1080, 1 spp, max depth 4, russian roulette from 3, plain wavefront path tracing")
PROFILE_SUMMARY = os.path.join(ROOT, "profiles", "trace_traversal_config1.txt")


def dist_info():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def over_ranks(seconds: float, units: float, ws: int, device=None) -> tuple:
    """(max of `seconds`, sum of `units`) over the ranks of the job: the job takes as
    long as its slowest rank, and its work is every rank's.  Uses the default
    process group (NCCL with CUDA tensors in the benchmark; gloo with CPU tensors
    in the tests)."""
    if ws <= 1:
        return float(seconds), float(units)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    u = torch.tensor([float(units)], dtype=torch.float64, device=device)
    dist.all_reduce(u)
    return float(t.item()), float(u.item())


class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "50"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
            return
        # the sampler's first line comes after nvidia-smi has started: wait for it
        # (up to 3 s) so that the timed region is covered from its start
        t0 = time.time()
        while time.time() - t0 < 3.0:
            self.f.flush()
            if os.path.getsize(self.path) > 0:
                break
            time.sleep(0.02)

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        with open(self.path) as f:
            res = self.parse(f)
        os.unlink(self.path)
        return res

    @staticmethod
    def parse(lines) -> dict | None:
        """Summary of nvidia-smi samples in FIELDS order (csv, noheader, nounits):
        median SM clock, highest max clock, the throttle reasons seen active."""
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for line in lines:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(mx)), "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic():
    """DRAM bytes of the traversal launches of one frame (closest hits and shadow
    rays, read + write) from the committed ncu summary of this build."""
    if not os.path.exists(PROFILE_SUMMARY):
        return None
    for line in open(PROFILE_SUMMARY):
        if line.startswith("dram_bytes_per_frame:"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def cpu_baseline(scene, view, settings):
    import oracle as O
    osc = O.OracleScene(scene)
    n = O.threads()
    ctr = np.zeros(5, np.uint64)
    t0 = time.perf_counter()
    osc.render_path(view, settings, nthreads=n, counters=ctr)
    dt = time.perf_counter() - t0
    rays = int(ctr[:3].sum())
    return {"value": rays / dt / 1e6, "unit": UNIT, "cores": n, "kind": "port",
            "sample": f"one full 1920x1080 frame of the same workload ({rays} rays, {dt:.2f} s wall)"}


def cache_vs_plain(pt_mod, abi, scenes, device, frames=120, check=(60,), ref_spp=4096, plain_max_spp=64):
    """Second half of the metric: ms/frame to equal relMSE vs an FP64-accumulated
    converged render, MLP cache vs plain, on the config-4 scene at 1080p.

    The cache trains online along the 120-frame seeded spline (one cache frame per
    spline frame).  At each checked frame: reference = FP64 accumulation of ref_spp
    plain samples per pixel (depth 8, frames of 16 spp); relMSE(x) = mean (x - ref)^2 / (ref^2 + 0.01); the
    plain tracer's relMSE is measured for the mean of k 1-spp frames, k = 1..64,
    and the k matching the cache's 1-spp relMSE is interpolated in log-log.
    Frame times: CUDA events around each render call on the library's stream."""
    import torch
    W, H = 1920, 1080
    sc = scenes.config4(width=W, height=H, frames=frames)
    stream = torch.cuda.Stream(device=device)
    pt = pt_mod.PathTracer(device.index or 0, stream=stream)
    pt.load_scene(sc)
    out = pt_mod.alloc_outputs(W, H, device=device, names=("radiance",))

    def timed(view, st):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        pt.render([view], st, [out])
        b.record(stream)
        b.synchronize()
        return a.elapsed_time(b)

    def relmse(x, ref):
        return float(np.mean((x[:, :3] - ref[:, :3]) ** 2 / (ref[:, :3] ** 2 + 1e-2)))

    pt.cache_reset(1)
    results = []
    cache_ms = []
    for f in range(frames):
        v = sc.views[f]
        st = abi.settings(mode=abi.MODE_PATH_CACHE, spp=1, max_depth=6, seed=10_000 + f, frame_index=f)
        ms = timed(v, st)
        if f >= 10:
            cache_ms.append(ms)
        if f not in check:
            continue
        x_cache = out["radiance"].cpu().numpy().astype(np.float64)
        for k in range(ref_spp // 16):   # converged reference of this frame: 16 spp per call
            flags = abi.RENDER_ACCUMULATE_F64 | (abi.RENDER_RESET_ACCUM if k == 0 else 0)
            pt.render([v], abi.settings(spp=16, max_depth=8, seed=500_000 + k, flags=flags), [{}])
        ref, _ = pt.read_accumulator(W, H)
        ref = ref.astype(np.float64)
        acc = np.zeros((W * H, 4))
        curve, plain_ms = {}, []
        for k in range(1, plain_max_spp + 1):
            plain_ms.append(timed(v, abi.settings(spp=1, max_depth=6, seed=900_000 + k)))
            acc += out["radiance"].cpu().numpy()
            if k & (k - 1) == 0:
                curve[k] = relmse(acc / k, ref)
        e_cache = relmse(x_cache, ref)
        ks = sorted(curve)
        k_eq = float(ks[-1])
        for k0, k1 in zip(ks, ks[1:]):
            if curve[k0] >= e_cache >= curve[k1]:
                t = (np.log(curve[k0]) - np.log(e_cache)) / (np.log(curve[k0]) - np.log(curve[k1]))
                k_eq = float(np.exp(np.log(k0) + t * (np.log(k1) - np.log(k0))))
                break
        if e_cache > curve[1]:
            k_eq = curve[1] / e_cache
        t_plain = float(np.median(plain_ms))
        results.append({"frame": f, "cache_relmse_1spp": e_cache, "plain_relmse_vs_spp": curve,
                        "plain_spp_for_equal_relmse": k_eq, "plain_ms_per_spp": t_plain,
                        "plain_ms_for_equal_relmse": k_eq * t_plain,
                        "mean_radiance": {"reference": float(ref[:, :3].mean()), "cache": float(x_cache[:, :3].mean())}})
    t_cache = float(np.median(cache_ms))
    ratio = float(np.mean([t_cache / r["plain_ms_for_equal_relmse"] for r in results]))
    return {"metric": "ms/frame to equal relMSE vs converged: MLP-cache vs plain", "unit": "ratio",
            "value": ratio, "higher_is_better": False, "cache_ms_per_frame": t_cache,
            "workload": "config 4: 64 value-noise terrain tiles + 200 icospheres, 1920x1080, 1 spp, depth 6, "
                        "cache MLP 64-4x64-3 BF16, 65536 samples/frame, Adam 1e-2, spread threshold 0.01",
            "reference": f"FP64 accumulation of {ref_spp} plain samples per pixel (depth 8; {ref_spp // 16} frames "
                         f"of 16 spp)", "checked_frames": list(check),
            "frames": frames, "checks": results}


def batched_views(snkpt, abi, scenes, device, stream, tuning, frames=5, warmup=3, scale=1):
    """Eight uneven views (640x360 .. 3840x2160, 19.2 Mpixels; each side divided
    by `scale`) of the terrain scene in one render call, 1 spp, depth 6: direct
    stream launches against CUDA-graph replay of the same frame.  Device-resident
    outputs; events on the library's stream around each frame, which include the
    host's launch (or capture + graph update) work."""
    import torch
    res_list = [(w // scale, h // scale) for w, h in scenes.CONFIG3_RESOLUTIONS]
    sc = scenes.config3(resolutions=res_list)
    pt = snkpt.PathTracer(device.index or 0, stream=stream)
    pt.load_scene(sc)
    if tuning:
        pt.set_tuning(tuning)
    outs = [snkpt.alloc_outputs(int(v["width"]), int(v["height"]), device=device, names=("radiance",))
            for v in sc.views]
    npx = sum(w * h for w, h in res_list)
    res = {"workload": f"config 3: 64 terrain tiles (256x256 grid) + 200 icospheres, 8 views "
                       f"{res_list[0][0]}x{res_list[0][1]}..{res_list[-1][0]}x{res_list[-1][1]} ({npx:,} px) in one "
                       f"call, 1 spp, depth 6",
           "blas_triangles": int(pt.stats()["triangles"]), "views": len(sc.views)}
    for name, flags in (("stream", 0), ("graph", abi.RENDER_USE_GRAPH)):
        for k in range(warmup):
            pt.render(sc.views, abi.settings(spp=1, max_depth=6, rr_depth=3, seed=500 + k, flags=flags), outs)
            pt.stats()
        torch.cuda.synchronize()
        ms, rays = 0.0, 0
        for k in range(frames):
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(stream)
            pt.render(sc.views, abi.settings(spp=1, max_depth=6, rr_depth=3, seed=600 + k, flags=flags), outs)
            b.record(stream)
            s = pt.stats()
            rays += s["rays_camera"] + s["rays_extension"] + s["rays_shadow"]
            b.synchronize()
            ms += a.elapsed_time(b)
        res[name] = {"Mrays_per_s": rays / (ms / 1e3) / 1e6, "ms_per_frame": ms / frames,
                     "rays_per_frame": rays / frames}
    del outs, pt
    torch.cuda.empty_cache()
    return res


def taa_bench(snkpt, device, stream, frames=20, warmup=3):
    """TAA resolve of a 1920x1080 RGBA32F frame with RG32F motion (device buffers,
    CUDA events on the resolver's stream, L2 flushed between frames).  Algorithmic
    bytes: 88 per pixel (16 radiance + 8 motion + 16 history + 8 previous motion
    read; 16 out + 16 next history + 8 next previous motion written)."""
    import torch
    W, H = 1920, 1080
    g = torch.Generator(device=device)
    g.manual_seed(7)
    rad = torch.rand((W * H, 4), device=device, generator=g)
    mot = (torch.rand((W * H, 2), device=device, generator=g) - 0.5) * 0.01
    out = torch.empty_like(rad)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=device)
    t = snkpt.TaaResolve(W, H, device=device.index or 0, stream=stream)
    for _ in range(warmup):
        t.resolve(rad, mot, out)
    ms = 0.0
    for _ in range(frames):
        with torch.cuda.stream(stream):
            flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        t.resolve(rad, mot, out)
        b.record(stream)
        b.synchronize()
        ms += a.elapsed_time(b)
    ms /= frames
    gbs = 88.0 * W * H / (ms / 1e3) / 1e9
    peak, kind = measured_peaks()
    return {"workload": "TAA resolve, 1920x1080 RGBA32F + RG32F motion", "kernel": "k_taa_resolve",
            "ms_per_frame": ms, "Mpixels_per_s": W * H / (ms / 1e3) / 1e6, "achieved_GBs": gbs,
            "peak_GBs": peak, "frac": gbs / peak, "bytes_per_pixel": 88}


def particle_bench(pt, abi, scene, device, n=100_000, steps=20, warmup=3):
    """Particle collision queries on the benchmark scene: per step, the scene probe
    of 100k particles (3 collision rays for each awake particle + 1 gravity ray)
    through snk_pt_particle_probe with device buffers; particles placed just
    short of surfaces hit by random rays (traced by the library itself)."""
    import torch
    rng = np.random.default_rng(11)
    lo = np.min([np.min(m.positions, 0) for m in scene.meshes], 0) - 60.0
    hi = np.max([np.max(m.positions, 0) for m in scene.meshes], 0) + 60.0
    rays = np.zeros(4 * n, abi.RAY_DTYPE)
    rays["o"] = rng.uniform([0.0, 1.0, 0.0], [100.0, 60.0, 100.0], (4 * n, 3))
    d = rng.normal(size=(4 * n, 3))
    rays["d"] = d / np.linalg.norm(d, axis=1, keepdims=True)
    rays["tmax"] = 1e4
    hits = pt.trace_rays(rays)
    ok = np.nonzero(hits["flags"] == 1)[0][:n]
    p = np.zeros(len(ok), abi.PARTICLE_DTYPE)
    p["position_radius"][:, :3] = rays["o"][ok] + rays["d"][ok] * (hits["t"][ok, None] - 0.3)
    p["position_radius"][:, 3] = 0.25
    p["velocity"][:, :3] = rng.normal(0.0, 3.0, (len(ok), 3))
    p["velocity"][:, 3] = 1.0
    t = torch.from_numpy(p.view(np.float32).reshape(-1, 12).copy()).to(device)
    for _ in range(warmup):
        pt.particle_probe(t, 1.0 / 120.0)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        pt.particle_probe(t, 1.0 / 120.0)
    torch.cuda.synchronize()
    ms = (time.perf_counter() - t0) / steps * 1e3
    del lo, hi
    return {"workload": f"{len(ok)} particles, 4 rays each (3 collision + gravity), config 1 scene",
            "ms_per_step": ms, "Mrays_per_s": 4 * len(ok) / (ms / 1e3) / 1e6,
            "note": "wall clock around the C-ABI call (synchronising), device buffers"}


def bvh_bench(snkpt, scenes, device, stream, reps=3):
    """BVH builds (wall clock around synchronising C-ABI calls, median of reps):
    the mesh BVHs of config 3 (a 131,072-triangle terrain tile and a 1,280-triangle
    icosphere: Morton sort, hierarchy, 3 treelet passes, 8-wide collapse) from
    uploaded meshes, and one per-frame instance-BVH rebuild (set_instances + build)
    at config 1's 201 instances (single-launch builder) and config 2's 4,297
    instances (multi-launch builder), every instance moved between rebuilds
    (instance records, emissive-light records, light CDF and the BVH all redone)."""
    import torch
    sc3 = scenes.config3(resolutions=[(64, 36)])
    tris = int(sum(m.num_triangles for m in sc3.meshes))
    mesh_ms = []
    for _ in range(reps):
        pt = snkpt.PathTracer(device.index or 0, stream=stream)
        pt.upload_meshes(sc3.meshes)
        pt.set_materials(sc3.materials)
        pt.set_lights(sc3.dir_light, sc3.point_lights)
        pt.set_instances(sc3.instances[:1])
        pt.synchronize()
        t0 = time.perf_counter()
        pt.build()
        pt.synchronize()
        mesh_ms.append((time.perf_counter() - t0) * 1e3)
        del pt
    out = {"mesh_bvh": {"workload": "config 3 meshes: 131,072 + 1,280 triangles", "triangles": tris,
                        "ms": float(np.median(mesh_ms)), "Mtris_per_s": tris / (float(np.median(mesh_ms)) / 1e3) / 1e6}}
    for name, sc in (("instance_bvh_201", scenes.config1(width=64, height=36)),
                     ("instance_bvh_4297", scenes.config2(width=64, height=36, frames=1))):
        pt = snkpt.PathTracer(device.index or 0, stream=stream)
        pt.load_scene(sc)
        inst = np.array(sc.instances, copy=True)
        for _ in range(3):
            pt.set_instances(inst); pt.build(); pt.synchronize()
        ms = []
        for k in range(20):
            # every instance moves (all table rows and boxes change, as in an animated frame)
            inst["transform"][:, [3, 7, 11]] += 1e-3 if k % 2 == 0 else -1e-3
            t0 = time.perf_counter()
            pt.set_instances(inst); pt.build(); pt.synchronize()
            ms.append((time.perf_counter() - t0) * 1e3)
        # the same updates with the instance BVH refitted (topology kept, boxes redone)
        pt.set_tuning({"tlas_refit_interval": 1000})
        refits0 = pt.stats()["instance_bvh_refits"]
        ms_refit = []
        for k in range(21):
            inst["transform"][:, [3, 7, 11]] += 1e-3 if k % 2 == 0 else -1e-3
            t0 = time.perf_counter()
            pt.set_instances(inst); pt.build(); pt.synchronize()
            if k > 0:   # (the first update after the tuning change rebuilds)
                ms_refit.append((time.perf_counter() - t0) * 1e3)
        out[name] = {"instances": len(inst), "ms_per_rebuild": float(np.median(ms)),
                     "ms_per_refit": float(np.median(ms_refit)),
                     "refits": int(pt.stats()["instance_bvh_refits"] - refits0),
                     "note": "every instance moved; per update: instance records, light tables, then the BVH "
                             "rebuilt or refitted"}
        del pt
    torch.cuda.synchronize()
    return out


def restir_bench(snkpt, abi, scenes, device, stream, tuning, frames=16, warmup=3, mode=None):
    """ReSTIR on the stress scene (config 2: the 1080p sphere field + 4096
    emissive quads, camera moving 0.05 units per frame): per frame the G-buffer,
    32 initial light candidates + 1 visibility ray with temporal reuse (M cap 20),
    and spatial reuse over 5 neighbours in a 30-pixel radius.  mode
    MODE_RESTIR_DI: direct light only; MODE_RESTIR_PT: the reference's whole pass-2
    output, direct light plus one 4-segment indirect path per pixel (roulette from
    segment 3), the paths' first segment giving the G-buffer.  Device-resident
    outputs; CUDA events on the library's stream."""
    import torch
    mode = abi.MODE_RESTIR_DI if mode is None else mode
    sc = scenes.config2(frames=frames)
    pt = snkpt.PathTracer(device.index or 0, stream=stream)
    pt.load_scene(sc)
    if tuning:
        pt.set_tuning(tuning)
    out = snkpt.alloc_outputs(1920, 1080, device=device, names=("radiance", "albedo", "normal", "motion", "depth"))

    def st(f, flags=0):
        return abi.settings(mode=mode, spp=1, max_depth=4, rr_depth=3, frame_index=f, seed=1, flags=flags)
    for k in range(warmup):
        pt.render([sc.views[0]], st(k), [out])
        pt.stats()
    ms, rays = 0.0, 0
    per_stage = {}
    for f in range(frames):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        pt.render([sc.views[f]], st(warmup + f, abi.RENDER_PROFILE), [out])
        b.record(stream)
        s = pt.stats()
        b.synchronize()
        ms += a.elapsed_time(b)
        rays += s["rays_camera"] + s["rays_extension"] + s["rays_shadow"]
        for k, v in s["stage_ms"].items():
            if v > 0:
                per_stage[k] = per_stage.get(k, 0.0) + v / frames
    del pt, out
    what = ("ReSTIR DI" if mode == abi.MODE_RESTIR_DI else
            "ReSTIR DI + path-traced indirect (1 path/pixel, 4 segments, roulette from 3)")
    return {"workload": f"config 2: {what}, 1920x1080, 4096 emissive quads + 16 sphere lights + sun, 32 "
                        "candidates, temporal (M cap 20) + 5 spatial neighbours in 30 px, camera +0.05/frame",
            "frames": frames, "ms_per_frame": ms / frames, "Mrays_per_s": rays / (ms / 1e3) / 1e6,
            "rays_per_frame": rays / frames, "stage_ms_per_frame": per_stage}


def run_reference(args):
    ws, rank, _ = dist_info()
    if rank != 0:
        return 0
    import oracle as O
    from snkpt import abi, scenes
    sc = scenes.config1()
    view = sc.views[0]
    osc = O.OracleScene(sc)
    n = O.threads()
    W, H = int(view["width"]), int(view["height"])
    rows = np.arange(H)

    def step(k):
        sel = rows[(rows % 8) == (k % 8)]
        px = (sel[:, None] * W + np.arange(W)[None, :]).reshape(-1).astype(np.uint32)
        ctr = np.zeros(5, np.uint64)
        st = abi.settings(spp=1, max_depth=4, rr_depth=3, seed=1 + k)
        t0 = time.perf_counter()
        osc.render_path(view, st, pixels=px, nthreads=n, counters=ctr)
        return int(ctr[:3].sum()), time.perf_counter() - t0

    for k in range(args.warmup):
        step(k)
    rays, secs = 0, 0.0
    for k in range(args.steps):
        r, s = step(args.warmup + k)
        rays += r
        secs += s
    value = rays / secs / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": secs / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": {"workload": WORKLOAD, "sample": "every 8th row of the 1080p frame per step"},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": n, "kind": "port",
                             "sample": "every 8th row of the 1080p frame per step (CPU oracle: the reference's "
                                       "ray-gen/closest-hit/miss logic in multithreaded C++; the reference's own "
                                       "Vulkan ray-tracing path is unavailable on this box)"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


def run_ours(args):
    import torch
    import snkpt
    from snkpt import abi, scenes

    ws, rank, local = dist_info()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    sc = scenes.config1()
    view = sc.views[0]
    W, H = int(view["width"]), int(view["height"])
    stream = torch.cuda.Stream(device=dev)
    pt = snkpt.PathTracer(local, stream=stream)
    pt.load_scene(sc)
    outs = snkpt.alloc_outputs(W, H, device=dev)
    torch.cuda.synchronize()
    tuning = pt.get_tuning()
    if not args.no_autotune:
        # untimed: the project's autotuner picks the launch knobs for this workload
        tuning = pt.autotune([view], abi.settings(spp=1, max_depth=4, rr_depth=3, seed=7), frames_per_trial=3)

    def settings(seed, flags=abi.RENDER_PROFILE):
        return abi.settings(spp=1, max_depth=4, rr_depth=3, seed=seed, flags=flags)

    # traversal counts for the algorithmic bytes (one untimed instrumented frame)
    pt.render([view], settings(1, abi.RENDER_COUNT_NODES), [outs])
    cnt = pt.stats()
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)

    def barrier():
        if ws > 1:
            import torch.distributed as dist
            dist.barrier()

    for k in range(args.warmup):
        pt.render([view], settings(100 + k), [outs])
        pt.stats()
    clocks = ClockSampler(local)
    clocks.start()
    barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    rays = 0
    launches = 0
    stage_ms = {k: 0.0 for k in abi.STAGES}
    stage_n = {k: 0 for k in abi.STAGES}
    rays_closest = 0
    rays_shadow = 0
    for k in range(args.steps):
        with torch.cuda.stream(stream):
            flush.zero_()
        ev[k][0].record(stream)
        pt.render([view], settings(1000 + k), [outs])
        ev[k][1].record(stream)
        s = pt.stats()
        rays += s["rays_camera"] + s["rays_extension"] + s["rays_shadow"]
        rays_closest += s["rays_camera"] + s["rays_extension"]
        rays_shadow += s["rays_shadow"]
        launches += sum(s["stage_launches"].values())
        for name in abi.STAGES:
            stage_ms[name] += s["stage_ms"][name]
            stage_n[name] += s["stage_launches"][name]
    torch.cuda.synchronize()
    barrier()
    total_ms = sum(a.elapsed_time(b) for a, b in ev)
    total_ms, rays_all = over_ranks(total_ms, rays, ws, dev)
    value = rays_all / (total_ms / 1e3) / 1e6

    # roofline of the dominant kernel: the traversal core.  Its closest-hit and
    # shadow launches overlap (the shadow rays of segment d run beside the closest
    # hits of segment d + 1 on a second stream), so the unit is the frame's
    # traversal: the algorithmic bytes of all its closest-hit and shadow rays over
    # the time during which a traversal launch runs (the union of their spans,
    # stage "trace_any", from CUDA events on the streams the kernels run on).  The
    # per-ray node and triangle counts are each ray's own traversal (the counting
    # frame traces ray by ray), also for the camera rays, which the timed frames
    # trace in warp packets.
    peak, peak_kind = measured_peaks()
    c_rays = cnt["rays_camera"] + cnt["rays_extension"]
    s_rays = cnt["rays_shadow"]
    b_closest = 32 + 24 + 80.0 * cnt["node_visits"] / max(c_rays, 1) + 48.0 * cnt["triangle_tests"] / max(c_rays, 1)
    b_shadow = 32 + 16 + 80.0 * cnt["shadow_node_visits"] / max(s_rays, 1) + \
        48.0 * cnt["shadow_triangle_tests"] / max(s_rays, 1)
    trav_bytes = b_closest * rays_closest + b_shadow * rays_shadow   # over the timed frames
    trav_s = stage_ms["trace_any"] / 1e3
    achieved = trav_bytes / trav_s / 1e9
    traffic = profile_traffic()
    roofline = {"bound": "hbm", "kernel": "k_trace_packet (camera rays) + k_trace_closest + k_trace_shadow "
                                                 "(one traversal core, overlapped)",
                "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak, "peak_kind": peak_kind,
                "traffic": traffic, "traffic_source": os.path.relpath(PROFILE_SUMMARY, ROOT) if traffic else None,
                "bytes_per_closest_ray": b_closest, "bytes_per_shadow_ray": b_shadow,
                "traversal_ms_per_frame": stage_ms["trace_any"] / args.steps,
                "algorithmic_bytes_per_frame": trav_bytes / args.steps,
                "nodes_per_ray": cnt["node_visits"] / max(c_rays, 1), "tris_per_ray": cnt["triangle_tests"] / max(c_rays, 1),
                "shadow_nodes_per_ray": cnt["shadow_node_visits"] / max(s_rays, 1),
                "stage_ms_per_frame": {k: v / args.steps for k, v in stage_ms.items() if v > 0}}

    # end to end through the C ABI with host buffers
    host_rad = torch.empty((W * H, 4), dtype=torch.float32, pin_memory=True).numpy()
    inst = np.array(sc.instances, copy=True)
    e2e_rays = 0

    def move(k):
        # every instance moves by 1e-3 each frame (back and forth), so the instance
        # table really crosses to the device and every derived table is redone
        inst["transform"][:, [3, 7, 11]] += 1e-3 if k % 2 == 0 else -1e-3
        inst["prev_transform"][:, [3, 7, 11]] = inst["transform"][:, [3, 7, 11]]
    for k in range(max(1, args.warmup)):
        move(k)
        pt.set_instances(inst)
        pt.render([view], settings(2000 + k, 0), [{"radiance": host_rad}])
    barrier()
    t0 = time.perf_counter()
    for k in range(args.steps):
        move(k)
        pt.set_instances(inst)
        pt.render([view], settings(3000 + k, 0), [{"radiance": host_rad}])
        s = pt.stats()
        e2e_rays += s["rays_camera"] + s["rays_extension"] + s["rays_shadow"]
    e2e_s = time.perf_counter() - t0
    e2e_s, e2e_rays_all = over_ranks(e2e_s, e2e_rays, ws, dev)
    e2e_value = e2e_rays_all / e2e_s / 1e6
    # the same, refitting the instance BVH between full rebuilds every 16 updates
    pt.set_tuning(dict(tuning, tlas_refit_interval=16))
    for k in range(max(1, args.warmup)):
        move(k)
        pt.set_instances(inst)
        pt.render([view], settings(2000 + k, 0), [{"radiance": host_rad}])
    barrier()
    t0 = time.perf_counter()
    refit_rays = 0
    for k in range(args.steps):
        move(k)
        pt.set_instances(inst)
        pt.render([view], settings(3000 + k, 0), [{"radiance": host_rad}])
        s = pt.stats()
        refit_rays += s["rays_camera"] + s["rays_extension"] + s["rays_shadow"]
    refit_s = time.perf_counter() - t0
    refit_s, refit_rays = over_ranks(refit_s, refit_rays, ws, dev)
    pt.set_tuning(tuning)
    clk = clocks.stop()   # sampled over the device-timed and the end-to-end frames
    h2d = inst.nbytes + abi.VIEW_DTYPE.itemsize + abi.SETTINGS_DTYPE.itemsize
    d2h = host_rad.nbytes

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": total_ms / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded scene generator)",
            "config": {"workload": WORKLOAD, "width": W, "height": H, "spp": 1, "max_depth": 4,
                       "rays_per_frame": rays / args.steps, "parallelism": f"replicas x{ws}",
                       "l2": "flushed between steps (256 MiB memset on the same stream, untimed)",
                       "tuning": tuning},
            "gpu_launches": launches,
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                    "ms_per_step": e2e_s / args.steps * 1e3},
            "e2e_instance_refit": {"value": refit_rays / refit_s / 1e6, "unit": UNIT,
                                   "ms_per_step": refit_s / args.steps * 1e3,
                                   "note": "as e2e, instance BVH refitted, rebuilt every 16th update"},
            "roofline": roofline}
    if clk:
        line["clocks"] = clk
    if rank == 0:
        if ws == 1 and not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(sc, view, settings(1, 0))
        line["taa"] = taa_bench(snkpt, dev, stream)
        line["particles"] = particle_bench(pt, abi, sc, dev)
        # (the ReSTIR frames use the default launch knobs: the autotuned ones are the
        # path-tracing frame's, and its visibility queues trace best at the defaults)
        line["restir"] = restir_bench(snkpt, abi, scenes, dev, stream, None)
        line["restir_pt"] = restir_bench(snkpt, abi, scenes, dev, stream, None, mode=abi.MODE_RESTIR_PT)
        line["bvh_build"] = bvh_bench(snkpt, scenes, dev, stream)
        if not args.no_batched:
            line["batched_views"] = batched_views(snkpt, abi, scenes, dev, stream, tuning)
            line["batched_views_small"] = batched_views(snkpt, abi, scenes, dev, stream, tuning, frames=20, scale=8)
        if args.cache_eval != "off":
            checks = (60,) if args.cache_eval == "quick" else tuple(range(9, 120, 10))
            line["cache_vs_plain"] = cache_vs_plain(snkpt, abi, scenes, dev, check=checks)
        print(json.dumps(line))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--no-batched", action="store_true", help="skip the 8-view batched (config 3) measurement")
    ap.add_argument("--cache-eval", default="full", choices=["off", "quick", "full"],
                    help="MLP cache vs plain at equal relMSE: quick = one checked frame, full = every 10th frame")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
