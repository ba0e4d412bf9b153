"""GPU frame parity: the wavefront path tracer and ReSTIR DI against the CPU
oracle.  Tolerance: per-pixel radiance within 1e-4 relative (the arithmetic is
specified to the operation, so in practice the values are identical); hit ids,
hit distances and the G-buffer must be identical."""
import numpy as np
import pytest

import oracle as O
import snkpt
from helpers import assert_hits_equal, camera_rays, max_rel, random_rays
from snkpt import abi, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-4
GBUF = ("albedo", "normal", "position", "rma", "motion", "depth", "mat_flags", "inst_id", "prim_id")


def _gpu_frame(pt, views, st, device):
    outs = [snkpt.alloc_outputs(int(v["width"]), int(v["height"]), device=device) for v in views]
    pt.render(views, st, outs)
    pt.synchronize()
    res = []
    for o in outs:
        d = {}
        for k, t in o.items():
            a = t.cpu().numpy()
            d[k] = a.view(np.uint32) if k in ("mat_flags", "inst_id", "prim_id") else a
        res.append(d)
    return res


def _compare(g, r, what):
    for k in GBUF:
        assert np.array_equal(g[k], r[k]), f"{what}: G-buffer '{k}' differs at {int((g[k] != r[k]).sum())} entries"
    m = max_rel(g["radiance"][:, :3], r["radiance"][:, :3])
    assert m <= RTOL, f"{what}: radiance max relative error {m}"


def test_path_config0_full(cuda, built_lib):
    sc = scenes.config0()
    st = abi.settings(spp=4, max_depth=4, rr_depth=3, seed=1)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    g = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    ctr = np.zeros(5, np.uint64)
    r = O.OracleScene(sc).render_path(sc.views[0], st, counters=ctr)
    _compare(g, r, "config 0")
    s = pt.stats()
    assert (s["rays_camera"], s["rays_extension"], s["rays_shadow"]) == tuple(int(x) for x in ctr[:3])
    assert g["radiance"][:, :3].mean() > 0.0


@pytest.mark.parametrize("max_depth,rr_depth", [(1, 1), (8, 2)])
def test_path_depth_and_roulette(cuda, built_lib, max_depth, rr_depth):
    """Direct light only (one segment) and long paths with early Russian roulette."""
    sc = scenes.config0(width=96, height=96)
    st = abi.settings(spp=2, max_depth=max_depth, rr_depth=rr_depth, seed=9)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    g = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    ctr = np.zeros(5, np.uint64)
    r = O.OracleScene(sc).render_path(sc.views[0], st, counters=ctr)
    _compare(g, r, f"depth {max_depth}, roulette from {rr_depth}")
    s = pt.stats()
    assert (s["rays_camera"], s["rays_extension"], s["rays_shadow"]) == tuple(int(x) for x in ctr[:3])
    if max_depth == 1:
        assert s["rays_extension"] == 0


def test_light_tables_follow_instance_updates(cuda, built_lib):
    """Instance and light tables across rebuilds of one context: emissive
    instances present (device-built triangle lights), removed (sphere-light
    table built on the host), back and moved, and set again unchanged (tables
    kept); every frame matches the oracle scene with the same instances."""
    sc = scenes.config1(width=64, height=48)
    em_mat = len(sc.materials)
    mats = np.concatenate([sc.materials, sc.materials[:1]])
    mats["flags"][-1] |= abi.MAT_EMISSIVE
    mats["albedo"][-1][:3] = (3.0, 2.5, 2.0)
    sc.materials = mats
    base = np.array(sc.instances, copy=True)
    lamps = np.array(base[1:5], copy=True)   # four icospheres turned into emitters
    lamps["material_id"] = em_mat
    with_lamps = np.concatenate([base, lamps])
    moved = np.array(with_lamps, copy=True)
    moved["transform"][-4:, [3, 7, 11]] += 0.25
    st = abi.settings(spp=1, max_depth=3, rr_depth=3, seed=5)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    osc = O.OracleScene(sc)
    for step, inst in enumerate((with_lamps, base, moved, moved)):
        pt.set_instances(inst)
        osc.set_instances(inst)
        g = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
        r = osc.render_path(sc.views[0], st)
        _compare(g, r, f"update {step}")


def test_path_config1_reduced_full_frame(cuda, built_lib):
    sc = scenes.config1(width=480, height=270)
    st = abi.settings(spp=1, max_depth=4, rr_depth=3, seed=1)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    g = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    ctr = np.zeros(5, np.uint64)
    r = O.OracleScene(sc).render_path(sc.views[0], st, counters=ctr)
    _compare(g, r, "config 1 (480x270)")
    s = pt.stats()
    assert (s["rays_camera"], s["rays_extension"], s["rays_shadow"]) == tuple(int(x) for x in ctr[:3])


def test_path_config1_1080p_sampled_pixels_and_determinism(cuda, built_lib):
    sc = scenes.config1()
    st = abi.settings(spp=1, max_depth=4, rr_depth=3, seed=1)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    a = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    b = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    for k in a:
        assert np.array_equal(a[k], b[k]), f"run-to-run difference in {k}"
    rng = np.random.default_rng(42)
    px = np.sort(rng.choice(1920 * 1080, 20000, replace=False)).astype(np.uint32)
    r = O.OracleScene(sc).render_path(sc.views[0], st, pixels=px)
    sub = {k: v[px] for k, v in a.items()}
    _compare(sub, r, "config 1 1080p (20k sampled pixels)")


def test_path_config1_720p_camera_packets_full_frame(cuda, built_lib):
    """A 1280x720 view (the smallest size whose camera rays are queued in 8x4
    tiles and traced in warp packets): the whole frame equals the oracle's."""
    sc = scenes.config1(width=1280, height=720)
    st = abi.settings(spp=1, max_depth=4, rr_depth=3, seed=6)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    g = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    _compare(g, O.OracleScene(sc).render_path(sc.views[0], st), "config 1 720p")


@pytest.mark.parametrize("case", ["config1 path", "config2 path spp2", "config2 restir", "two views"])
def test_camera_packets_match_ray_by_ray(cuda, built_lib, case):
    """Camera rays traced in warp packets (views of at least 1280x720) give every
    output bit for bit as when each ray is traced by itself (a lowered step cap
    turns the packets off): path frames with 1 and 2 samples per pixel, a ReSTIR
    DI frame's G-buffer and shading, and a batch of two views."""
    cfg = 1 if case.startswith("config1") or case == "two views" else 2
    sc = scenes.config1(width=1280, height=720) if cfg == 1 else scenes.config2(width=1280, height=720, frames=2)
    views = [sc.views[0]] if case != "two views" else \
        [sc.views[0], scenes.look_at_view((20.0, 12.0, 5.0), (60.0, 0.0, 70.0), 50.0, 1280, 720)]
    if case == "config2 restir":
        st = abi.settings(mode=abi.MODE_RESTIR_DI, frame_index=0, seed=2)
    else:
        st = abi.settings(spp=2 if "spp2" in case else 1, max_depth=4, rr_depth=3, seed=8)
    outs = []
    for knobs in ({}, {"max_traversal_steps": 65535}):
        pt = snkpt.PathTracer(0)
        if knobs:
            pt.set_tuning(knobs)
        pt.load_scene(sc)
        outs.append(_gpu_frame(pt, views, st, cuda))
        del pt
    for v in range(len(views)):
        for k in outs[0][v]:
            assert np.array_equal(outs[0][v][k], outs[1][v][k]), f"{case}: view {v} '{k}' differs"
    assert (outs[0][0]["inst_id"] != 0xFFFFFFFF).mean() > 0.3


@pytest.mark.parametrize("spp", [1, 3])
def test_path_multi_view_batch(cuda, built_lib, spp):
    res = [(160, 90), (96, 54), (200, 120)]
    sc = scenes.config3(resolutions=res)
    st = abi.settings(spp=spp, max_depth=6, rr_depth=3, seed=3)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    gs = _gpu_frame(pt, sc.views, st, cuda)
    osc = O.OracleScene(sc)
    base = 0
    for v, g in zip(sc.views, gs):
        r = osc.render_path(v, st, pixel_base=base)
        _compare(g, r, f"multi-view {int(v['width'])}x{int(v['height'])}")
        base += int(v["width"]) * int(v["height"])


@pytest.mark.parametrize("spp", [1, 2])
def test_host_outputs_match_device_outputs(cuda, built_lib, spp):
    """Device outputs of one-sample frames are written as each path ends (no resolve
    pass); host outputs, and frames of several samples, by the resolve pass."""
    sc = scenes.config0(width=128, height=128)
    st = abi.settings(spp=spp, max_depth=4)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    g = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    host = snkpt.alloc_outputs(128, 128)
    pt.render([sc.views[0]], st, [host])
    for k in g:
        h = host[k].view(np.uint32) if k in ("mat_flags", "inst_id", "prim_id") else host[k]
        assert np.array_equal(g[k], h), k
    # page-locked host outputs are written in place by the kernels (no staging copy)
    import torch
    pinned = {}
    for k, a in snkpt.alloc_outputs(128, 128).items():
        t = torch.empty(a.shape, dtype=torch.float32 if a.dtype == np.float32 else torch.int32, pin_memory=True)
        t.fill_(-7)
        pinned[k] = t.numpy()
    pt.render([sc.views[0]], st, [pinned])
    for k in g:
        h = pinned[k].view(np.uint32) if k in ("mat_flags", "inst_id", "prim_id") else pinned[k]
        assert np.array_equal(g[k], h), ("pinned", k)


def test_fp64_accumulator_device_outputs(cuda, built_lib):
    """The FP64 accumulator gets the same sums whether the frame's outputs are on the
    device (pixels written as their paths end) or on the host (resolve pass)."""
    import torch
    sc = scenes.config1(width=160, height=90)
    sums = []
    for device in (True, False):
        pt = snkpt.PathTracer(0)
        pt.load_scene(sc)
        for f in range(3):
            flags = abi.RENDER_ACCUMULATE_F64 | (abi.RENDER_RESET_ACCUM if f == 0 else 0)
            st = abi.settings(spp=1, max_depth=4, seed=30 + f, flags=flags)
            out = snkpt.alloc_outputs(160, 90, device=cuda if device else None, names=("radiance",))
            pt.render([sc.views[0]], st, [out])
        pt.synchronize()
        sums.append(pt.read_accumulator(160, 90))
    assert sums[0][1] == sums[1][1] == 3
    assert np.array_equal(sums[0][0], sums[1][0])


def test_fp64_accumulator(cuda, built_lib):
    sc = scenes.config0(width=64, height=64)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    frames = []
    for f in range(4):
        flags = abi.RENDER_ACCUMULATE_F64 | (abi.RENDER_RESET_ACCUM if f == 0 else 0)
        st = abi.settings(spp=1, max_depth=4, seed=10 + f, flags=flags)
        host = snkpt.alloc_outputs(64, 64, names=("radiance",))
        pt.render([sc.views[0]], st, [host])
        frames.append(host["radiance"].astype(np.float64))
    acc, n = pt.read_accumulator(64, 64)
    assert n == 4
    mean = np.mean(frames, 0)
    assert np.allclose(acc[:, :3], mean[:, :3], rtol=1e-6, atol=1e-7)


def test_restir_config2_frames(cuda, built_lib):
    W, H, F = 192, 108, 4
    sc = scenes.config2(width=W, height=H, frames=F)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    osc = O.OracleScene(sc)
    ors = O.OracleRestir(osc, W, H)
    for f in range(F):
        st = abi.settings(mode=abi.MODE_RESTIR_DI, frame_index=f, seed=1)
        g = _gpu_frame(pt, [sc.views[f]], st, cuda)[0]
        ctr = np.zeros(5, np.uint64)
        r, _ = ors.frame(sc.views[f], st, counters=ctr)
        _compare(g, r, f"ReSTIR frame {f}")
        s = pt.stats()
        # every visibility test of the oracle is either traced or answered by an identical earlier test
        tests = s["rays_shadow"] + s["shadow_tests_reused"]
        assert tests == int(ctr[2]), f"frame {f}: visibility tests {tests} vs {int(ctr[2])}"
        if f > 0:
            assert s["shadow_tests_reused"] > 0.15 * tests
        assert g["radiance"][:, :3].mean() > 0.0


@pytest.mark.parametrize("temporal,spatial", [(0, 0), (1, 3), (0, 5)])
def test_restir_reuse_settings(cuda, built_lib, temporal, spatial):
    """The reference's RtSettings (num_temporal_resamples, num_spatial_resamples):
    no reuse, its defaults (temporal on, 3 neighbours), spatial reuse only."""
    W, H, F = 128, 72, 3
    sc = scenes.config2(width=W, height=H, frames=F)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    ors = O.OracleRestir(O.OracleScene(sc), W, H)
    for f in range(F):
        st = abi.settings(mode=abi.MODE_RESTIR_DI, frame_index=f, seed=4, restir_temporal=temporal,
                          restir_spatial=spatial)
        g = _gpu_frame(pt, [sc.views[f]], st, cuda)[0]
        ctr = np.zeros(5, np.uint64)
        r, _ = ors.frame(sc.views[f], st, counters=ctr)
        _compare(g, r, f"ReSTIR temporal {temporal} spatial {spatial} frame {f}")
        s = pt.stats()
        assert s["rays_shadow"] + s["shadow_tests_reused"] == int(ctr[2])


def test_restir_two_views_per_call(cuda, built_lib):
    """Two views of different sizes rendered by one call in ReSTIR mode: each view
    keeps its own reservoirs, and the second view's random streams are keyed by
    its global pixel offset (the width x height of the first)."""
    F = 3
    a = scenes.config2(width=160, height=90, frames=F)
    b = scenes.config2(width=96, height=54, frames=F)
    pt = snkpt.PathTracer(0)
    pt.load_scene(a)
    osc = O.OracleScene(a)
    ra, rb = O.OracleRestir(osc, 160, 90), O.OracleRestir(osc, 96, 54)
    for f in range(F):
        st = abi.settings(mode=abi.MODE_RESTIR_DI, frame_index=f, seed=1)
        ga, gb = _gpu_frame(pt, [a.views[f], b.views[f]], st, cuda)
        ca, cb = np.zeros(5, np.uint64), np.zeros(5, np.uint64)
        oa, _ = ra.frame(a.views[f], st, pixel_base=0, counters=ca)
        ob, _ = rb.frame(b.views[f], st, pixel_base=160 * 90, counters=cb)
        _compare(ga, oa, f"ReSTIR view 0 frame {f}")
        _compare(gb, ob, f"ReSTIR view 1 frame {f}")
        s = pt.stats()
        assert s["rays_shadow"] + s["shadow_tests_reused"] == int(ca[2] + cb[2])


def test_restir_history_of_a_larger_scene(cuda, built_lib):
    """Frames after the instance list shrinks: history reservoirs that point at
    instances which no longer exist are dropped, on the GPU as in the oracle."""
    W, H, F = 128, 72, 4
    sc = scenes.config2(width=W, height=H, frames=F)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    osc = O.OracleScene(sc)
    ors = O.OracleRestir(osc, W, H)
    smaller = np.ascontiguousarray(sc.instances[:len(sc.instances) - 4000])   # most emissive quads removed
    for f in range(F):
        if f == 2:
            pt.set_instances(smaller)
            pt.build()
            osc.set_instances(smaller)
        st = abi.settings(mode=abi.MODE_RESTIR_DI, frame_index=f, seed=1)
        g = _gpu_frame(pt, [sc.views[f]], st, cuda)[0]
        r, _ = ors.frame(sc.views[f], st)
        _compare(g, r, f"ReSTIR frame {f}")
    pt.synchronize()   # no device error


@pytest.mark.parametrize("spp,max_depth", [(1, 4), (2, 6)])
def test_restir_pt_config2_frames(cuda, built_lib, spp, max_depth):
    """The reference's whole pass-2 output (RayGen.rgen:530-570): ReSTIR DI plus
    path-traced indirect light, over 4 frames of the moving config-2 camera.  The
    G-buffer is identical, radiance within 1e-4, and every ray is accounted for:
    one camera ray per path (the first path's camera ray is the G-buffer's), the
    paths' extension rays, and the paths' shadow rays plus ReSTIR's visibility
    tests (traced or answered by an identical earlier test)."""
    W, H, F = 192, 108, 4
    sc = scenes.config2(width=W, height=H, frames=F)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    ors = O.OracleRestir(O.OracleScene(sc), W, H)
    for f in range(F):
        st = abi.settings(mode=abi.MODE_RESTIR_PT, spp=spp, max_depth=max_depth, rr_depth=3, frame_index=f, seed=1)
        g = _gpu_frame(pt, [sc.views[f]], st, cuda)[0]
        ctr = np.zeros(5, np.uint64)
        r, _ = ors.frame(sc.views[f], st, counters=ctr)
        _compare(g, r, f"ReSTIR + indirect frame {f}")
        s = pt.stats()
        assert s["rays_camera"] == W * H * spp == int(ctr[0])
        assert s["rays_extension"] == int(ctr[1]) > 0
        assert s["rays_shadow"] + s["shadow_tests_reused"] == int(ctr[2])


def test_restir_pt_is_restir_di_plus_indirect(cuda, built_lib):
    """Frame by frame, the combined mode equals the DI-only mode plus a
    non-negative indirect term on surface pixels, and equals it exactly on
    background and emissive pixels; with one path segment (no continuation) the
    indirect term is zero and the two modes agree bit for bit."""
    W, H, F = 160, 90, 3
    sc = scenes.config2(width=W, height=H, frames=F)
    di, ptm, one = (snkpt.PathTracer(0) for _ in range(3))
    for p in (di, ptm, one):
        p.load_scene(sc)
    for f in range(F):
        a = _gpu_frame(di, [sc.views[f]], abi.settings(mode=abi.MODE_RESTIR_DI, frame_index=f, seed=3), cuda)[0]
        b = _gpu_frame(ptm, [sc.views[f]], abi.settings(mode=abi.MODE_RESTIR_PT, frame_index=f, seed=3), cuda)[0]
        c = _gpu_frame(one, [sc.views[f]], abi.settings(mode=abi.MODE_RESTIR_PT, max_depth=1, frame_index=f, seed=3),
                       cuda)[0]
        for k in GBUF:
            assert np.array_equal(a[k], b[k]) and np.array_equal(a[k], c[k]), k
        assert np.array_equal(a["radiance"], c["radiance"]), f"frame {f}: depth-1 combined mode differs from DI"
        surf = (a["inst_id"] != abi.INVALID_INDEX) & ((a["mat_flags"] & abi.MAT_EMISSIVE) == 0)
        ind = b["radiance"][:, :3].astype(np.float64) - a["radiance"][:, :3]
        assert np.array_equal(b["radiance"][~surf], a["radiance"][~surf])
        assert (ind[surf] >= -1e-5 * np.abs(a["radiance"][surf, :3]) - 1e-7).all()
        assert ind[surf].mean() > 1e-3 * a["radiance"][surf, :3].mean()


def test_restir_pt_two_views_per_call(cuda, built_lib):
    """Two views in one call: the indirect paths are batched over both views (keyed
    by global pixel), the ReSTIR passes run per view."""
    F = 2
    a = scenes.config2(width=128, height=72, frames=F)
    b = scenes.config2(width=80, height=45, frames=F)
    pt = snkpt.PathTracer(0)
    pt.load_scene(a)
    osc = O.OracleScene(a)
    ra, rb = O.OracleRestir(osc, 128, 72), O.OracleRestir(osc, 80, 45)
    for f in range(F):
        st = abi.settings(mode=abi.MODE_RESTIR_PT, spp=1, max_depth=4, frame_index=f, seed=2)
        ga, gb = _gpu_frame(pt, [a.views[f], b.views[f]], st, cuda)
        oa, _ = ra.frame(a.views[f], st, pixel_base=0)
        ob, _ = rb.frame(b.views[f], st, pixel_base=128 * 72)
        _compare(ga, oa, f"view 0 frame {f}")
        _compare(gb, ob, f"view 1 frame {f}")


@pytest.mark.parametrize("mode", [abi.MODE_RESTIR_DI, abi.MODE_RESTIR_PT])
def test_restir_full_size_config2(cuda, built_lib, mode):
    """Config 2 at its own size, 1920x1080 with 4096 emissive quads: two frames of
    the moving camera (the second reuses the first's reservoirs), every pixel
    against a full-frame oracle run (the reservoir passes read neighbours, so the
    oracle renders whole frames); G-buffer identical, radiance within 1e-4."""
    W, H, F = 1920, 1080, 2
    sc = scenes.config2(width=W, height=H, frames=F)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    ors = O.OracleRestir(O.OracleScene(sc), W, H)
    for f in range(F):
        st = abi.settings(mode=mode, spp=1, max_depth=4, rr_depth=3, frame_index=f, seed=1)
        g = _gpu_frame(pt, [sc.views[f]], st, cuda)[0]
        ctr = np.zeros(5, np.uint64)
        r, _ = ors.frame(sc.views[f], st, counters=ctr)
        _compare(g, r, f"1080p mode {mode} frame {f}")
        s = pt.stats()
        assert s["rays_shadow"] + s["shadow_tests_reused"] == int(ctr[2])


def test_launch_knobs_do_not_change_results(cuda, built_lib):
    """Every autotuner candidate must render the same bits (the knobs only move work)."""
    sc = scenes.config1(width=320, height=180)
    st = abi.settings(spp=1, max_depth=4, rr_depth=3, seed=5)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    base = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    for knobs in [dict(trace_blocks_per_sm=4, ray_chunk=32, refill_idle=1, prim_bias=2, trace_variant=1),
                  dict(trace_blocks_per_sm=32, ray_chunk=256, refill_idle=16, prim_bias=8, shade_blocks_per_sm=4),
                  dict(shadow_blocks_per_sm=8, shadow_ray_chunk=128, shadow_refill_idle=8, shadow_prim_bias=2,
                       shadow_variant=3)]:
        pt.set_tuning(knobs)
        g = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
        for k in g:
            assert np.array_equal(g[k], base[k]), (knobs, k)
    best = pt.autotune([sc.views[0]], st, frames_per_trial=1)
    assert best["trace_blocks_per_sm"] > 0 and best["ray_chunk"] > 0
    g = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    for k in g:
        assert np.array_equal(g[k], base[k]), ("autotuned", k)


def test_graph_replay_matches_stream_launches(cuda, built_lib):
    """SNK_RENDER_USE_GRAPH captures the frame into a CUDA graph and replays it,
    updating the instantiated graph as frame parameters change; the images (and
    the online-trained cache weights) must equal those of direct launches."""
    res = [(160, 90), (96, 54), (200, 120)]
    sc = scenes.config3(resolutions=res)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    for f in range(3):
        st = abi.settings(spp=1, max_depth=6, rr_depth=3, seed=20 + f, frame_index=f)
        base = _gpu_frame(pt, sc.views, st, cuda)
        st["flags"] = abi.RENDER_USE_GRAPH
        got = _gpu_frame(pt, sc.views, st, cuda)
        for g, b in zip(got, base):
            for k in b:
                assert np.array_equal(g[k], b[k]), (f, k)
    # new seeds, frame indices, camera poses and output buffers replay the one capture
    s = pt.stats()
    assert (s["graph_launches"], s["graph_captures"]) == (3, 1)
    moved = [v.copy() for v in sc.views]
    for v in moved:
        v["pos"] += np.float32(0.5)
    st = abi.settings(spp=1, max_depth=6, rr_depth=3, seed=99, frame_index=7)
    base = _gpu_frame(pt, moved, st, cuda)
    st["flags"] = abi.RENDER_USE_GRAPH
    got = _gpu_frame(pt, moved, st, cuda)
    for g, b in zip(got, base):
        for k in b:
            assert np.array_equal(g[k], b[k]), ("moved views", k)
    assert pt.stats()["graph_captures"] == 1
    # a different depth is a different frame: captured again
    st = abi.settings(spp=1, max_depth=3, rr_depth=3, seed=5, flags=abi.RENDER_USE_GRAPH)
    _gpu_frame(pt, sc.views, st, cuda)
    assert pt.stats()["graph_captures"] == 2
    # cache mode: training kernels (Adam step counters) are captured each frame
    weights = []
    for flags in (0, abi.RENDER_USE_GRAPH):
        pt.cache_reset(2)
        imgs = []
        for f in range(4):
            st = abi.settings(mode=abi.MODE_PATH_CACHE, spp=1, max_depth=6, seed=50 + f, frame_index=f, flags=flags)
            imgs.append(_gpu_frame(pt, sc.views[:1], st, cuda)[0]["radiance"])
        weights.append((pt.cache_get_weights(), imgs))
    assert np.array_equal(weights[0][0], weights[1][0])
    for a, b in zip(weights[0][1], weights[1][1]):
        assert np.array_equal(a, b)


def test_full_size_eight_view_batch_sampled_pixels(cuda, built_lib):
    """The largest workload in one call: config 3's eight views (640x360 .. 3840x2160,
    19,238,400 pixels, depth 6) rendered together; 1500 seeded pixels of every view
    against the oracle, and the ray count against the per-view pixel counts."""
    sc = scenes.config3()
    st = abi.settings(spp=1, max_depth=6, rr_depth=3, seed=17)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    outs = [snkpt.alloc_outputs(int(v["width"]), int(v["height"]), device=cuda,
                                names=("radiance", "albedo", "normal", "depth", "inst_id", "prim_id"))
            for v in sc.views]
    pt.render(sc.views, st, outs)
    pt.synchronize()
    assert pt.stats()["rays_camera"] == sum(int(v["width"]) * int(v["height"]) for v in sc.views) == 19_238_400
    osc = O.OracleScene(sc)
    rng = np.random.default_rng(99)
    base = 0
    for v, o in zip(sc.views, outs):
        n = int(v["width"]) * int(v["height"])
        px = np.sort(rng.choice(n, 1500, replace=False)).astype(np.uint32)
        r = osc.render_path(v, st, pixels=px, pixel_base=base)
        g = {k: t.cpu().numpy() for k, t in o.items()}
        for k in ("inst_id", "prim_id"):
            assert np.array_equal(g[k].view(np.uint32)[px], r[k]), (int(v["width"]), k)
        for k in ("albedo", "normal", "depth"):
            assert np.array_equal(g[k][px], r[k]), (int(v["width"]), k)
        m = max_rel(g["radiance"][px, :3], r["radiance"][:, :3])
        assert m <= RTOL, (int(v["width"]), m)
        base += n


def test_instances_of_empty_meshes_are_skipped(cuda, built_lib):
    """A scene mixing empty meshes (0 triangles) with real ones renders as if the
    empty instances were absent."""
    sc = scenes.config0(width=96, height=96)
    empty = scenes.Mesh(np.zeros((0, 3), np.float32), None, np.zeros((0, 3), np.uint32))
    meshes = list(sc.meshes) + [empty]
    inst = np.concatenate([sc.instances, scenes.make_instances([(scenes.affine(t=(1.0, 2.0, 3.0)), len(meshes) - 1, 0)])])
    mixed = scenes.Scene(meshes, inst, sc.materials, sc.dir_light, sc.point_lights, sc.views, "mixed")
    st = abi.settings(spp=1, max_depth=3, seed=2)
    a = _gpu_frame(_tracer(mixed), [sc.views[0]], st, cuda)[0]
    b = _gpu_frame(_tracer(sc), [sc.views[0]], st, cuda)[0]
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def _tracer(sc):
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    return pt


def _odd_geometry_scene():
    """Config 1 (reduced) with transforms and triangles the regular scenes do not
    have: mirrored, non-uniformly scaled and sheared icospheres; a mesh of
    degenerate triangles (repeated vertex, collinear, a sliver) with a triangle
    listed twice; and two coincident instances of it (ties in t broken by
    instance, then triangle index)."""
    sc = scenes.config1(width=96, height=64)
    inst = np.array(sc.instances, copy=True)
    odd = {1: scenes.affine(scale=(-1.0, 1.0, 1.0)), 2: scenes.affine(scale=(2.0, 0.5, 1.0)),
           3: scenes.affine(R=[[1.0, 0.6, 0.0], [0.0, 1.0, 0.0], [0.0, 0.3, 1.0]]),
           4: scenes.affine(scale=(-1.5, -0.7, 1.2))}
    for i, m in odd.items():
        t = inst["transform"][i].reshape(3, 4).astype(np.float64)
        m = m.astype(np.float64)
        # keep the instance where it was, change the linear part
        new = np.concatenate([m[:, :3] @ t[:, :3], t[:, 3:]], 1).astype(np.float32)
        inst["transform"][i] = new.reshape(12)
        inst["prev_transform"][i] = new.reshape(12)
    p = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0], [2, 0, 0], [1, 1e-7, 0], [0, 2, 0], [1, 1, 0]], np.float32)
    tri = np.array([[0, 1, 2], [0, 0, 1], [0, 1, 3], [1, 4, 3], [2, 1, 6], [0, 1, 2], [2, 5, 6]], np.uint32)
    nrm = np.tile(np.array([[0, 0, 1]], np.float32), (len(p), 1))
    sc.meshes.append(scenes.Mesh(p, nrm, tri))
    mid = len(sc.meshes) - 1
    extra = np.zeros(3, inst.dtype)
    for k, (x, z) in enumerate([(0.0, 2.0), (1.5, 3.0), (1.5, 3.0)]):
        m = scenes.affine(R=scenes.rot_x(-0.4), scale=(1.5, 1.5, 1.5), t=(x, 0.5, z)).reshape(12)
        extra[k]["transform"] = m
        extra[k]["prev_transform"] = m
        extra[k]["mesh_id"] = mid
        extra[k]["material_id"] = k % len(sc.materials)
    sc.instances = np.concatenate([inst, extra])
    return sc


def test_odd_transforms_and_degenerate_triangles(cuda, built_lib):
    sc = _odd_geometry_scene()
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    osc = O.OracleScene(sc)
    st = abi.settings(spp=2, max_depth=3, rr_depth=3, seed=13)
    g = _gpu_frame(pt, [sc.views[0]], st, cuda)[0]
    r = osc.render_path(sc.views[0], st)
    _compare(g, r, "odd transforms / degenerate triangles")
    rays = np.concatenate([camera_rays(sc.views[0]), random_rays(sc, 200_000, np.random.default_rng(31))])
    assert_hits_equal(pt.trace_rays(rays), osc.trace(rays), "odd geometry closest")
    assert_hits_equal(pt.trace_rays(rays, any_hit=True), osc.trace(rays, any_hit=True), "odd geometry any")
    # the coincident instances: every hit on either is reported on the lower instance index
    n = len(sc.instances)
    h = osc.trace(rays)
    assert not (h["inst"] == n - 1).any() and (h["inst"] == n - 2).any()
