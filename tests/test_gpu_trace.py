"""GPU per-ray parity: closest hit (t, instance, triangle, barycentrics) and any
hit of the CUDA traversal must equal the CPU oracle bit for bit."""
import numpy as np
import pytest

import oracle as O
import snkpt
from helpers import assert_hits_equal, camera_rays, random_rays, scene_bounds, shadow_rays
from snkpt import abi, scenes

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes_loaded(cuda, built_lib):
    out = {}
    for cfg, kw in [(0, {}), (1, {"width": 1920, "height": 1080}), (2, {"width": 640, "height": 360, "frames": 1}),
                    (3, {"resolutions": [(1280, 720)]}), (4, {"width": 960, "height": 540, "frames": 2})]:
        sc = scenes.make(cfg, **kw)
        pt = snkpt.PathTracer(0)
        pt.load_scene(sc)
        out[cfg] = (sc, pt, O.OracleScene(sc))
    return out


# at least 1M rays per configuration: every camera ray of the view (400k sampled
# at 1080p) plus random rays through the scene box
@pytest.mark.parametrize("cfg,n_rand", [(0, 1_000_000), (1, 600_000), (2, 800_000), (3, 200_000), (4, 600_000)])
def test_closest_hit_bit_exact(scenes_loaded, cfg, n_rand):
    sc, pt, osc = scenes_loaded[cfg]
    rng = np.random.default_rng(100 + cfg)
    v = sc.views[0]
    npix = int(v["width"]) * int(v["height"])
    cam = camera_rays(v) if npix <= 1 << 20 else camera_rays(v, 400_000, rng)
    rays = np.concatenate([cam, random_rays(sc, n_rand, rng)])
    assert len(rays) >= 1_000_000
    gpu = pt.trace_rays(rays)
    ref = osc.trace(rays)
    assert_hits_equal(gpu, ref, f"config {cfg} closest")
    assert (ref["flags"] == 1).mean() > 0.3   # the ray sets actually hit geometry


@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4])
def test_any_hit_bit_exact(scenes_loaded, cfg):
    sc, pt, osc = scenes_loaded[cfg]
    rng = np.random.default_rng(200 + cfg)
    rays = shadow_rays(sc, 300_000, rng)
    gpu = pt.trace_rays(rays, any_hit=True)
    ref = osc.trace(rays, any_hit=True)
    assert np.array_equal(gpu["flags"], ref["flags"]), f"{int((gpu['flags'] != ref['flags']).sum())} differ"
    occluded = ref["flags"].mean()
    assert 0.02 < occluded < 0.98


def test_device_buffers_match_host_buffers(scenes_loaded, cuda):
    import torch
    sc, pt, _ = scenes_loaded[1]
    rng = np.random.default_rng(7)
    rays = random_rays(sc, 100_000, rng)
    host = pt.trace_rays(rays)
    t = torch.from_numpy(rays.view(np.float32).reshape(-1, 8).copy()).to(cuda)
    dev = pt.trace_rays(t).cpu().numpy().view(abi.HIT_DTYPE).reshape(-1)
    assert_hits_equal(dev, host, "device vs host buffers")


def test_watertight_floor_grid(scenes_loaded):
    sc, pt, _ = scenes_loaded[0]
    xs = np.arange(0, 33) * (10.0 / 32) - 5.0
    hx = (xs[:-1] + xs[1:]) / 2
    pts = [(x, z) for x in xs[1:-1] for z in xs[1:-1]] + [(x, z) for x in hx for z in xs[1:-1]] + \
          [(x, z) for x in xs[1:-1] for z in hx]
    rays = np.zeros(len(pts), abi.RAY_DTYPE)
    rays["o"] = [(x, 0.5, z) for x, z in pts]
    rays["d"] = (0, -1, 0)
    rays["tmax"] = 1e4
    h = pt.trace_rays(rays)
    assert (h["inst"] == 0).all() and (h["t"] == 0.5).all()


def test_degenerate_rays(scenes_loaded):
    sc, pt, osc = scenes_loaded[1]
    rng = np.random.default_rng(9)
    r = random_rays(sc, 4096, rng)
    # axis-aligned directions (zero components), empty intervals, tiny tmax
    r["d"][:1024] = np.eye(3)[rng.integers(0, 3, 1024)] * rng.choice([-1.0, 1.0], (1024, 1))
    r["tmin"][1024:2048] = 5.0
    r["tmax"][1024:2048] = 5.0
    r["tmax"][2048:3072] = 1e-6
    # negative and NaN tmin (taken as 0, as traceRayEXT requires tmin >= 0)
    r["tmin"][3072:3584] = -1.0
    r["tmin"][3584:] = np.nan
    h = pt.trace_rays(r)
    assert_hits_equal(h, osc.trace(r), "degenerate rays")
    assert (h["flags"][1024:2048] == 0).all()
    r0 = r[3072:].copy()
    r0["tmin"] = 0.0
    assert_hits_equal(h[3072:], pt.trace_rays(r0), "tmin below 0 as 0")


def test_box_test_edge_cases(scenes_loaded):
    """Rays that stress the rounding of the quantised box test: origins far
    outside the scene, origins on mesh vertices with axis-parallel directions,
    and rays grazing the ground plane (y = 0) from points on it."""
    sc, pt, osc = scenes_loaded[1]
    rng = np.random.default_rng(21)
    lo, hi = scene_bounds(sc)
    n = 100_000
    # far origins (1e4 outside the box) aimed at random points inside it
    target = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3)); d /= np.linalg.norm(d, axis=1, keepdims=True)
    far = np.zeros(n, abi.RAY_DTYPE)
    far["o"] = target - 1e4 * d
    far["d"] = d
    far["tmax"] = 3e4
    # world-space vertices of random instances, axis-parallel directions
    verts = []
    for i in rng.integers(0, len(sc.instances), 64):
        m = sc.meshes[int(sc.instances[i]["mesh_id"])]
        M = sc.instances[i]["transform"].reshape(3, 4).astype(np.float64)
        p = m.positions[rng.integers(0, len(m.positions), n // 64)].astype(np.float64)
        verts.append(p @ M[:, :3].T + M[:, 3])
    verts = np.concatenate(verts)
    axis = np.zeros(len(verts), abi.RAY_DTYPE)
    axis["o"] = verts
    axis["d"] = np.eye(3)[rng.integers(0, 3, len(verts))] * rng.choice([-1.0, 1.0], (len(verts), 1))
    axis["tmax"] = 1e4
    # grazing: from points of the ground plane, nearly parallel to it
    g = np.zeros(n, abi.RAY_DTYPE)
    g["o"] = np.stack([rng.uniform(lo[0], hi[0], n), np.zeros(n), rng.uniform(lo[2], hi[2], n)], 1)
    phi = rng.uniform(0, 2 * np.pi, n)
    elev = rng.choice([-1.0, 1.0], n) * 10.0 ** rng.uniform(-7, -2, n)
    g["d"] = np.stack([np.cos(phi), elev, np.sin(phi)], 1) / np.sqrt(1 + elev ** 2)[:, None]
    g["tmax"] = 1e4
    for name, rays in (("far origins", far), ("vertex origins, axis-parallel", axis), ("grazing", g)):
        assert_hits_equal(pt.trace_rays(rays), osc.trace(rays), name)


def test_deep_instance_bvh(cuda, built_lib):
    """More than 1024 instances (the multi-launch instance BVH) in a layout whose
    Morton hierarchy is deep: 40 cubes at halving distances along the diagonal
    (1e5 down to 1e-7) plus 1,100 small cubes in a cluster.  The collapse then
    runs past its multi-block levels into the single-block finish; hits must
    still equal the oracle's and no device error may be reported."""
    rng = np.random.default_rng(31)
    cube = scenes.cube_mesh()
    rows = []
    for k in range(40):
        c = 1e5 * 0.5 ** k
        rows.append((scenes.affine(scale=(0.3 * 0.5 ** k,) * 3, t=(c, c, c)), 0, 0))
    for p in rng.uniform(-2.0, 2.0, (1100, 3)):
        rows.append((scenes.affine(scale=(0.05, 0.05, 0.05), t=tuple(p)), 0, 0))
    sc = scenes.Scene([cube], scenes.make_instances(rows), scenes.make_materials([((0.5, 0.5, 0.5), 0.5, 0.0, 0)]),
                      scenes.no_dir_light(), scenes.point_lights([]), [], "deep")
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    osc = O.OracleScene(sc)
    n = 200_000
    rays = np.zeros(n, abi.RAY_DTYPE)
    # half the rays aim at the diagonal chain, half at the cluster
    tgt = np.concatenate([np.repeat(1e5 * 0.5 ** rng.uniform(0.0, 20.0, (n // 2, 1)), 3, 1),
                          rng.uniform(-2.0, 2.0, (n // 2, 3))])
    d = rng.normal(size=(n, 3)); d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays["o"] = tgt - 0.5 * np.linalg.norm(tgt, axis=1, keepdims=True).clip(4.0, None) * d
    rays["d"] = d
    rays["tmax"] = 1e6
    h = pt.trace_rays(rays)
    assert_hits_equal(h, osc.trace(rays), "deep instance BVH")
    assert (h["flags"] == 1).mean() > 0.05
    pt.synchronize()   # raises on a device error (bit 8: instance BVH build)


def test_empty_scene(cuda, built_lib):
    pt = snkpt.PathTracer(0)
    pt.upload_meshes([scenes.Mesh(np.zeros((0, 3), np.float32), None, np.zeros((0, 3), np.uint32))])
    pt.set_materials(scenes.make_materials([((0.5, 0.5, 0.5), 0.5, 0.0, 0)]))
    pt.set_lights(scenes.no_dir_light(), scenes.point_lights([]))
    pt.set_instances(scenes.make_instances([(scenes.affine(), 0, 0)]))
    pt.build()
    rays = random_rays(scenes.config0(width=8, height=8), 1000, np.random.default_rng(1))
    h = pt.trace_rays(rays)
    assert (h["flags"] == 0).all() and (h["inst"] == abi.INVALID_INDEX).all()


def test_invalid_scene_is_rejected(cuda, built_lib):
    sc = scenes.config0(width=8, height=8)
    pt = snkpt.PathTracer(0)
    pt.upload_meshes(sc.meshes)
    pt.set_materials(sc.materials)
    pt.set_lights(sc.dir_light, sc.point_lights)
    bad = sc.instances.copy()
    bad[0]["mesh_id"] = 99
    pt.set_instances(bad)
    with pytest.raises(snkpt.SnkError) as e:
        pt.build()
    assert e.value.code == 1
    bad = sc.instances.copy()
    bad[0]["transform"][0] = np.nan
    with pytest.raises(snkpt.SnkError):
        pt.set_instances(bad)


def test_traversal_bounds_report_limit_and_recover(cuda, built_lib):
    """The traversal's step cap and stack bound are software loop bounds the
    context can lower: a ray that reaches one stops, the error word gets the
    bound's bit (2 steps, 1 stack) and the next synchronising call returns
    SNK_ERR_LIMIT naming it.  With the defaults back the same context traces
    bit-exactly again (the error word was cleared)."""
    sc = scenes.config1(width=64, height=36)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    rng = np.random.default_rng(5)
    rays = np.concatenate([camera_rays(sc.views[0]), random_rays(sc, 20_000, rng)])
    for knob, bit in (("max_traversal_steps", 2), ("stack_limit", 1)):
        pt.set_tuning({knob: 1})
        with pytest.raises(snkpt.SnkError) as e:
            pt.trace_rays(rays)
        assert e.value.code == abi.ERR_LIMIT
        assert f"error word {bit})" in str(e.value), str(e.value)
    pt.set_tuning({"max_traversal_steps": 1})
    out = snkpt.alloc_outputs(64, 36, names=("radiance",))
    with pytest.raises(snkpt.SnkError) as e:   # a frame with host outputs synchronises and reports it too
        pt.render([sc.views[0]], abi.settings(), [out])
    assert e.value.code == abi.ERR_LIMIT
    pt.set_tuning({})
    assert_hits_equal(pt.trace_rays(rays), O.OracleScene(sc).trace(rays), "after the bounds were restored")
    with pytest.raises(snkpt.SnkError):
        pt.set_tuning({"stack_limit": 65})


def test_treelet_restructuring_lowers_sah_and_keeps_hits(cuda, built_lib):
    """The restructured BVH must have a lower SAH cost and fewer node visits than
    the plain LBVH while every hit stays identical (hits do not depend on the tree)."""
    sc = scenes.config3(resolutions=[(320, 180)])
    rng = np.random.default_rng(11)
    rays = np.concatenate([camera_rays(sc.views[0]), random_rays(sc, 100_000, rng)])
    st = abi.settings(spp=1, max_depth=4, seed=3, flags=abi.RENDER_COUNT_NODES)
    res = {}
    for passes in (snkpt.TREELET_PASSES_NONE, 1, 0):   # none, one pass, default (3)
        pt = snkpt.PathTracer(0)
        pt.set_tuning({"bvh_treelet_passes": passes})
        pt.load_scene(sc)
        hits = pt.trace_rays(rays)
        pt.render([sc.views[0]], st, [{}])
        s = pt.stats()
        res[passes] = (s["blas_sah_cost"], hits, s["node_visits"] / (s["rays_camera"] + s["rays_extension"]))
    plain, one, full = res[snkpt.TREELET_PASSES_NONE], res[1], res[0]
    assert_hits_equal(one[1], plain[1], "one treelet pass vs plain LBVH")
    assert_hits_equal(full[1], plain[1], "three treelet passes vs plain LBVH")
    assert full[0] < one[0] < plain[0], (plain[0], one[0], full[0])
    assert full[2] < plain[2], (plain[2], full[2])
    assert_hits_equal(full[1], O.OracleScene(sc).trace(rays), "restructured BVH vs oracle")
    # the least-SAH choice of each wide node's children against the greedy one
    # (open the largest child until 8): lower cost, identical hits
    pt = snkpt.PathTracer(0)
    pt.set_tuning({"bvh_collapse": 1})
    pt.load_scene(sc)
    greedy_hits = pt.trace_rays(rays)
    greedy_sah = pt.stats()["blas_sah_cost"]
    assert full[0] < greedy_sah, (full[0], greedy_sah)
    assert_hits_equal(greedy_hits, full[1], "greedy vs least-SAH collapse")


@pytest.mark.parametrize("knobs", [{"bvh_leaf_max": 2}, {"bvh_leaf_max": 1, "bvh_leaf_pack": 4},
                                   {"tlas_leaf_max": 3}, {"bvh_leaf_max": 4, "tlas_leaf_max": 2},
                                   {"bvh_collapse": 1}, {"bvh_collapse": 1, "tlas_leaf_max": 2}])
def test_multi_primitive_leaves_keep_hits(cuda, built_lib, knobs):
    """Leaves of several primitives (mesh or instance level) use the general
    primitive groups in traversal; single-primitive leaves use the slot-mask form.
    The greedy collapse (bvh_collapse 1) makes other trees of either kind.  Hits,
    any-hit answers and a rendered frame must not depend on any of it."""
    sc = scenes.config1(width=320, height=180)
    rng = np.random.default_rng(23)
    rays = np.concatenate([camera_rays(sc.views[0]), random_rays(sc, 100_000, rng)])
    srays = shadow_rays(sc, 100_000, rng)
    single = snkpt.PathTracer(0)
    single.load_scene(sc)
    multi = snkpt.PathTracer(0)
    multi.set_tuning(knobs)
    multi.load_scene(sc)
    assert_hits_equal(multi.trace_rays(rays), single.trace_rays(rays), f"{knobs} vs single-primitive leaves")
    assert np.array_equal(multi.trace_rays(srays, any_hit=True)["flags"], single.trace_rays(srays, any_hit=True)["flags"])
    assert_hits_equal(multi.trace_rays(rays), O.OracleScene(sc).trace(rays), f"{knobs} vs oracle")
    st = abi.settings(spp=1, max_depth=4, seed=9)
    outs = [snkpt.alloc_outputs(320, 180, device=cuda) for _ in range(2)]
    single.render([sc.views[0]], st, [outs[0]])
    multi.render([sc.views[0]], st, [outs[1]])
    single.synchronize(); multi.synchronize()
    for k in outs[0]:
        assert np.array_equal(outs[0][k].cpu().numpy(), outs[1][k].cpu().numpy()), k


def _small_meshes():
    """Meshes of 1, 2, 4 and 8 triangles (mesh BVHs of one wide node, whose
    children are all leaves when leaves hold one triangle) and the 12-triangle
    cube (a root with an internal child)."""
    tri = scenes.Mesh(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), None, np.array([[0, 1, 2]], np.uint32))
    tet = scenes.Mesh(np.array([[1, 1, 1], [1, -1, -1], [-1, 1, -1], [-1, -1, 1]], np.float32), None,
                      np.array([[0, 1, 2], [0, 3, 1], [0, 2, 3], [1, 3, 2]], np.uint32))
    octa = scenes.Mesh(np.array([[1, 0, 0], [-1, 0, 0], [0, 1, 0], [0, -1, 0], [0, 0, 1], [0, 0, -1]], np.float32),
                       None, np.array([[0, 2, 4], [2, 1, 4], [1, 3, 4], [3, 0, 4], [2, 0, 5], [1, 2, 5], [3, 1, 5],
                                       [0, 3, 5]], np.uint32))
    return [tri, scenes.quad_mesh(), tet, octa, scenes.cube_mesh()]


@pytest.mark.parametrize("knobs", [{}, {"tlas_leaf_max": 2}, {"bvh_leaf_max": 2}])
def test_small_meshes_bit_exact(cuda, built_lib, knobs):
    """600 instances of meshes of 1 to 12 triangles, most of them a single wide
    node: single-primitive leaves in both levels (slot-mask primitive groups),
    multi-primitive instance leaves, multi-primitive mesh leaves.  Closest hits
    and any-hit answers equal the oracle's in all three."""
    rng = np.random.default_rng(41)
    rows = []
    for k in range(600):
        R = scenes.random_rotation(rng)
        s = rng.uniform(0.2, 2.0, 3)
        rows.append((scenes.affine(R, tuple(s), tuple(rng.uniform(-20.0, 20.0, 3))), k % 5, 0))
    sc = scenes.Scene(_small_meshes(), scenes.make_instances(rows),
                      scenes.make_materials([((0.5, 0.5, 0.5), 0.5, 0.0, 0)]), scenes.no_dir_light(),
                      scenes.point_lights([]), [], "small meshes")
    pt = snkpt.PathTracer(0)
    if knobs:
        pt.set_tuning(knobs)
    pt.load_scene(sc)
    osc = O.OracleScene(sc)
    rays = random_rays(sc, 300_000, rng)
    h = pt.trace_rays(rays)
    assert_hits_equal(h, osc.trace(rays), f"small meshes {knobs}")
    assert (h["flags"] == 1).mean() > 0.2
    hit_mesh = np.array([r[1] for r in rows])[h["inst"][h["flags"] == 1]]
    assert len(np.unique(hit_mesh)) == 5
    srays = shadow_rays(sc, 200_000, rng)
    a = pt.trace_rays(srays, any_hit=True)
    assert np.array_equal(a["flags"], osc.trace(srays, any_hit=True)["flags"])
    assert 0.02 < a["flags"].mean() < 0.98
    pt.synchronize()


@pytest.mark.parametrize("cfg", [1, 2])
def test_instance_bvh_refit_keeps_hits(cuda, built_lib, cfg):
    """Refitting the instance BVH (tlas_refit_interval) while instances move must
    give the same hits as rebuilding it every update, and as the oracle: config 1's
    201 instances (single-launch builder) and config 2's 4,297 (multi-launch
    builder)."""
    sc = scenes.config1(width=320, height=180) if cfg == 1 else scenes.config2(width=320, height=180, frames=1)
    rng = np.random.default_rng(21)
    rays = np.concatenate([camera_rays(sc.views[0]), random_rays(sc, 100_000, rng)])
    refit = snkpt.PathTracer(0)
    refit.set_tuning({"tlas_refit_interval": 1000})
    refit.load_scene(sc)
    build = snkpt.PathTracer(0)
    build.load_scene(sc)
    inst = np.array(sc.instances, copy=True)
    for f in range(5):
        prev = inst["transform"].copy()
        move = rng.normal(0.0, 2.0 + 4.0 * f, (len(inst), 3)).astype(np.float32)
        move[inst["mesh_id"] == 1] = 0.0                    # the ground stays
        t = inst["transform"].reshape(-1, 3, 4)
        t[:, :, 3] += move
        inst["transform"] = t.reshape(inst["transform"].shape)
        inst["prev_transform"] = prev
        refit.set_instances(inst)
        build.set_instances(inst)
        a, b = refit.trace_rays(rays), build.trace_rays(rays)
        assert_hits_equal(a, b, f"refit vs rebuild, update {f}")
    assert refit.stats()["instance_bvh_refits"] == 5
    assert build.stats()["instance_bvh_refits"] == 0
    sc.instances = inst
    assert_hits_equal(a, O.OracleScene(sc).trace(rays), "refit vs oracle")
    st = abi.settings(spp=1, max_depth=3, seed=4)
    outs = [snkpt.alloc_outputs(320, 180, device=cuda) for _ in range(2)]
    refit.render([sc.views[0]], st, [outs[0]])
    build.render([sc.views[0]], st, [outs[1]])
    refit.synchronize(); build.synchronize()
    for k in outs[0]:
        assert np.array_equal(outs[0][k].cpu().numpy(), outs[1][k].cpu().numpy()), k


def test_meshdata_asset_traces_bit_exact(cuda, built_lib):
    """Submeshes of a .meshdata asset (one BLAS each, as the reference builds them)
    instanced in a scene: hits equal the oracle's on the same meshes."""
    import os
    from snkpt import meshdata as MD
    md = MD.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "two_submeshes.meshdata"))
    rng = np.random.default_rng(8)
    meshes = md.meshes()
    rows, mats = [], []
    for k in range(40):
        sm = k % 2
        mats.append((*scenes.random_material(rng), 0))
        rows.append((scenes.affine(scenes.random_rotation(rng), (rng.uniform(0.5, 3.0),) * 3,
                                   rng.uniform(-10.0, 10.0, 3)), sm, len(mats) - 1))
    view = scenes.look_at_view((0.0, 8.0, -25.0), (0.0, 0.0, 0.0), 60.0, 320, 180)
    sc = scenes.Scene(meshes, scenes.make_instances(rows), scenes.make_materials(mats),
                      scenes.dir_light((0.3, 1.0, 0.2), (2.0, 2.0, 2.0)), scenes.point_lights([]), [view], "meshdata")
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    rays = np.concatenate([camera_rays(view), random_rays(sc, 200_000, rng)])
    ref = O.OracleScene(sc).trace(rays)
    assert_hits_equal(pt.trace_rays(rays), ref, "meshdata submeshes")
    assert (ref["flags"] == 1).mean() > 0.01
