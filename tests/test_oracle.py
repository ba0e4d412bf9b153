"""CPU tests of the oracle: pinned against published vectors, the golden float64
transcription of the reference GLSL, closed-form intersection answers and a
brute-force closest-hit search."""
import os

import numpy as np
import pytest

import oracle as O
from helpers import assert_hits_equal, camera_rays, random_rays, shadow_rays
from snkpt import abi, scenes

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_pcg32_published_vector():
    # pcg32-demo (pcg-c-basic): pcg32_srandom_r(&rng, 42u, 54u), first six outputs
    expect = [0xA15C02B7, 0x7B47F409, 0xBA1D3330, 0x83D2F293, 0xBFA4784B, 0xCBED606E]
    assert O.pcg32(42, 54, 6).tolist() == expect


def test_pcg_stream_properties():
    a = O.pcg_stream(7, 0, 0, 1, 4096)
    b = O.pcg_stream(7, 0, 0, 1, 4096)
    c = O.pcg_stream(8, 0, 0, 1, 4096)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)
    assert a.min() >= 0.0 and a.max() < 1.0
    assert abs(a.mean() - 0.5) < 0.02


def test_sincos2pi_accuracy():
    u = np.concatenate([np.linspace(0, 1, 100001, endpoint=False), np.float32([0.25, 0.5, 0.75, 0.9999999])])
    u = u.astype(np.float32)
    s, c = O.sincos2pi(u)
    ref = 2 * np.pi * u.astype(np.float64)
    assert np.abs(s - np.sin(ref)).max() < 4e-7
    assert np.abs(c - np.cos(ref)).max() < 4e-7
    assert s[0] == 0.0 and c[0] == 1.0


def _rel(a, b, floor):
    return np.abs(np.asarray(a, np.float64) - b) / np.maximum(np.abs(b), floor)


# binary32 vs the float64 transcription: near the GGX peak at low roughness the
# NDF denominator n.h^2 (a^2 - 1) + 1 cancels, which costs ~1e-4 relative.
BRDF_RTOL = 3e-4


def test_brdf_matches_golden_glsl_transcription():
    g = np.load(os.path.join(GOLDEN, "brdf.npz"))
    out = O.brdf(g["brdf_in"])
    ref = g["brdf_out"]
    assert _rel(out, ref, 1e-3).max() < BRDF_RTOL
    assert np.median(_rel(out, ref, 1e-3)) < 1e-6


def test_directional_light_matches_golden():
    g = np.load(os.path.join(GOLDEN, "brdf.npz"))
    out = O.directional(g["dir_in"])
    assert _rel(out, g["dir_out"], 1e-3).max() < BRDF_RTOL


def test_pointlight_matches_golden():
    g = np.load(os.path.join(GOLDEN, "brdf.npz"))
    out = O.pointlight(g["pl_in"])
    assert _rel(out, g["pl_out"], 1e-4).max() < BRDF_RTOL


def _tri_rows(o, d, v0, v1, v2, tmin=0.0, tmax=1e4):
    return np.array([list(o) + list(d) + list(v0) + list(v1) + list(v2) + [tmin, tmax]], np.float32)


def test_watertight_known_answers():
    v0, v1, v2 = (0, 0, 0), (1, 0, 0), (0, 0, 1)
    r = O.tri(_tri_rows((0.25, 1, 0.25), (0, -1, 0), v0, v1, v2))[0]
    assert r.tolist() == [1.0, 1.0, 0.25, 0.25]
    # behind the origin, outside, parallel, beyond tmax, before tmin
    assert O.tri(_tri_rows((0.25, -1, 0.25), (0, -1, 0), v0, v1, v2))[0][0] == 0.0
    assert O.tri(_tri_rows((0.75, 1, 0.75), (0, -1, 0), v0, v1, v2))[0][0] == 0.0
    assert O.tri(_tri_rows((0.25, 0, 0.25), (1, 0, 0), v0, v1, v2))[0][0] == 0.0
    assert O.tri(_tri_rows((0.25, 1, 0.25), (0, -1, 0), v0, v1, v2, 0.0, 0.5))[0][0] == 0.0
    assert O.tri(_tri_rows((0.25, 1, 0.25), (0, -1, 0), v0, v1, v2, 1.5, 2.0))[0][0] == 0.0
    # exactly on the shared edge of two triangles of a quad: at least one reports the hit
    q = [(0, 0, 0), (1, 0, 0), (1, 0, 1), (0, 0, 1)]
    for p in [(0.5, 1, 0.5), (0.25, 1, 0.25), (1, 1, 1), (0, 1, 0)]:
        a = O.tri(_tri_rows(p, (0, -1, 0), q[0], q[2], q[1]))[0][0]
        b = O.tri(_tri_rows(p, (0, -1, 0), q[0], q[3], q[2]))[0][0]
        assert a + b >= 1.0, p


def test_invert_affine():
    rng = np.random.default_rng(3)
    for _ in range(20):
        M = scenes.affine(scenes.random_rotation(rng), rng.uniform(0.5, 4, 3), rng.uniform(-50, 50, 3))
        inv, nm, det = O.invert_affine(M)
        A = np.vstack([M.astype(np.float64), [0, 0, 0, 1]])
        B = np.vstack([inv.reshape(3, 4).astype(np.float64), [0, 0, 0, 1]])
        assert np.abs(A @ B - np.eye(4)).max() < 1e-5
        assert np.allclose(nm.reshape(3, 3), np.linalg.inv(A[:3, :3]).T, atol=1e-6)
        assert abs(det - np.linalg.det(A[:3, :3])) < 1e-3 * abs(det)


def _brute_closest(scene, rays):
    """Closest hit by testing every triangle of every instance (oracle's own
    intersection routine on the object-space ray, no BVH)."""
    hits = np.zeros(len(rays), abi.HIT_DTYPE)
    hits["t"] = -1.0
    hits["inst"] = abi.INVALID_INDEX
    hits["prim"] = abi.INVALID_INDEX
    best_t = np.full(len(rays), np.inf)
    for ii, inst in enumerate(scene.instances):
        m = scene.meshes[int(inst["mesh_id"])]
        inv, _, _ = O.invert_affine(inst["transform"])
        inv = inv.reshape(3, 4)
        # object-space rays in float32, same order as the oracle
        o = rays["o"].astype(np.float32)
        d = rays["d"].astype(np.float32)
        oo = ((inv[:, 0] * o[:, :1] + inv[:, 1] * o[:, 1:2]) + inv[:, 2] * o[:, 2:3]) + inv[:, 3]
        od = (inv[:, 0] * d[:, :1] + inv[:, 1] * d[:, 1:2]) + inv[:, 2] * d[:, 2:3]
        tri = m.positions[m.indices]  # (T,3,3)
        for r in range(len(rays)):
            rows = np.concatenate([np.tile(np.concatenate([oo[r], od[r]]), (len(tri), 1)), tri.reshape(-1, 9),
                                   np.tile([rays["tmin"][r], rays["tmax"][r]], (len(tri), 1))], 1).astype(np.float32)
            res = O.tri(rows)
            for p in np.flatnonzero(res[:, 0] > 0):
                t = res[p, 1]
                key = (t, ii, p)
                if t < best_t[r] or (t == best_t[r] and (ii, p) < (int(hits["inst"][r]), int(hits["prim"][r]))):
                    best_t[r] = t
                    hits[r] = (t, ii, p, res[p, 2], res[p, 3], 1)
                del key
    return hits


def test_oracle_bvh_matches_brute_force():
    sc = scenes.config0(width=32, height=32)
    osc = O.OracleScene(sc)
    rng = np.random.default_rng(11)
    rays = np.concatenate([camera_rays(sc.views[0], 40, rng), random_rays(sc, 40, rng)])
    assert_hits_equal(osc.trace(rays), _brute_closest(sc, rays), "oracle BVH vs brute force")


def test_oracle_any_hit_consistent_with_closest():
    sc = scenes.config1(width=64, height=36)
    osc = O.OracleScene(sc)
    rng = np.random.default_rng(5)
    rays = shadow_rays(sc, 20000, rng)
    closest = osc.trace(rays)
    anyh = osc.trace(rays, any_hit=True)
    assert np.array_equal(closest["flags"], anyh["flags"])


def test_oracle_watertight_floor_grid():
    sc = scenes.config0(width=16, height=16)
    osc = O.OracleScene(sc)
    xs = np.arange(0, 33) * (10.0 / 32) - 5.0
    hx = (xs[:-1] + xs[1:]) / 2
    pts = [(x, z) for x in xs[1:-1] for z in xs[1:-1]] + [(x, z) for x in hx for z in xs[1:-1]] + \
          [(x, z) for x in xs[1:-1] for z in hx]
    rays = np.zeros(len(pts), abi.RAY_DTYPE)
    rays["o"] = [(x, 0.5, z) for x, z in pts]
    rays["d"] = (0, -1, 0)
    rays["tmax"] = 1e4
    h = osc.trace(rays)
    assert (h["inst"] == 0).all() and (h["t"] == 0.5).all()


def test_oracle_render_thread_independent():
    sc = scenes.config0(width=48, height=48)
    osc = O.OracleScene(sc)
    st = abi.settings(spp=2, max_depth=4, rr_depth=3)
    a = osc.render_path(sc.views[0], st, nthreads=1)
    b = osc.render_path(sc.views[0], st, nthreads=8)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert np.isfinite(a["radiance"]).all() and (a["radiance"][:, :3] >= 0).all()
    # pixel subsets render the same values as the full frame
    px = np.array([0, 17, 48 * 20 + 7, 48 * 48 - 1], np.uint32)
    c = osc.render_path(sc.views[0], st, pixels=px)
    assert np.array_equal(c["radiance"], a["radiance"][px])


def test_oracle_cache_termination():
    """The oracle's cache-mode paths: without termination (a huge threshold) they
    are the plain paths; with it, a path that ends in the cache has gathered no
    more than its plain continuation (the same random numbers up to its end), the
    others are unchanged, and every query record is a unit direction and normal."""
    sc = scenes.config1(width=64, height=36)
    osc = O.OracleScene(sc)
    plain = osc.render_path(sc.views[0], abi.settings(spp=1, max_depth=6, seed=3))["radiance"]
    none = osc.render_path_cache(sc.views[0], abi.settings(spp=1, max_depth=6, seed=3, cache_spread=1e30))
    assert not none["qbeta"].any()
    assert np.array_equal(none["radiance"], plain)
    c = osc.render_path_cache(sc.views[0], abi.settings(spp=1, max_depth=6, seed=3))
    q = c["qbeta"][:, 3] > 0
    assert 0.02 < q.mean() < 0.9
    assert np.array_equal(c["radiance"][~q], plain[~q])
    assert (c["radiance"][q, :3] <= plain[q, :3] * (1 + 1e-6) + 1e-12).all()
    assert np.allclose(np.linalg.norm(c["qrec"][q, 4:7], axis=1), 1.0, atol=1e-4)
    assert np.allclose(np.linalg.norm(c["qrec"][q, 8:11], axis=1), 1.0, atol=1e-4)
    assert (c["qbeta"][q, :3] >= 0).all()


def test_oracle_restir_frames():
    sc = scenes.config2(width=48, height=27, frames=3)
    osc = O.OracleScene(sc)
    rs = O.OracleRestir(osc, 48, 27)
    ms = []
    for f in range(3):
        out, res = rs.frame(sc.views[f], abi.settings(mode=abi.MODE_RESTIR_DI, frame_index=f))
        assert np.isfinite(out["radiance"]).all()
        assert (out["radiance"][:, :3] >= 0).all()
        ms.append(int(res["m_em"].max()))
    # temporal reuse accumulates history (M grows past one frame's candidates)
    assert ms[0] >= 32 and ms[2] > ms[0]


def test_oracle_restir_pt_is_di_plus_indirect_paths():
    """The oracle's combined mode: on surface pixels the DI-only frame plus the mean
    of the pixel's indirect paths; the indirect paths of frame 0 are the plain path
    tracer's paths minus what their primary vertex gathers (emission, NEE), so a
    path frame with that vertex's light removed restates them."""
    W, H = 48, 27
    sc = scenes.config2(width=W, height=H, frames=2)
    osc = O.OracleScene(sc)
    a, b, c = (O.OracleRestir(osc, W, H) for _ in range(3))
    for f in range(2):
        di, _ = a.frame(sc.views[f], abi.settings(mode=abi.MODE_RESTIR_DI, frame_index=f, seed=5))
        ctr = np.zeros(5, np.uint64)
        pt, _ = b.frame(sc.views[f], abi.settings(mode=abi.MODE_RESTIR_PT, spp=2, max_depth=4, frame_index=f, seed=5),
                        counters=ctr)
        one, _ = c.frame(sc.views[f], abi.settings(mode=abi.MODE_RESTIR_PT, max_depth=1, frame_index=f, seed=5))
        assert np.array_equal(one["radiance"], di["radiance"])
        surf = (di["inst_id"] != abi.INVALID_INDEX) & ((di["mat_flags"] & abi.MAT_EMISSIVE) == 0)
        assert np.array_equal(pt["radiance"][~surf], di["radiance"][~surf])
        assert (pt["radiance"][surf, :3] >= di["radiance"][surf, :3]).all()
        assert (pt["radiance"][surf, :3] > di["radiance"][surf, :3]).any()
        assert int(ctr[0]) == W * H * 2   # one camera ray per path, none extra for the G-buffer
    # frame 0: seed + 0 x 0x9E3779B9 = seed, the plain tracer's own streams; a path
    # of depth 1 gathers only primary-vertex light, so (depth 4) - (depth 1) is the indirect part
    st4 = abi.settings(spp=1, max_depth=4, rr_depth=3, seed=5)
    st1 = abi.settings(spp=1, max_depth=1, rr_depth=3, seed=5)
    p4 = osc.render_path(sc.views[0], st4)["radiance"][:, :3].astype(np.float64)
    p1 = osc.render_path(sc.views[0], st1)["radiance"][:, :3].astype(np.float64)
    d = O.OracleRestir(osc, W, H)
    di0, _ = O.OracleRestir(osc, W, H).frame(sc.views[0], abi.settings(mode=abi.MODE_RESTIR_DI, seed=5))
    pt0, _ = d.frame(sc.views[0], abi.settings(mode=abi.MODE_RESTIR_PT, spp=1, max_depth=4, rr_depth=3, seed=5))
    surf = (di0["inst_id"] != abi.INVALID_INDEX) & ((di0["mat_flags"] & abi.MAT_EMISSIVE) == 0)
    ind = pt0["radiance"][surf, :3].astype(np.float64) - di0["radiance"][surf, :3]
    assert np.allclose(ind, (p4 - p1)[surf], rtol=1e-4, atol=1e-5)


def test_scene_configs():
    c0 = scenes.config0()
    assert c0.num_instanced_triangles == 2048 + 10 + 60 + 2
    c1 = scenes.config1(width=64, height=36)
    assert c1.meshes[0].num_triangles == 1280 and c1.meshes[1].num_triangles == 131072
    assert len(c1.instances) == 201 and len(c1.point_lights) == 16
    c2 = scenes.config2(width=64, height=36, frames=2)
    assert int((c2.materials["flags"] & abi.MAT_EMISSIVE).sum()) == 4096
    c3 = scenes.config3(resolutions=[(64, 36)])
    assert c3.meshes[1].num_triangles == 131072 and len(c3.instances) == 264
    assert sum(w * h for w, h in scenes.CONFIG3_RESOLUTIONS) == 19_238_400


@pytest.mark.parametrize("cfg", [0, 1])
def test_oracle_deterministic_hits(cfg):
    sc = scenes.make(cfg, width=32, height=18)
    osc = O.OracleScene(sc)
    rng = np.random.default_rng(cfg)
    rays = random_rays(sc, 5000, rng)
    assert_hits_equal(osc.trace(rays, nthreads=1), osc.trace(rays, nthreads=8), "thread count")


def test_oracle_negative_tmin_is_zero():
    """A negative or NaN tmin is taken as 0 (traceRayEXT requires tmin >= 0)."""
    sc = scenes.make(1, width=32, height=18)
    osc = O.OracleScene(sc)
    rays = random_rays(sc, 2000, np.random.default_rng(4))
    ref = osc.trace(rays)
    for v in (-1.0, -1e30, np.nan):
        r = rays.copy()
        r["tmin"] = v
        assert_hits_equal(osc.trace(r), ref, f"tmin {v}")


def test_light_table_sphere_lights_restated():
    """Sphere lights only: the oracle's selection table equals a numpy restatement
    of its definition bit for bit (w = 4 pi lum(colour); q = max(1, rint(w / w_max
    2^40)); cdf = acc / total, pmf = q / total in double rounded to float)."""
    sc = scenes.config1(width=32, height=18)
    pl = sc.point_lights
    keep = pl["radius"] > 0
    col = pl["colour"][keep].astype(np.float64)
    w = 4.0 * np.pi * (0.2126 * col[:, 0] + 0.7152 * col[:, 1] + 0.0722 * col[:, 2])
    q = np.where(w > 0, np.maximum(1, np.rint(w / w.max() * 2.0 ** 40)), 0).astype(np.uint64)
    acc = np.cumsum(q, dtype=np.uint64)
    total = float(acc[-1])
    cdf = (acc.astype(np.float64) / total).astype(np.float32)
    cdf[-1] = 1.0
    pmf = (q.astype(np.float64) / total).astype(np.float32)
    c, p, kind = O.OracleScene(sc).light_table()
    assert (kind == 0).all() and len(c) == int(keep.sum())
    assert np.array_equal(c.view(np.uint32), cdf.view(np.uint32))
    assert np.array_equal(p.view(np.uint32), pmf.view(np.uint32))


def test_light_table_properties():
    """Sphere lights and 8,192 emissive triangles: the CDF rises to exactly 1,
    each PMF entry is the CDF's step, a dark light is never chosen and a light
    2^-60 as bright as the brightest still is (its integer weight is 1)."""
    sc = scenes.config2(width=32, height=18, frames=1)
    sc.point_lights = np.array(sc.point_lights, copy=True)
    sc.point_lights["colour"][3] = 0.0
    mats = np.array(sc.materials, copy=True)
    em = np.flatnonzero((mats["flags"] & abi.MAT_EMISSIVE) != 0)
    mats["albedo"][em[7]][:3] = np.float32(2.0 ** -60)
    sc.materials = mats
    osc = O.OracleScene(sc)
    c, p, kind = osc.light_table()
    n_sph = int((sc.point_lights["radius"] > 0).sum())
    assert (kind[:n_sph] == 0).all() and (kind[n_sph:] == 1).all() and len(kind) == n_sph + 8192
    assert (np.diff(c) >= 0).all() and c[-1] == 1.0 and (p >= 0).all()
    step = np.diff(np.concatenate([[0.0], c.astype(np.float64)]))
    assert np.abs(step - p).max() < 1e-6
    assert abs(float(p.astype(np.float64).sum()) - 1.0) < 1e-5
    assert p[3] == 0.0 and c[3] == c[2]
    # the dim emitter's two triangles: instance order follows the material order of config 2
    inst = np.flatnonzero(sc.instances["material_id"] == em[7])
    assert len(inst) == 1
    tri_k = n_sph + 2 * int(np.searchsorted(np.flatnonzero(np.isin(sc.instances["material_id"], em)), inst[0]))
    assert p[tri_k] > 0.0 and p[tri_k + 1] > 0.0 and p[tri_k] < 1e-9


def test_taa_oracle_matches_golden_restatement():
    """The oracle's TAA resolve equals the independent numpy binary32 restatement
    (tests/golden/make_taa_golden.py) bit for bit over a 3-frame sequence."""
    d = np.load(os.path.join(GOLDEN, "taa.npz"))
    w, h = int(d["width"]), int(d["height"])
    t = O.OracleTaa(w, h)
    for f in range(d["radiance"].shape[0]):
        o = t.resolve(d["radiance"][f], d["motion"][f])
        assert np.array_equal(o.view(np.uint32), d["resolved"][f].view(np.uint32)), f
