"""GPU tests of path tracing with the online-trained MLP radiance cache."""
import numpy as np
import pytest

import snkpt
from snkpt import abi, scenes

pytestmark = pytest.mark.gpu


def frame(pt, view, st, cuda, names=("radiance",)):
    w, h = int(view["width"]), int(view["height"])
    out = snkpt.alloc_outputs(w, h, device=cuda, names=names)
    pt.render([view], st, [out])
    pt.synchronize()
    return {k: v.cpu().numpy() for k, v in out.items()}


def rel_mse(x, ref, eps=1e-2):
    x = np.asarray(x, np.float64)[:, :3]
    ref = np.asarray(ref, np.float64)[:, :3]
    return float(np.mean((x - ref) ** 2 / (ref ** 2 + eps)))


def test_cache_mode_without_termination_matches_plain(cuda, built_lib):
    sc = scenes.config1(width=320, height=180)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    names = ("radiance", "albedo", "normal", "depth", "inst_id", "prim_id", "motion")
    plain = frame(pt, sc.views[0], abi.settings(spp=1, max_depth=6, seed=9), cuda, names)
    cached = frame(pt, sc.views[0], abi.settings(mode=abi.MODE_PATH_CACHE, spp=1, max_depth=6, seed=9,
                                                 cache_spread=1e30), cuda, names)
    for k in names:
        assert np.array_equal(plain[k], cached[k]), k
    s = pt.stats()
    assert s["cache_queries"] == 0 and s["cache_samples"] == 16384 * 4


@pytest.mark.parametrize("cfg", [1, 4])
def test_cache_termination_matches_oracle(cuda, built_lib, cfg):
    """Cache-mode frames with termination against the oracle: which paths end in
    the cache, where, with what throughput, and the radiance they gathered before
    must equal the oracle's restatement of the spread heuristic.  With a zero
    network the image is exactly the truncated one; with the network of a cache
    reset, each ended path adds throughput x max(network(record), 0), the network
    evaluated on the oracle's query records by the same inference kernel."""
    import oracle as O
    sc = scenes.config1(width=320, height=180) if cfg == 1 else scenes.config4(width=320, height=180, frames=1)
    view = sc.views[0]
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    st = abi.settings(mode=abi.MODE_PATH_CACHE, spp=1, max_depth=6, seed=21, cache_lr=-1.0)   # no update
    ref = O.OracleScene(sc).render_path_cache(view, st)
    q = ref["qbeta"][:, 3] > 0
    assert 0.02 < q.mean() < 0.9, q.mean()   # the heuristic really ends paths here
    pt.cache_set_weights(np.zeros(snkpt.CACHE_NUM_WEIGHTS, np.float32))
    g = frame(pt, view, st, cuda)["radiance"]
    assert np.array_equal(g, ref["radiance"]), "truncated radiance"
    assert pt.stats()["cache_queries"] == int(q.sum())
    pt.cache_reset(5)
    g = frame(pt, view, st, cuda)["radiance"].astype(np.float64)
    y = pt.cache_infer(ref["qrec"][q]).astype(np.float64)
    expect = ref["radiance"][:, :3].astype(np.float64)
    expect[q] += ref["qbeta"][q, :3].astype(np.float64) * np.maximum(y, 0.0)
    err = np.abs(g[:, :3] - expect) / np.maximum(np.abs(expect), 1e-3)
    assert float(err.max()) <= 1e-4, float(err.max())
    assert float(np.abs(g[q, :3] - ref["radiance"][q, :3]).max()) > 0.0   # the network added something


def test_cache_learns_what_truncation_loses(cuda, built_lib):
    """Against an FP64-accumulated converged image: the trained cache must recover
    most of the energy that the same cache-truncated paths lose without it."""
    W, H = 160, 90
    sc = scenes.config3(resolutions=[(W, H)])
    view = sc.views[0]
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    for f in range(256):   # converged reference: 256 spp, depth 8, FP64 accumulation
        flags = abi.RENDER_ACCUMULATE_F64 | (abi.RENDER_RESET_ACCUM if f == 0 else 0)
        pt.render([view], abi.settings(spp=1, max_depth=8, seed=100 + f, flags=flags), [{}])
    ref, nf = pt.read_accumulator(W, H)
    assert nf == 256

    def mean_frames(mode_kw, seeds):
        acc = np.zeros((W * H, 4))
        for s in seeds:
            acc += frame(pt, view, abi.settings(spp=1, max_depth=6, seed=s, **mode_kw), cuda)["radiance"]
        return acc / len(seeds)

    # truncation without the cache: zero network, no training
    pt.cache_set_weights(np.zeros(snkpt.CACHE_NUM_WEIGHTS, np.float32))
    trunc = mean_frames(dict(mode=abi.MODE_PATH_CACHE, cache_lr=-1.0, frame_index=0), range(1000, 1032))
    assert pt.stats()["cache_queries"] > 0
    # trained cache
    pt.cache_reset(1)
    for f in range(60):
        frame(pt, view, abi.settings(mode=abi.MODE_PATH_CACHE, spp=1, max_depth=6, seed=2000 + f, frame_index=f), cuda)
    cached = mean_frames(dict(mode=abi.MODE_PATH_CACHE, cache_lr=-1.0, frame_index=99), range(3000, 3032))
    plain = mean_frames(dict(mode=abi.MODE_PATH), range(4000, 4032))
    e_trunc, e_cache, e_plain = rel_mse(trunc, ref), rel_mse(cached, ref), rel_mse(plain, ref)
    assert np.isfinite(cached).all()
    # energy: truncation is dark, the cache restores the missing radiance
    lum = lambda x: float(np.mean(x[:, :3]))
    assert lum(trunc) < lum(ref)
    assert abs(lum(cached) - lum(ref)) < 0.5 * abs(lum(trunc) - lum(ref))
    assert e_cache < e_trunc, (e_cache, e_trunc, e_plain)


def test_quality_guard_falls_back_and_recovers(cuda, built_lib):
    """A trained cache passes the guard's probe; a broken one (large constant
    weights) fails it, the frame is then rendered plainly (bit-identical to plain
    path tracing) while the network keeps training, and the probe error falls."""
    from snkpt.cache_guard import RadianceCacheGuard
    W, H = 160, 90
    sc = scenes.config3(resolutions=[(W, H)])
    view = sc.views[0]
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    pt.cache_reset(1)
    for f in range(40):
        frame(pt, view, abi.settings(mode=abi.MODE_PATH_CACHE, spp=1, max_depth=6, seed=500 + f, frame_index=f), cuda)
    g = RadianceCacheGuard(pt, relmse_budget=0.05, check_every=1, probe_scale=2, probe_spp=8, device=cuda)
    out = snkpt.alloc_outputs(W, H, device=cuda, names=("radiance",))
    st = abi.settings(mode=abi.MODE_PATH_CACHE, spp=1, max_depth=6, seed=3, frame_index=40)
    g.render(view, st, out)                                      # frame 0 of the guard: no probe
    st["frame_index"] = 41
    r = g.render(view, st, out)
    assert r["mode"] == "cache" and r["probe_relmse"] < 0.05, r
    pt.cache_set_weights(np.full(snkpt.CACHE_NUM_WEIGHTS, 0.05, np.float32))   # radiance far too large
    st["frame_index"], st["seed"] = 42, 4
    r = g.render(view, st, out)
    assert r["mode"] == "plain" and r["probe_relmse"] > 0.05, r
    pt.synchronize()
    got = out["radiance"].cpu().numpy()
    plain = frame(pt, view, abi.settings(spp=1, max_depth=6, seed=4, frame_index=42), cuda)["radiance"]
    assert np.array_equal(got, plain)
    first_bad = r["probe_relmse"]
    for f in range(43, 70):
        st["frame_index"], st["seed"] = f, 100 + f
        g.render(view, st, out)
    assert g.history[-1][1] < 0.1 * first_bad, g.history[-5:]
