"""Host logic of the MLP-cache quality guard (snkpt.cache_guard) with a stand-in
tracer: when it probes, what it renders for a probe, when it falls back to plain
path tracing and when it returns to the cache.  No GPU: the stand-in fills host
buffers with an image whose cache-mode version carries a chosen bias."""
import numpy as np

from snkpt import abi, scenes
from snkpt.cache_guard import RadianceCacheGuard, block_means, rel_mse


class FakeTracer:
    def __init__(self):
        self.bias = 0.0
        self.calls = []   # (width, height, mode, spp, cache_spread, cache_lr)

    def render(self, views, settings, outputs):
        v, st, out = views[0], settings.reshape(-1)[0] if settings.ndim else settings, outputs[0]
        w, h = int(v["width"]), int(v["height"])
        self.calls.append((w, h, int(st["mode"]), int(st["spp"]), float(st["cache_spread"]), float(st["cache_lr"])))
        y, x = np.mgrid[0:h, 0:w]
        img = (0.2 + 0.5 * (x / max(w - 1, 1)) + 0.3 * (y / max(h - 1, 1))).reshape(-1)
        cached = int(st["mode"]) == abi.MODE_PATH_CACHE and float(st["cache_spread"]) < 1e29
        scale = 1.0 + (self.bias if cached else 0.0)
        out["radiance"][:, :3] = (img * scale)[:, None]
        out["radiance"][:, 3] = 1.0

    def synchronize(self):
        pass


def _setup(budget=0.05, every=2, scale=4, spp=8):
    view = scenes.config1(width=64, height=32).views[0]
    t = FakeTracer()
    g = RadianceCacheGuard(t, relmse_budget=budget, check_every=every, probe_scale=scale, probe_spp=spp)
    out = {"radiance": np.zeros((64 * 32, 4), np.float32)}
    st = abi.settings(mode=abi.MODE_PATH_CACHE, spp=1, max_depth=4, seed=7, frame_index=0)
    return view, t, g, out, st


def test_probe_schedule_and_probe_renders():
    view, t, g, out, st = _setup()
    modes = []
    for f in range(5):
        st["frame_index"] = f
        r = g.render(view, st, out)
        modes.append((r["mode"], r["probe_relmse"] is not None))
    # probes on frames 2 and 4 (not on the first frame), every frame in cache mode
    assert modes == [("cache", False), ("cache", False), ("cache", True), ("cache", False), ("cache", True)]
    probes = [c for c in t.calls if c[0] == 16]
    assert len(probes) == 4                                            # two renders per probe
    assert {c[3] for c in probes} == {8}                               # probe_spp
    assert sorted(c[2] for c in probes) == [abi.MODE_PATH, abi.MODE_PATH, abi.MODE_PATH_CACHE, abi.MODE_PATH_CACHE]
    assert all(c[5] < 0 for c in probes if c[2] == abi.MODE_PATH_CACHE)   # no training step in a probe
    frames = [c for c in t.calls if c[0] == 64]
    assert len(frames) == 5 and all(c[2] == abi.MODE_PATH_CACHE and c[4] < 1e29 for c in frames)


def test_fallback_and_recovery():
    view, t, g, out, st = _setup(budget=0.05, every=1)
    g.render(view, st, out)
    t.bias = 0.5                                      # relMSE of a 50 % bias is ~0.2 > budget
    r = g.render(view, st, out)
    assert r["mode"] == "plain" and r["probe_relmse"] > 0.05
    assert t.calls[-1][2] == abi.MODE_PATH_CACHE and t.calls[-1][4] >= 1e29   # plain image, training goes on
    np.testing.assert_array_equal(out["radiance"][:, 0], out["radiance"][:, 1])
    t.bias = 0.01                                     # the cache has recovered
    r = g.render(view, st, out)
    assert r["mode"] == "cache" and r["probe_relmse"] < 0.05
    assert [h[2] for h in g.history] == [True, False]


def test_rel_mse_of_block_means():
    w, h = 8, 4
    ref = np.ones((w * h, 4))
    x = ref.copy()
    x[:, :3] *= 1.1
    assert abs(rel_mse(x, ref) - 0.01 / 1.01) < 1e-12
    b = block_means(np.arange(w * h * 4, dtype=np.float64).reshape(-1, 4), w, h, 2)
    assert b.shape == ((w // 2) * (h // 2), 3)
