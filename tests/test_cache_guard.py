"""CPU tests of the MLP-cache quality guard: the library's error measure
(snk_cache_guard_relmse, host code) against its numpy statement, and the Python
face of the guard (what it asks the library to set, how it reports the library's
guard state) with a stand-in tracer.  The guard's probes and fallback run on the
GPU (tests/test_gpu_cache.py)."""
import numpy as np
import pytest

import snkpt
from snkpt import abi, scenes
from snkpt.cache_guard import RadianceCacheGuard, block_means, rel_mse, relmse_library


@pytest.mark.parametrize("w,h,block", [(64, 32, 4), (37, 21, 4), (16, 9, 1), (8, 4, 16), (50, 30, 7)])
def test_library_measure_matches_numpy_statement(built_lib, w, h, block):
    rng = np.random.default_rng(w * 100 + h)
    plain = rng.uniform(0.0, 2.0, (w * h, 4)).astype(np.float32)
    cached = (plain * rng.uniform(0.7, 1.4, (w * h, 4))).astype(np.float32)
    b = min(block, w, h)
    want = rel_mse(block_means(cached, w, h, b), block_means(plain, w, h, b))
    got = relmse_library(cached, plain, w, h, block)
    assert abs(got - want) <= 1e-12 * max(1.0, want), (got, want)
    assert relmse_library(plain, plain, w, h, block) == 0.0


def test_library_measure_rejects_bad_arguments(built_lib):
    with pytest.raises(snkpt.SnkError):
        relmse_library(np.zeros((4, 4)), np.zeros((4, 4)), 0, 4, 1)


class FakeTracer:
    """Keeps the guard settings and a guard state the test scripts."""

    def __init__(self):
        self.guard = None
        self.state = {"frames": 0, "probes": 0, "fallback_frames": 0, "last_probe_relmse": -1.0, "fallback": False}
        self.script = []     # per render: (probe relMSE or None, fallback after it)
        self.rendered = []

    def set_cache_guard(self, **kw):
        self.guard = kw

    def cache_guard_state(self):
        return dict(self.state)

    def render(self, views, settings, outputs):
        self.rendered.append(int(np.asarray(settings).reshape(-1)[0]["mode"]))
        probe, fallback = self.script.pop(0)
        if probe is not None:
            self.state["probes"] += 1
            self.state["last_probe_relmse"] = probe
            self.state["fallback"] = fallback
        self.state["frames"] += 1
        if self.state["fallback"]:
            self.state["fallback_frames"] += 1


def test_python_guard_sets_the_library_guard_and_reports_its_state():
    t = FakeTracer()
    g = RadianceCacheGuard(t, relmse_budget=0.02, check_every=3, probe_scale=2, probe_spp=8, block=5)
    assert t.guard == dict(relmse_budget=0.02, check_every=3, probe_scale=2, probe_spp=8, block=5)
    view = scenes.config1(width=16, height=8).views[0]
    st = abi.settings(mode=abi.MODE_PATH, spp=1)
    t.script = [(None, False), (0.5, True), (None, True), (0.01, False)]
    res = [g.render(view, st, {}) for _ in range(4)]
    assert [r["mode"] for r in res] == ["cache", "plain", "plain", "cache"]
    assert [r["probe_relmse"] for r in res] == [None, 0.5, None, 0.01]
    assert g.history == [(1, 0.5, True), (3, 0.01, False)]
    assert t.rendered == [abi.MODE_PATH_CACHE] * 4   # every guarded frame is a cache frame
