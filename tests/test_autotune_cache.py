"""Host logic of PathTracer.autotune's JSON cache: a result stored under (device
name, key) is reused instead of searching again, other keys search and are
added, and an unreadable file is replaced.  The library's search itself needs a
GPU; here a stand-in returns fixed knobs and counts the searches."""
import ctypes as C
import json

import pytest

import snkpt
from snkpt import abi, scenes


class FakeLib:
    def __init__(self):
        self.searches = 0
        self.applied = []

    def snk_pt_autotune(self, h, views, n, settings, frames, best_ref):
        self.searches += 1
        best = C.cast(best_ref, C.POINTER(snkpt.Tuning)).contents
        best.trace_blocks_per_sm = 12
        best.prim_bias = 3 + self.searches
        return 0

    def snk_pt_set_tuning(self, h, t_ref):
        self.applied.append(C.cast(t_ref, C.POINTER(snkpt.Tuning)).contents.as_dict())
        return 0


@pytest.fixture
def tracer(monkeypatch):
    torch = pytest.importorskip("torch")
    fake = FakeLib()
    monkeypatch.setattr(snkpt, "lib", lambda: fake)
    monkeypatch.setattr(torch.cuda, "get_device_name", lambda *a: "GB300 (stand-in)")
    pt = object.__new__(snkpt.PathTracer)
    pt._h = None
    return pt, fake


def test_autotune_cache_reuse_and_keys(tracer, tmp_path):
    pt, fake = tracer
    view = scenes.config1(width=32, height=18).views[0]
    st = abi.settings(spp=1, max_depth=4, rr_depth=3, seed=1)
    path = str(tmp_path / "sub" / "tune.json")
    a = pt.autotune([view], st, cache=path, key="config1")
    assert fake.searches == 1 and a["trace_blocks_per_sm"] == 12 and a["prim_bias"] == 4
    data = json.load(open(path))
    assert data == {"GB300 (stand-in)|config1": a}
    b = pt.autotune([view], st, cache=path, key="config1")        # stored: applied, no search
    assert b == a and fake.searches == 1 and fake.applied[-1] == a
    c = pt.autotune([view], st, cache=path, key="config2")        # another key: searched and added
    assert fake.searches == 2 and c["prim_bias"] == 5
    assert set(json.load(open(path))) == {"GB300 (stand-in)|config1", "GB300 (stand-in)|config2"}
    open(path, "w").write("{not json")                            # unreadable: searched and rewritten
    d = pt.autotune([view], st, cache=path, key="config1")
    assert fake.searches == 3 and json.load(open(path)) == {"GB300 (stand-in)|config1": d}


def test_autotune_without_cache_always_searches(tracer):
    pt, fake = tracer
    view = scenes.config1(width=32, height=18).views[0]
    st = abi.settings(spp=1, max_depth=4, rr_depth=3, seed=1)
    pt.autotune([view], st)
    pt.autotune([view], st)
    assert fake.searches == 2 and not fake.applied
