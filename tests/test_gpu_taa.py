"""GPU TAA resolve (snk_taa_*) against the CPU oracle: bit-exact (every
operation is a binary32 basic operation in a fixed order on both sides)."""
import numpy as np
import pytest

import oracle as O
import snkpt
from snkpt import abi, scenes

pytestmark = pytest.mark.gpu


def frames(rng, w, h, n):
    out = []
    for _ in range(n):
        r = rng.lognormal(-0.5, 1.2, (h * w, 4)).astype(np.float32)
        r[rng.uniform(size=(h * w, 4)) < 0.05] *= -1.0
        r[:, 3] = 1.0
        mv = rng.normal(0.0, 0.02, (h * w, 2)).astype(np.float32)
        mv[rng.uniform(size=h * w) < 0.1] *= 30.0
        out.append((r, mv))
    return out


def test_golden_sequence_host_buffers(cuda, built_lib):
    import os
    d = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "taa.npz"))
    w, h = int(d["width"]), int(d["height"])
    t = snkpt.TaaResolve(w, h)
    for f in range(d["radiance"].shape[0]):
        o = t.resolve(d["radiance"][f], d["motion"][f])
        assert np.array_equal(o.view(np.uint32), d["resolved"][f].view(np.uint32)), f


@pytest.mark.parametrize("w,h", [(640, 360), (97, 53), (1, 1), (33, 9)])
def test_device_buffers_match_oracle(cuda, w, h):
    import torch
    rng = np.random.default_rng(w * 1000 + h)
    seq = frames(rng, w, h, 3)
    t = snkpt.TaaResolve(w, h)
    ot = O.OracleTaa(w, h)
    for k, (r, mv) in enumerate(seq):
        rt = torch.from_numpy(r).to(cuda)
        mt = torch.from_numpy(mv).to(cuda)
        inplace = k == 1
        out = t.resolve(rt, mt, out=rt if inplace else None)
        torch.cuda.synchronize()
        g = out.cpu().numpy()
        ref = ot.resolve(r, mv)
        assert np.array_equal(g.view(np.uint32), ref.view(np.uint32)), (w, h, k, float(np.abs(g - ref).max()))


def test_reset_restarts_history(cuda):
    rng = np.random.default_rng(5)
    (r0, m0), (r1, m1) = frames(rng, 48, 32, 2)
    t = snkpt.TaaResolve(48, 32)
    t.resolve(r0, m0)
    t.reset()
    a = t.resolve(r1, m1)
    ot = O.OracleTaa(48, 32)
    b = ot.resolve(r1, m1)
    assert np.array_equal(a.view(np.uint32), b.view(np.uint32))


def test_resolves_path_traced_frames_with_motion(cuda, built_lib):
    """The render pass's radiance and motion outputs feed the resolve directly
    (config 2's camera moving 0.05 units per frame)."""
    sc = scenes.config2(width=160, height=90, frames=4)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    t = snkpt.TaaResolve(160, 90)
    ot = O.OracleTaa(160, 90)
    for f, v in enumerate(sc.views):
        out = snkpt.alloc_outputs(160, 90, device=cuda, names=("radiance", "motion"))
        pt.render([v], abi.settings(spp=1, max_depth=3, seed=f, frame_index=f), [out])
        pt.synchronize()
        res = t.resolve(out["radiance"], out["motion"])
        import torch
        torch.cuda.synchronize()
        ref = ot.resolve(out["radiance"].cpu().numpy(), out["motion"].cpu().numpy())
        assert np.array_equal(res.cpu().numpy().view(np.uint32), ref.view(np.uint32)), f
        if f > 0:
            assert np.abs(out["motion"].cpu().numpy()).max() > 0.0
