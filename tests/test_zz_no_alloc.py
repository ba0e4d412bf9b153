"""The allocation-free render entry point (snk_pt_render_noalloc) against the
regular one (snk_pt_render).

snk_pt_render_noalloc exists for callers that must not allocate device memory
while they render -- an engine frame loop that hands out every device byte from
its own allocator, or code where the device-wide synchronisation of
cudaMalloc/cudaFree would stall other work.  It runs the same wavefront kernels
with their scratch in a fixed array inside the library, so its output must match
the regular entry point's within the frame-parity tolerance (1e-4 relative;
G-buffer identical), call after call, even though every call reuses the same
scratch.  This file is collected last on purpose."""
import numpy as np
import pytest

import snkpt
from helpers import max_rel
from snkpt import abi, scenes

pytestmark = pytest.mark.gpu

RTOL = 1e-4
INT_OUT = ("mat_flags", "inst_id", "prim_id")


def _host(outs):
    r = {}
    for k, t in outs.items():
        a = t.cpu().numpy()
        r[k] = a.view(np.uint32) if k in INT_OUT else a
    return r


def _assert_same(a, b, what):
    for k in a:
        if k == "radiance":
            m = max_rel(a[k][:, :3], b[k][:, :3])
            assert m <= RTOL, f"{what}: radiance max relative error {m}"
        else:
            assert np.array_equal(a[k], b[k]), f"{what}: {k} differs"


def test_noalloc_matches_regular_render_on_consecutive_calls(cuda, built_lib):
    W, H = 128, 128
    sc = scenes.config0(width=W, height=H)
    st = abi.settings(spp=2, max_depth=4, rr_depth=3, seed=7)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    ref_out = snkpt.alloc_outputs(W, H, device=cuda)
    pt.render([sc.views[0]], st, [ref_out])
    pt.synchronize()
    ref = _host(ref_out)
    ref_stats = pt.stats()
    outs = [snkpt.alloc_outputs(W, H, device=cuda) for _ in range(3)]
    import torch
    torch.cuda.synchronize()
    free_before = None
    for call in range(3):
        out = outs[call]
        pt.render_noalloc(sc.views[0], st, out)
        pt.synchronize()
        if call == 0:   # the first call may load kernels; later calls must not change free memory
            free_before = torch.cuda.mem_get_info(cuda)[0]
        _assert_same(_host(out), ref, f"no-alloc call {call}")
        s = pt.stats()
        assert (s["rays_camera"], s["rays_extension"], s["rays_shadow"]) == \
               (ref_stats["rays_camera"], ref_stats["rays_extension"], ref_stats["rays_shadow"])
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(cuda)[0] == free_before, "device free memory changed across no-alloc calls"


def test_noalloc_rejects_views_beyond_its_scratch(cuda, built_lib):
    sc = scenes.config0(width=256, height=256)
    pt = snkpt.PathTracer(0)
    pt.load_scene(sc)
    out = snkpt.alloc_outputs(256, 256, device=cuda, names=("radiance",))
    assert 256 * 256 * 2 > snkpt.NOALLOC_MAX_PATHS
    with pytest.raises(snkpt.SnkError) as e:
        pt.render_noalloc(sc.views[0], abi.settings(spp=2), out)
    assert e.value.code == 1 and "65536" in str(e.value)
