"""CPU tests of the Python side of snk_pt_render_noalloc: the wrapper refuses
output buffers that the library would write through as device memory (host
arrays, CPU tensors, tensors on another device, wrong dtype, non-contiguous or
too small) before any library call is made."""
import numpy as np
import pytest
import torch

import snkpt
from snkpt import abi, scenes


@pytest.fixture
def tracer(monkeypatch):
    """A PathTracer without a library context; any library call fails the test."""
    def no_lib():
        raise AssertionError("the library was called")
    monkeypatch.setattr(snkpt, "lib", no_lib)
    pt = snkpt.PathTracer.__new__(snkpt.PathTracer)
    pt._h = None
    pt.device = 0
    return pt


class FakeCuda:
    """Stands in for a CUDA tensor (this container has no GPU)."""

    def __init__(self, t: torch.Tensor, index=0, contiguous=True):
        self.t, self.is_cuda, self.dtype = t, True, t.dtype
        self.device = torch.device("cuda", index)
        self._contiguous = contiguous

    def is_contiguous(self):
        return self._contiguous

    def numel(self):
        return self.t.numel()

    def data_ptr(self):
        raise AssertionError("a pointer was taken")


def _view(w=16, h=8):
    return scenes.config0(width=w, height=h).views[0]


@pytest.mark.parametrize("bad, what", [
    (lambda n: np.zeros((n, 4), np.float32), "CUDA"),
    (lambda n: torch.zeros((n, 4)), "CUDA"),
    (lambda n: FakeCuda(torch.zeros((n, 4)), index=1), "cuda:1"),
    (lambda n: FakeCuda(torch.zeros((n, 4), dtype=torch.float64)), "dtype"),
    (lambda n: FakeCuda(torch.zeros((n, 4)), contiguous=False), "contiguous"),
    (lambda n: FakeCuda(torch.zeros((n - 1, 4))), "elements"),
])
def test_noalloc_rejects_bad_radiance_buffers(tracer, bad, what):
    n = 16 * 8
    with pytest.raises(ValueError, match=what):
        tracer.render_noalloc(_view(), abi.settings(), {"radiance": bad(n)})


def test_noalloc_rejects_bad_integer_outputs(tracer):
    n = 16 * 8
    with pytest.raises(ValueError, match="dtype"):
        tracer.render_noalloc(_view(), abi.settings(), {"inst_id": FakeCuda(torch.zeros(n, dtype=torch.float32))})
    with pytest.raises(ValueError, match="unknown"):
        tracer.render_noalloc(_view(), abi.settings(), {"colour": FakeCuda(torch.zeros(n))})


def test_noalloc_accepts_well_formed_outputs_up_to_the_library_call(tracer):
    n = 16 * 8
    outs = {"radiance": FakeCuda(torch.zeros((n, 4))), "depth": FakeCuda(torch.zeros(n)),
            "prim_id": FakeCuda(torch.zeros(n, dtype=torch.int32))}
    # validation passes; the next step takes the buffers' pointers
    with pytest.raises(AssertionError, match="pointer"):
        tracer.render_noalloc(_view(), abi.settings(), outs)
