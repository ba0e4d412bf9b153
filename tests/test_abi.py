"""CPU tests of the C ABI: the library builds, loads, exports every declared
entry point, its structs have the declared layouts, and it fails cleanly
without a GPU (no compute calls)."""
import ctypes as C
import os
import re
import subprocess

import numpy as np
import pytest

import snkpt
from snkpt import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "snk_pt.h")


def declared_functions():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^int\s+(snk_(?:pt|taa|meshdata|cache)_\w+)\s*\(", src, re.M)))


def test_header_declares_entry_points():
    fns = declared_functions()
    assert "snk_pt_render" in fns and "snk_pt_trace_rays" in fns and len(fns) >= 14
    assert set(fns) == set(snkpt.EXPORTS)


def test_library_exports_every_declared_symbol(built_lib):
    L = C.CDLL(built_lib)
    missing = [f for f in declared_functions() if not hasattr(L, f)]
    assert not missing, missing


def test_struct_layouts_match_header(tmp_path):
    prog = tmp_path / "sizes.c"
    prog.write_text('#include "snk_pt.h"\n#include <stdio.h>\n#include <stddef.h>\nint main(void){'
                    'printf("%zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu %zu\\n", sizeof(snk_instance), sizeof(snk_material),'
                    'sizeof(snk_directional_light), sizeof(snk_point_light), sizeof(snk_view), sizeof(snk_render_settings),'
                    'sizeof(snk_ray), sizeof(snk_hit), sizeof(snk_pt_stats), sizeof(snk_view_outputs), sizeof(snk_mesh),'
                    'sizeof(snk_tuning), offsetof(snk_tuning, max_traversal_steps), offsetof(snk_tuning, shadow_variant));'
                    'return 0;}\n')
    exe = tmp_path / "sizes"
    subprocess.check_call(["gcc", "-std=c99", "-I", os.path.dirname(HEADER), str(prog), "-o", str(exe)])
    got = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    expect = [abi.INSTANCE_DTYPE.itemsize, abi.MATERIAL_DTYPE.itemsize, abi.DIR_LIGHT_DTYPE.itemsize,
              abi.POINT_LIGHT_DTYPE.itemsize, abi.VIEW_DTYPE.itemsize, abi.SETTINGS_DTYPE.itemsize,
              abi.RAY_DTYPE.itemsize, abi.HIT_DTYPE.itemsize, abi.STATS_DTYPE.itemsize,
              C.sizeof(snkpt.ViewOutputs), C.sizeof(snkpt.Mesh), C.sizeof(snkpt.Tuning),
              snkpt.Tuning.max_traversal_steps.offset, snkpt.Tuning.shadow_variant.offset]
    assert got == expect


def test_abi_version(built_lib):
    v = C.c_uint32()
    assert snkpt.lib().snk_pt_abi_version(C.byref(v)) == 0
    hdr = open(HEADER).read()
    assert v.value == int(re.search(r"#define\s+SNK_PT_ABI_VERSION\s+(\d+)u", hdr).group(1)) == 2


def test_status_codes_match_header():
    hdr = open(HEADER).read()
    for name in ("OK", "ERR_INVALID_ARG", "ERR_CUDA", "ERR_OUT_OF_MEMORY", "ERR_STATE", "ERR_LIMIT", "ERR_UNSUPPORTED"):
        m = re.search(rf"#define\s+SNK_{name}\s+(\d+)", hdr)
        assert m and int(m.group(1)) == getattr(abi, name), name


def test_null_arguments_are_rejected(built_lib):
    L = snkpt.lib()
    assert L.snk_pt_create(None, None) == abi.ERR_INVALID_ARG
    assert L.snk_pt_destroy(None) == abi.ERR_INVALID_ARG
    assert L.snk_pt_render(None, None, 0, None, None) == abi.ERR_INVALID_ARG
    assert L.snk_pt_trace_rays(None, None, 0, None, 0, 0) == abi.ERR_INVALID_ARG


def test_create_without_gpu_fails_cleanly(built_lib):
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(snkpt.SnkError) as e:
        snkpt.PathTracer(0)
    assert e.value.code == 2   # SNK_ERR_CUDA


def test_settings_defaults_mirror_reference():
    # RT::RtSettings defaults (Core/headers/rendering/Raytracing.h:13-16)
    s = snkpt.RT.RtSettings()
    assert (s.num_temporal_resamples, s.num_spatial_resamples) == (1, 3)
    st = abi.settings(mode=abi.MODE_RESTIR_DI)
    assert int(st["restir_candidates"]) == 32 and int(st["restir_mcap"]) == 20   # RayGen.rgen:95-97
    assert np.dtype(abi.SETTINGS_DTYPE).itemsize == 64
