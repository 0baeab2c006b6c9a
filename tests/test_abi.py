"""CPU checks of the C-ABI library: it loads without a GPU, exports every entry point
include/jbgpu.h declares, its host-side mass properties agree with the oracle, and it
refuses to run without a device instead of falling back to the CPU."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from jbgpu import _abi, scenes

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    txt = open(os.path.join(ROOT, "include", "jbgpu.h")).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"^\s*(?:const\s+)?\w+\**\s+\**(jbgpu_\w+)\s*\(", txt, flags=re.M)))


def test_header_lists_the_entry_points():
    fns = header_functions()
    assert "jbgpu_world_step" in fns and "jbgpu_world_create" in fns
    assert len(fns) >= 20


def test_library_exports_every_declared_symbol(gpu_lib):
    L = C.CDLL(gpu_lib.LIB if hasattr(gpu_lib, "LIB") else gpu_lib._build.LIB)
    missing = [f for f in header_functions() if not hasattr(L, f)]
    assert not missing, missing
    assert set(gpu_lib.EXPORTED) <= set(header_functions())


def test_struct_sizes_match_header(tmp_path):
    # sizes as the C compiler lays the header's structs out, against the ctypes mirror
    src = tmp_path / "sz.c"
    src.write_text('#include <stdio.h>\n#include "jbgpu.h"\nint main(void){printf("%zu %zu %zu %zu %zu %zu %zu\\n",'
                   'sizeof(jbgpu_config),sizeof(jbgpu_shape_desc),sizeof(jbgpu_body_desc),sizeof(jbgpu_state),'
                   'sizeof(jbgpu_manifolds),sizeof(jbgpu_counters),sizeof(jbgpu_ray_hit));return 0;}\n')
    exe = tmp_path / "sz"
    import subprocess
    subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), str(src), "-o", str(exe)])
    sizes = [int(x) for x in subprocess.check_output([str(exe)]).split()]
    mirror = [C.sizeof(t) for t in (_abi.Config, _abi.ShapeDesc, _abi.BodyDesc, _abi.State, _abi.Manifolds, _abi.Counters,
                                    _abi.RayHit)]
    assert sizes == mirror
    assert C.sizeof(_abi.RayHit) == _abi.RAY_HIT_DTYPE.itemsize
    assert C.sizeof(_abi.BodyDesc) == scenes.BODY_DTYPE.itemsize


def test_host_inertia_matches_oracle(gpu_lib, oracle_lib):
    import pyoracle
    rng = np.random.default_rng(3)
    d = rng.standard_normal((32, 3)); d /= np.linalg.norm(d, axis=1, keepdims=True)
    pts = (d * [0.4, 0.9, 0.6]).astype(np.float32)
    for s in [{"type": _abi.SHAPE_BOX, "params": (0.3, 0.45, 0.6, 0), "points": None},
              {"type": _abi.SHAPE_SPHERE, "params": (0.33, 0, 0, 0), "points": None},
              {"type": _abi.SHAPE_CAPSULE, "params": (0.25, 0.9, 0, 0), "points": None},
              {"type": _abi.SHAPE_CONVEX_HULL, "params": (0, 0, 0, 0), "points": pts}]:
        a = gpu_lib.shape_local_inertia(s, 3.7)
        b = pyoracle.shape_local_inertia(s, 3.7)
        assert np.array_equal(a, b), (s["type"], a, b)


def _has_device():
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


@pytest.mark.skipif(_has_device(), reason="checks the no-device error path")
def test_no_device_is_an_error_not_a_fallback(gpu_lib):
    with pytest.raises(gpu_lib.JbgpuError) as e:
        gpu_lib.GpuWorld(scenes.box_stack(2))
    assert e.value.code == _abi.ERR_NO_DEVICE


def test_randomised_order_is_rejected_before_device_use(gpu_lib):
    cfg = _abi.default_config(solver_mode=_abi.SOLVER_CACHE_FRIENDLY | _abi.SOLVER_RANDMIZE_ORDER)
    with pytest.raises(gpu_lib.JbgpuError) as e:
        gpu_lib.GpuWorld(config=cfg)
    assert e.value.code == _abi.ERR_UNSUPPORTED
