"""The C-ABI library builds, loads and exports every entry point of include/lbgpu.h.

No compute call is made here: these tests run without a GPU.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from laboetie_gb300 import LbgpuError, Box, library, library_path

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            text = open(os.path.join(ROOT, "include", fn)).read()
            text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
            names |= set(re.findall(r"\b(lbgpu_[a-z0-9_]+)\s*\(", text))
    return sorted(names)


def test_library_builds_and_loads():
    L = library()
    assert os.path.exists(library_path())
    assert L is not None


def test_every_declared_symbol_is_exported():
    L = library()
    names = declared_symbols()
    assert len(names) >= 15
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, f"declared in include/*.h but not exported: {missing}"


def test_default_params_are_the_reference_defaults():
    from laboetie_gb300.lbgpu import Params

    p = Params()
    library().lbgpu_default_params(ctypes.byref(p), 4, 5, 6)
    assert (p.lx, p.ly, p.lz) == (4, 5, 6)
    assert p.relaxation_time == 1.0      # module_collision.f90:38
    assert p.target_error == 1e-10       # equilibration.f90:57
    assert p.rho0 == 1.0                 # init_simu.f90:31
    assert list(p.f_ext) == [0.0, 0.0, 0.0]


def test_invalid_arguments_fail_before_touching_the_gpu():
    nat = np.zeros((4, 4, 4), dtype=np.int8)
    with pytest.raises(LbgpuError) as e:
        Box(nat, relaxation_time=0.4)
    assert "relaxation_time" in str(e.value)
    bad = nat.copy()
    bad[0, 0, 0] = 3
    with pytest.raises(LbgpuError):
        Box(bad)


def test_no_gpu_means_a_loud_failure_not_a_cpu_fallback():
    import subprocess

    has_gpu = subprocess.run(["sh", "-c", "nvidia-smi -L"], capture_output=True).returncode == 0
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(LbgpuError) as e:
        Box(np.zeros((4, 4, 4), dtype=np.int8))
    assert e.value.status & 2  # LBGPU_ERR_CUDA


def test_batch_footprint_and_struct_layout():
    """lbgpu_batch_footprint is host logic, an upper bound over both layouts: populations, flags,
    previous velocity and the nature byte per node, the compact-layout positions, flags and row
    table (256-byte aligned parts), plus the tracer buffers when Db > 0 (V, P twice and the fixed
    (u*, D): four float4 records per node, two more with adsorption)."""
    from laboetie_gb300.lbgpu import Cell, Request, RequestResult, footprint, make_cell

    assert (ctypes.sizeof(Cell), ctypes.sizeof(Request), ctypes.sizeof(RequestResult)) == (144, 200, 88)
    up = lambda x: (x + 255) // 256 * 256
    N = 1 * 50 * 50
    base = up(76 * N) + up(4 * N) + up(16 * N) + up(N) + 2 * up(4 * N) + up(8 * 50 * 50)
    assert footprint(make_cell((1, 50, 50))) == base
    tiles = (N + 255) // 256
    mp = 4 * up(16 * N) + up(8 * (9 * tiles + 1))
    assert footprint(make_cell((1, 50, 50), tracer=dict(Db=0.01))) == base + mp
    ads = footprint(make_cell((1, 50, 50), tracer=dict(Db=0.01, ka=0.02, kd=0.01)))
    assert ads == base + mp + 2 * up(16 * N)
    assert footprint(make_cell((0, 4, 4))) == 0


def test_batch_without_gpu_fails_loudly():
    import subprocess

    from laboetie_gb300.lbgpu import Batch

    has_gpu = subprocess.run(["sh", "-c", "nvidia-smi -L"], capture_output=True).returncode == 0
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(LbgpuError) as e:
        Batch()
    assert e.value.status & 2  # LBGPU_ERR_CUDA
