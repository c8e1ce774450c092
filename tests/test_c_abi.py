"""include/lbgpu.h compiled by a C compiler, checked against the Fortran host's bind(C) types.

The reference's host is Fortran; it binds the C ABI through iso_c_binding with the derived types
written in INTEGRATION.md.  A C compiler lays out a bind(C) type exactly as the C struct with the
same members in the same order (Fortran 2008 15.3.4): c_int 4 bytes, c_long_long 8, c_double 8,
c_ptr 8, each member at the next multiple of its alignment, arrays as their element, nested
bind(C) types as their own layout.  So the layout of each type is computed here from its Fortran
declaration and compared with what gcc reports for include/lbgpu.h (tests/c_abi/conformance.c),
and with the ctypes mirrors of the Python binding.  The same C program then runs the reference's
C1 flow phase through the C ABI from C: without a GPU it must fail loudly (LBGPU_ERR_CUDA from
lbgpu_create), with one (-m gpu) its l2err history and flux must equal the oracle's bit for bit.
"""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_abi", "conformance.c")
STRUCTS = ["lbgpu_params", "lbgpu_tracer", "lbgpu_pnp_params", "lbgpu_cell", "lbgpu_request",
           "lbgpu_request_result", "lbgpu_batch_tuning"]
KIND = {"c_int": (4, 4), "c_long_long": (8, 8), "c_double": (8, 8), "c_ptr": (8, 8),
        "c_int8_t": (1, 1), "c_size_t": (8, 8), "c_float": (4, 4)}


def fortran_types():
    """{name: [(field, kind, count)]} from the `type, bind(C) :: name` blocks of INTEGRATION.md."""
    text = open(os.path.join(ROOT, "INTEGRATION.md")).read()
    out = {}
    for name, body in re.findall(r"type, bind\(C\) :: (\w+)\n(.*?)\n\s*end type", text, re.S):
        fields = []
        for line in body.splitlines():
            line = line.split("!")[0].strip()
            if not line:
                continue
            m = re.match(r"(integer|real|type)\((\w+)\)\s*::\s*(.*)", line)
            assert m, f"unparsed bind(C) line in {name}: {line!r}"
            kind = m.group(2)
            for item in re.findall(r"(\w+)(?:\((\d+)\))?", m.group(3)):
                fields.append((item[0], kind, int(item[1] or 1)))
        out[name] = fields
    return out


def fortran_layout(types, name, cache=None):
    """(offsets {field: (offset, size)}, sizeof, alignment) under the C interoperability rules."""
    cache = {} if cache is None else cache
    if name in cache:
        return cache[name]
    off, align, fields = 0, 1, {}
    for field, kind, count in types[name]:
        if kind in KIND:
            size, al = KIND[kind]
        else:
            _, size, al = fortran_layout(types, kind, cache)
        off = (off + al - 1) // al * al
        fields[field] = (off, size * count)
        off += size * count
        align = max(align, al)
    res = (fields, (off + align - 1) // align * align, align)
    cache[name] = res
    return res


@pytest.fixture(scope="module")
def conformance_exe(tmp_path_factory):
    from laboetie_gb300 import library, library_path

    library()   # builds liblbgpu.so when it is missing
    gcc = shutil.which("gcc") or shutil.which("cc")
    if not gcc:
        pytest.skip("no C compiler")
    lib_dir = os.path.dirname(library_path())
    exe = str(tmp_path_factory.mktemp("c_abi") / "conformance")
    subprocess.run([gcc, "-std=c11", "-Wall", "-Werror", "-O1", "-I", os.path.join(ROOT, "include"),
                    SRC, "-o", exe, "-L", lib_dir, "-llbgpu", "-Wl,-rpath," + lib_dir],
                   check=True, capture_output=True, text=True)
    return exe


def c_layout(exe):
    out = subprocess.run([exe, "layout"], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.splitlines():
        parts = line.split()
        if parts[1] == "sizeof":
            res.setdefault(parts[0], [{}, 0])[1] = int(parts[2])
        else:
            res.setdefault(parts[0], [{}, 0])[0][parts[1]] = (int(parts[2]), int(parts[3]))
    return res


def test_fortran_bind_c_types_are_all_written_out():
    types = fortran_types()
    assert set(STRUCTS) <= set(types), set(STRUCTS) - set(types)


@pytest.mark.parametrize("name", STRUCTS)
def test_header_layout_equals_the_fortran_bind_c_type(conformance_exe, name):
    types = fortran_types()
    want_fields, want_size, _ = fortran_layout(types, name)
    got_fields, got_size = c_layout(conformance_exe)[name]
    assert list(got_fields) == list(want_fields), "member order differs"
    assert got_fields == want_fields
    assert got_size == want_size


@pytest.mark.parametrize("name,cls", [
    ("lbgpu_params", "Params"), ("lbgpu_tracer", "Tracer"), ("lbgpu_pnp_params", "PnpParams"),
    ("lbgpu_cell", "Cell"), ("lbgpu_request", "Request"), ("lbgpu_request_result", "RequestResult"),
    ("lbgpu_batch_tuning", "BatchTuning")])
def test_python_mirrors_equal_the_header(conformance_exe, name, cls):
    import ctypes

    from laboetie_gb300 import lbgpu

    S = getattr(lbgpu, cls)
    got_fields, got_size = c_layout(conformance_exe)[name]
    assert ctypes.sizeof(S) == got_size
    for field, _ in S._fields_:
        assert getattr(S, field).offset == got_fields[field][0], field
        assert getattr(S, field).size == got_fields[field][1], field


def _has_gpu():
    return subprocess.run(["sh", "-c", "nvidia-smi -L"], capture_output=True).returncode == 0


def test_c_client_without_gpu_fails_loudly(conformance_exe):
    if _has_gpu():
        pytest.skip("a GPU is present")
    r = subprocess.run([conformance_exe, "c1"], capture_output=True, text=True)
    assert r.returncode == 3
    assert r.stderr.startswith("status 2 lbgpu_create")   # LBGPU_ERR_CUDA, no CPU result
    assert "steps" not in r.stdout


@pytest.mark.gpu
def test_c_client_runs_c1_bit_exact(conformance_exe, oracle_mod):
    from laboetie_gb300 import geometry as geo

    r = subprocess.run([conformance_exe, "c1"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.splitlines()
    steps = int(lines[0].split()[1])
    l2 = np.array([float.fromhex(x.split()[2]) for x in lines if x.startswith("l2err")])
    jx = np.array([float.fromhex(x.split()[2]) for x in lines if x.startswith("jx")])
    nat = geo.slit(4, 4, 34)
    ref = oracle_mod.equilibration(nat, tau=1.0, target_error=1e-10, f_ext=(1e-5, 0.0, 0.0))
    assert steps == ref["steps"]
    assert np.array_equal(l2, ref["l2err"])
    assert np.array_equal(jx, ref["j"][0].ravel())
