"""In-tree build of liblbgpu.so (CUDA kernels + C ABI) for sm_103a.

Every translation unit is compiled by nvcc in parallel into laboetie_gb300/_build/, then linked
into one shared library with the CUDA runtime linked statically.  The FP64 strict units are
compiled with ``-fmad=false`` so that no multiply-add is fused: their results equal the
reference's separately rounded operations.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "liblbgpu.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "--expt-relaxed-constexpr",
          "-Xcompiler", "-fPIC,-ffp-contract=off", "-I", os.path.join(ROOT, "include"), "-I", CSRC]
# translation units whose FP64 arithmetic must match the reference operation for operation
STRICT = {"flow_f64.cu", "mp_f64.cu", "pnp.cu", "ek.cu", "noalloc_moments.cu", "profiles.cu",
          "geometry_build.cu"}


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build liblbgpu")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _stale(obj: str, deps) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(ROOT, "include", "lbgpu.h"))
    cc = nvcc()

    def compile_one(src):
        obj = os.path.join(OUT_DIR, src[:-3] + ".o")
        path = os.path.join(CSRC, src)
        if not _stale(obj, [path] + headers):
            return obj, None
        cmd = [cc, *ARCH, *COMMON, "-c", path, "-o", obj]
        if src in STRICT:
            cmd.insert(1, "-fmad=false")
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            return obj, f"{' '.join(cmd)}\n{r.stdout}\n{r.stderr}"
        if verbose and r.stderr.strip():
            print(r.stderr, file=sys.stderr)
        return obj, None

    srcs = sources()
    with ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        results = list(ex.map(compile_one, srcs))
    errs = [e for _, e in results if e]
    if errs:
        raise RuntimeError("nvcc failed:\n" + "\n".join(errs))
    objs = [o for o, _ in results]
    # objects of translation units that no longer exist: dropped, and the library relinked
    gone = [os.path.join(OUT_DIR, f) for f in os.listdir(OUT_DIR) if f.endswith(".o")]
    gone = [o for o in gone if o not in objs]
    for o in gone:
        os.remove(o)
    if gone or _stale(LIB, objs):
        cmd = [cc, *ARCH, "-shared", "-Xcompiler", "-fPIC", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
