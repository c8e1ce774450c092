"""laboetie_gb300 -- GB300-native lattice-Boltzmann hot path for laboetie.

The product is ``liblbgpu.so`` (CUDA kernels for sm_103a behind the C ABI in
``include/lbgpu.h``).  This package builds it in-tree and exposes a thin ctypes mirror of the
reference's Fortran interfaces (``collide``, the bounce-back/stream block and moments of
``equilibration.f90``, ``equilibration`` itself, the tracer moment propagation and the
Poisson/Nernst-Planck routines).  There is no CPU fallback: if the library or a GPU is missing,
every call raises.
"""
from .lbgpu import (  # noqa: F401
    LbgpuError,
    Box,
    Params,
    Tracer,
    PnpParams,
    FP64,
    FP32_DEV,
    FP64_FUSED,
    library,
    library_path,
)

__all__ = ["LbgpuError", "Box", "Params", "Tracer", "PnpParams", "FP64", "FP32_DEV", "FP64_FUSED",
           "library",
           "library_path"]
