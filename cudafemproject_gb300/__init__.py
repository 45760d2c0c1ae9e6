"""GB300 (sm_103a) element-by-element linear elasticity: CST triangles and
linear tetrahedra, Jacobi-PCG with a matrix-free EbE operator, FP32 + FP64
iterative refinement, GN22 explicit / implicit dynamics, adjoint sensitivities.

A drop-in for the EbE path of moarseniy/CudaFEMproject (femfunc.cpp solver
entry points, run_config keys, prepared-mesh and VTK formats). The compute
path is the in-tree CUDA library ``_lib/libcfem_gb300.so``; there is no CPU
fallback.
"""
from .meshio import Problem, RunConfig, WaveletParams, load_run_config, read_task, write_task  # noqa: F401

__all__ = ["Problem", "RunConfig", "WaveletParams", "load_run_config", "read_task", "write_task", "FemContext",
           "lib"]


def lib():
    from . import capi
    return capi.lib()


def __getattr__(name):
    if name == "FemContext":
        from .solver import FemContext
        return FemContext
    raise AttributeError(name)
