"""ctypes declarations of the C-ABI in include/cfem.h.

The library is loaded from the package's in-tree ``_lib/`` folder. There is no
CPU fallback: if the library is missing the import of :func:`lib` raises.
"""
from __future__ import annotations

import ctypes as C
import os

from . import build as _build

LIB_PATH = _build.LIB

# enums (cfem.h)
OK, ERR_INVALID_ARGUMENT, ERR_CUDA, ERR_OUT_OF_MEMORY, ERR_NOT_CONVERGED, ERR_DIVERGED, ERR_MESH, \
    ERR_UNSUPPORTED, ERR_IO = range(9)
COMPAT, CONSISTENT = 0, 1
FP64, FP32, FP32_REFINE = 0, 1, 2
STOP_REFERENCE, STOP_RESIDUAL = 0, 1
FORM_AUTO, FORM_GRADIENT, FORM_STORED_KE, FORM_GRADIENT_FAN, FORM_GEOMETRY_FAN = 0, 1, 2, 3, 4

STATUS_NAMES = {0: "CFEM_OK", 1: "CFEM_ERR_INVALID_ARGUMENT", 2: "CFEM_ERR_CUDA", 3: "CFEM_ERR_OUT_OF_MEMORY",
                4: "CFEM_ERR_NOT_CONVERGED", 5: "CFEM_ERR_DIVERGED", 6: "CFEM_ERR_MESH", 7: "CFEM_ERR_UNSUPPORTED",
                8: "CFEM_ERR_IO"}

i32, i64, f64, vp = C.c_int32, C.c_int64, C.c_double, C.c_void_p


class Mesh(C.Structure):
    _fields_ = [("dim", i32), ("n_nodes", i64), ("nodes", vp), ("n_elems", i64), ("elems", vp),
                ("n_constraints", i64), ("constraints", vp), ("n_loads", i64), ("load_nodes", vp),
                ("load_vectors", vp), ("n_faces", i64), ("face_nodes", vp), ("face_elems", vp),
                ("face_normals", vp), ("face_pressures", vp), ("elem_young", vp)]


class Material(C.Structure):
    _fields_ = [("young_modulus", f64), ("poisson_ratio", f64), ("rho", f64)]


class Options(C.Structure):
    _fields_ = [("semantics", i32), ("matvec_form", i32), ("patch_elems", i32), ("verbose", i32)]


class Wavelet(C.Structure):
    _fields_ = [("type", i32), ("freq", f64), ("timeshift", f64), ("ampl", f64)]


class SolveParams(C.Structure):
    _fields_ = [("precision", i32), ("stop_rule", i32), ("tol", f64), ("max_iter", i32), ("outer_tol", f64),
                ("max_outer", i32)]


class SolveInfo(C.Structure):
    _fields_ = [("status", i32), ("iterations", i32), ("outer_iterations", i32), ("rel_residual", f64),
                ("gamma0", f64), ("gamma", f64), ("solve_ms", f64), ("kernel_launches", i64)]


class DynParams(C.Structure):
    _fields_ = [("beta1", f64), ("beta2", f64), ("dt", f64), ("endtime", f64), ("precision", i32),
                ("pcg_tol", f64), ("stop_rule", i32), ("max_iter", i32), ("warm_start", i32),
                ("n_receivers", i32), ("receiver_nodes", vp), ("receiver_trace", vp)]


class DynInfo(C.Structure):
    _fields_ = [("status", i32), ("steps", i32), ("pcg_iterations", i64), ("solve_ms", f64)]


# (name, restype, argtypes) for every entry point declared in include/cfem.h
SIGNATURES = [
    ("cfem_abi_version", i32, []),
    ("cfem_last_error_string", C.c_char_p, []),
    ("cfem_create", i32, [C.POINTER(vp), C.POINTER(Mesh), C.POINTER(Material), C.POINTER(Options), vp]),
    ("cfem_destroy", None, [vp]),
    ("cfem_set_stream", i32, [vp, vp]),
    ("cfem_selftest_copy_timeout", i32, [vp]),
    ("cfem_synchronize", i32, [vp]),
    ("cfem_get_counts", i32, [vp, vp]),
    ("cfem_dof_map", i32, [vp, vp]),
    ("cfem_adjacency", i32, [vp, vp]),
    ("cfem_bc_mask", i32, [vp, vp]),
    ("cfem_renumbering", i32, [vp, vp, vp]),
    ("cfem_element_matrices", i32, [vp, i64, i64, vp]),
    ("cfem_diagonal", i32, [vp, vp]),
    ("cfem_rhs", i32, [vp, C.POINTER(Wavelet), f64, vp]),
    ("cfem_matvec", i32, [vp, i32, vp, vp]),
    ("cfem_pcg", i32, [vp, C.POINTER(SolveParams), vp, vp, C.POINTER(SolveInfo)]),
    ("cfem_static_solve", i32, [vp, C.POINTER(Wavelet), C.POINTER(SolveParams), vp, C.POINTER(SolveInfo)]),
    ("cfem_dyn", i32, [vp, C.POINTER(DynParams), C.POINTER(Wavelet), vp, C.POINTER(DynInfo)]),
    ("cfem_pcg_multi", i32, [vp, C.POINTER(SolveParams), i32, vp, vp, C.POINTER(SolveInfo)]),
    ("cfem_autotune_patch_elems", i32, [C.POINTER(Mesh), C.POINTER(Material), C.POINTER(Options), vp, i32,
                                        C.POINTER(i32), vp]),
    ("cfem_kfile_read", i32, [C.c_char_p, i32, C.POINTER(vp)]),
    ("cfem_kfile_sizes", i32, [vp, vp, vp, vp, vp, vp]),
    ("cfem_kfile_get", i32, [vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]),
    ("cfem_kfile_free", None, [vp]),
    ("cfem_create_batch", i32, [C.POINTER(vp), i32, C.POINTER(Mesh), C.POINTER(Material), C.POINTER(Options), vp]),
    ("cfem_batch_info", i32, [vp, C.POINTER(i32), vp, vp]),
    ("cfem_batch_static_solve", i32, [vp, C.POINTER(SolveParams), vp, C.POINTER(SolveInfo)]),
    ("cfem_adjoint", i32, [vp, C.POINTER(SolveParams), vp, vp, vp, vp, C.POINTER(SolveInfo)]),
    ("cfem_set_young", i32, [vp, vp]),
    ("cfem_dyn_adjoint", i32, [vp, C.POINTER(DynParams), C.POINTER(Wavelet), i32, vp, vp, C.POINTER(f64), vp,
                                C.POINTER(DynInfo)]),
    ("cfem_element_stress", i32, [vp, vp, vp, vp, vp]),
    ("cfem_profile_matvec", i32, [vp, i32, i32, C.POINTER(f64), C.POINTER(f64)]),
    ("cfem_matvec_energy_noalloc", i32, [vp, vp, vp, vp]),
    ("cfem_run_task", i32, [C.c_char_p, C.c_char_p, i32, vp, i64, C.POINTER(SolveInfo), C.POINTER(DynInfo)]),
    ("cfem_write_vtk", i32, [C.c_char_p, i32, vp, i64, vp, i64, vp]),
]

_lib = None


def lib():
    """Load the library (building it in-tree first if the toolchain is present)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            _build.build()
        L = C.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


class CfemError(RuntimeError):
    def __init__(self, status: int, where: str):
        self.status = status
        msg = lib().cfem_last_error_string().decode(errors="replace")
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {msg}")


def check(status: int, where: str, allow=(OK,)):
    if status not in allow:
        raise CfemError(status, where)
    return status
