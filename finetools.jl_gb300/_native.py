"""ctypes binding of libfegpu.so (the C ABI declared in include/fegpu.h).

The library is built in-tree by ``build.py``; this module never falls back to
anything else: if the shared object is missing or no GPU is present, the
calls fail with an exception.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
# FEGPU_DEVICE_CHECKS=1 loads the build with device index checks
# (build.py --device-checks)
LIBPATH = os.path.join(HERE, "libfegpu_checked.so" if os.environ.get("FEGPU_DEVICE_CHECKS") == "1"
                       else "libfegpu.so")

OK = 0
Q4, H8, H20, T4, T10 = 0, 1, 2, 3, 4
COEF_CONST, COEF_PER_ELEMENT, COEF_PER_QP, COEF_ISO_LAME = 0, 1, 2, 3
FP64, MIXED, FP64_FAST = 0, 1, 2
FORM_DIFFUSION, FORM_LIN_ELASTIC, FORM_DOT = 0, 1, 2
REQUEST_COEF, REQUEST_COORDS = 0, 1
ASM_SPARSE, ASM_SPARSE_SYMM, ASM_SPARSE_DIAG, ASM_HRZ_LUMPING_SYMM = 0, 1, 2, 3

EXPORTS = [
    "fegpu_last_error", "fegpu_context_create", "fegpu_context_destroy",
    "fegpu_context_synchronize", "fegpu_context_stream", "fegpu_context_timing",
    "fegpu_context_kernel_stats", "fegpu_context_device_checks", "fegpu_selftest_soft_add",
    "fegpu_femm_create", "fegpu_femm_destroy",
    "fegpu_femm_set_geometry", "fegpu_femm_set_axisymmetric", "fegpu_femm_colors", "fegpu_dofmap_create",
    "fegpu_dofmap_destroy", "fegpu_dofmap_copy_pattern", "fegpu_matrix_create",
    "fegpu_matrix_destroy", "fegpu_matrix_set_symmetric_assembly", "fegpu_bilform_diffusion", "fegpu_bilform_lin_elastic",
    "fegpu_bilform_dot", "fegpu_bilform_div_grad", "fegpu_bilform_convection", "fegpu_linform_dot", "fegpu_bilform_dot_lumped", "fegpu_matrix_nnz", "fegpu_matrix_copy_csc",
    "fegpu_matrix_copy_values", "fegpu_matrix_copy_values_async", "fegpu_matrix_wait_export", "fegpu_matrix_copy_block_csc", "fegpu_matrix_spmv",
    "fegpu_matrix_cg", "fegpu_assembler_create",
    "fegpu_assembler_destroy", "fegpu_assembler_assemble", "fegpu_assembler_make",
    "fegpu_assembler_copy_csc", "fegpu_bilform_masslike", "fegpu_bilform_lin_elastic_noalloc",
    "fegpu_batch_create", "fegpu_batch_destroy", "fegpu_batch_add", "fegpu_batch_set_coef",
    "fegpu_batch_tune", "fegpu_batch_tile", "fegpu_batch_set_wait_limit", "fegpu_batch_withhold", "fegpu_batch_launch",
    "fegpu_batch_wait", "fegpu_batch_run", "fegpu_batch_stats",
    "fegpu_server_create", "fegpu_server_destroy", "fegpu_server_set_precision",
    "fegpu_server_set_slice", "fegpu_server_set_memory_limit", "fegpu_server_add_mesh",
    "fegpu_server_remove_mesh", "fegpu_server_mesh_bytes", "fegpu_estimate_mesh_bytes",
    "fegpu_server_submit", "fegpu_server_cancel",
    "fegpu_server_wait", "fegpu_server_drain", "fegpu_server_hold", "fegpu_server_stats",
    "fegpu_server_memory",
]


class Coef(C.Structure):
    _fields_ = [("kind", C.c_int), ("ncomp", C.c_int), ("data", C.c_void_p)]


class FegpuError(RuntimeError):
    """A libfegpu call returned a nonzero status."""


_lib = None


def load(path: str = LIBPATH):
    """Load libfegpu.so and declare the prototypes (no GPU needed)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise FegpuError(f"{path} is missing: build it with finetools.jl_gb300/build.py "
                         "(there is no CPU fallback)")
    L = C.CDLL(path)
    vp, i64, i32, d = C.c_void_p, C.c_int64, C.c_int, C.c_double
    pp = C.POINTER(C.c_void_p)
    p64 = C.POINTER(C.c_int64)
    proto = {
        "fegpu_last_error": ([], C.c_char_p),
        "fegpu_context_create": ([i32, pp], i32),
        "fegpu_context_destroy": ([vp], i32),
        "fegpu_context_synchronize": ([vp], i32),
        "fegpu_context_stream": ([vp, pp], i32),
        "fegpu_context_timing": ([vp, i32], i32),
        "fegpu_context_kernel_stats": ([vp, C.POINTER(C.c_double), p64, i32], i32),
        "fegpu_context_device_checks": ([vp, C.POINTER(C.c_int)], i32),
        "fegpu_selftest_soft_add": ([vp, C.c_int64, C.c_uint64, C.POINTER(C.c_int64),
                                     C.POINTER(C.c_int64)], i32),
        "fegpu_femm_create": ([vp, i32, i64, vp, i64, i32, vp, vp, vp, d, pp], i32),
        "fegpu_femm_destroy": ([vp], i32),
        "fegpu_femm_set_geometry": ([vp, i32, vp], i32),
        "fegpu_femm_set_axisymmetric": ([vp, i32], i32),
        "fegpu_femm_colors": ([vp, vp, p64], i32),
        "fegpu_dofmap_create": ([vp, i32, vp, i64, pp, p64], i32),
        "fegpu_dofmap_destroy": ([vp], i32),
        "fegpu_dofmap_copy_pattern": ([vp, vp, vp], i32),
        "fegpu_matrix_create": ([vp, pp], i32),
        "fegpu_matrix_destroy": ([vp], i32),
        "fegpu_matrix_set_symmetric_assembly": ([vp, i32], i32),
        "fegpu_bilform_diffusion": ([vp, C.POINTER(Coef), i32], i32),
        "fegpu_bilform_lin_elastic": ([vp, C.POINTER(Coef), i32], i32),
        "fegpu_bilform_div_grad": ([vp, C.POINTER(Coef), i32], i32),
        "fegpu_bilform_convection": ([vp, i32, vp], i32),
        "fegpu_bilform_dot": ([vp, C.POINTER(Coef), i32, i32, i32], i32),
        "fegpu_linform_dot": ([vp, C.POINTER(Coef), i32, vp], i32),
        "fegpu_bilform_dot_lumped": ([vp, C.POINTER(Coef), i32, i32, vp], i32),
        "fegpu_matrix_nnz": ([vp, i32, p64], i32),
        "fegpu_matrix_copy_csc": ([vp, i32, vp, vp, vp], i32),
        "fegpu_matrix_copy_values": ([vp, vp], i32),
        "fegpu_matrix_copy_values_async": ([vp, vp], i32),
        "fegpu_matrix_wait_export": ([vp], i32),
        "fegpu_matrix_copy_block_csc": ([vp, i64, i64, i64, i64, i32, p64, vp, vp, vp], i32),
        "fegpu_matrix_spmv": ([vp, vp, vp], i32),
        "fegpu_matrix_cg": ([vp, vp, vp, i32, vp], i32),
        "fegpu_assembler_create": ([vp, i32, i64, i64, pp], i32),
        "fegpu_assembler_destroy": ([vp], i32),
        "fegpu_assembler_assemble": ([vp, vp, i32, i32, vp, vp], i32),
        "fegpu_assembler_make": ([vp, p64], i32),
        "fegpu_assembler_copy_csc": ([vp, vp, vp, vp], i32),
        "fegpu_bilform_masslike": ([vp, C.POINTER(Coef), i32, vp, vp], i32),
        "fegpu_bilform_lin_elastic_noalloc": ([vp, C.POINTER(Coef)], i32),
        "fegpu_batch_create": ([vp, pp], i32),
        "fegpu_batch_destroy": ([vp], i32),
        "fegpu_batch_add": ([vp, vp, i32, C.POINTER(Coef), i32, p64], i32),
        "fegpu_batch_set_coef": ([vp, i64, C.POINTER(Coef)], i32),
        "fegpu_batch_tune": ([vp, C.c_char_p], i32),
        "fegpu_batch_tile": ([vp, i64, C.POINTER(C.c_int)], i32),
        "fegpu_batch_set_wait_limit": ([vp, d], i32),
        "fegpu_batch_withhold": ([vp, i64], i32),
        "fegpu_batch_launch": ([vp], i32),
        "fegpu_batch_wait": ([vp], i32),
        "fegpu_batch_run": ([vp], i32),
        "fegpu_batch_stats": ([vp, p64, p64], i32),
        "fegpu_server_create": ([vp, i32, i32, pp], i32),
        "fegpu_server_destroy": ([vp], i32),
        "fegpu_server_set_precision": ([vp, i32], i32),
        "fegpu_server_set_slice": ([vp, i64], i32),
        "fegpu_server_set_memory_limit": ([vp, i64], i32),
        "fegpu_server_remove_mesh": ([vp, i64], i32),
        "fegpu_server_mesh_bytes": ([vp, i64, p64], i32),
        "fegpu_estimate_mesh_bytes": ([i32, i64, i64, i32, p64], i32),
        "fegpu_server_cancel": ([vp, i64], i32),
        "fegpu_server_add_mesh": ([vp, vp, i32, C.POINTER(Coef), i32, p64], i32),
        "fegpu_server_submit": ([vp, i64, i32, vp, i64, p64], i32),
        "fegpu_server_wait": ([vp, i64, C.POINTER(C.c_double)], i32),
        "fegpu_server_drain": ([vp], i32),
        "fegpu_server_hold": ([vp, i32], i32),
        "fegpu_server_stats": ([vp, p64, p64, p64], i32),
        "fegpu_server_memory": ([vp, p64, p64], i32),
    }
    for name, (args, res) in proto.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def check(status: int):
    if status != OK:
        msg = load().fegpu_last_error().decode()
        raise FegpuError(msg or f"libfegpu status {status}")


def ptr(a) -> int:
    return a.ctypes.data


_contexts: dict[int, int] = {}


def context(device: int = 0) -> int:
    """One library context (CUDA stream) per device, created on first use."""
    if device not in _contexts:
        h = C.c_void_p()
        check(load().fegpu_context_create(device, C.byref(h)))
        _contexts[device] = h.value
    return _contexts[device]
