"""GPU assemblers: drop-in replacements of SysmatAssemblerSparseSymm /
SysmatAssemblerSparse and SysvecAssembler (src/AssemblyModule.jl:88-583,
853-917).

Passing ``SysmatAssemblerGPU()`` where a reference caller passes
``SysmatAssemblerSparseSymm()`` switches the form to the device path; the
result is the same SparseMatrixCSC (here a scipy CSC matrix, 1-based arrays
converted to 0-based) or, with ``result="device"``, a handle to the matrix
left on the GPU.  The generic startassembly!/assemble!/makematrix! protocol
is also provided, for element matrices computed by the caller.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np
import scipy.sparse as sp

from . import _native as nat


def _is_assembler(x) -> bool:
    return isinstance(x, (SysmatAssemblerGPU, SysvecAssemblerGPU))


class DeviceMatrix:
    """Assembled matrix resident on the GPU (CSR == CSC: symmetric pattern)."""

    def __init__(self, h, dm, drop_zeros):
        self.h, self.dm, self.drop_zeros = h, dm, drop_zeros
        self.shape = (dm.ndof, dm.ndof)

    def values(self):
        """Values in the structural pattern order (no zero dropping)."""
        v = np.empty(self.dm.nnz)
        nat.check(nat.load().fegpu_matrix_copy_values(self.h, nat.ptr(v)))
        return v

    def spmv(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty_like(x)
        nat.check(nat.load().fegpu_matrix_spmv(self.h, nat.ptr(x), nat.ptr(y)))
        return y

    def __matmul__(self, x):
        return self.spmv(x)

    def cg(self, b, x0, maxiter):
        """conjugategradient(K, b, x0, maxiter) on the device."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x0 = np.ascontiguousarray(x0, dtype=np.float64)
        if b.shape != (self.shape[0],) or x0.shape != (self.shape[0],):
            raise ValueError("Size mismatch")
        x = np.empty_like(b)
        nat.check(nat.load().fegpu_matrix_cg(self.h, nat.ptr(b), nat.ptr(x0), int(maxiter),
                                             nat.ptr(x)))
        return x

    def nnz(self, drop_zeros=None):
        dz = self.drop_zeros if drop_zeros is None else drop_zeros
        n = C.c_int64()
        nat.check(nat.load().fegpu_matrix_nnz(self.h, int(dz), C.byref(n)))
        return n.value

    def to_scipy(self, drop_zeros=None):
        dz = self.drop_zeros if drop_zeros is None else drop_zeros
        nnz = self.nnz(dz)
        colptr = np.empty(self.dm.ndof + 1, dtype=np.int64)
        rowval = np.empty(nnz, dtype=np.int64)
        nzval = np.empty(nnz)
        nat.check(nat.load().fegpu_matrix_copy_csc(self.h, int(dz), nat.ptr(colptr),
                                                   nat.ptr(rowval), nat.ptr(nzval)))
        return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=self.shape)


class SysmatAssemblerGPU:
    """GPU system-matrix assembler.

    symmetric=True reproduces SysmatAssemblerSparseSymm (the default of the
    symmetric forms: exact zeros of S + S' are not stored), symmetric=False
    SysmatAssemblerSparse (structural pattern kept).  precision "fp64" or
    "mixed" (FP32 element arithmetic, FP64 global accumulation).
    """

    def __init__(self, symmetric: bool = True, precision: str = "fp64", result: str = "host",
                 drop_zeros=None, device: int = 0):
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        if result not in ("host", "device"):
            raise ValueError("result must be 'host' or 'device'")
        self.symmetric = symmetric
        self.precision = precision
        self.precision_code = nat.FP64 if precision == "fp64" else nat.MIXED
        self.result = result
        self.drop_zeros = symmetric if drop_zeros is None else bool(drop_zeros)
        self.device = device
        self._generic = None
        self._nomatrixresult = False

    def eltype(self):
        return np.float64

    # ---- device forms --------------------------------------------------------
    def _matrix_for(self, dm):
        key = id(self)
        h = dm.matrices.get(key)
        if h is None:
            out = C.c_void_p()
            nat.check(nat.load().fegpu_matrix_create(dm.h, C.byref(out)))
            h = out.value
            dm.matrices[key] = h
        return h

    def _run(self, dm, call):
        h = self._matrix_for(dm)
        nat.check(call(h))
        M = DeviceMatrix(h, dm, self.drop_zeros)
        return M if self.result == "device" else M.to_scipy()

    # ---- generic protocol (element matrices from the caller) -----------------
    def startassembly(self, elem_mat_nrows, elem_mat_ncols, n_elem_mats, row_nalldofs,
                      col_nalldofs, force_init=False):
        if self.symmetric and elem_mat_nrows != elem_mat_ncols:
            raise ValueError("Symmetric sparse matrix is assumed to be assembled from square "
                             "matrices")
        if self._generic is None:
            out = C.c_void_p()
            nat.check(nat.load().fegpu_assembler_create(nat.context(self.device),
                                                        int(self.symmetric), row_nalldofs,
                                                        col_nalldofs, C.byref(out)))
            self._generic = out.value
            self._shape = (row_nalldofs, col_nalldofs)
            weakref.finalize(self, nat.load().fegpu_assembler_destroy, self._generic)
        return self

    def assemble(self, mat, dofnums_row, dofnums_col):
        if self._generic is None:
            raise RuntimeError("startassembly must be called first")
        m = np.asfortranarray(mat, dtype=np.float64)
        r = np.ascontiguousarray(np.ravel(dofnums_row), dtype=np.int64)
        c = np.ascontiguousarray(np.ravel(dofnums_col), dtype=np.int64)
        if m.shape != (len(r), len(c)):
            raise ValueError("Wrong size of matrix")
        nat.check(nat.load().fegpu_assembler_assemble(self._generic, nat.ptr(m), m.shape[0],
                                                      m.shape[1], nat.ptr(r), nat.ptr(c)))
        return self

    def makematrix(self):
        if self._nomatrixresult:
            return sp.csc_matrix(self._shape)
        nnz = C.c_int64()
        nat.check(nat.load().fegpu_assembler_make(self._generic, C.byref(nnz)))
        colptr = np.empty(self._shape[1] + 1, dtype=np.int64)
        rowval = np.empty(nnz.value, dtype=np.int64)
        nzval = np.empty(nnz.value)
        nat.check(nat.load().fegpu_assembler_copy_csc(self._generic, nat.ptr(colptr),
                                                      nat.ptr(rowval), nat.ptr(nzval)))
        return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=self._shape)


class SysvecAssemblerGPU:
    """GPU system-vector assembler (SysvecAssembler semantics)."""

    def __init__(self, device: int = 0):
        self.device = device

    def _run(self, dm, coef, m):
        F = np.zeros(dm.ndof)
        nat.check(nat.load().fegpu_linform_dot(dm.h, C.byref(coef), m, nat.ptr(F)))
        return F


def conjugategradient(A, b, x0, maxiter):
    """conjugategradient (src/AlgoBaseModule.jl:425-445) for a matrix resident
    on the GPU (a DeviceMatrix: ``SysmatAssemblerGPU(result="device")``)."""
    if not isinstance(A, DeviceMatrix):
        raise TypeError("conjugategradient runs on a DeviceMatrix (assemble with "
                        "SysmatAssemblerGPU(result=\"device\")); there is no CPU path")
    return A.cg(b, x0, maxiter)


def startassembly(a, *args, **kw):
    return a.startassembly(*args, **kw)


def assemble(a, *args):
    return a.assemble(*args)


def makematrix(a):
    return a.makematrix()
