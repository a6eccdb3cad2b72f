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
import itertools
import weakref

import numpy as np
import scipy.sparse as sp

from . import _native as nat


# per-assembler keys of the device matrices a DOF map holds (an object's id
# can be reused once it is freed, which would hand a new assembler the matrix
# of an earlier device result)
_assembler_serial = itertools.count()


def _is_assembler(x) -> bool:
    return isinstance(x, (SysmatAssemblerGPU, SysmatAssemblerFFBlockGPU, SysvecAssemblerGPU,
                          SysvecAssemblerFBlockGPU))


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

    def block(self, rows, cols, drop_zeros=None):
        """CSC (scipy) of the block rows x cols (0-based ranges) of the matrix;
        exact zeros left out as the assembler's result does (drop_zeros)."""
        dz = int(self.drop_zeros if drop_zeros is None else drop_zeros)
        r0, r1 = rows
        c0, c1 = cols
        L = nat.load()
        nnz = C.c_int64()
        nat.check(L.fegpu_matrix_copy_block_csc(self.h, r0, r1, c0, c1, dz, C.byref(nnz), None,
                                                None, None))
        colptr = np.empty(c1 - c0 + 1, dtype=np.int64)
        rowval = np.empty(nnz.value, dtype=np.int64)
        nzval = np.empty(nnz.value)
        nat.check(L.fegpu_matrix_copy_block_csc(self.h, r0, r1, c0, c1, dz, C.byref(nnz),
                                                nat.ptr(colptr), nat.ptr(rowval), nat.ptr(nzval)))
        return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(r1 - r0, c1 - c0))

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
    SysmatAssemblerSparse (structural pattern kept).  precision "fp64" (the
    reference's operation order: bilform_diffusion and bilform_lin_elastic
    return the reference algorithm's matrix bit for bit), "fp64_fast" (FP64
    with fused multiply-adds: within 1e-12 |K_ij| + 1e-14 max_k |K_ik|) or
    "mixed" (FP32 element arithmetic, FP64 global accumulation).  lumping
    "diag" / "hrz" reproduces SysmatAssemblerSparseDiag /
    SysmatAssemblerSparseHRZLumpingSymm (diagonal results; bilform_dot and the
    generic protocol).
    """

    def __init__(self, symmetric: bool = True, precision: str = "fp64", result: str = "host",
                 drop_zeros=None, device: int = 0, lumping=None):
        if precision not in ("fp64", "fp64_fast", "mixed"):
            raise ValueError("precision must be 'fp64', 'fp64_fast' or 'mixed'")
        if lumping not in (None, "diag", "hrz"):
            raise ValueError("lumping must be None, 'diag' or 'hrz'")
        self.lumping = lumping
        if result not in ("host", "device"):
            raise ValueError("result must be 'host' or 'device'")
        self.symmetric = symmetric
        self.precision = precision
        self.precision_code = {"fp64": nat.FP64, "fp64_fast": nat.FP64_FAST,
                               "mixed": nat.MIXED}[precision]
        self.result = result
        self.drop_zeros = symmetric if drop_zeros is None else bool(drop_zeros)
        self.device = device
        self._generic = None
        self._generic_kind = None
        self._generic_fin = None
        self._shape = None
        self._nomatrixresult = False
        self._key = ("assembler", next(_assembler_serial))

    def eltype(self):
        return np.float64

    def _post(self, A):
        """The result handed to the caller (the wrapping FF-block assembler
        cuts its block out)."""
        return A

    # ---- device forms --------------------------------------------------------
    def _matrix_for(self, dm):
        """The device matrix this assembler fills on the DOF map dm: one per
        (assembler, DOF map), so a device result stays valid until the same
        assembler assembles again on the same DOF map."""
        key = self._key
        h = dm.matrices.get(key)
        if h is None:
            out = C.c_void_p()
            nat.check(nat.load().fegpu_matrix_create(dm.h, C.byref(out)))
            h = out.value
            dm.matrices[key] = h
        nat.check(nat.load().fegpu_matrix_set_symmetric_assembly(h, int(bool(self.symmetric))))
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
        kind = {None: nat.ASM_SPARSE_SYMM if self.symmetric else nat.ASM_SPARSE,
                "diag": nat.ASM_SPARSE_DIAG, "hrz": nat.ASM_HRZ_LUMPING_SYMM}[self.lumping]
        self._open_generic(kind, row_nalldofs, col_nalldofs)
        return self

    def _open_generic(self, kind, nrows, ncols):
        """A fresh device COO assembler of this kind and size: startassembly!
        restarts the buffers, dropping triples assembled before."""
        if self._generic_fin is not None:
            self._generic_fin()
        out = C.c_void_p()
        nat.check(nat.load().fegpu_assembler_create(nat.context(self.device), kind,
                                                    int(nrows), int(ncols), C.byref(out)))
        self._generic = out.value
        self._generic_kind = kind
        self._shape = (int(nrows), int(ncols))
        self._generic_fin = weakref.finalize(self, nat.load().fegpu_assembler_destroy,
                                             self._generic)
        return self._generic

    def _generic_csc(self, nnz):
        """Copy the made matrix of the device COO assembler out as scipy CSC."""
        colptr = np.empty(self._shape[1] + 1, dtype=np.int64)
        rowval = np.empty(nnz, dtype=np.int64)
        nzval = np.empty(nnz)
        nat.check(nat.load().fegpu_assembler_copy_csc(self._generic, nat.ptr(colptr),
                                                      nat.ptr(rowval), nat.ptr(nzval)))
        return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=self._shape)

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
        return self._generic_csc(nnz.value)


class SysmatAssemblerFFBlockGPU:
    """SysmatAssemblerFFBlock (src/AssemblyModule.jl:1144-1236): the assembly
    is delegated to a wrapped GPU assembler (by default
    SysmatAssemblerGPU(symmetric=False), the reference's
    SysmatAssemblerSparse) and the result is its free-free block
    (matrix_blocked_ff: rows 1..row_nfreedofs, columns 1..col_nfreedofs),
    cut out on the device for the device forms.  The result is a scipy CSC
    matrix."""

    def __init__(self, row_nfreedofs, col_nfreedofs=None, a=None, device: int = 0):
        if isinstance(row_nfreedofs, SysmatAssemblerGPU):
            # SysmatAssemblerFFBlock(a, row_nfreedofs, col_nfreedofs)
            a, row_nfreedofs, col_nfreedofs = row_nfreedofs, col_nfreedofs, a
        self._a = a if a is not None else SysmatAssemblerGPU(symmetric=False, device=device)
        self._row_nfreedofs = int(row_nfreedofs)
        self._col_nfreedofs = int(row_nfreedofs if col_nfreedofs is None else col_nfreedofs)

    # the wrapped assembler's settings
    symmetric = property(lambda self: self._a.symmetric)
    precision = property(lambda self: self._a.precision)
    precision_code = property(lambda self: self._a.precision_code)
    lumping = property(lambda self: self._a.lumping)
    drop_zeros = property(lambda self: self._a.drop_zeros)

    def eltype(self):
        return self._a.eltype()

    def _post(self, A):
        return _blocked(A, "ff", self._row_nfreedofs, self._col_nfreedofs)

    def _run(self, dm, call):
        h = self._a._matrix_for(dm)
        nat.check(call(h))
        return self._post(DeviceMatrix(h, dm, self._a.drop_zeros))

    def startassembly(self, *args, **kw):
        self._a.startassembly(*args, **kw)
        return self

    def assemble(self, mat, dofnums_row, dofnums_col):
        self._a.assemble(mat, dofnums_row, dofnums_col)
        return self

    def makematrix(self):
        return self._post(self._a.makematrix())


def SysmatAssemblerSparseDiagGPU(device: int = 0):
    """SysmatAssemblerSparseDiag on the GPU (src/AssemblyModule.jl:599-794)."""
    return SysmatAssemblerGPU(symmetric=True, lumping="diag", device=device)


def SysmatAssemblerSparseHRZLumpingSymmGPU(device: int = 0):
    """SysmatAssemblerSparseHRZLumpingSymm on the GPU (src/AssemblyModule.jl:943-1145)."""
    return SysmatAssemblerGPU(symmetric=True, lumping="hrz", device=device)


class SysvecAssemblerGPU:
    """GPU system-vector assembler (SysvecAssembler semantics,
    src/AssemblyModule.jl:853-917).  linform_dot / distribloads run on the
    device; the generic protocol (startassembly / assemble / makevector) takes
    element vectors from the caller and sums them on the device, each entry in
    assembly order, through the generic COO assembler with one column."""

    def __init__(self, device: int = 0):
        self.device = device
        self._generic = None
        self._fin = None
        self._n = 0

    def eltype(self):
        return np.float64

    def _run(self, dm, coef, m):
        F = np.zeros(dm.ndof)
        nat.check(nat.load().fegpu_linform_dot(dm.h, C.byref(coef), m, nat.ptr(F)))
        return self._post(F)

    def _post(self, F):
        return F

    def startassembly(self, row_nalldofs):
        if self._fin is not None:
            self._fin()
        out = C.c_void_p()
        nat.check(nat.load().fegpu_assembler_create(nat.context(self.device), nat.ASM_SPARSE,
                                                    int(row_nalldofs), 1, C.byref(out)))
        self._generic = out.value
        self._n = int(row_nalldofs)
        self._fin = weakref.finalize(self, nat.load().fegpu_assembler_destroy, self._generic)
        return self

    def assemble(self, vec, dofnums):
        if self._generic is None:
            raise RuntimeError("startassembly must be called first")
        v = np.ascontiguousarray(np.ravel(vec), dtype=np.float64)
        r = np.ascontiguousarray(np.ravel(dofnums), dtype=np.int64)
        if len(v) != len(r):
            raise ValueError("Size mismatch")
        one = np.ones(1, dtype=np.int64)
        nat.check(nat.load().fegpu_assembler_assemble(self._generic, nat.ptr(v), len(r), 1,
                                                      nat.ptr(r), nat.ptr(one)))
        return self

    def makevector(self):
        nnz = C.c_int64()
        nat.check(nat.load().fegpu_assembler_make(self._generic, C.byref(nnz)))
        colptr = np.empty(2, dtype=np.int64)
        rowval = np.empty(nnz.value, dtype=np.int64)
        nzval = np.empty(nnz.value)
        nat.check(nat.load().fegpu_assembler_copy_csc(self._generic, nat.ptr(colptr),
                                                      nat.ptr(rowval), nat.ptr(nzval)))
        F = np.zeros(self._n)
        F[rowval - 1] = nzval
        return self._post(F)


class SysvecAssemblerFBlockGPU:
    """SysvecAssemblerFBlock (src/AssemblyModule.jl:1238-1284): the vector
    assembly of the wrapped GPU assembler, cut to the free DOFs
    (vector_blocked_f)."""

    def __init__(self, row_nfreedofs, a=None, device: int = 0):
        self._a = a if a is not None else SysvecAssemblerGPU(device=device)
        self._row_nfreedofs = int(row_nfreedofs)

    def eltype(self):
        return self._a.eltype()

    def _post(self, F):
        return vector_blocked_f(F, self._row_nfreedofs)

    def _run(self, dm, coef, m):
        return self._post(self._a._run(dm, coef, m))

    def startassembly(self, row_nalldofs):
        self._a.startassembly(row_nalldofs)
        return self

    def assemble(self, vec, dofnums):
        self._a.assemble(vec, dofnums)
        return self

    def makevector(self):
        return self._post(self._a.makevector())


def vector_blocked_f(V, nfreedofs):
    """vector_blocked_f (src/MatrixUtilityModule.jl:807-830): the free part."""
    V = np.asarray(V)
    if nfreedofs > V.shape[0]:
        raise ValueError("The f block has too many rows")
    return V[:nfreedofs].copy()


def vector_blocked_d(V, nfreedofs):
    """vector_blocked_d (src/MatrixUtilityModule.jl:832-855): the data part."""
    V = np.asarray(V)
    if nfreedofs > V.shape[0]:
        raise ValueError("The f block has too many rows")
    return V[nfreedofs:].copy()


def _blocked(A, which, row_nfreedofs, col_nfreedofs):
    """One of the four blocks of A: on the device for a DeviceMatrix, else
    by slicing the (scipy) matrix as the reference slices its
    SparseMatrixCSC (stored entries kept)."""
    col_nfreedofs = row_nfreedofs if col_nfreedofs is None else col_nfreedofs
    n, m = A.shape
    if row_nfreedofs > n:
        raise ValueError("The ff block has too many rows")
    if col_nfreedofs > m:
        raise ValueError("The ff block has too many columns")
    rows = (0, row_nfreedofs) if which[0] == "f" else (row_nfreedofs, n)
    cols = (0, col_nfreedofs) if which[1] == "f" else (col_nfreedofs, m)
    if isinstance(A, DeviceMatrix):
        return A.block(rows, cols)
    if not sp.issparse(A):
        raise TypeError("blocked extraction takes a DeviceMatrix or a scipy sparse matrix")
    return sp.csc_matrix(A)[rows[0]:rows[1], cols[0]:cols[1]]


def matrix_blocked_ff(A, row_nfreedofs, col_nfreedofs=None):
    """matrix_blocked_ff (src/MatrixUtilityModule.jl:675-688): the free-free block."""
    return _blocked(A, "ff", row_nfreedofs, col_nfreedofs)


def matrix_blocked_fd(A, row_nfreedofs, col_nfreedofs=None):
    """matrix_blocked_fd (src/MatrixUtilityModule.jl:708-723)."""
    return _blocked(A, "fd", row_nfreedofs, col_nfreedofs)


def matrix_blocked_df(A, row_nfreedofs, col_nfreedofs=None):
    """matrix_blocked_df (src/MatrixUtilityModule.jl:743-758)."""
    return _blocked(A, "df", row_nfreedofs, col_nfreedofs)


def matrix_blocked_dd(A, row_nfreedofs, col_nfreedofs=None):
    """matrix_blocked_dd (src/MatrixUtilityModule.jl:778-793)."""
    return _blocked(A, "dd", row_nfreedofs, col_nfreedofs)


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


def makevector(a):
    return a.makevector()
