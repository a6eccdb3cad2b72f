"""ctypes front end of the CPU oracle (``oracle/fe_oracle.c``).

TEST INFRASTRUCTURE ONLY.  The oracle is a serial C restatement of the
FinEtools.jl assembly path; it is the checker for the GPU library and the
timed CPU baseline.  Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU
baseline legs of ``bench.py`` import this module.  The product package never
does.

All node and DOF numbers are 1-based, as in the reference.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np
import scipy.sparse as sp

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_build", "libfe_oracle.so")

Q4, H8, H20, T4, T10 = 0, 1, 2, 3, 4
L2 = 5  # oracle-only two-node line (runs the reference's 1-D known-answer tests)
DIFFUSION, LIN_ELASTIC, DOT, DIV_GRAD = 0, 1, 2, 3
COEF_CONST, COEF_PER_ELEMENT, COEF_PER_QP = 0, 1, 2
ASM_SPARSE, ASM_SPARSE_SYMM, ASM_DIAG, ASM_HRZ = 0, 1, 2, 3
NNE = {Q4: 4, H8: 8, H20: 20, T4: 4, T10: 10}
MDIM = {Q4: 2, H8: 3, H20: 3, T4: 3, T10: 3}

_lib = None


def build() -> str:
    """Compile the oracle with its Makefile (gcc, seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIBPATH


class _Problem(C.Structure):
    _fields_ = [
        ("etype", C.c_int), ("nelem", C.c_int64), ("conn", C.c_void_p),
        ("nnodes", C.c_int64), ("sdim", C.c_int), ("xyz", C.c_void_p),
        ("ndn", C.c_int), ("dofnums", C.c_void_p), ("nalldofs", C.c_int64),
        ("npts", C.c_int), ("pc", C.c_void_p), ("w", C.c_void_p),
        ("otherdim", C.c_double), ("rm", C.c_void_p), ("axisymmetric", C.c_int),
        ("Ns", C.c_void_p), ("dNs", C.c_void_p),
    ]


class _Coef(C.Structure):
    _fields_ = [("kind", C.c_int), ("ncomp", C.c_int), ("data", C.c_void_p)]


def lib():
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH) or os.path.getmtime(LIBPATH) < os.path.getmtime(
        os.path.join(HERE, "fe_oracle.c")
    ):
        build()
    L = C.CDLL(LIBPATH)
    vp, i64, i32, d = C.c_void_p, C.c_int64, C.c_int, C.c_double
    L.orc_gauss_rule.argtypes = [i32, i32, vp, vp]
    L.orc_tet_rule.argtypes = [i32, vp, vp]
    L.orc_bfun.argtypes = [i32, vp, vp]
    L.orc_bfundpar.argtypes = [i32, vp, vp]
    L.orc_linearspace.argtypes = [d, d, i64, vp]
    L.orc_h8blockx.argtypes = [vp, i64, vp, i64, vp, i64, vp, vp]
    L.orc_t4blockx.argtypes = [vp, i64, vp, i64, vp, i64, vp, vp]
    L.orc_q4blockx.argtypes = [vp, i64, vp, i64, vp, vp]
    L.orc_quadratic_upgrade.argtypes = [i32, i64, vp, i64, vp, vp, vp]
    L.orc_quadratic_upgrade.restype = i64
    L.orc_element_coloring.argtypes = [i64, i32, vp, i64, vp]
    L.orc_element_coloring.restype = i64
    L.orc_connection_degrees.argtypes = [i64, i32, vp, i64, vp]
    L.orc_connection_degrees.restype = i64
    L.orc_matrix_nnz.argtypes = [vp]
    L.orc_matrix_nnz.restype = i64
    L.orc_matrix_nrows.argtypes = [vp]
    L.orc_matrix_nrows.restype = i64
    L.orc_matrix_ncols.argtypes = [vp]
    L.orc_matrix_ncols.restype = i64
    L.orc_matrix_zeros_dropped.argtypes = [vp]
    L.orc_matrix_zeros_dropped.restype = i64
    L.orc_matrix_copy.argtypes = [vp, vp, vp, vp]
    L.orc_matrix_free.argtypes = [vp]
    L.orc_assembler_create.argtypes = [i32, i64, i64]
    L.orc_assembler_create.restype = vp
    L.orc_assembler_assemble.argtypes = [vp, vp, i32, i32, vp, vp]
    L.orc_assembler_make.argtypes = [vp]
    L.orc_assembler_make.restype = vp
    L.orc_assembler_free.argtypes = [vp]
    L.orc_bilform.argtypes = [C.POINTER(_Problem), i32, C.POINTER(_Coef), i32, i32, vp]
    L.orc_bilform.restype = vp
    L.orc_linform_dot.argtypes = [C.POINTER(_Problem), C.POINTER(_Coef), i32, vp]
    L.orc_bilform_convection.argtypes = [C.POINTER(_Problem), vp, i32]
    L.orc_bilform_convection.restype = vp
    L.orc_bilform_masslike.argtypes = [C.POINTER(_Problem), C.POINTER(_Coef), i32]
    L.orc_bilform_masslike.restype = vp
    L.orc_last_error.restype = C.c_char_p
    _lib = L
    return L


def _p(a):
    return a.ctypes.data


def _err():
    return lib().orc_last_error().decode()


# ---------------------------------------------------------------- rules
def gauss_rule(dim, order):
    pc = np.zeros((order**dim, dim))
    w = np.zeros(order**dim)
    n = lib().orc_gauss_rule(dim, order, _p(pc), _p(w))
    if n < 0:
        raise ValueError(_err())
    return pc, w


def tet_rule(npts):
    pc = np.zeros((npts, 3))
    w = np.zeros(npts)
    if lib().orc_tet_rule(npts, _p(pc), _p(w)) < 0:
        raise ValueError(_err())
    return pc, w


def bfun(etype, pc):
    pc = np.ascontiguousarray(pc, dtype=np.float64)
    N = np.zeros(NNE[etype])
    lib().orc_bfun(etype, _p(pc), _p(N))
    return N


def bfundpar(etype, pc):
    pc = np.ascontiguousarray(pc, dtype=np.float64)
    d = np.zeros((NNE[etype], MDIM[etype]))
    lib().orc_bfundpar(etype, _p(pc), _p(d))
    return d


# ---------------------------------------------------------------- meshes
def linearspace(a, b, n):
    out = np.zeros(n)
    lib().orc_linearspace(float(a), float(b), int(n), _p(out))
    return out


def h8blockx(xs, ys, zs):
    xs, ys, zs = (np.ascontiguousarray(v, dtype=np.float64) for v in (xs, ys, zs))
    nn = len(xs) * len(ys) * len(zs)
    ne = (len(xs) - 1) * (len(ys) - 1) * (len(zs) - 1)
    xyz = np.zeros((nn, 3))
    conn = np.zeros((ne, 8), dtype=np.int64)
    lib().orc_h8blockx(_p(xs), len(xs), _p(ys), len(ys), _p(zs), len(zs), _p(xyz), _p(conn))
    return xyz, conn


def t4blockx(xs, ys, zs):
    xs, ys, zs = (np.ascontiguousarray(v, dtype=np.float64) for v in (xs, ys, zs))
    nn = len(xs) * len(ys) * len(zs)
    ne = 6 * (len(xs) - 1) * (len(ys) - 1) * (len(zs) - 1)
    xyz = np.zeros((nn, 3))
    conn = np.zeros((ne, 4), dtype=np.int64)
    lib().orc_t4blockx(_p(xs), len(xs), _p(ys), len(ys), _p(zs), len(zs), _p(xyz), _p(conn))
    return xyz, conn


def q4blockx(xs, ys):
    xs, ys = (np.ascontiguousarray(v, dtype=np.float64) for v in (xs, ys))
    nn = len(xs) * len(ys)
    ne = (len(xs) - 1) * (len(ys) - 1)
    xyz = np.zeros((nn, 2))
    conn = np.zeros((ne, 4), dtype=np.int64)
    lib().orc_q4blockx(_p(xs), len(xs), _p(ys), len(ys), _p(xyz), _p(conn))
    return xyz, conn


def quadratic_upgrade(etype_from, xyz, conn):
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    ne = 12 if etype_from == H8 else 6
    nv = conn.shape[1]
    cap = xyz.shape[0] + conn.shape[0] * ne
    xo = np.zeros((cap, 3))
    co = np.zeros((conn.shape[0], nv + ne), dtype=np.int64)
    n = lib().orc_quadratic_upgrade(etype_from, conn.shape[0], _p(conn), xyz.shape[0],
                                    _p(xyz), _p(xo), _p(co))
    return xo[:n].copy(), co


def block(etype, L, W, H, nL, nW, nH):
    """H8block/H20block/T4block/T10block on [0,L]x[0,W]x[0,H]."""
    xs, ys, zs = linearspace(0, L, nL + 1), linearspace(0, W, nW + 1), linearspace(0, H, nH + 1)
    if etype in (H8, H20):
        xyz, conn = h8blockx(xs, ys, zs)
        if etype == H20:
            xyz, conn = quadratic_upgrade(H8, xyz, conn)
    else:
        xyz, conn = t4blockx(xs, ys, zs)
        if etype == T10:
            xyz, conn = quadratic_upgrade(T4, xyz, conn)
    return xyz, conn


def element_coloring(conn, nnodes):
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    colors = np.zeros(conn.shape[0], dtype=np.int64)
    nc = lib().orc_element_coloring(conn.shape[0], conn.shape[1], _p(conn), nnodes, _p(colors))
    return colors, int(nc)


def connection_degrees(conn, nnodes):
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    deg = np.zeros(nnodes, dtype=np.int64)
    lib().orc_connection_degrees(conn.shape[0], conn.shape[1], _p(conn), nnodes, _p(deg))
    return deg


# ---------------------------------------------------------------- matrices
def _take_matrix(h):
    L = lib()
    if not h:
        raise RuntimeError(_err())
    nr = L.orc_matrix_nrows(h)
    n = L.orc_matrix_ncols(h)
    nnz = L.orc_matrix_nnz(h)
    colptr = np.zeros(n + 1, dtype=np.int64)
    rowval = np.zeros(nnz, dtype=np.int64)
    nzval = np.zeros(nnz)
    L.orc_matrix_copy(h, _p(colptr), _p(rowval), _p(nzval))
    dropped = L.orc_matrix_zeros_dropped(h)
    L.orc_matrix_free(h)
    K = sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(nr, n))
    return K, int(dropped)


class Assembler:
    """SysmatAssemblerSparse / SysmatAssemblerSparseSymm / SysmatAssemblerSparseDiag
    / SysmatAssemblerSparseHRZLumpingSymm restated (kind overrides symmetric)."""

    def __init__(self, symmetric, nrows, ncols, kind=None):
        k = kind if kind is not None else (ASM_SPARSE_SYMM if symmetric else ASM_SPARSE)
        self.h = lib().orc_assembler_create(k, nrows, ncols)
        if not self.h:
            raise ValueError(_err())
        self.zeros_dropped = 0

    def assemble(self, mat, rows, cols):
        mat = np.ascontiguousarray(mat, dtype=np.float64)
        r = np.ascontiguousarray(np.ravel(rows), dtype=np.int64)
        c = np.ascontiguousarray(np.ravel(cols), dtype=np.int64)
        if lib().orc_assembler_assemble(self.h, _p(mat), mat.shape[0], mat.shape[1],
                                        _p(r), _p(c)) != 0:
            raise ValueError(_err())

    def make(self):
        K, self.zeros_dropped = _take_matrix(lib().orc_assembler_make(self.h))
        return K

    def __del__(self):
        if getattr(self, "h", None):
            lib().orc_assembler_free(self.h)
            self.h = None


def _problem(etype, conn, xyz, dofnums, nalldofs, pc, w, otherdim, keep, rm=None,
             axisymmetric=False, tables=None):
    conn = np.ascontiguousarray(conn, dtype=np.int64)
    xyz = np.ascontiguousarray(xyz, dtype=np.float64)
    dofnums = np.ascontiguousarray(dofnums, dtype=np.int64)
    if dofnums.ndim == 1:
        dofnums = dofnums.reshape(-1, 1)
    pc = np.ascontiguousarray(pc, dtype=np.float64)
    w = np.ascontiguousarray(w, dtype=np.float64)
    keep += [conn, xyz, dofnums, pc, w]
    rmp = None
    if rm is not None:
        rm = np.ascontiguousarray(rm, dtype=np.float64).reshape(3, 3)
        keep.append(rm)
        rmp = _p(rm)
    nsp = dnp = None
    if tables is not None:
        Ns = np.ascontiguousarray(tables[0], dtype=np.float64)
        dN = np.ascontiguousarray(tables[1], dtype=np.float64)
        if Ns.size != len(w) * NNE.get(etype, 2) or dN.size != Ns.size * MDIM.get(etype, 1):
            raise ValueError("tables: npts x nne and npts x nne x mdim expected")
        keep += [Ns, dN]
        nsp, dnp = _p(Ns), _p(dN)
    return _Problem(etype, conn.shape[0], _p(conn), xyz.shape[0], xyz.shape[1], _p(xyz),
                    dofnums.shape[1], _p(dofnums), int(nalldofs), len(w), _p(pc), _p(w),
                    float(otherdim), rmp, int(bool(axisymmetric)), nsp, dnp)


def _coef(kind, data, keep):
    data = np.ascontiguousarray(data, dtype=np.float64)
    keep.append(data)
    if kind == COEF_CONST:
        ncomp = data.size
    elif kind == COEF_PER_ELEMENT:
        ncomp = data.shape[1] if data.ndim > 1 else 1
        ncomp = int(np.prod(data.shape[1:])) if data.ndim > 1 else 1
    else:
        ncomp = int(np.prod(data.shape[2:])) if data.ndim > 2 else 1
    return _Coef(kind, ncomp, _p(data))


def bilform(form, etype, conn, xyz, dofnums, nalldofs, pc, w, coef, coef_kind=COEF_CONST,
            otherdim=1.0, m=3, symmetric=True, phases=False, asm=None, rm=None,
            axisymmetric=False, tables=None):
    """One bilinear form, assembled like the reference's 4/5-argument call.

    tables = (Ns, dN): the integrationdata() basis tables the caller hands
    over (as the GPU library receives them); None computes them here.
    Returns the scipy CSC matrix (and, optionally, the number of exact zeros
    dropped by the symmetric completion and the phase timings).
    """
    keep = []
    P = _problem(etype, conn, xyz, dofnums, nalldofs, pc, w, otherdim, keep, rm, axisymmetric,
                 tables)
    Cf = _coef(coef_kind, coef, keep)
    ph = np.zeros(3)
    kind = asm if asm is not None else (ASM_SPARSE_SYMM if symmetric else ASM_SPARSE)
    h = lib().orc_bilform(C.byref(P), form, C.byref(Cf), m, kind, _p(ph))
    K, dropped = _take_matrix(h)
    if phases:
        return K, dropped, ph
    return K


def bilform_convection(etype, conn, xyz, dofnums, nalldofs, pc, w, velocity, otherdim=1.0,
                       axisymmetric=False):
    """bilform_convection (scalar field) with SysmatAssemblerSparse; velocity
    nnodes x nsd."""
    keep = []
    P = _problem(etype, conn, xyz, dofnums, nalldofs, pc, w, otherdim, keep,
                 axisymmetric=axisymmetric)
    v = np.ascontiguousarray(velocity, dtype=np.float64)
    h = lib().orc_bilform_convection(C.byref(P), _p(v), v.shape[1])
    K, _ = _take_matrix(h)
    return K


def bilform_masslike(etype, conn, xyz, dofnums, nalldofs, pc, w, coef, coef_kind=COEF_CONST,
                     otherdim=1.0, m=3, axisymmetric=False):
    """bilform_masslike with SysmatAssemblerSparse: the nelem*ndn x nalldofs
    matrix whose rows (i-1)*ndn+1 .. i*ndn belong to element i; coef ndn x ndn
    (constant, per element or per quadrature point)."""
    keep = []
    P = _problem(etype, conn, xyz, dofnums, nalldofs, pc, w, otherdim, keep,
                 axisymmetric=axisymmetric)
    Cf = _coef(coef_kind, coef, keep)
    K, _ = _take_matrix(lib().orc_bilform_masslike(C.byref(P), C.byref(Cf), m))
    return K


def linform_dot(etype, conn, xyz, dofnums, nalldofs, pc, w, force, coef_kind=COEF_CONST,
                otherdim=1.0, m=3, axisymmetric=False):
    keep = []
    P = _problem(etype, conn, xyz, dofnums, nalldofs, pc, w, otherdim, keep,
                 axisymmetric=axisymmetric)
    Cf = _coef(coef_kind, force, keep)
    F = np.zeros(int(nalldofs))
    if lib().orc_linform_dot(C.byref(P), C.byref(Cf), m, _p(F)) != 0:
        raise ValueError(_err())
    return F


def conjugategradient(A, b, x0, maxiter):
    """conjugategradient (src/AlgoBaseModule.jl:425-445), restated in numpy:
    the same iteration (two products with A per step); A any matrix numpy or
    scipy can multiply."""
    x = np.array(x0, dtype=np.float64, copy=True)
    gt = A @ x - b                          # transpose of the gradient
    d = gt.copy()
    for _ in range(maxiter):
        Ad = A @ d
        rho = float(d @ Ad)
        alpha = -float(gt @ d) / rho
        x += alpha * d
        gt = A @ x - b
        beta = float(gt @ Ad) / rho
        d = beta * d - gt
    return x
