"""FEMMBase and the bilinear / linear forms, executed by libfegpu on the GPU.

Mirror of the reference's interface (src/FEMMBaseModule.jl):

    femm = FEMMBase(IntegDomain(fes, GaussRule(3, 2)))
    K = bilform_diffusion(femm, geom, u, DataCache(1.0))            # 4 args
    K = bilform_diffusion(femm, SysmatAssemblerGPU(), geom, u, cf)  # 5 args
    K = bilform_lin_elastic(femm, geom, u, DeforModelRed3D, DataCache(D))
    G = bilform_dot(femm, geom, u, DataCache(c), m=3)
    F = linform_dot(femm, geom, P, DataCache(f), m)
    F = distribloads(femm, geom, P, ForceIntensity(f), m)

As in the reference, the short forms use the symmetric assembler
(SysmatAssemblerSparseSymm semantics) and return a SparseMatrixCSC-like
scipy CSC matrix; the element computation and the assembly run in the
hand-written CUDA kernels of libfegpu.  There is no CPU path.
"""
from __future__ import annotations

import ctypes as C
import weakref

import numpy as np
import scipy.sparse as sp

from . import _native as nat
from .assembly import SysmatAssemblerGPU, SysvecAssemblerGPU, _is_assembler
from .fields import NodalField


class DeforModelRed3D:
    """Model reduction marker for 3-D elasticity (src/DeforModelRedModule.jl:64)."""

    nstressstrain = 6


class DataCache:
    """Coefficient supplier (src/DataCacheModule.jl:65-112).

    DataCache(data) is constant; DataCache(data, fill) calls
    fill(cache, XYZ, tangents, feid, qpid) -> value at every quadrature
    point (evaluated on the host over all points, then uploaded: slow, but
    with the reference's semantics).
    """

    def __init__(self, data, fill=None):
        self._cache = np.array(data, dtype=np.float64) if not callable(data) else data
        self._fill = fill

    def __call__(self, XYZ, tangents, feid, qpid):
        if self._fill is not None:
            self._cache = self._fill(self._cache, XYZ, tangents, feid, qpid)
        return self._cache

    def size(self):
        return np.shape(self._cache)


class ElementwiseData(DataCache):
    """Per-element coefficient: row e of `values` is the coefficient of
    element e (what a DataCache whose fill indexes by feid returns)."""

    def __init__(self, values):
        v = np.asarray(values, dtype=np.float64)
        self.values = v.reshape(v.shape[0], -1)
        super().__init__(self.values[0].reshape(v.shape[1:]) if v.ndim > 1 else v[0])

    def __call__(self, XYZ, tangents, feid, qpid):
        return self.values[feid - 1].reshape(np.shape(self._cache))


class IsotropicElementwise(DataCache):
    """Per-element isotropic elasticity given by Young's modulus and Poisson
    ratio; evaluates to the 6x6 Voigt D of element feid."""

    def __init__(self, E, nu):
        from .meshes import lame
        self.E = np.asarray(E, dtype=np.float64)
        self.nu = np.asarray(nu, dtype=np.float64)
        lam, mu = lame(self.E, self.nu)
        self.lame = np.ascontiguousarray(np.stack([lam, mu], axis=1))
        super().__init__(np.zeros((6, 6)))

    def __call__(self, XYZ, tangents, feid, qpid):
        from .meshes import isotropic_D
        return isotropic_D(self.E[feid - 1], self.nu[feid - 1])


class ForceIntensity:
    """Distributed load intensity (src/ForceIntensityModule.jl:34-89)."""

    def __init__(self, magn):
        if isinstance(magn, DataCache):
            self._cache = magn
        else:
            self._cache = DataCache(np.atleast_1d(np.asarray(magn, dtype=np.float64)))


class IntegDomain:
    """Element set + integration rule + other dimension, or an axisymmetric
    domain (src/IntegDomainModule.jl:43-143): a two-manifold measured as a
    volume is scaled by the constant other dimension or by 2 pi r.  Only
    constant other dimensions are supported on the GPU."""

    def __init__(self, fes, integration_rule, otherdimension=1.0, axisymmetric=False):
        if callable(otherdimension):
            raise NotImplementedError("the GPU path supports a constant other dimension")
        if isinstance(otherdimension, bool):  # IntegDomain(fes, rule, axisymmetric)
            otherdimension, axisymmetric = 1.0, otherdimension
        self.axisymmetric = bool(axisymmetric)
        self.fes = fes
        self.integration_rule = integration_rule
        self.otherdimension = float(otherdimension)

    def integrationdata(self):
        """npts, Ns (npts x nne), gradNparams (npts x nne x mdim), w, pc
        (src/IntegDomainModule.jl:610-648)."""
        r = self.integration_rule
        pc = r.param_coords
        Ns = np.stack([self.fes.bfun(p).ravel() for p in pc])
        dN = np.stack([self.fes.bfundpar(p) for p in pc])
        return r.npts, Ns, dN, r.weights, pc


class CSys:
    """Material coordinate system (src/CSysModule.jl:17-110): CSys(dim) is the
    identity; CSys(R) a constant rotation matrix R (columns: the material
    axes in global coordinates), as csmat returns it.  A frame that varies
    over the mesh (the reference's update function) is not taken by the
    device forms: evaluate the rotated coefficient per point with a
    DataCache fill function instead."""

    def __init__(self, spec):
        if callable(spec):
            raise NotImplementedError("a material frame that varies over the mesh: supply the "
                                      "rotated coefficient per point (DataCache with a fill)")
        if np.isscalar(spec):
            self.csmat = np.eye(int(spec))
        else:
            self.csmat = np.array(spec, dtype=np.float64)
            if self.csmat.ndim != 2 or self.csmat.shape[0] != self.csmat.shape[1]:
                raise ValueError("CSys: a square rotation matrix")
        self.isidentity = bool(np.array_equal(self.csmat, np.eye(self.csmat.shape[0])))


def _strain_rotation(R):
    """T with (local Voigt strain) = T (global Voigt strain), engineering
    shears, order xx, yy, zz, xy, xz, yz: the strain that blmat! forms with
    the gradients in the material frame and Rm (src/DeforModelRedModule.jl:
    447-472) is R' eps R."""
    T = np.zeros((6, 6))
    for k in range(6):
        e = np.zeros(6)
        e[k] = 1.0
        eps = np.array([[e[0], e[3] / 2, e[4] / 2], [e[3] / 2, e[1], e[5] / 2],
                        [e[4] / 2, e[5] / 2, e[2]]])
        loc = R.T @ eps @ R
        T[:, k] = [loc[0, 0], loc[1, 1], loc[2, 2], 2 * loc[0, 1], 2 * loc[0, 2], 2 * loc[1, 2]]
    return T


def _is_isotropic_D(D):
    """The 6 x 6 D of an isotropic material (invariant under rotation)."""
    D = np.asarray(D).reshape(6, 6)
    lam, mu = D[0, 1], D[3, 3]
    iso = np.zeros((6, 6))
    iso[:3, :3] = lam
    iso[np.arange(3), np.arange(3)] = lam + 2 * mu
    iso[np.arange(3, 6), np.arange(3, 6)] = mu
    return bool(np.array_equal(D, iso))


def _in_material_frame(femm, coef, keep, what):
    """A coefficient given in the material frame of femm.mcsys, expressed in
    global coordinates: K = sum B_l' D B_l with B_l = T B (elasticity: D ->
    T' D T) and gradients g_l = g R (diffusion: kappa -> R kappa R').  The
    identity frame, scalar conductivities and isotropic materials pass
    unchanged."""
    cs = femm.mcsys
    if cs is None or cs.isidentity:
        return coef
    R = cs.csmat
    v = keep[-1]
    n = coef.ncomp
    if what == "diffusion" and n == R.shape[0] ** 2:
        rows = v.reshape(-1, n)
        out = np.stack([(R @ r.reshape(R.shape) @ R.T).ravel() for r in rows])
    elif what == "elasticity" and n == 36:
        rows = v.reshape(-1, 36)
        if all(_is_isotropic_D(r) for r in rows):
            return coef
        T = _strain_rotation(R)
        out = np.stack([(T.T @ r.reshape(6, 6) @ T).ravel() for r in rows])
    else:
        return coef
    out = np.ascontiguousarray(out.reshape(v.shape))
    keep.append(out)
    return nat.Coef(coef.kind, n, nat.ptr(out))


class FEMMBase:
    """Finite-element machine (src/FEMMBaseModule.jl:72-93): the integration
    domain and the material frame (identity by default, or a constant
    CSys).  Holds the device-resident element set (connectivity, colouring,
    integration tables) once built."""

    def __init__(self, integdomain: IntegDomain, mcsys: CSys = None, device: int = 0):
        self.integdomain = integdomain
        self.mcsys = mcsys
        self.device = device
        self._h = None
        self._dofmaps = {}
        self._geom_key = None

    def finite_elements(self):
        return self.integdomain.fes

    # ---- native handles --------------------------------------------------
    def _handle(self):
        if self._h is None:
            L = nat.load()
            ctx = nat.context(self.device)
            fes = self.integdomain.fes
            npts, Ns, dN, w, _ = self.integdomain.integrationdata()
            Ns = np.ascontiguousarray(Ns, dtype=np.float64)
            dN = np.ascontiguousarray(dN, dtype=np.float64)
            w = np.ascontiguousarray(w, dtype=np.float64)
            conn = np.ascontiguousarray(fes.conn, dtype=np.int64)
            h = C.c_void_p()
            nnodes = int(conn.max()) if conn.size else 1
            nnodes = max(nnodes, getattr(self, "_nnodes_hint", 0))
            nat.check(L.fegpu_femm_create(ctx, fes.code, conn.shape[0], nat.ptr(conn), nnodes,
                                          npts, nat.ptr(Ns), nat.ptr(dN), nat.ptr(w),
                                          self.integdomain.otherdimension, C.byref(h)))
            self._h = h.value
            self._nnodes = nnodes
            weakref.finalize(self, _destroy, "fegpu_femm_destroy", self._h, self._dofmaps)
            if self.integdomain.axisymmetric:
                nat.check(L.fegpu_femm_set_axisymmetric(self._h, 1))
        return self._h

    def _ensure_nodes(self, nnodes):
        if self._h is not None and nnodes != self._nnodes:
            raise ValueError("the number of nodes of the geometry changed")
        self._nnodes_hint = nnodes

    def set_geometry(self, geom: NodalField):
        self._ensure_nodes(geom.values.shape[0])
        h = self._handle()
        xyz = np.asfortranarray(geom.values, dtype=np.float64)
        nat.check(nat.load().fegpu_femm_set_geometry(h, xyz.shape[1], nat.ptr(xyz)))

    def dofmap(self, u: NodalField):
        self._ensure_nodes(u.dofnums.shape[0])
        h = self._handle()
        dn = np.asfortranarray(u.dofnums, dtype=np.int64)
        key = (dn.shape, dn.tobytes(), u.nalldofs())
        dm = self._dofmaps.get(key)
        if dm is None:
            out = C.c_void_p()
            nnz = C.c_int64()
            nat.check(nat.load().fegpu_dofmap_create(h, dn.shape[1], nat.ptr(dn), u.nalldofs(),
                                                     C.byref(out), C.byref(nnz)))
            dm = _DofMap(out.value, nnz.value, u.nalldofs(), dn.shape[1])
            self._dofmaps[key] = dm
        return dm

    def colors(self):
        h = self._handle()
        n = self.integdomain.fes.count()
        col = np.zeros(n, dtype=np.int64)
        nc = C.c_int64()
        nat.check(nat.load().fegpu_femm_colors(h, nat.ptr(col), C.byref(nc)))
        return col, nc.value


class _DofMap:
    def __init__(self, h, nnz, ndof, ndn):
        self.h, self.nnz, self.ndof, self.ndn = h, nnz, ndof, ndn
        self.matrices = {}

    def pattern(self):
        colptr = np.zeros(self.ndof + 1, dtype=np.int64)
        rowval = np.zeros(self.nnz, dtype=np.int64)
        nat.check(nat.load().fegpu_dofmap_copy_pattern(self.h, nat.ptr(colptr), nat.ptr(rowval)))
        return colptr, rowval


def _destroy(fn, h, dofmaps):
    try:
        L = nat.load()
        for dm in dofmaps.values():
            for m in dm.matrices.values():
                L.fegpu_matrix_destroy(m)
            L.fegpu_dofmap_destroy(dm.h)
        getattr(L, fn)(h)
    except Exception:
        pass


# ---------------------------------------------------------------------------
# coefficient marshalling
def _qp_values(femm: FEMMBase, geom: NodalField, cf: DataCache, ncomp: int):
    """Evaluate a callable DataCache at every (element, point): loc and J
    computed as locjac! does (src/MatrixUtilityModule.jl:60-68)."""
    fes = femm.integdomain.fes
    npts, Ns, dN, w, _ = femm.integdomain.integrationdata()
    X = geom.values[fes.conn - 1]                       # E x nne x sdim
    loc = np.einsum("qk,eks->eqs", Ns, X)
    J = np.einsum("eks,qkm->eqsm", X, dN)
    out = np.empty((fes.count(), npts, ncomp))
    for e in range(fes.count()):
        for q in range(npts):
            out[e, q] = np.ravel(cf(loc[e, q][None, :], J[e, q], e + 1, q + 1))
    return out


def _coef(femm, geom, cf, keep):
    """DataCache -> fegpu_coef."""
    if isinstance(cf, IsotropicElementwise):
        keep.append(cf.lame)
        return nat.Coef(nat.COEF_ISO_LAME, 2, nat.ptr(cf.lame))
    if isinstance(cf, ElementwiseData):
        v = np.ascontiguousarray(cf.values)
        keep.append(v)
        return nat.Coef(nat.COEF_PER_ELEMENT, v.shape[1], nat.ptr(v))
    if cf._fill is not None:
        ncomp = int(np.prod(cf.size())) if cf.size() else 1
        v = np.ascontiguousarray(_qp_values(femm, geom, cf, ncomp))
        keep.append(v)
        return nat.Coef(nat.COEF_PER_QP, ncomp, nat.ptr(v))
    v = np.ascontiguousarray(np.asarray(cf._cache, dtype=np.float64).ravel())
    keep.append(v)
    return nat.Coef(nat.COEF_CONST, v.size, nat.ptr(v))


def _split(args, n_plain):
    """(assembler, rest) for the 4/5-argument forms of the reference."""
    if len(args) > 0 and _is_assembler(args[0]):
        return args[0], args[1:]
    if len(args) != n_plain:
        raise TypeError("wrong number of arguments")
    return None, args


def _prepare(femm: FEMMBase, geom: NodalField, u: NodalField):
    femm.set_geometry(geom)
    return femm.dofmap(u)


# ---------------------------------------------------------------------------
# the forms
def bilform_diffusion(femm: FEMMBase, *args):
    """K = int grad(w) . c . grad(u) dV (src/FEMMBaseModule.jl:1462-1545)."""
    assembler, (geom, u, cf) = _split(args, 3)
    assembler = assembler or SysmatAssemblerGPU()
    dm = _prepare(femm, geom, u)
    keep = []
    coef = _in_material_frame(femm, _coef(femm, geom, cf, keep), keep, "diffusion")
    return assembler._run(dm, lambda h: nat.load().fegpu_bilform_diffusion(
        h, C.byref(coef), assembler.precision_code))


def bilform_lin_elastic(femm: FEMMBase, *args):
    """K = int (B w)' D (B u) dV (src/FEMMBaseModule.jl:1774-1824)."""
    assembler, (geom, u, mr, cf) = _split(args, 4)
    if mr is not DeforModelRed3D:
        raise NotImplementedError("only DeforModelRed3D is supported")
    assembler = assembler or SysmatAssemblerGPU()
    dm = _prepare(femm, geom, u)
    keep = []
    coef = _in_material_frame(femm, _coef(femm, geom, cf, keep), keep, "elasticity")
    return assembler._run(dm, lambda h: nat.load().fegpu_bilform_lin_elastic(
        h, C.byref(coef), assembler.precision_code))


def bilform_dot(femm: FEMMBase, *args, m=3):
    """K = int w . c . u dV (src/FEMMBaseModule.jl:1335-1376)."""
    assembler, (geom, u, cf) = _split(args, 3)
    assembler = assembler or SysmatAssemblerGPU()
    dm = _prepare(femm, geom, u)
    keep = []
    coef = _coef(femm, geom, cf, keep)
    if getattr(assembler, "lumping", None):
        # SysmatAssemblerSparseDiag / HRZLumpingSymm: a diagonal matrix on the
        # DOFs of the element set (explicit zeros kept, as sparse() does)
        diag = np.empty(dm.ndof)
        nat.check(nat.load().fegpu_bilform_dot_lumped(
            dm.h, C.byref(coef), int(m), int(assembler.lumping == "hrz"), nat.ptr(diag)))
        conn = femm.integdomain.fes.conn - 1
        dofs = np.unique(u.dofnums[np.unique(conn)].ravel()) - 1
        return assembler._post(sp.csc_matrix((diag[dofs], (dofs, dofs)),
                                             shape=(dm.ndof, dm.ndof)))
    return assembler._run(dm, lambda h: nat.load().fegpu_bilform_dot(
        h, C.byref(coef), int(m), int(assembler.symmetric), assembler.precision_code))


def bilform_convection(femm: FEMMBase, *args):
    """K = int w u . grad(q) dV for a scalar field (src/FEMMBaseModule.jl:1583-1625):
    bilform_convection(femm, [assembler], geom, u, Q, rhof) with u the velocity
    NodalField; the reference's default assembler is SysmatAssemblerSparse
    (unsymmetric), and rhof does not enter the reference's matrix."""
    assembler, (geom, u, Q, rhof) = _split(args, 4)
    assembler = assembler or SysmatAssemblerGPU(symmetric=False)
    if assembler.symmetric:
        raise ValueError("convection: the element matrix is unsymmetric "
                         "(use SysmatAssemblerGPU(symmetric=False))")
    dm = _prepare(femm, geom, Q)
    vel = np.asfortranarray(u.values, dtype=np.float64)
    return assembler._run(dm, lambda h: nat.load().fegpu_bilform_convection(
        h, vel.shape[1], vel.ctypes.data))


def bilform_div_grad(femm: FEMMBase, *args):
    """K = int mu grad(w) : grad(u) dV (src/FEMMBaseModule.jl:1672-1723); the
    reference's default assembler is SysmatAssemblerSparse (unsymmetric)."""
    assembler, (geom, u, viscf) = _split(args, 3)
    assembler = assembler or SysmatAssemblerGPU(symmetric=False)
    dm = _prepare(femm, geom, u)
    keep = []
    coef = _coef(femm, geom, viscf, keep)
    return assembler._run(dm, lambda h: nat.load().fegpu_bilform_div_grad(
        h, C.byref(coef), assembler.precision_code))


def bilform_masslike(femm: FEMMBase, *args, m=3):
    """Rectangular "mass-like" matrix (src/FEMMBaseModule.jl:1865-1927):
    bilform_masslike(femm, [assembler], geom, phi, cf; m=3) with nelem*ndn
    rows (rows (i-1)*ndn+1 .. i*ndn belong to element i) and nalldofs(phi)
    columns, M[(i-1)*ndn+p, dof(b,q)] = int N_b c[p,q].  The reference's
    default assembler is SysmatAssemblerSparse: only an unsymmetric,
    unlumped GPU assembler applies (the matrix is not square)."""
    assembler, (geom, phi, cf) = _split(args, 3)
    assembler = assembler or SysmatAssemblerGPU(symmetric=False)
    inner = getattr(assembler, "_a", assembler)  # an FF-block assembler's wrapped one
    if inner.symmetric or inner.lumping:
        raise ValueError("masslike: the matrix is rectangular "
                         "(use SysmatAssemblerGPU(symmetric=False))")
    dm = _prepare(femm, geom, phi)
    keep = []
    coef = _coef(femm, geom, cf, keep)
    if coef.kind == nat.COEF_ISO_LAME:
        raise ValueError("masslike: the coefficient is a scalar or an ndn x ndn matrix")
    nelem = femm.integdomain.fes.count()
    inner._open_generic(nat.ASM_SPARSE, nelem * dm.ndn, dm.ndof)
    nnz = C.c_int64()
    nat.check(nat.load().fegpu_bilform_masslike(dm.h, C.byref(coef), int(m),
                                                inner._generic, C.byref(nnz)))
    return assembler._post(inner._generic_csc(nnz.value))


def innerproduct(femm: FEMMBase, *args):
    """Gram matrix: bilform_dot with the identity (src/FEMMBaseModule.jl:1388-1410)."""
    assembler, (geom, afield) = _split(args, 2)
    cf = DataCache(np.eye(afield.ndofs()))
    if assembler is None:
        return bilform_dot(femm, geom, afield, cf)
    return bilform_dot(femm, assembler, geom, afield, cf)


def linform_dot(femm: FEMMBase, *args):
    """F = int N f dV (src/FEMMBaseModule.jl:1207-1255)."""
    assembler, (geom, P, f, m) = _split(args, 4)
    assembler = assembler or SysvecAssemblerGPU()
    dm = _prepare(femm, geom, P)
    keep = []
    coef = _coef(femm, geom, f, keep)
    return assembler._run(dm, coef, int(m))


def distribloads(femm: FEMMBase, *args):
    """Distributed loads through linform_dot (src/FEMMBaseModule.jl:1277-1297)."""
    assembler, (geom, P, fi, m) = _split(args, 4)
    if assembler is None:
        return linform_dot(femm, geom, P, fi._cache, m)
    return linform_dot(femm, assembler, geom, P, fi._cache, m)


def connectionmatrix(femm: FEMMBase, nnodes: int):
    """Node-to-node connection pattern (src/FEMMBaseModule.jl:490-510), built
    on the device from a one-DOF-per-node numbering."""
    import scipy.sparse as sp
    femm._ensure_nodes(nnodes)
    u = NodalField(np.zeros((nnodes, 1)))
    from .fields import numberdofs
    numberdofs(u)
    dm = femm.dofmap(u)
    colptr, rowval = dm.pattern()
    return sp.csc_matrix((np.ones(len(rowval), dtype=np.int64), rowval - 1, colptr - 1),
                         shape=(nnodes, nnodes))
