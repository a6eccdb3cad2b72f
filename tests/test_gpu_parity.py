"""GPU parity: libfegpu (through its C ABI) against the CPU oracle.

Bar of the reference-order FP64 path (precision "fp64", the default) for
bilform_diffusion and bilform_lin_elastic: the matrix equals the oracle's bit
for bit -- structure, values and the exact zeros S + S' leaves out.
Bar of the other FP64 paths ("fp64_fast" and the remaining forms): the CSR
structure is bit-exact; every value satisfies
    |K_ij - Kref_ij| <= 1e-12 |Kref_ij| + 1e-14 max_k |Kref_ik|
and |(K - Kref) x| <= 1e-12 |Kref x|.  The absolute term covers entries
formed by cancellation (mathematically zero or nearly so, e.g. vertex /
opposite mid-edge couplings of straight-edged T10 under an exact rule): any
change of summation order, the reference's own LoopVectorization reordering
included, moves them by a few ulps of the row scale.  Structure is compared
on the structural pattern (SysmatAssemblerSparse semantics, zeros kept);
the symmetric assembler's dropping of exact zeros depends on bitwise values
and is checked on fully perturbed meshes, where no exact zeros arise.
Mixed precision: normwise 1e-6.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


def mixed_gate(K32, K64, tol=MIXED_TOL, seed=5):
    """The mixed-precision error gate against FP64, per nonzero and normwise:
        max_ij |dK_ij| / max_k |K_ik| <= tol   (the row's scale)
        |dK x| / |K x| <= tol                  (x uniform in [-1, 1])
    A raw per-entry relative bound cannot hold in FP32 for entries formed by
    cancellation (near zero in FP64: an FP32 rounding of the row's terms is
    larger than the entry); the row scale is what such an entry's accuracy
    is measured against.  Returns (row-scaled, normwise)."""
    A = K64.tocsr()
    B = K32.tocsr()
    rows = np.abs(A).max(axis=1).toarray().ravel()
    D = (B - A).tocsr()
    D.data = np.abs(D.data)
    dr = D.max(axis=1).toarray().ravel()
    nz = rows > 0
    row = float((dr[nz] / rows[nz]).max()) if nz.any() else 0.0
    assert np.all(dr[~nz] == 0)
    x = np.random.default_rng(seed).uniform(-1, 1, A.shape[1])
    kx = float(np.linalg.norm((B - A) @ x) / np.linalg.norm(A @ x))
    assert row <= tol, f"row-scaled per-nonzero error {row:.3e} > {tol:g}"
    assert kx <= tol, f"|dK x| / |K x| = {kx:.3e} > {tol:g}"
    return row, kx


def _rowmax(K):
    """max |K_ij| per row (0 for an empty row)."""
    R = K.tocsr()
    out = np.zeros(R.shape[0])
    full = np.diff(R.indptr) > 0
    if R.nnz:
        out[full] = np.maximum.reduceat(np.abs(R.data), R.indptr[:-1][full])
    return out


RTOL = 1e-12
ATOL_ROW = 1e-14


def bitwise(K, Kr):
    """The GPU matrix equals the oracle's bit for bit (structure and values)."""
    K = K.tocsc()
    R = Kr.tocsc()
    K.sort_indices()
    R.sort_indices()
    assert np.array_equal(K.indptr, R.indptr), "column pointers differ from the oracle's"
    assert np.array_equal(K.indices, R.indices), "row indices differ from the oracle's"
    diff = np.flatnonzero(K.data.view(np.int64) != R.data.view(np.int64))
    assert diff.size == 0, (f"{diff.size} values differ from the oracle's bitwise "
                            f"(first: {K.data[diff[0]]!r} vs {R.data[diff[0]]!r})")


def compare(K, Kr, tol=RTOL, structure=True, atol_row=ATOL_ROW):
    """Returns (max raw relative error, max |dK| / (rtol |K| + atol row scale), |dK x|/|K x|)."""
    K = K.tocsr()
    K.sort_indices()
    R = Kr.tocsr()
    R.sort_indices()
    same = np.array_equal(K.indptr, R.indptr) and np.array_equal(K.indices, R.indices)
    if structure:
        assert same, "CSR structure differs from the oracle's"
    rm = np.repeat(_rowmax(R), np.diff(R.indptr))
    if same:
        diff = np.abs(K.data - R.data)
    else:
        A = (K - R).tocsr()
        diff = np.abs(np.asarray(A[R.nonzero()]).ravel())
        off = abs(A) - abs(A).multiply(R != 0)
        if off.nnz:
            rmax = _rowmax(R)
            offr = off.tocsr()
            for i in range(offr.shape[0]):
                row = offr.data[offr.indptr[i]:offr.indptr[i + 1]]
                if row.size:
                    assert row.max() <= atol_row * rmax[i], "entry outside the oracle pattern"
    raw = float((diff / np.maximum(np.abs(R.data), 1e-300)).max()) if diff.size else 0.0
    gate = float((diff / (tol * np.abs(R.data) + atol_row * rm)).max()) if diff.size else 0.0
    x = np.random.default_rng(7).uniform(-1, 1, K.shape[1])
    kx = np.linalg.norm((K - R) @ x) / max(np.linalg.norm(R @ x), 1e-300)
    assert gate <= 1.0, f"value error {gate:.3g} x the bound (raw relative {raw:.3e})"
    assert kx <= tol, f"relative |dK x| {kx:.3e}"
    return raw, gate, kx


def _oracle_form(O, femm, form, geom, u, coef, kind=0, m=3, symmetric=True):
    """The oracle's form on the same inputs the GPU library receives,
    integrationdata() tables included."""
    fes = femm.integdomain.fes
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    return O.bilform(form, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc, w, coef,
                     coef_kind=kind, otherdim=femm.integdomain.otherdimension, m=m,
                     symmetric=symmetric, tables=(Ns, dN))


def _field(ft, n, ndn):
    return ft.numberdofs(ft.NodalField(np.zeros((n, ndn))))


# ---------------------------------------------------------------- diffusion
@pytest.mark.parametrize("et,n,rule", [("H8", 4, ("G", 3, 2)), ("H20", 3, ("G", 3, 3)),
                                       ("T4", 3, ("T", 1)), ("T10", 3, ("T", 4)),
                                       ("H8", 3, ("G", 3, 3)), ("T10", 2, ("T", 5))])
@pytest.mark.parametrize("coef", ["iso", "general", "per_element", "per_point",
                                  "per_point_general"])
@pytest.mark.parametrize("prec", ["fp64", "fp64_fast"])
def test_diffusion_fp64(ft, O, et, n, rule, coef, prec):
    gen = {"H8": ft.H8block, "H20": ft.H20block, "T4": ft.T4block, "T10": ft.T10block}[et]
    fens, fes = gen(1.0, 1.2, 0.9, n, n + 1, n)
    fens.xyz = ft.meshes.jitter_interior(fens.xyz, (n, n + 1, n), 0.2, 11, box=(1.0, 1.2, 0.9))
    if et in ("H20", "T10"):
        nv = fens.count()
        fens = ft.meshes.recompute_midpoints(fens, fes, nv)
    r = ft.GaussRule(*rule[1:]) if rule[0] == "G" else ft.TetRule(rule[1])
    femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 1)
    if coef == "iso":
        cf, oc, kind = ft.DataCache(2.5), np.array([2.5]), 0
    elif coef == "general":
        k = np.array([[2.0, 0.3, 0.1], [0.3, 1.5, -0.2], [0.1, -0.2, 1.0]])
        cf, oc, kind = ft.DataCache(k), k, 0
    elif coef == "per_element":
        v = np.random.default_rng(3).lognormal(0, 1, fes.count())
        cf, oc, kind = ft.ElementwiseData(v), v.reshape(-1, 1), 1
    elif coef == "per_point":
        # a DataCache whose fill! varies per element and point, evaluated on
        # the host at every point (src/DataCacheModule.jl:103-112)
        npts = femm.integdomain.integrationdata()[0]
        vals = np.random.default_rng(5).lognormal(0, 1, (fes.count(), npts))
        cf = ft.DataCache(1.0, lambda cache, XYZ, tangents, feid, qpid:
                          vals[feid - 1, qpid - 1])
        oc, kind = vals.reshape(fes.count(), npts, 1), 2
    else:
        # a 3x3 conductivity following the point's coordinates
        # (_bilform_diffusion_general: c = cf(loc, J, i, j) at every point)
        k0 = np.array([[2.0, 0.3, 0.1], [0.3, 1.5, -0.2], [0.1, -0.2, 1.0]])
        cf = ft.DataCache(k0, lambda cache, XYZ, tangents, feid, qpid:
                          k0 * (1.0 + XYZ[0, 0] + 0.5 * XYZ[0, 2]))
        oc, kind = ft.femm._qp_values(femm, geom, cf, 9), 2
    K = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(symmetric=False, precision=prec), geom,
                             u, cf)
    Kr = _oracle_form(O, femm, O.DIFFUSION, geom, u, oc, kind, symmetric=False)
    compare(K, Kr)
    assert abs(K - K.T).max() == 0.0
    Ksr = _oracle_form(O, femm, O.DIFFUSION, geom, u, oc, kind)
    if prec == "fp64":
        bitwise(K, Kr)
        K64 = ft.bilform_diffusion(femm, geom, u, cf)  # the 4-argument form
        bitwise(K64, Ksr)
        # the mixed path takes the same point values (rules with positive
        # weights: the 5-point tetrahedral rule's negative centroid weight
        # makes every entry a cancellation, 1.1e-6 of the row scale in FP32)
        if coef.startswith("per_point") and femm.integdomain.integrationdata()[3].min() > 0:
            mixed_gate(ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(precision="mixed"),
                                            geom, u, cf), K64)
    else:
        Ks = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(precision=prec), geom, u, cf)
        compare(Ks, Ksr, structure=False)


# ---------------------------------------------------------------- elasticity
@pytest.mark.parametrize("et,n,rule", [("H8", 3, ("G", 3, 2)), ("H20", 2, ("G", 3, 3)),
                                       ("T4", 3, ("T", 1)), ("T10", 3, ("T", 4))])
@pytest.mark.parametrize("coef", ["iso_const", "aniso_const", "per_element_iso", "per_element_D",
                                  "per_point_D"])
@pytest.mark.parametrize("prec", ["fp64", "fp64_fast"])
def test_elasticity_fp64(ft, O, et, n, rule, coef, prec):
    gen = {"H8": ft.H8block, "H20": ft.H20block, "T4": ft.T4block, "T10": ft.T10block}[et]
    fens, fes = gen(1.0, 1.0, 1.0, n, n, n)
    fens.xyz = ft.meshes.jitter_interior(fens.xyz, (n, n, n), 0.15, 5)
    if et in ("H20", "T10"):
        fens = ft.meshes.recompute_midpoints(fens, fes, 0)
    r = ft.GaussRule(*rule[1:]) if rule[0] == "G" else ft.TetRule(rule[1])
    femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    rng = np.random.default_rng(9)
    if coef == "iso_const":
        D = ft.isotropic_D(210e9, 0.3)
        cf, oc, kind = ft.DataCache(D), D, 0
    elif coef == "aniso_const":
        A = rng.uniform(-1, 1, (6, 6))
        D = A @ A.T + 6 * np.eye(6)
        cf, oc, kind = ft.DataCache(D), D, 0
    elif coef == "per_element_iso":
        E = rng.lognormal(np.log(70e9), 0.5, fes.count())
        nu = rng.uniform(0.2, 0.35, fes.count())
        cf = ft.IsotropicElementwise(E, nu)
        oc = np.stack([ft.isotropic_D(a, b) for a, b in zip(E, nu)]).reshape(-1, 36)
        kind = 1
    elif coef == "per_element_D":
        Ds = []
        for _ in range(fes.count()):
            A = rng.uniform(-1, 1, (6, 6))
            Ds.append(A @ A.T + 6 * np.eye(6))
        oc = np.stack(Ds).reshape(-1, 36)
        cf, kind = ft.ElementwiseData(oc), 1
    else:
        # C = cf(loc, J, i, j) varying per point (src/FEMMBaseModule.jl:1802):
        # an isotropic D whose modulus follows x, evaluated on the host
        npts = femm.integdomain.integrationdata()[0]
        def fill(cache, XYZ, tangents, feid, qpid):
            return ft.isotropic_D(70e9 * (1.0 + XYZ[0, 0]), 0.3)
        cf = ft.DataCache(ft.isotropic_D(70e9, 0.3), fill)
        oc = ft.femm._qp_values(femm, geom, cf, 36)
        kind = 2
        if prec != "fp64":
            # the fused paths need one D per element
            with pytest.raises(ft.FegpuError, match="varies over the points"):
                ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision=prec), geom, u,
                                       ft.DeforModelRed3D, cf)
            return
    K = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(symmetric=False, precision=prec),
                               geom, u, ft.DeforModelRed3D, cf)
    Kr = _oracle_form(O, femm, O.LIN_ELASTIC, geom, u, oc, kind, symmetric=False)
    compare(K, Kr)
    assert abs(K - K.T).max() == 0.0
    Ksr = _oracle_form(O, femm, O.LIN_ELASTIC, geom, u, oc, kind)
    if prec == "fp64":
        bitwise(K, Kr)
        bitwise(ft.bilform_lin_elastic(femm, geom, u, ft.DeforModelRed3D, cf), Ksr)
    else:
        Ks = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision=prec), geom, u,
                                    ft.DeforModelRed3D, cf)
        compare(Ks, Ksr, structure=False)


# ---------------------------------------------------------------- convection
@pytest.mark.parametrize("et", ["H8", "T10", "H20", "Q4"])
def test_convection_fp64(ft, O, et):
    """bilform_convection (src/FEMMBaseModule.jl:1583-1625) with its default
    SysmatAssemblerSparse, a nonuniform nodal velocity."""
    rng = np.random.default_rng(21)
    if et == "Q4":
        fens, fes = ft.Q4block(1.0, 0.6, 5, 3)
        fens.xyz = ft.meshes.jitter_interior(fens.xyz, (5, 3), 0.15, 7, box=(1.0, 0.6))
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, 2), 0.3))
    else:
        gen = {"H8": ft.H8block, "H20": ft.H20block, "T10": ft.T10block}[et]
        fens, fes = gen(1.0, 0.7, 1.3, 3, 2, 2)
        fens.xyz = ft.meshes.jitter_interior(fens.xyz, (3, 2, 2), 0.15, 7, box=(1.0, 0.7, 1.3))
        if et in ("H20", "T10"):
            fens = ft.meshes.recompute_midpoints(fens, fes, 0)
        r = ft.TetRule(4) if et == "T10" else ft.GaussRule(3, 3 if et == "H20" else 2)
        femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(fens.xyz)
    sd = fens.xyz.shape[1]
    vel = ft.NodalField(rng.uniform(-1, 1, (fens.count(), sd)) + np.arange(1, sd + 1))
    Q = _field(ft, fens.count(), 1)
    K = ft.bilform_convection(femm, geom, vel, Q, ft.DataCache(1.2))
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    Kr = O.bilform_convection(fes.code, fes.conn, geom.values, Q.dofnums, Q.nalldofs(), pc, w,
                              vel.values, otherdim=femm.integdomain.otherdimension)
    compare(K, Kr)


# ---------------------------------------------------------------- div_grad
@pytest.mark.parametrize("et,n,rule", [("H8", 3, ("G", 3, 2)), ("T10", 2, ("T", 4)),
                                       ("H20", 2, ("G", 3, 3))])
@pytest.mark.parametrize("coef", ["const", "per_element"])
def test_div_grad_fp64(ft, O, et, n, rule, coef):
    """bilform_div_grad (src/FEMMBaseModule.jl:1672-1723) with its default
    SysmatAssemblerSparse; mixed precision within 1e-6 of FP64."""
    gen = {"H8": ft.H8block, "H20": ft.H20block, "T10": ft.T10block}[et]
    fens, fes = gen(1.0, 0.7, 1.3, n, n, n)
    fens.xyz = ft.meshes.jitter_interior(fens.xyz, (n, n, n), 0.15, 6, box=(1.0, 0.7, 1.3))
    if et in ("H20", "T10"):
        fens = ft.meshes.recompute_midpoints(fens, fes, 0)
    r = ft.GaussRule(*rule[1:]) if rule[0] == "G" else ft.TetRule(rule[1])
    femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    rng = np.random.default_rng(12)
    if coef == "const":
        cf, oc, kind = ft.DataCache(1.8e-3), np.array([1.8e-3]), 0
    else:
        mu = rng.lognormal(np.log(1e-3), 0.5, fes.count())
        cf, oc, kind = ft.ElementwiseData(mu), mu.reshape(-1, 1), 1
    K = ft.bilform_div_grad(femm, geom, u, cf)
    Kr = _oracle_form(O, femm, O.DIV_GRAD, geom, u, oc, kind, symmetric=False)
    compare(K, Kr)
    Km = ft.bilform_div_grad(femm, ft.SysmatAssemblerGPU(symmetric=False, precision="mixed"),
                             geom, u, cf)
    x = rng.uniform(-1, 1, K.shape[0])
    assert np.linalg.norm((Km - K) @ x) <= MIXED_TOL * np.linalg.norm(K @ x)
    mixed_gate(Km, K)


# ---------------------------------------------------------------- dot / linform
@pytest.mark.parametrize("et,ndn", [("H8", 1), ("H8", 3), ("T10", 3), ("H20", 1)])
def test_dot_volume(ft, O, et, ndn):
    gen = {"H8": ft.H8block, "H20": ft.H20block, "T10": ft.T10block}[et]
    fens, fes = gen(12.0, 1.1, 0.32, 2, 4, 3)
    r = ft.TetRule(4) if et == "T10" else ft.GaussRule(3, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), ndn)
    c = np.eye(ndn) * 1.7
    if ndn == 3:
        c[0, 1] = c[1, 0] = 0.2
    for symmetric in (True, False):
        asm = ft.SysmatAssemblerGPU(symmetric=symmetric)
        K = ft.bilform_dot(femm, asm, geom, u, ft.DataCache(c))
        Kr = _oracle_form(O, femm, O.DOT, geom, u, c, symmetric=symmetric)
        compare(K, Kr, structure=not symmetric)
    # test/test_forms.jl:1-27: v' G v = volume for the Gram matrix
    G = ft.innerproduct(femm, geom, u)
    v = np.ones(G.shape[0])
    V = 12.0 * 1.1 * 0.32
    assert abs(v @ G @ v - ndn * V) / V <= 1e-5


def test_dot_unsymmetric_coefficient(ft, O):
    """An unsymmetric ndn x ndn coefficient with SysmatAssemblerSparse gives an
    unsymmetric matrix: the CSC export must read the values by columns."""
    fens, fes = ft.H8block(1.0, 0.8, 0.6, 3, 2, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    c = np.array([[2.0, 0.3, -0.1], [0.7, 1.5, 0.2], [0.05, -0.4, 1.1]])
    K = ft.bilform_dot(femm, ft.SysmatAssemblerGPU(symmetric=False), geom, u, ft.DataCache(c))
    Kr = _oracle_form(O, femm, O.DOT, geom, u, c, symmetric=False)
    compare(K, Kr)
    assert abs(K - K.T).max() > 0.0


def test_dot_surface_q4_thickness(ft, O):
    """Q4 surface mass with thickness (IntegDomain(fes, rule, 0.01)), in 3-D
    space (m = 3 -> surface Jacobian x thickness) and m = 2."""
    fens, fes = ft.Q4block(2.0, 1.5, 5, 4)
    rng = np.random.default_rng(1)
    xyz = np.hstack([fens.xyz, rng.uniform(-0.05, 0.05, (fens.count(), 1))])
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, 2), 0.01))
    geom = ft.NodalField(xyz)
    for ndn in (1, 3):
        u = _field(ft, fens.count(), ndn)
        for m in (2, 3):
            K = ft.bilform_dot(femm, geom, u, ft.DataCache(np.eye(ndn)), m=m)
            Kr = _oracle_form(O, femm, O.DOT, geom, u, np.eye(ndn), m=m)
            compare(K, Kr, structure=False)


def test_diffusion_q4_planar(ft, O):
    """2-D diffusion with thickness (test/test_forms.jl:106-156 pattern on Q4)."""
    fens, fes = ft.Q4block(12.0, 1.1, 6, 4)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, 2), 0.32))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 1)
    for cf, oc in ((ft.DataCache(1.0), np.array([1.0])), (ft.DataCache(np.eye(2)), np.eye(2))):
        K = ft.bilform_diffusion(femm, geom, u, cf)
        Kr = _oracle_form(O, femm, O.DIFFUSION, geom, u, oc)
        compare(K, Kr, structure=False)
    a, b, c = -0.1, 0.3, 0.4
    v = a + b * fens.xyz[:, 0] + c * fens.xyz[:, 1]
    V = 12.0 * 1.1 * 0.32
    assert abs(v @ K @ v - (b * b + c * c) * V) / V <= 1e-5


@pytest.mark.parametrize("et,ndn", [("H8", 1), ("T10", 3), ("H20", 3)])
def test_linform(ft, O, et, ndn):
    gen = {"H8": ft.H8block, "H20": ft.H20block, "T10": ft.T10block}[et]
    fens, fes = gen(12.0, 1.1, 4.32, 2, 4, 3)
    r = ft.TetRule(4) if et == "T10" else ft.GaussRule(3, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(fens.xyz)
    P = _field(ft, fens.count(), ndn)
    f = np.arange(1, ndn + 1) * 11.0
    F = ft.linform_dot(femm, geom, P, ft.DataCache(f), 3)
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    Fr = O.linform_dot(fes.code, fes.conn, fens.xyz, P.dofnums, P.nalldofs(), pc, w, f)
    assert np.abs(F - Fr).max() <= 1e-12 * np.abs(Fr).max()
    # test/test_forms.jl:158-194: sum(F) = volume * force
    F = ft.distribloads(femm, geom, P, ft.ForceIntensity(f), 3)
    V = 12.0 * 1.1 * 4.32
    assert abs(F.sum() - V * f.sum()) / (V * f.sum()) <= 1e-5


# ---------------------------------------------------------------- numbering, determinism
def test_general_dof_numbering_with_ebcs(ft, O):
    """Fixed DOFs numbered last (non-contiguous per node): general slot path."""
    fens, fes = ft.T10block(1.0, 1.0, 1.0, 2, 3, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
    geom = ft.NodalField(fens.xyz)
    u = ft.NodalField(np.zeros((fens.count(), 3)))
    on_face = np.flatnonzero(np.abs(fens.xyz[:, 0]) < 1e-12) + 1
    ft.setebc(u, on_face, True, [1], 0.0)
    ft.setebc(u, on_face[::2], True, [3], 0.0)
    ft.numberdofs(u)
    D = ft.isotropic_D(1.0, 0.25)
    K = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(symmetric=False), geom, u,
                               ft.DeforModelRed3D, ft.DataCache(D))
    Kr = _oracle_form(O, femm, O.LIN_ELASTIC, geom, u, D, symmetric=False)
    compare(K, Kr)


# ---------------------------------------------------------------- empty and ragged inputs
def test_empty_element_set(ft):
    """An element set without elements: every form returns the all-zero result
    of the full size (FP64 and mixed), as makematrix! of an assembler that
    received no triples does."""
    fens, _ = ft.H8block(1.0, 1.0, 1.0, 2, 2, 2)
    femm = ft.FEMMBase(ft.IntegDomain(ft.FESetH8(np.zeros((0, 8), dtype=np.int64)),
                                      ft.GaussRule(3, 2)))
    geom = ft.NodalField(fens.xyz)
    u1 = _field(ft, fens.count(), 1)
    u3 = _field(ft, fens.count(), 3)
    for prec in ("fp64", "mixed"):
        K = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(precision=prec), geom, u1,
                                 ft.DataCache(1.0))
        assert K.shape == (u1.nalldofs(), u1.nalldofs()) and K.nnz == 0
        K = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision=prec), geom, u3,
                                   ft.DeforModelRed3D, ft.DataCache(ft.isotropic_D(1.0, 0.3)))
        assert K.shape == (u3.nalldofs(), u3.nalldofs()) and K.nnz == 0
    F = ft.linform_dot(femm, geom, u3, ft.DataCache(np.array([1.0, 2.0, 3.0])), 3)
    assert F.shape == (u3.nalldofs(),) and not F.any()


def test_isolated_nodes_and_single_element(ft, O):
    """Nodes that no element references, numbered among the others (their
    rows and columns are empty), and a mesh of one element: FP64 against the
    oracle, mixed against FP64."""
    fens, fes = ft.H8block(1.0, 0.7, 0.5, 2, 2, 1)
    rng = np.random.default_rng(8)
    xyz = np.vstack([fens.xyz, rng.uniform(0, 1, (5, 3))])  # five nodes of no element
    n = xyz.shape[0]
    perm = rng.permutation(n)
    where = np.empty(n, dtype=np.int64)
    where[perm] = np.arange(n)
    xyz = xyz[perm]
    for conn in (where[fes.conn - 1] + 1, where[fes.conn[:1] - 1] + 1):
        femm = ft.FEMMBase(ft.IntegDomain(ft.FESetH8(conn), ft.GaussRule(3, 2)))
        geom = ft.NodalField(xyz)
        u = _field(ft, n, 3)
        D = ft.isotropic_D(1.0, 0.3)
        # structural pattern (SysmatAssemblerSparse): the regular block has
        # exact-zero couplings, which S + S' drops only when bitwise zero
        K = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(symmetric=False), geom, u,
                                   ft.DeforModelRed3D, ft.DataCache(D))
        compare(K, _oracle_form(O, femm, O.LIN_ELASTIC, geom, u, D, symmetric=False))
        K32 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(symmetric=False,
                                                                 precision="mixed"),
                                     geom, u, ft.DeforModelRed3D, ft.DataCache(D))
        x = rng.uniform(-1, 1, K.shape[0])
        assert np.linalg.norm((K32 - K) @ x) / np.linalg.norm(K @ x) <= MIXED_TOL
        mixed_gate(K32, K)
        untouched = np.setdiff1d(np.arange(1, n + 1), np.unique(conn))
        rows = u.dofnums[untouched - 1].ravel() - 1
        assert abs(K.tocsr()[rows]).sum() == 0 and abs(K32.tocsr()[rows]).sum() == 0


@pytest.mark.parametrize("form", ["elastic", "convection"])
def test_blocked_extraction(ft, form):
    """matrix_blocked_ff / fd / df / dd (src/MatrixUtilityModule.jl:675-806) of a
    device matrix with the free DOFs numbered first equal the corresponding
    slices of the full CSC export (symmetric and unsymmetric values)."""
    fens, fes = ft.H8block(1.0, 0.8, 0.6, 3, 3, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    geom = ft.NodalField(fens.xyz)
    on_face = np.flatnonzero(np.abs(fens.xyz[:, 0]) < 1e-12) + 1
    asm = ft.SysmatAssemblerGPU(symmetric=False, result="device")
    if form == "elastic":
        u = ft.NodalField(np.zeros((fens.count(), 3)))
        ft.setebc(u, on_face, True, [1, 2], 0.0)
        ft.numberdofs(u)
        K = ft.bilform_lin_elastic(femm, asm, geom, u, ft.DeforModelRed3D,
                                   ft.DataCache(ft.isotropic_D(1.0, 0.3)))
    else:
        u = ft.NodalField(np.zeros((fens.count(), 1)))
        ft.setebc(u, on_face, True, [1], 0.0)
        ft.numberdofs(u)
        vel = ft.NodalField(np.tile([1.0, 0.5, -0.2], (fens.count(), 1)))
        K = ft.bilform_convection(femm, asm, geom, vel, u, ft.DataCache(1.0))
    nf = u.nfreedofs()
    full = K.to_scipy(drop_zeros=False).tocsc()
    n = full.shape[0]
    for fn, rows, cols in ((ft.matrix_blocked_ff, slice(0, nf), slice(0, nf)),
                           (ft.matrix_blocked_fd, slice(0, nf), slice(nf, n)),
                           (ft.matrix_blocked_df, slice(nf, n), slice(0, nf)),
                           (ft.matrix_blocked_dd, slice(nf, n), slice(nf, n))):
        B = fn(K, nf)
        R = full[rows, cols].tocsc()
        R.sort_indices()
        B.sort_indices()
        assert B.shape == R.shape
        assert np.array_equal(B.indptr, R.indptr) and np.array_equal(B.indices, R.indices)
        assert np.array_equal(B.data, R.data)
    if form == "convection":
        assert abs(full - full.T).max() > 0


def test_permuted_node_numbering(ft, O):
    fens, fes = ft.H8block(1.0, 1.0, 1.0, 3, 3, 3)
    u = ft.NodalField(np.zeros((fens.count(), 3)))
    perm = np.random.default_rng(4).permutation(fens.count()) + 1
    ft.numberdofs(u, entperm=perm)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    geom = ft.NodalField(fens.xyz)
    D = ft.isotropic_D(3.0, 0.2)
    K = ft.bilform_lin_elastic(femm, geom, u, ft.DeforModelRed3D, ft.DataCache(D))
    Kr = _oracle_form(O, femm, O.LIN_ELASTIC, geom, u, D)
    compare(K, Kr, structure=False)


def test_determinism(ft):
    """test/test_basics.jl:3043-3045: repeated assembly is bitwise identical."""
    fens, fes = ft.t10_elastic_mesh(n=4)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    D = ft.isotropic_D(210e9, 0.3)
    asm = ft.SysmatAssemblerGPU(result="device")
    v1 = ft.bilform_lin_elastic(femm, asm, geom, u, ft.DeforModelRed3D, ft.DataCache(D)).values()
    v2 = ft.bilform_lin_elastic(femm, asm, geom, u, ft.DeforModelRed3D, ft.DataCache(D)).values()
    assert np.array_equal(v1, v2)


def test_device_results_do_not_alias(ft):
    """A device result keeps its values while other (short-lived) assemblers
    assemble on the same mesh: each assembler fills its own device matrix,
    whatever object ids the interpreter reuses."""
    fens, fes = ft.h8_diffusion_mesh(n=4, seed=3)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 1)
    K1 = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(result="device"), geom, u,
                              ft.DataCache(1.0))
    v1 = K1.values().copy()
    for prec in ("fp64", "mixed", "fp64", "mixed"):
        K2 = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(precision=prec, result="device"),
                                  geom, u, ft.DataCache(2.0))
        assert np.abs(K2.values() - 2.0 * v1).max() <= 1e-6 * np.abs(v1).max()
    assert np.array_equal(K1.values(), v1)


def test_colouring_matches_reference(ft, O, kats):
    k = kats["coloring_t4"]
    fens, fes = ft.T4block(*k["block"])
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(1)))
    femm.set_geometry(ft.NodalField(fens.xyz))
    col, nc = femm.colors()
    ref, nref = O.element_coloring(fes.conn, fens.count())
    assert nc == nref == len(k["unique_colors_in_order"])
    assert np.array_equal(col, ref)


def test_connection_matrix_degree(ft, kats):
    k = kats["connection_degree"]
    fens, fes = ft.H8block(*k["block"])
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    C = ft.connectionmatrix(femm, fens.count())
    deg = np.diff(C.indptr)
    assert deg.max() == k["max_degree"] and deg.min() == k["min_degree"]


def _gpu_dropped(ft, femm, geom, u, form, cf):
    """(exported symmetric matrix, number of exact zeros it left out)."""
    asm = ft.SysmatAssemblerGPU(result="device")
    if form == "diffusion":
        M = ft.bilform_diffusion(femm, asm, geom, u, cf)
    else:
        M = ft.bilform_lin_elastic(femm, asm, geom, u, ft.DeforModelRed3D, cf)
    return M.to_scipy(), M.nnz(drop_zeros=False) - M.nnz(drop_zeros=True)


@pytest.mark.parametrize("case", ["h8_regular_diffusion", "t10_boundary_elasticity"])
def test_zero_dropping_on_regular_mesh(ft, O, case):
    """Meshes on which the reference's S + S' step (src/AssemblyModule.jl:576)
    meets exact zeros: a regular H8 block (the edge couplings of a cube
    element cancel exactly) and a T10 block whose boundary nodes stay on the
    block faces (the benchmark jitter).  The default symmetric assembler
    (SysmatAssemblerSparseSymm, reference-order FP64) leaves out exactly the
    entries the oracle leaves out, and the result equals the oracle's bit for
    bit; the structural result (SysmatAssemblerSparse) keeps them."""
    if case == "h8_regular_diffusion":
        fens, fes = ft.H8block(1.0, 1.0, 1.0, 3, 3, 3)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
        u = _field(ft, fens.count(), 1)
        form, cf, oc, ofm = "diffusion", ft.DataCache(1.0), np.array([1.0]), O.DIFFUSION
    else:
        fens, fes = ft.t10_elastic_mesh(n=6, seed=2)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
        u = _field(ft, fens.count(), 3)
        D = ft.isotropic_D(210e9, 0.3)
        form, cf, oc, ofm = "elasticity", ft.DataCache(D), D, O.LIN_ELASTIC
    geom = ft.NodalField(fens.xyz)
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    Kr, dropped, _ = O.bilform(ofm, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc,
                               w, oc, phases=True, tables=(Ns, dN))
    assert dropped > 0, "the mesh should meet exact zeros"
    K, gpu_dropped = _gpu_dropped(ft, femm, geom, u, form, cf)
    assert gpu_dropped == dropped
    bitwise(K, Kr)
    Kn = (ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(symmetric=False), geom, u, cf)
          if form == "diffusion" else
          ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(symmetric=False), geom, u,
                                 ft.DeforModelRed3D, cf))
    bitwise(Kn, _oracle_form(O, femm, ofm, geom, u, oc, symmetric=False))


@pytest.mark.parametrize("et", ["H8", "T10", "H20"])
def test_symmetric_structure_fully_perturbed(ft, O, et):
    """Every node moved: no exact zeros, so the S + S' zero dropping of the
    symmetric assembler leaves the structural pattern, bit-exactly."""
    gen = {"H8": ft.H8block, "H20": ft.H20block, "T10": ft.T10block}[et]
    fens, fes = gen(1.0, 1.0, 1.0, 3, 2, 3)
    rng = np.random.default_rng(12)
    fens.xyz = fens.xyz + rng.uniform(-0.05, 0.05, fens.xyz.shape)
    if et != "H8":
        fens = ft.meshes.recompute_midpoints(fens, fes, 0)
    r = ft.TetRule(4) if et == "T10" else ft.GaussRule(3, 3 if et == "H20" else 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    D = ft.isotropic_D(210e9, 0.3)
    K = ft.bilform_lin_elastic(femm, geom, u, ft.DeforModelRed3D, ft.DataCache(D))
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    Kr, dropped, _ = O.bilform(O.LIN_ELASTIC, fes.code, fes.conn, geom.values, u.dofnums,
                               u.nalldofs(), pc, w, D, phases=True)
    assert dropped == 0
    compare(K, Kr)


# ---------------------------------------------------------------- generic assembler
def test_generic_assembler_kats(ft, kats):
    k = kats["assembler"]["sparse_rect"]
    a = ft.SysmatAssemblerGPU(symmetric=False)
    a.startassembly(5, 5, 3, 7, 7)
    for m, r, c in zip(k["mats"], k["rows"], k["cols"]):
        a.assemble(np.array(m), r, c)
    A = a.makematrix().toarray()
    assert np.abs(np.array(k["expected"]) - A).max() < 1e-5
    k = kats["assembler"]["symm_mtm"]
    a = ft.SysmatAssemblerGPU(symmetric=True)
    a.startassembly(5, 5, 3, 7, 7)
    for m, r, c in zip(k["mats"], k["rows"], k["cols"]):
        m = np.array(m)
        a.assemble(m.T @ m, r, c)
    A = a.makematrix().toarray()
    assert np.abs(np.array(k["expected"]) - A).max() < 1e-5
    assert np.abs(A - A.T).max() == 0.0


def test_generic_lumping_assemblers(ft, kats):
    """SysmatAssemblerSparseDiag (test/test_basics.jl:135) and the HRZ recipe
    (test/test_basics.jl:923-960) through the device assembler."""
    k = kats["assembler"]["sparse_diag_mtm"]
    a = ft.SysmatAssemblerSparseDiagGPU()
    a.startassembly(5, 5, 3, 7, 7)
    for m, d in zip(k["mats"], k["dofs"]):
        m = np.array(m)
        a.assemble(m.T @ m, d, d)
    A = a.makematrix().toarray()
    assert np.abs(np.diag(np.diag(np.array(k["expected"]))) - A).max() < 1e-5
    rng = np.random.default_rng(5)
    N, el = 30, rng.random((8, 8))
    el = el + el.T
    a = ft.SysmatAssemblerSparseHRZLumpingSymmGPU()
    a.startassembly(8, 8, 3, N, N)
    ref = np.zeros(N)
    for d in ([10, 29, 15, 1, 7, 3, 6, 2], [15, 1, 7, 11, 29, 3, 8, 4],
              [25, 1, 17, 13, 30, 13, 18, 14]):
        a.assemble(el, d, d)
        f = el.sum(axis=0).sum() / np.trace(el)
        for i, dd in enumerate(d):
            ref[dd - 1] += f * el[i, i]
    M = a.makematrix()
    assert np.abs(M.diagonal() - ref).sum() / np.linalg.norm(el) <= 1e-9


@pytest.mark.parametrize("et,ndn,coef", [("H8", 3, "const"), ("T10", 3, "per_element"),
                                         ("H20", 1, "const"), ("Q4", 3, "const")])
@pytest.mark.parametrize("lumping", ["diag", "hrz"])
def test_lumped_mass(ft, O, et, ndn, coef, lumping):
    """bilform_dot with the lumping assemblers on the device against the
    oracle's restatement of the same assembly."""
    rng = np.random.default_rng(14)
    if et == "Q4":
        fens, fes = ft.Q4block(2.0, 1.5, 5, 4)
        xyz = np.hstack([fens.xyz, rng.uniform(-0.05, 0.05, (fens.count(), 1))])
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, 2), 0.01))
    else:
        gen = {"H8": ft.H8block, "H20": ft.H20block, "T10": ft.T10block}[et]
        fens, fes = gen(1.0, 0.7, 1.3, 3, 2, 2)
        xyz = ft.meshes.jitter_interior(fens.xyz, (3, 2, 2), 0.15, 4, box=(1.0, 0.7, 1.3))
        if et in ("H20", "T10"):
            fens.xyz = xyz
            xyz = ft.meshes.recompute_midpoints(fens, fes, 0).xyz
        r = ft.TetRule(4) if et == "T10" else ft.GaussRule(3, 3 if et == "H20" else 2)
        femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(xyz)
    u = _field(ft, fens.count(), ndn)
    if coef == "const":
        c = np.eye(ndn) * 7.8e3
        if ndn == 3:
            c[0, 1] = c[1, 0] = 40.0
        cf, oc, kind = ft.DataCache(c), c, 0
    else:
        rho = rng.uniform(1e3, 8e3, fes.count())
        cf = ft.ElementwiseData(rho)
        oc = np.stack([np.eye(ndn) * v for v in rho]).reshape(-1, ndn * ndn)
        kind = 1
    asm = (ft.SysmatAssemblerSparseDiagGPU() if lumping == "diag"
           else ft.SysmatAssemblerSparseHRZLumpingSymmGPU())
    M = ft.bilform_dot(femm, asm, geom, u, cf)
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    Mr = O.bilform(O.DOT, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc, w, oc,
                   coef_kind=kind, otherdim=femm.integdomain.otherdimension, m=3,
                   asm=O.ASM_DIAG if lumping == "diag" else O.ASM_HRZ)
    compare(M, Mr)


def test_generic_assembler_random(ft, O):
    """test/test_basics.jl:2100-2175: random symmetric matrices vs the oracle."""
    rng = np.random.default_rng(2)
    N = 133
    for symm in (False, True):
        a = ft.SysmatAssemblerGPU(symmetric=symm)
        a.startassembly(6, 6, 100, N, N)
        o = O.Assembler(symm, N, N)
        for _ in range(200):
            k = int(rng.integers(2, 7))
            M = rng.uniform(-1, 1, (k, k))
            M = M + M.T
            d = rng.permutation(N)[:k] + 1
            a.assemble(M, d, d)
            o.assemble(M, d, d)
        A = a.makematrix()
        Ar = o.make()
        compare(A, Ar)


# ---------------------------------------------------------------- mixed precision
@pytest.mark.parametrize("et", ["H20", "T10", "H8"])
def test_mixed_precision(ft, O, et):
    if et == "H20":
        fens, fes, flagged = ft.h20_elastic_mesh(n=4, distort_fraction=0.05)
        r = ft.GaussRule(3, 3)
    elif et == "T10":
        fens, fes = ft.t10_elastic_mesh(n=4)
        r = ft.TetRule(4)
    else:
        fens, fes = ft.h8_diffusion_mesh(n=5)
        r = ft.GaussRule(3, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    rng = np.random.default_rng(4)
    E = rng.lognormal(np.log(70e9), 0.5, fes.count())
    nu = rng.uniform(0.2, 0.35, fes.count())
    cf = ft.IsotropicElementwise(E, nu)
    K64 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(), geom, u, ft.DeforModelRed3D, cf)
    K32 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="mixed"), geom, u,
                                 ft.DeforModelRed3D, cf)
    x = rng.uniform(-1, 1, K64.shape[0])
    assert np.linalg.norm((K32 - K64) @ x) / np.linalg.norm(K64 @ x) <= MIXED_TOL
    assert abs(K32 - K64).max() / abs(K64).max() <= MIXED_TOL
    mixed_gate(K32, K64)
    assert abs(K32 - K32.T).max() == 0.0


@pytest.mark.parametrize("curved", [False, True])
def test_mixed_t10_straight_and_curved(ft, O, curved):
    """Mixed T10 elasticity within the mixed bound of FP64 on straight-sided
    elements (affine: the FP32 corner Jacobian) and on elements whose
    mid-edge nodes are moved off the edges (curved: FP64 geometry), and on a
    mesh that mixes both."""
    fens, fes = ft.t10_elastic_mesh(n=5, seed=9)
    xyz = fens.xyz.copy()
    if curved:
        rng = np.random.default_rng(12)
        mids = np.unique(fes.conn[:, 4:].ravel() - 1)
        pick = mids[rng.random(mids.size) < 0.5]  # about half the mid-edge nodes
        interior = np.all((xyz[pick] > 1e-9) & (xyz[pick] < 1 - 1e-9), axis=1)
        pick = pick[interior]
        xyz[pick] += rng.uniform(-0.02, 0.02, (pick.size, 3)) / 5
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
    geom = ft.NodalField(xyz)
    u = _field(ft, fens.count(), 3)
    rng = np.random.default_rng(5)
    cf = ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 0.5, fes.count()),
                                 rng.uniform(0.2, 0.35, fes.count()))
    K64 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(), geom, u, ft.DeforModelRed3D, cf)
    K32 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="mixed"), geom, u,
                                 ft.DeforModelRed3D, cf)
    x = rng.uniform(-1, 1, K64.shape[0])
    assert np.linalg.norm((K32 - K64) @ x) / np.linalg.norm(K64 @ x) <= MIXED_TOL
    assert abs(K32 - K64).max() / abs(K64).max() <= MIXED_TOL
    mixed_gate(K32, K64)
    assert abs(K32 - K32.T).max() == 0.0
    # the FP64 path against the oracle: corner Jacobians on the straight
    # elements, isoparametric ones on the curved
    D = ft.isotropic_D(70e9, 0.3)
    K = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(symmetric=False), geom, u,
                               ft.DeforModelRed3D, ft.DataCache(D))
    compare(K, _oracle_form(O, femm, O.LIN_ELASTIC, geom, u, D, symmetric=False))


# ---------------------------------------------------------------- masslike
def _masslike_case(ft, et, seed=17):
    rng = np.random.default_rng(seed)
    if et == "Q4":
        fens, fes = ft.Q4block(2.0, 1.5, 5, 4)
        xyz = np.hstack([fens.xyz, rng.uniform(-0.05, 0.05, (fens.count(), 1))])
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, 2), 0.01))
    else:
        gen = {"H8": ft.H8block, "H20": ft.H20block, "T10": ft.T10block, "T4": ft.T4block}[et]
        fens, fes = gen(1.0, 0.7, 1.3, 3, 2, 2)
        xyz = ft.meshes.jitter_interior(fens.xyz, (3, 2, 2), 0.15, 4, box=(1.0, 0.7, 1.3))
        if et in ("H20", "T10"):
            fens.xyz = xyz
            xyz = ft.meshes.recompute_midpoints(fens, fes, 0).xyz
        r = {"T10": ft.TetRule(4), "T4": ft.TetRule(1), "H20": ft.GaussRule(3, 3),
             "H8": ft.GaussRule(3, 2)}[et]
        femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    return rng, fens, fes, femm, ft.NodalField(xyz)


@pytest.mark.parametrize("et,ndn,coef,m", [("H8", 1, "const", 3), ("T10", 3, "matrix", 3),
                                           ("H20", 3, "per_element", 3), ("T4", 1, "per_qp", 3),
                                           ("Q4", 3, "matrix", 3), ("Q4", 1, "const", 2)])
def test_masslike(ft, O, et, ndn, coef, m):
    """bilform_masslike (src/FEMMBaseModule.jl:1865-1917): the nelem*ndn x
    nalldofs matrix through SysmatAssemblerSparse semantics (every element
    block entry stored, explicit zeros included) against the oracle."""
    rng, fens, fes, femm, geom = _masslike_case(ft, et)
    u = _field(ft, fens.count(), ndn)
    npts = femm.integdomain.integrationdata()[0]
    if coef == "const":
        cf, oc, kind = ft.DataCache(np.eye(ndn) * 2.5), np.eye(ndn) * 2.5, 0
    elif coef == "matrix":
        c = rng.uniform(0.5, 1.5, (ndn, ndn))
        cf, oc, kind = ft.DataCache(c), c, 0
    elif coef == "per_element":
        rho = rng.uniform(1e3, 8e3, fes.count())
        cf = ft.ElementwiseData(rho)
        oc, kind = np.stack([np.eye(ndn) * v for v in rho]).reshape(-1, ndn * ndn), 1
    else:
        vals = rng.uniform(1.0, 2.0, (fes.count(), npts))
        cf = ft.DataCache(np.eye(ndn), lambda cache, XYZ, tangents, feid, qpid:
                          np.eye(ndn) * vals[feid - 1, qpid - 1])
        oc = np.stack([[np.eye(ndn) * v for v in row] for row in vals]).reshape(
            fes.count(), npts, ndn * ndn)
        kind = 2
    M = ft.bilform_masslike(femm, geom, u, cf, m=m)
    _, Ns, dN, w, pc = femm.integdomain.integrationdata()
    Mr = O.bilform_masslike(fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc, w, oc,
                            coef_kind=kind, otherdim=femm.integdomain.otherdimension, m=m)
    assert M.shape == (fes.count() * ndn, u.nalldofs()) == Mr.shape
    assert M.nnz == Mr.nnz == fes.count() * ndn * fes.nne * ndn
    compare(M, Mr)
    # each element row integrates its basis functions (partition of unity):
    # the row sums of the scalar case are the element measures times c
    if ndn == 1 and coef == "const":
        assert np.all(np.asarray(M.sum(axis=1)).ravel() > 0)


def test_masslike_errors(ft):
    _, fens, fes, femm, geom = _masslike_case(ft, "H8")
    u = _field(ft, fens.count(), 1)
    with pytest.raises(ValueError, match="rectangular"):
        ft.bilform_masslike(femm, ft.SysmatAssemblerGPU(symmetric=True), geom, u,
                            ft.DataCache(1.0))
    with pytest.raises(ft.FegpuError, match="only acceptable"):
        ft.bilform_masslike(femm, geom, u, ft.DataCache(1.0), m=2)


# ---------------------------------------------------------------- FF block
def test_ffblock_assembler(ft, O):
    """SysmatAssemblerFFBlock (src/AssemblyModule.jl:1144-1236): the device
    forms, the generic protocol and masslike return the free-free block of
    what the wrapped assembler makes."""
    fens, fes = ft.H8block(1.0, 0.8, 0.6, 3, 3, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    geom = ft.NodalField(fens.xyz)
    on_face = np.flatnonzero(np.abs(fens.xyz[:, 0]) < 1e-12) + 1
    u = ft.NodalField(np.zeros((fens.count(), 3)))
    ft.setebc(u, on_face, True, [1, 2], 0.0)
    ft.numberdofs(u)
    nf = u.nfreedofs()
    D = ft.DataCache(ft.isotropic_D(1.0, 0.3))
    full = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(symmetric=False), geom, u,
                                  ft.DeforModelRed3D, D).tocsc()
    B = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerFFBlockGPU(nf), geom, u,
                               ft.DeforModelRed3D, D)
    R = full[:nf, :nf].tocsc()
    assert B.shape == (nf, nf)
    assert np.array_equal(B.indptr, R.indptr) and np.array_equal(B.indices, R.indices)
    assert np.array_equal(B.data, R.data)
    # symmetric wrapped assembler: exact zeros of S + S' are not stored
    Bs = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerFFBlockGPU(
        ft.SysmatAssemblerGPU(symmetric=True), nf), geom, u, ft.DeforModelRed3D, D)
    Rs = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(symmetric=True), geom, u,
                                ft.DeforModelRed3D, D).tocsc()[:nf, :nf]
    Rs.eliminate_zeros()
    assert Bs.nnz == Rs.nnz and abs(Bs - Rs).max() == 0.0
    # the generic protocol
    rng = np.random.default_rng(5)
    a = ft.SysmatAssemblerFFBlockGPU(7, 5)
    a.startassembly(4, 4, 10, 11, 9)
    o = O.Assembler(False, 11, 9)
    for _ in range(10):
        Mk = rng.uniform(-1, 1, (4, 4))
        r, c = rng.permutation(11)[:4] + 1, rng.permutation(9)[:4] + 1
        a.assemble(Mk, r, c)
        o.assemble(Mk, r, c)
    A = a.makematrix()
    Ar = o.make().tocsc()[:7, :5]
    assert A.shape == (7, 5) and A.nnz == Ar.nnz and abs(A - Ar).max() == 0.0
    # masslike through the block assembler
    q = _field(ft, fens.count(), 1)
    Mfull = ft.bilform_masslike(femm, geom, q, ft.DataCache(1.0))
    Mb = ft.bilform_masslike(femm, ft.SysmatAssemblerFFBlockGPU(10, 30), geom, q,
                             ft.DataCache(1.0))
    assert Mb.shape == (10, 30) and abs(Mb - Mfull.tocsc()[:10, :30]).max() == 0.0


def test_generic_assembler_rectangular(ft, O):
    """SysmatAssemblerSparse with rows != columns and repeated DOFs (sums in
    input order) through the device makematrix! and CSC export."""
    rng = np.random.default_rng(8)
    a = ft.SysmatAssemblerGPU(symmetric=False)
    a.startassembly(3, 5, 300, 41, 67)
    o = O.Assembler(False, 41, 67)
    for _ in range(300):
        Mk = rng.uniform(-1, 1, (3, 5))
        r = rng.integers(1, 42, 3)
        c = rng.integers(1, 68, 5)
        a.assemble(Mk, r, c)
        o.assemble(Mk, r, c)
    A = a.makematrix()
    Ar = o.make()
    assert A.shape == Ar.shape == (41, 67)
    A, Ar = A.tocsc(), Ar.tocsc()
    assert np.array_equal(A.indptr, Ar.indptr) and np.array_equal(A.indices, Ar.indices)
    assert np.array_equal(A.data, Ar.data)


def test_async_export_pipeline(ft):
    """fegpu_matrix_copy_values_async: two matrices of one dofmap assembled in
    turn while the other's values travel to the host; a form that writes a
    matrix waits for its copy in flight, so every exported buffer holds the
    values of its own assembly."""
    import ctypes as C
    import torch
    nat = ft._native
    L = nat.load()
    fens, fes = ft.H8block(1.0, 0.8, 0.6, 6, 5, 4)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    asm = ft.SysmatAssemblerGPU(result="device")
    K = ft.bilform_lin_elastic(femm, asm, geom, u, ft.DeforModelRed3D,
                               ft.DataCache(ft.isotropic_D(1.0, 0.3)))
    nnz = K.dm.nnz
    k2 = C.c_void_p()
    nat.check(L.fegpu_matrix_create(K.dm.h, C.byref(k2)))
    mats = [K.h, k2.value]
    bufs = [torch.empty(nnz, dtype=torch.float64, pin_memory=True).numpy() for _ in range(4)]
    scales = [1.0, 2.0, 3.0, 4.0]
    try:
        for i, sc in enumerate(scales):
            D = np.ascontiguousarray(ft.isotropic_D(sc, 0.3).ravel())
            cf = nat.Coef(nat.COEF_CONST, 36, D.ctypes.data)
            nat.check(L.fegpu_bilform_lin_elastic(mats[i & 1], C.byref(cf), nat.FP64))
            nat.check(L.fegpu_matrix_copy_values_async(mats[i & 1], bufs[i].ctypes.data))
        for h in mats:
            nat.check(L.fegpu_matrix_wait_export(h))
        last2 = np.empty(nnz)
        nat.check(L.fegpu_matrix_copy_values(k2.value, nat.ptr(last2)))
    finally:
        nat.check(L.fegpu_matrix_destroy(k2.value))
    # each buffer holds exactly the values of its own assembly
    assert np.array_equal(K.values(), bufs[2]) and np.array_equal(last2, bufs[3])
    # the elasticity matrix is linear in E: buffer i = scale_i x buffer 0 (to
    # rounding; entries formed by cancellation get an absolute bound)
    top = np.abs(bufs[0]).max()
    for i, sc in enumerate(scales):
        assert np.allclose(bufs[i], sc * bufs[0], rtol=1e-12, atol=1e-13 * sc * top)


@pytest.mark.parametrize("et", ["H20", "T10", "H8", "T4", "H20_mirrored"])
def test_mixed_tensor_core_blocks(ft, et, monkeypatch):
    """The tensor-core element blocks (tcgen05 kind::tf32, split hi/lo
    operands) against the FP64 path, beside the FP32-pipe blocks: both within
    the mixed tolerance, exactly symmetric, and not the same arithmetic.  The
    mirrored mesh (every det J < 0) takes the two-operand products instead of
    the symmetric rank-K ones."""
    rng = np.random.default_rng(9)
    if et.startswith("H20"):
        fens, fes, _ = ft.h20_elastic_mesh(n=4, distort_fraction=0.05)
        if et == "H20_mirrored":
            fens.xyz = fens.xyz * np.array([-1.0, 1.0, 1.0])
        r = ft.GaussRule(3, 3)
    elif et == "T10":
        fens, fes = ft.t10_elastic_mesh(n=3)
        r = ft.TetRule(4)
    elif et == "H8":
        fens, fes = ft.H8block(1.0, 0.8, 0.6, 5, 4, 3)
        fens.xyz = ft.meshes.jitter_interior(fens.xyz, (5, 4, 3), 0.2, 3, box=(1.0, 0.8, 0.6))
        r = ft.GaussRule(3, 3)
    else:
        fens, fes = ft.T4block(1.0, 0.8, 0.6, 4, 3, 3)
        fens.xyz = ft.meshes.jitter_interior(fens.xyz, (4, 3, 3), 0.2, 3, box=(1.0, 0.8, 0.6))
        r = ft.TetRule(1)
    femm = ft.FEMMBase(ft.IntegDomain(fes, r))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    E = rng.lognormal(np.log(70e9), 0.5, fes.count())
    nu = rng.uniform(0.2, 0.35, fes.count())
    cf = ft.IsotropicElementwise(E, nu)
    K64 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(), geom, u, ft.DeforModelRed3D, cf)
    out = {}
    for flag in ("1", "0"):  # tensor-core blocks (opt-in) and the default FP32-pipe tile
        monkeypatch.setenv("FEGPU_MIXED_TC", flag)
        out[flag] = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="mixed"), geom,
                                           u, ft.DeforModelRed3D, cf)
    x = rng.uniform(-1, 1, K64.shape[0])
    for flag, K in out.items():
        err_kx = np.linalg.norm((K - K64) @ x) / np.linalg.norm(K64 @ x)
        err_max = abs(K - K64).max() / abs(K64).max()
        assert err_kx <= MIXED_TOL and err_max <= MIXED_TOL, (flag, err_kx, err_max)
        mixed_gate(K, K64)
        assert abs(K - K.T).max() == 0.0
    assert abs(out["1"] - out["0"]).max() > 0.0


# ------------------------------------------------- reference identities on the GPU
@pytest.mark.parametrize("idx", range(3))
def test_div_grad_reference_identities(ft, kats, idx):
    """test/test_forms.jl mbilform_div_grad_1..3 through the GPU entry point:
    no energy for a constant velocity, 2 mu V |sym grad u|^2 for a linear
    one, the elasticity energy with C = diag(2mu x3, mu x3) for a polynomial
    one; the reference's default (unsymmetric) assembler."""
    rec = kats["div_grad"][idx]
    L, W, t, nl, nw, nt = rec["block"]
    fens, fes = ft.H8block(L, W, t, nl, nw, nt)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, rec["gauss_order"])))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    mu, V, tol = rec["mu"], rec["volume"], rec["tol"]
    G = ft.bilform_div_grad(femm, geom, u, ft.DataCache(mu))
    x, y, z = fens.xyz[:, 0], fens.xyz[:, 1], fens.xyz[:, 2]
    if rec["kind"] == "constant_field":
        v = np.tile(rec["uxyz"], fens.count())
        assert abs(v @ G @ v) / V <= tol
        return
    a, b, c, d = rec["abcd"]
    if rec["kind"] == "linear_field":
        U = np.stack([a + b * x + c * y + d * z, b + c * x + d * y + a * z,
                      c + d * x + a * y + b * z], axis=1)
        gradu = np.array([[b, c, d], [c, d, a], [d, a, b]])
        exact = 2 * mu * V * (((gradu + gradu.T) / 2) ** 2).sum()
        v = U.ravel()
        assert abs(v @ G @ v - exact) / exact <= tol
    else:
        U = np.stack([a + b * x ** 2 + c * y ** 3 + d * z, b + c * x + d * y ** 2 + a * z ** 4,
                      c + d * x ** 3 + a * y + b * z ** 2], axis=1)
        C = np.diag([2 * mu] * 3 + [mu] * 3)
        G2 = ft.bilform_lin_elastic(femm, geom, u, ft.DeforModelRed3D, ft.DataCache(C))
        v = U.ravel()
        e1, e2 = v @ G @ v, v @ G2 @ v
        assert abs(e1 - e2) / e1 <= tol


def test_ffblock_reference_case(ft, kats):
    """test/test_forms.jl mbilform_diffusion_assembly_1: the free-free block by
    SysmatAssemblerFFBlock equals matrix_blocked_ff of the full matrix (here
    exactly, and the reference's energy check)."""
    k = kats["ffblock"]
    L, W, t, nl, nw, nt = k["block"]
    fens, fes = ft.H8block(L, W, t, nl, nw, nt)
    geom = ft.NodalField(fens.xyz)
    psi = ft.NodalField(np.ones((fens.count(), 1)))
    ft.setebc(psi, k["fixed_nodes"], True, [1] * len(k["fixed_nodes"]), 0.0)
    ft.numberdofs(psi)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, k["gauss_order"])))
    v_f = ft.gathersysvec(psi)
    cf = ft.DataCache(np.eye(3))
    K = ft.bilform_diffusion(femm, geom, psi, cf)
    K_ff = ft.matrix_blocked_ff(K, psi.nfreedofs())
    result = abs(v_f @ K_ff @ v_f)
    B = ft.bilform_diffusion(femm, ft.SysmatAssemblerFFBlockGPU(psi.nfreedofs()), geom, psi, cf)
    assert B.shape == K_ff.shape
    assert abs(v_f @ B @ v_f - result) <= k["tol"] * max(result, 1e-300)


def test_generic_vector_assembly(ft):
    """SysvecAssembler's generic protocol (src/AssemblyModule.jl:885-917) on
    the device: element vectors summed into the global vector in assembly
    order (the same numbers as a host accumulation), bounds errors with the
    reference's messages, and the free block (SysvecAssemblerFBlock)."""
    rng = np.random.default_rng(12)
    n = 57
    a = ft.SysvecAssemblerGPU()
    a.startassembly(n)
    ref = np.zeros(n)
    for _ in range(200):
        k = int(rng.integers(1, 9))
        v = rng.uniform(-1, 1, k)
        d = rng.integers(1, n + 1, k)
        a.assemble(v, d)
        for vi, di in zip(v, d):
            ref[di - 1] += vi
    F = a.makevector()
    assert np.array_equal(F, ref)
    b = ft.SysvecAssemblerFBlockGPU(40)
    b.startassembly(n)
    b.assemble(np.array([1.0, 2.0]), np.array([3, 50]))
    Fb = b.makevector()
    assert Fb.shape == (40,) and Fb[2] == 1.0 and Fb.sum() == 1.0
    a.startassembly(n)
    with pytest.raises(ft.FegpuError, match="Row degree of freedom > size"):
        a.assemble(np.array([1.0]), np.array([n + 1]))


def test_linform_free_block(ft):
    """linform_dot through SysvecAssemblerFBlock: the free part of the full
    load vector."""
    fens, fes = ft.H8block(1.0, 0.8, 0.6, 3, 3, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    geom = ft.NodalField(fens.xyz)
    u = ft.NodalField(np.zeros((fens.count(), 3)))
    ft.setebc(u, np.flatnonzero(np.abs(fens.xyz[:, 0]) < 1e-12) + 1, True, [1], 0.0)
    ft.numberdofs(u)
    f = ft.DataCache(np.array([1.0, -2.0, 0.5]))
    F = ft.linform_dot(femm, geom, u, f, 3)
    Ff = ft.linform_dot(femm, ft.SysvecAssemblerFBlockGPU(u.nfreedofs()), geom, u, f, 3)
    assert np.array_equal(Ff, F[:u.nfreedofs()])


@pytest.mark.parametrize("form", ["diffusion", "elasticity"])
def test_material_frame(ft, O, form):
    """A constant material frame (CSys with a rotation matrix,
    src/CSysModule.jl): the oracle follows the reference (gradients in the
    frame, RmTJ = Rm' J, blmat! with Rm); the device forms take the
    coefficient rotated to global coordinates."""
    rng = np.random.default_rng(23)
    fens, fes = ft.H8block(1.0, 0.7, 1.3, 3, 2, 2)
    fens.xyz = ft.meshes.jitter_interior(fens.xyz, (3, 2, 2), 0.15, 5, box=(1.0, 0.7, 1.3))
    Q, _ = np.linalg.qr(rng.normal(size=(3, 3)))
    R = Q * np.sign(np.linalg.det(Q))           # a proper rotation
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)), mcsys=ft.CSys(R))
    geom = ft.NodalField(fens.xyz)
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    if form == "diffusion":
        kap = np.diag([3.0, 1.0, 0.2])
        kap[0, 1] = kap[1, 0] = 0.4
        u = _field(ft, fens.count(), 1)
        K = ft.bilform_diffusion(femm, geom, u, ft.DataCache(kap))
        Kr = O.bilform(O.DIFFUSION, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(),
                       pc, w, kap, rm=R)
    else:
        D = np.zeros((6, 6))
        D[:3, :3] = [[12.0, 3.0, 2.0], [3.0, 9.0, 2.5], [2.0, 2.5, 7.0]]
        D[3, 3], D[4, 4], D[5, 5] = 3.0, 2.0, 2.6
        u = _field(ft, fens.count(), 3)
        K = ft.bilform_lin_elastic(femm, geom, u, ft.DeforModelRed3D, ft.DataCache(D))
        Kr = O.bilform(O.LIN_ELASTIC, fes.code, fes.conn, geom.values, u.dofnums,
                       u.nalldofs(), pc, w, D, rm=R)
    compare(K, Kr, structure=False)
    # the frame matters: the identity frame gives another matrix
    femm0 = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    if form == "diffusion":
        K0 = ft.bilform_diffusion(femm0, geom, u, ft.DataCache(kap))
    else:
        K0 = ft.bilform_lin_elastic(femm0, geom, u, ft.DeforModelRed3D, ft.DataCache(D))
    assert abs(K - K0).max() > 1e-3 * abs(K).max()


@pytest.mark.parametrize("et,form,order", [("H8", "elasticity", 4), ("H20", "diffusion", 4),
                                           ("H8", "diffusion", 6), ("Q4", "dot", 6)])
def test_high_order_gauss_rules(ft, O, et, form, order):
    """Gauss rules beyond order 3 (the reference tabulates orders 1-10): the
    FP64 forms against the oracle with the same tables, and the mixed path
    (smaller tiles for the larger tables) within the mixed bound."""
    rng = np.random.default_rng(31)
    if et == "Q4":
        fens, fes = ft.Q4block(2.0, 1.5, 5, 4)
        xyz = np.hstack([fens.xyz, rng.uniform(-0.05, 0.05, (fens.count(), 1))])
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, order), 0.01))
    else:
        gen = ft.H8block if et == "H8" else ft.H20block
        fens, fes = gen(1.0, 0.7, 1.3, 3, 2, 2)
        xyz = ft.meshes.jitter_interior(fens.xyz, (3, 2, 2), 0.15, 4, box=(1.0, 0.7, 1.3))
        if et == "H20":
            fens.xyz = xyz
            xyz = ft.meshes.recompute_midpoints(fens, fes, 0).xyz
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, order)))
    geom = ft.NodalField(xyz)
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    assert npts == order ** (2 if et == "Q4" else 3)
    od = femm.integdomain.otherdimension
    if form == "elasticity":
        u = _field(ft, fens.count(), 3)
        D = ft.isotropic_D(1.0, 0.3)
        K = ft.bilform_lin_elastic(femm, geom, u, ft.DeforModelRed3D, ft.DataCache(D))
        Kr = O.bilform(O.LIN_ELASTIC, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(),
                       pc, w, D)
        K32 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="mixed"), geom, u,
                                     ft.DeforModelRed3D, ft.DataCache(D))
        x = rng.uniform(-1, 1, K.shape[0])
        assert np.linalg.norm((K32 - K) @ x) <= MIXED_TOL * np.linalg.norm(K @ x)
        mixed_gate(K32, K)
    elif form == "diffusion":
        u = _field(ft, fens.count(), 1)
        K = ft.bilform_diffusion(femm, geom, u, ft.DataCache(1.3))
        Kr = O.bilform(O.DIFFUSION, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(),
                       pc, w, np.array([1.3]))
    else:
        u = _field(ft, fens.count(), 1)
        K = ft.bilform_dot(femm, geom, u, ft.DataCache(np.eye(1) * 2.0))
        Kr = O.bilform(O.DOT, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc, w,
                       np.eye(1) * 2.0, otherdim=od, m=3)
    compare(K, Kr)


def test_rule_too_large_is_refused(ft):
    """A rule whose per-element tables exceed a CTA's shared memory is refused
    with an error, not run."""
    fens, fes = ft.H20block(1.0, 1.0, 1.0, 2, 2, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 10)))
    u = _field(ft, fens.count(), 3)
    with pytest.raises(ft.FegpuError, match="too large"):
        ft.bilform_lin_elastic(femm, ft.NodalField(fens.xyz), u, ft.DeforModelRed3D,
                               ft.DataCache(ft.isotropic_D(1.0, 0.3)))


def _axisym_case(ft, kats, jitter=True):
    k = kats["axisymmetric"]
    fens, fes = ft.Q4block(k["a"], k["b"], k["na"] + 3, k["nb"] + 2)
    if jitter:
        fens.xyz = ft.meshes.jitter_interior(fens.xyz, (k["na"] + 3, k["nb"] + 2), 0.15, 9,
                                             box=(k["a"], k["b"]))
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, k["gauss_order"]), True))
    return k, fens, fes, femm, ft.NodalField(fens.xyz)


def test_axisymmetric_volume(ft, kats):
    """test/test_basics.jl mbas010x1 through the GPU forms: the rectangle
    revolved about the axis has volume pi a^2 b (1' M 1 of bilform_dot with
    m = 3), FP64 and mixed; m = 2 measures the area."""
    k, fens, fes, femm, geom = _axisym_case(ft, kats, jitter=False)
    u = _field(ft, fens.count(), 1)
    one = np.ones(fens.count())
    V = np.pi * k["a"] ** 2 * k["b"]
    for prec in ("fp64", "mixed"):
        M = ft.bilform_dot(femm, ft.SysmatAssemblerGPU(precision=prec), geom, u,
                           ft.DataCache(np.eye(1)), m=3)
        assert abs(one @ M @ one - V) <= (1e-12 if prec == "fp64" else 1e-6) * V
    S = ft.bilform_dot(femm, geom, u, ft.DataCache(np.eye(1)), m=2)
    assert abs(one @ S @ one - k["a"] * k["b"]) <= 1e-12 * k["a"] * k["b"]


@pytest.mark.parametrize("form", ["dot", "diffusion", "diffusion_general", "linform", "lumped",
                                  "masslike", "convection"])
def test_axisymmetric_forms(ft, O, kats, form):
    """Axisymmetric Q4 domains (2 pi r in place of the other dimension) for
    every form that measures a two-manifold as a volume, against the oracle;
    the mixed path within the mixed bound."""
    k, fens, fes, femm, geom = _axisym_case(ft, kats)
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    n = fens.count()
    kw = dict(otherdim=1.0, axisymmetric=True)
    if form == "dot":
        u = _field(ft, n, 3)
        c = np.diag([1.0, 2.0, 3.0])
        K = ft.bilform_dot(femm, geom, u, ft.DataCache(c), m=3)
        Kr = O.bilform(O.DOT, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc, w, c,
                       m=3, **kw)
        K32 = ft.bilform_dot(femm, ft.SysmatAssemblerGPU(precision="mixed"), geom, u,
                             ft.DataCache(c), m=3)
    elif form in ("diffusion", "diffusion_general"):
        u = _field(ft, n, 1)
        c = 1.7 if form == "diffusion" else np.array([[2.0, 0.3], [0.3, 1.0]])
        K = ft.bilform_diffusion(femm, geom, u, ft.DataCache(c))
        Kr = O.bilform(O.DIFFUSION, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(),
                       pc, w, np.atleast_1d(c), **kw)
        K32 = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(precision="mixed"), geom, u,
                                   ft.DataCache(c))
    elif form == "linform":
        u = _field(ft, n, 2)
        f = np.array([1.0, -0.5])
        F = ft.linform_dot(femm, geom, u, ft.DataCache(f), 3)
        Fr = O.linform_dot(fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc, w, f,
                           m=3, **kw)
        assert np.allclose(F, Fr, rtol=1e-12, atol=1e-14 * np.abs(Fr).max())
        return
    elif form == "lumped":
        u = _field(ft, n, 1)
        K = ft.bilform_dot(femm, ft.SysmatAssemblerSparseHRZLumpingSymmGPU(), geom, u,
                           ft.DataCache(np.eye(1) * 7.0), m=3)
        Kr = O.bilform(O.DOT, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc, w,
                       np.eye(1) * 7.0, m=3, asm=O.ASM_HRZ, **kw)
        compare(K, Kr)
        return
    elif form == "masslike":
        u = _field(ft, n, 1)
        K = ft.bilform_masslike(femm, geom, u, ft.DataCache(np.eye(1) * 2.0))
        Kr = O.bilform_masslike(fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc, w,
                                np.eye(1) * 2.0, **kw)
        compare(K, Kr)
        return
    else:
        q = _field(ft, n, 1)
        vel = ft.NodalField(np.column_stack([np.full(n, 0.7), np.full(n, -1.1)]))
        K = ft.bilform_convection(femm, geom, vel, q, ft.DataCache(1.0))
        Kr = O.bilform_convection(fes.code, fes.conn, geom.values, q.dofnums, q.nalldofs(), pc,
                                  w, vel.values, **kw)
        compare(K, Kr)
        return
    compare(K, Kr)
    x = np.random.default_rng(5).uniform(-1, 1, K.shape[0])
    assert np.linalg.norm((K32 - K) @ x) <= MIXED_TOL * np.linalg.norm(K @ x)
    mixed_gate(K32, K)


def test_integer_unit_addition_matches_fp64_unit(ft):
    """sf_add (the T10 elasticity kernel's point sums on the integer units)
    against the FP64 unit's __dadd_rn on the device: 4 million operand pairs
    of four kinds (uniform bit patterns, exponent differences 0..70,
    near-cancellations, ties to even), every result equal in every bit."""
    import ctypes as C
    from importlib import import_module
    nat = import_module(ft.__name__ + "._native")
    L = nat.load()
    bad, first = C.c_int64(), C.c_int64()
    for seed in (1, 20261204):
        nat.check(L.fegpu_selftest_soft_add(nat.context(0), 4_000_000, seed, C.byref(bad),
                                            C.byref(first)))
        assert bad.value == 0 and first.value == -1, (seed, bad.value, first.value)
