"""The CPU oracle against the known answers of the reference's own tests.

Every case cites the reference test it restates; the numbers come from
tests/golden/reference_kats.json (extracted from the reference test files by
tests/golden/make_golden.py).
"""
import numpy as np
import pytest


def _dense(A):
    return np.asarray(A.todense())


def test_kat_sparse_rectangular(O, kats):
    # test/test_miscellaneous.jl:1939 (mmassembly): SysmatAssemblerSparse
    k = kats["assembler"]["sparse_rect"]
    a = O.Assembler(False, 7, 7)
    for m, r, c in zip(k["mats"], k["rows"], k["cols"]):
        a.assemble(np.array(m), r, c)
    A = _dense(a.make())
    # the reference checks abs(maximum(ref - A)) < 1e-5; max-abs is stricter
    assert np.abs(np.array(k["expected"]) - A).max() < 1e-5


def test_kat_symmetric_mtm(O, kats):
    # test/test_miscellaneous.jl:1980 (mmassembly2): SysmatAssemblerSparseSymm
    k = kats["assembler"]["symm_mtm"]
    a = O.Assembler(True, 7, 7)
    for m, r, c in zip(k["mats"], k["rows"], k["cols"]):
        m = np.array(m)
        a.assemble(m.T @ m, r, c)
    A = _dense(a.make())
    assert np.abs(np.array(k["expected"]) - A).max() < 1e-5
    assert np.abs(A - A.T).max() == 0.0


def test_kat_sparse_and_symm_agree(O, kats):
    # test/test_basics.jl:78 (mmassembly2ya1)
    k = kats["assembler"]["sparse_and_symm_mtm"]
    ref = np.array(k["expected"])
    out = []
    for symm in (False, True):
        a = O.Assembler(symm, 7, 7)
        for m, d in zip(k["mats"], k["dofs"]):
            m = np.array(m)
            a.assemble(m.T @ m, d, d)
        out.append(_dense(a.make()))
    assert np.abs(ref - out[0]).max() < 1e-5
    assert np.abs(out[0] - out[1]).max() < 1e-5
    assert np.abs(ref - out[1]).max() < 1e-5


def test_kat_sparse_diag(O, kats):
    # test/test_basics.jl:135 (mmassembly2ya2): SysmatAssemblerSparseDiag keeps
    # the element diagonals: the diagonal of the full assembly
    k = kats["assembler"]["sparse_diag_mtm"]
    ref = np.array(k["expected"])
    a = O.Assembler(True, 7, 7, kind=O.ASM_DIAG)
    for m, d in zip(k["mats"], k["dofs"]):
        m = np.array(m)
        a.assemble(m.T @ m, d, d)
    A = _dense(a.make())
    assert np.abs(np.diag(np.diag(ref)) - A).max() < 1e-5


def test_hrz_lumping_recipe(O):
    # test/test_basics.jl:923-960 (mmhrzass1): the HRZ diagonal against its
    # definition, on the test's DOF lists (seeded matrix instead of rand)
    rng = np.random.default_rng(5)
    N, el = 30, rng.random((8, 8))
    el = el + el.T
    a = O.Assembler(True, N, N, kind=O.ASM_HRZ)
    ref = np.zeros(N)
    for d in ([10, 29, 15, 1, 7, 3, 6, 2], [15, 1, 7, 11, 29, 3, 8, 4],
              [25, 1, 17, 13, 30, 13, 18, 14]):
        a.assemble(el, d, d)
        f = el.sum(axis=0).sum() / np.trace(el)
        for i, dd in enumerate(d):
            ref[dd - 1] += f * el[i, i]
    M = a.make()
    assert np.abs(M.diagonal() - ref).sum() / np.linalg.norm(el) <= 1e-9


def test_kat_spot_values(O, kats):
    # test/test_basics.jl:1577 (massnomat1): entries after the deferred makematrix!
    k = kats["assembler"]["nomatrixresult"]
    a = O.Assembler(False, 7, 7)
    for m, r, c in zip(k["mats"], k["rows"], k["cols"]):
        a.assemble(np.array(m), r, c)
    A = _dense(a.make())
    for r, c, v in k["spots"]:
        assert A[r - 1, c - 1] == pytest.approx(v, rel=1e-6)


def test_assembler_errors(O):
    # src/AssemblyModule.jl:265-273, 519-524
    a = O.Assembler(True, 4, 4)
    with pytest.raises(ValueError, match="Row degree of freedom > size"):
        a.assemble(np.eye(2), [1, 5], [1, 5])
    with pytest.raises(ValueError, match="Column degree of freedom < 1"):
        a.assemble(np.eye(2), [0, 1], [0, 1])
    with pytest.raises(ValueError, match="do not agree"):
        O.Assembler(True, 4, 5)


def _block(O, gen, blk):
    et = {"H8block": O.H8, "H20block": O.H20, "T4block": O.T4, "T10block": O.T10}[gen]
    return et, O.block(et, *blk)


@pytest.mark.parametrize("key", ["coloring_h8", "coloring_t4"])
def test_kat_coloring(O, kats, key):
    # test/test_meshing.jl:7185-7244: the greedy colouring of an 11^3 block
    k = kats[key]
    et, (xyz, conn) = _block(O, k["generator"], k["block"])
    colors, nc = O.element_coloring(conn, xyz.shape[0])
    _, first = np.unique(colors, return_index=True)
    assert list(colors[np.sort(first)]) == k["unique_colors_in_order"]
    assert nc == len(k["unique_colors_in_order"])
    # no two elements of one colour share a node
    for n in range(xyz.shape[0]):
        c = colors[np.any(conn == n + 1, axis=1)]
        assert len(c) == len(np.unique(c))


def test_kat_connection_degree(O, kats):
    # test/test_miscellaneous.jl:931 (mmconnection1)
    k = kats["connection_degree"]
    _, (xyz, conn) = _block(O, k["generator"], k["block"])
    deg = O.connection_degrees(conn, xyz.shape[0])
    assert deg.max() == k["max_degree"] and deg.min() == k["min_degree"]


def _patch(O, rec):
    et, (xyz, conn) = _block(O, rec["generator"], rec["block"])
    pc, w = O.gauss_rule(3, rec["gauss_order"])
    return et, xyz, conn, pc, w


def _scalar_field(xyz):
    return np.arange(1, xyz.shape[0] + 1)


@pytest.mark.parametrize("idx", range(8))
def test_kat_patch(O, kats, idx):
    """Energy/patch identities of test/test_forms.jl and test/test_basics.jl."""
    rec = kats["patch"][idx] if idx < len(kats["patch"]) else None
    if rec is None:
        pytest.skip("no such record")
    et, xyz, conn, pc, w = _patch(O, rec)
    V, tol = rec["volume"], rec["tol"]
    n = xyz.shape[0]
    kind = rec["kind"]
    if kind == "dot_volume":
        v = np.ones(n)
        G = O.bilform(O.DOT, et, conn, xyz, _scalar_field(xyz), n, pc, w, np.eye(1))
        assert abs(v @ G @ v - V) / V <= tol
    elif kind == "dot_volume_3dof":
        v = np.ones(3 * n)
        dofs = np.arange(1, 3 * n + 1).reshape(n, 3)
        G = O.bilform(O.DOT, et, conn, xyz, dofs, 3 * n, pc, w, np.eye(3))
        assert abs(v @ G @ v - 3 * V) / V <= tol
    elif kind == "diffusion_constant_field":
        v = np.ones(n)
        K = O.bilform(O.DIFFUSION, et, conn, xyz, _scalar_field(xyz), n, pc, w, np.eye(3))
        assert abs(v @ K @ v) / V <= tol
    elif kind == "diffusion_linear_field":
        a, b, c, d = rec["abcd"]
        v = a + b * xyz[:, 0] + c * xyz[:, 1] + d * xyz[:, 2]
        K = O.bilform(O.DIFFUSION, et, conn, xyz, _scalar_field(xyz), n, pc, w, np.eye(3))
        assert abs(v @ K @ v - (b * b + c * c + d * d) * V) / V <= tol
    elif kind == "distribloads_sum":
        F = O.linform_dot(et, conn, xyz, _scalar_field(xyz), n, pc, w, np.array([rec["force"]]))
        assert abs(F.sum() - V * rec["force"]) / rec["norm"] <= tol
    elif kind == "elastic_rigid_translation":
        mu = rec["mu"]
        D = np.diag([2 * mu] * 3 + [mu] * 3)
        dofs = np.arange(1, 3 * n + 1).reshape(n, 3)
        v = np.tile(rec["uxyz"], n)
        G = O.bilform(O.LIN_ELASTIC, et, conn, xyz, dofs, 3 * n, pc, w, D)
        assert abs(v @ G @ v) / V <= tol
    elif kind == "elastic_linear_field":
        a, b, c, d = rec["abcd"]
        mu = rec["mu"]
        D = np.diag([2 * mu] * 3 + [mu] * 3)
        x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
        U = np.stack([a + b * x + c * y + d * z, b + c * x + d * y + a * z,
                      c + d * x + a * y + b * z], axis=1)
        gradu = np.array([[b, c, d], [c, d, a], [d, a, b]])
        sym = (gradu + gradu.T) / 2
        exact = 2 * mu * V * (sym ** 2).sum()
        dofs = np.arange(1, 3 * n + 1).reshape(n, 3)
        G = O.bilform(O.LIN_ELASTIC, et, conn, xyz, dofs, 3 * n, pc, w, D)
        v = U.ravel()
        assert abs(v @ G @ v - exact) / exact <= tol
    elif kind == "elastic_symmetry_linear_field":
        # test/test_forms.jl:456 (mbilform_div_grad_5): exact symmetry and the
        # energy of u = (x + 3y, y - 2z, x - 2z), here against its closed form
        mu = rec["mu"]
        D = np.diag([2 * mu] * 3 + [mu] * 3)
        dofs = np.arange(1, 3 * n + 1).reshape(n, 3)
        G = O.bilform(O.LIN_ELASTIC, et, conn, xyz, dofs, 3 * n, pc, w, D)
        assert abs(G - G.T).max() == 0.0
        x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
        v = np.stack([x + 3 * y, y - 2 * z, x - 2 * z], axis=1).ravel()
        eps = np.array([1.0, 1.0, -2.0])            # xx, yy, zz
        gam = np.array([3.0 + 0.0, 0.0 + 1.0, -2.0 + 0.0])  # xy, xz, yz (engineering)
        exact = V * (2 * mu * (eps ** 2).sum() + mu * (gam ** 2).sum())
        assert abs(v @ G @ v - exact) / exact <= tol
    else:
        pytest.fail(kind)


@pytest.mark.parametrize("et,rule", [("H8", (3, 2)), ("H20", (3, 3)), ("T4", 4), ("T10", 4),
                                     ("Q4", (2, 2))])
def test_basis_gradients_fd(O, et, rule):
    """bfundpar is the derivative of bfun (central differences)."""
    e = getattr(O, et)
    pc, _ = O.gauss_rule(*rule) if isinstance(rule, tuple) else O.tet_rule(rule)
    h = 1e-6
    for p in pc:
        G = O.bfundpar(e, p)
        N = O.bfun(e, p)
        assert abs(N.sum() - 1) < 1e-12
        for d in range(len(p)):
            dp = np.zeros_like(p)
            dp[d] = h
            fd = (O.bfun(e, p + dp) - O.bfun(e, p - dp)) / (2 * h)
            assert np.abs(fd - G[:, d]).max() < 1e-8


def test_element_kernels_vs_dense(O):
    """test/test_basics.jl:508-575: upper-triangle kernels + complete_lt! equal
    the dense products; exercised through one-element forms."""
    xyz, conn = O.block(O.H8, 1.0, 1.0, 1.0, 1, 1, 1)
    rng = np.random.default_rng(0)
    xyz = xyz + rng.uniform(-0.1, 0.1, xyz.shape)
    pc, w = O.gauss_rule(3, 2)
    dofs = np.arange(1, 9)
    kap = rng.uniform(0.5, 1.0, (3, 3))
    kap = kap + kap.T
    K = O.bilform(O.DIFFUSION, O.H8, conn, xyz, dofs, 8, pc, w, kap).toarray()
    # dense restatement: sum_q grad N kappa grad N' detJ w
    X = xyz[conn[0] - 1]
    loc = np.zeros((8, 8))
    for p, wq in zip(pc, w):
        dN = O.bfundpar(O.H8, p)
        J = X.T @ dN
        g = dN @ np.linalg.inv(J)
        loc += g @ kap @ g.T * np.linalg.det(J) * wq
    ref = np.zeros((8, 8))
    ref[np.ix_(conn[0] - 1, conn[0] - 1)] = loc
    assert np.linalg.norm(K - ref) / np.linalg.norm(ref) <= 1e-9


def test_conjugategradient_on_reference_system(O, kats):
    """The system of the reference's conjugategradient test: 20 iterations on
    the 6x6 Lehmer matrix reach the solution."""
    c = kats["conjugategradient"]
    A, b = np.array(c["A"]), np.array(c["b"])
    x = O.conjugategradient(A, b, np.zeros(len(b)), c["maxiter"])
    assert np.linalg.norm(A @ x - b) <= 1e-12 * np.linalg.norm(b)
    assert np.allclose(x, np.linalg.solve(A, b), rtol=1e-10, atol=1e-12)


def test_kat_masslike(O, kats):
    """bilform_masslike on the reference's two-element line mesh: each element
    owns one row; the row holds the integrals of the element's basis functions
    (exact equality, as the reference asserts)."""
    c = kats["masslike"]
    xyz = np.stack([c["xs"], c["ys"]], axis=1)
    conn = np.array([[i + 1, i + 2] for i in range(len(c["xs"]) - 1)], dtype=np.int64)
    dofnums = np.arange(1, len(c["xs"]) + 1, dtype=np.int64).reshape(-1, 1)
    pc, w = O.gauss_rule(1, c["gauss_order"])
    G = O.bilform_masslike(O.L2, conn, xyz, dofnums, len(c["xs"]), pc, w, np.eye(1))
    assert G.shape == (len(conn), len(c["xs"]))
    assert np.array_equal(G.toarray(), np.array(c["G"]))
    # SysmatAssemblerSparse keeps the explicit structure: one entry per
    # (element row, element DOF)
    assert G.nnz == conn.size


def _div_grad_field(rec, xyz):
    """The velocity fields of the reference's div_grad tests."""
    x, y, z = xyz[:, 0], xyz[:, 1], xyz[:, 2]
    if rec["kind"] == "constant_field":
        return np.tile(rec["uxyz"], (xyz.shape[0], 1))
    a, b, c, d = rec["abcd"]
    if rec["kind"] == "linear_field":
        return np.stack([a + b * x + c * y + d * z, b + c * x + d * y + a * z,
                         c + d * x + a * y + b * z], axis=1)
    return np.stack([a + b * x ** 2 + c * y ** 3 + d * z, b + c * x + d * y ** 2 + a * z ** 4,
                     c + d * x ** 3 + a * y + b * z ** 2], axis=1)


@pytest.mark.parametrize("idx", range(3))
def test_kat_div_grad(O, kats, idx):
    """bilform_div_grad identities of test/test_forms.jl (mbilform_div_grad_1
    to _3): no energy for a constant velocity, 2 mu V |sym grad u|^2 for a
    linear one, and the elasticity energy with C = diag(2mu x3, mu x3) for a
    polynomial one."""
    rec = kats["div_grad"][idx]
    et, (xyz, conn) = O.H8, O.block(O.H8, *rec["block"])
    pc, w = O.gauss_rule(3, rec["gauss_order"])
    n, mu, V, tol = xyz.shape[0], rec["mu"], rec["volume"], rec["tol"]
    dofs = np.arange(1, 3 * n + 1).reshape(n, 3)
    G = O.bilform(O.DIV_GRAD, et, conn, xyz, dofs, 3 * n, pc, w, np.array([mu]),
                  symmetric=False)
    v = _div_grad_field(rec, xyz).ravel()
    if rec["kind"] == "constant_field":
        assert abs(v @ G @ v) / V <= tol
    elif rec["kind"] == "linear_field":
        a, b, c, d = rec["abcd"]
        gradu = np.array([[b, c, d], [c, d, a], [d, a, b]])
        sym = (gradu + gradu.T) / 2
        exact = 2 * mu * V * (sym ** 2).sum()
        assert abs(v @ G @ v - exact) / exact <= tol
    else:
        C = np.diag([2 * mu] * 3 + [mu] * 3)
        G2 = O.bilform(O.LIN_ELASTIC, et, conn, xyz, dofs, 3 * n, pc, w, C)
        e1, e2 = v @ G @ v, v @ G2 @ v
        assert abs(e1 - e2) / e1 <= tol


def test_kat_axisymmetric_volume(O, kats):
    """test/test_basics.jl mbas010x1: the a x b rectangle revolved about the
    axis has volume pi a^2 b (there integrated on Q8; here the same identity
    through bilform_dot on Q4 of an axisymmetric domain: 1' M 1 = volume,
    exact for the rule since 2 pi r is linear)."""
    k = kats["axisymmetric"]
    xyz, conn = O.q4blockx(O.linearspace(0.0, k["a"], k["na"] + 1),
                           O.linearspace(0.0, k["b"], k["nb"] + 1))
    n = xyz.shape[0]
    pc, w = O.gauss_rule(2, k["gauss_order"])
    M = O.bilform(O.DOT, O.Q4, conn, xyz, np.arange(1, n + 1), n, pc, w, np.eye(1),
                  m=3, axisymmetric=True)
    one = np.ones(n)
    V = np.pi * k["a"] ** 2 * k["b"]
    assert abs(one @ M @ one - V) <= 1e-12 * V
    # the surface measure (m = 2) ignores the axisymmetry: the area a b
    S = O.bilform(O.DOT, O.Q4, conn, xyz, np.arange(1, n + 1), n, pc, w, np.eye(1),
                  m=2, axisymmetric=True)
    assert abs(one @ S @ one - k["a"] * k["b"]) <= 1e-12 * k["a"] * k["b"]
