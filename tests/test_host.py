"""Host-side logic of the package, checked against the oracle (no GPU)."""
import numpy as np
import pytest


@pytest.mark.parametrize("gen,et", [("H8block", "H8"), ("H20block", "H20"), ("T4block", "T4"),
                                    ("T10block", "T10")])
@pytest.mark.parametrize("blk", [(12.0, 1.1, 0.32, 2, 4, 3), (1.0, 1.0, 1.0, 3, 3, 3),
                                 (25.0, 50.0, 50.0, 5, 4, 3)])
def test_generators_match_oracle(ft, O, gen, et, blk):
    fens, fes = getattr(ft, gen)(*blk)
    xyz, conn = O.block(getattr(O, et), *blk)
    assert np.array_equal(fes.conn, conn)
    assert np.array_equal(fens.xyz, xyz)


def test_q4_generator_matches_oracle(ft, O):
    fens, fes = ft.Q4block(3.0, 2.0, 3, 4)
    xyz, conn = O.q4blockx(O.linearspace(0, 3.0, 4), O.linearspace(0, 2.0, 5))
    assert np.array_equal(fes.conn, conn) and np.array_equal(fens.xyz, xyz)


@pytest.mark.parametrize("n,L", [(2, 12.0), (4, 1.1), (33, 7.32), (61, 1.0)])
def test_linearspace(ft, O, n, L):
    a = ft.linearspace(0.0, L, n)
    b = O.linearspace(0.0, L, n)
    assert np.abs(a - b).max() <= 2 * np.finfo(float).eps * L


@pytest.mark.parametrize("cls,et,rule", [("FESetH8", "H8", ("G", 3, 3)), ("FESetH20", "H20", ("G", 3, 3)),
                                         ("FESetT4", "T4", ("T", 4)), ("FESetT10", "T10", ("T", 5)),
                                         ("FESetQ4", "Q4", ("G", 2, 3))])
def test_basis_functions(ft, O, cls, et, rule):
    r = ft.GaussRule(*rule[1:]) if rule[0] == "G" else ft.TetRule(rule[1])
    fs = getattr(ft, cls)(np.zeros((0, getattr(ft, cls).nne), dtype=np.int64))
    for p in r.param_coords:
        assert np.abs(fs.bfun(p).ravel() - O.bfun(getattr(O, et), p)).max() <= 1e-15
        assert np.abs(fs.bfundpar(p) - O.bfundpar(getattr(O, et), p)).max() <= 1e-15


@pytest.mark.parametrize("dim,order", [(1, 2), (2, 2), (2, 3), (3, 2), (3, 3)])
def test_gauss_rule(ft, O, dim, order):
    r = ft.GaussRule(dim, order)
    pc, w = O.gauss_rule(dim, order)
    assert np.array_equal(r.param_coords, pc) and np.array_equal(r.weights, w)


@pytest.mark.parametrize("npts", [1, 4])
def test_tet_rule(ft, O, npts):
    r = ft.TetRule(npts)
    pc, w = O.tet_rule(npts)
    assert np.array_equal(r.param_coords, pc) and np.array_equal(r.weights, w)


def test_numberdofs_free_then_fixed(ft):
    # src/FieldModule.jl:328-377: free DOFs node by node, then the fixed ones
    u = ft.NodalField(np.zeros((4, 3)))
    ft.setebc(u, [2], True, [2], 0.0)
    ft.setebc(u, [4], True, [1], 0.0)
    ft.numberdofs(u)
    assert u.nfreedofs() == 10 and u.nalldofs() == 12
    assert u.dofnums.tolist() == [[1, 2, 3], [4, 11, 5], [6, 7, 8], [12, 9, 10]]


def test_numberdofs_permuted(ft):
    u = ft.NodalField(np.zeros((3, 1)))
    ft.numberdofs(u, entperm=[3, 1, 2])
    assert u.dofnums.ravel().tolist() == [2, 3, 1]


def test_datacache_semantics(ft):
    # test/test_miscellaneous.jl vectorcachetest1/2
    c = ft.DataCache([10.0])
    assert list(c(np.zeros((1, 2)), np.zeros((2, 1)), 0, 1)) == [10.0]

    def fill(v, XYZ, tangents, feid, qpid):
        return np.array([10.0 + feid])
    c = ft.DataCache(np.array([1.0]), fill)
    assert list(c(np.zeros((1, 2)), np.zeros((2, 1)), 3, 1)) == [13.0]


@pytest.mark.parametrize("maker", ["h8", "t10", "h20"])
def test_synthetic_meshes_valid(ft, maker):
    """The seeded benchmark meshes (small versions) have positive Jacobians."""
    if maker == "h8":
        fens, fes = ft.h8_diffusion_mesh(n=6)
        rule = ft.GaussRule(3, 2)
    elif maker == "t10":
        fens, fes = ft.t10_elastic_mesh(n=6)
        rule = ft.TetRule(4)
    else:
        fens, fes, flagged = ft.h20_elastic_mesh(n=6, distort_fraction=0.05)
        rule = ft.GaussRule(3, 3)
        assert len(flagged) >= 1
    dN = np.stack([fes.bfundpar(p) for p in rule.param_coords])
    X = fens.xyz[fes.conn - 1]
    dets = np.linalg.det(np.einsum("eks,qkm->eqsm", X, dN))
    assert dets.min() > 0
    if maker == "h20":
        r = dets.min(axis=1) / dets.mean(axis=1)
        assert (r[flagged] < 0.05).all()


def test_element_coloring_restatement(ft, O):
    """The library's colouring equals the restated reference colouring; checked
    through the oracle on the host side only (the GPU test checks the library)."""
    fens, fes = ft.T4block(1.0, 1.0, 1.0, 4, 3, 5)
    col, nc = O.element_coloring(fes.conn, fens.count())
    assert nc >= 1 and col.min() == 1


def test_vector_blocked(ft):
    """vector_blocked_f / _d (src/MatrixUtilityModule.jl:807-855): the free
    and data parts; too many free DOFs is an error."""
    v = np.arange(7.0)
    assert np.array_equal(ft.vector_blocked_f(v, 3), v[:3])
    assert np.array_equal(ft.vector_blocked_d(v, 3), v[3:])
    assert ft.vector_blocked_f(v, 0).size == 0 and ft.vector_blocked_d(v, 7).size == 0
    with pytest.raises(ValueError, match="too many rows"):
        ft.vector_blocked_f(v, 8)


def test_assembler_matrix_keys_unique(ft):
    """Device matrices are keyed per assembler by a serial number, never by
    an object id that a freed assembler leaves for the next one."""
    keys = set()
    for _ in range(200):
        keys.add(ft.SysmatAssemblerGPU()._key)  # each assembler freed at once
    assert len(keys) == 200
