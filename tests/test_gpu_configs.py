"""Entry-by-entry parity at the benchmark configurations themselves.

The reference-order FP64 path (precision "fp64", the drop-in default) is run
through the C ABI on the seeded configuration meshes and compared with the
CPU oracle, which restates the reference's bilform_* + makematrix!
(src/FEMMBaseModule.jl:1462-1545, 1774-1824; src/AssemblyModule.jl:454-583),
on the same inputs (mesh, coefficients and the integrationdata() tables the
library is handed):
  - H8 20^3 diffusion, interior nodes jittered +-0.2 h, isotropic (1.0) and
    general (the identity 3x3) conductivity;
  - T10 24^3 linear elasticity with the T10 60^3 configuration's jitter
    (+-0.15 h, boundary nodes on the block faces), E = 210e9, nu = 0.3:
    the mesh on which S + S' meets exact zeros;
  - H20 40^3 linear elasticity in FP64 (the mixed configuration's mesh: +-0.25 h
    jitter, 1 % of the elements distorted to det J ratio < 0.05, per-element
    lognormal E and uniform nu).
For each: colptr / rowval bit-exact against the symmetric assembler's result
(exact zeros left out as the reference leaves them out, with the same count),
every value equal bit for bit, hence |dK| <= 1e-12 |K| per nonzero and
|dK x| <= 1e-12 |K x|, which are asserted as well.
"""
import numpy as np
import pytest

from test_gpu_parity import bitwise, compare

pytestmark = pytest.mark.gpu


def _field(ft, n, ndn):
    return ft.numberdofs(ft.NodalField(np.zeros((n, ndn))))


def _check(ft, O, femm, fes, geom, u, form, cf, oc, okind):
    npts, Ns, dN, w, pc = femm.integdomain.integrationdata()
    ofm = O.DIFFUSION if form == "diffusion" else O.LIN_ELASTIC
    Kr, dropped, _ = O.bilform(ofm, fes.code, fes.conn, geom.values, u.dofnums, u.nalldofs(), pc,
                               w, oc, coef_kind=okind, phases=True, tables=(Ns, dN))
    asm = ft.SysmatAssemblerGPU(result="device")
    if form == "diffusion":
        M = ft.bilform_diffusion(femm, asm, geom, u, cf)
    else:
        M = ft.bilform_lin_elastic(femm, asm, geom, u, ft.DeforModelRed3D, cf)
    K = M.to_scipy()
    assert M.nnz(drop_zeros=False) - M.nnz(drop_zeros=True) == dropped
    bitwise(K, Kr)
    raw, gate, kx = compare(K, Kr)
    assert raw == 0.0 and kx == 0.0
    return K.nnz, dropped


@pytest.mark.parametrize("coef", ["iso", "general"])
def test_config_h8_20_diffusion(ft, O, coef):
    fens, fes = ft.h8_diffusion_mesh(n=20, seed=1)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 1)
    if coef == "iso":
        cf, oc = ft.DataCache(1.0), np.array([1.0])
    else:
        cf, oc = ft.DataCache(np.eye(3)), np.eye(3)
    nnz, _ = _check(ft, O, femm, fes, geom, u, "diffusion", cf, oc, O.COEF_CONST)
    assert nnz == 226981


def test_config_t10_24_elasticity(ft, O):
    fens, fes = ft.t10_elastic_mesh(n=24, seed=2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    D = ft.isotropic_D(210e9, 0.3)
    _, dropped = _check(ft, O, femm, fes, geom, u, "elasticity", ft.DataCache(D), D, O.COEF_CONST)
    assert dropped > 0


def test_config_h20_40_elasticity_fp64(ft, O):
    fens, fes, flagged = ft.h20_elastic_mesh(n=40)
    assert len(flagged) > 0
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 3)))
    geom = ft.NodalField(fens.xyz)
    u = _field(ft, fens.count(), 3)
    rng = np.random.default_rng(4)
    E = rng.lognormal(np.log(70e9), 0.5, fes.count())
    nu = rng.uniform(0.2, 0.35, fes.count())
    cf = ft.IsotropicElementwise(E, nu)
    oc = np.stack([ft.isotropic_D(a, b) for a, b in zip(E, nu)]).reshape(-1, 36)
    nnz, _ = _check(ft, O, femm, fes, geom, u, "elasticity", cf, oc, O.COEF_PER_ELEMENT)
    assert nnz == 136823049
