"""conjugategradient on a matrix resident on the GPU (fegpu_matrix_cg)
against the oracle's restatement of the same iteration
(src/AlgoBaseModule.jl:425-445) on the same matrix.

Bar: |x_gpu - x_oracle| <= 1e-10 |x_oracle| after the same number of
iterations (the products and dot products sum in different orders), and the
iteration reduces the residual as the oracle's does on these mass matrices
(H8 2x2x2 and H20 3x3x3 Gauss: symmetric positive definite).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("et,ndn,maxiter,bound", [("H8", 1, 60, 1e-5), ("H20", 3, 20, 0.3)])
def test_cg_matches_oracle(ft, O, et, ndn, maxiter, bound):
    fens, fes = ft.nearest_block(et, 3000 if et == "H8" else 600, seed=3)
    rule = ft.GaussRule(3, 2) if et == "H8" else ft.GaussRule(3, 3)
    femm = ft.FEMMBase(ft.IntegDomain(fes, rule))
    geom = ft.NodalField(fens.xyz)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), ndn))))
    # mass matrix (SPD, well conditioned)
    M = ft.bilform_dot(femm, ft.SysmatAssemblerGPU(result="device"), geom, u,
                       ft.DataCache(np.eye(ndn) * 7.8))
    rng = np.random.default_rng(1)
    b = rng.uniform(-1, 1, M.shape[0])
    x0 = np.zeros_like(b)
    x = ft.conjugategradient(M, b, x0, maxiter)
    xr = O.conjugategradient(M.to_scipy(drop_zeros=False), b, x0, maxiter)
    assert np.linalg.norm(x - xr) <= 1e-10 * np.linalg.norm(xr)
    assert np.linalg.norm(M.spmv(x) - b) <= bound * np.linalg.norm(b)


def test_cg_zero_iterations_returns_x0(ft):
    fens, fes = ft.nearest_block("H8", 200, seed=4)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 1))))
    M = ft.bilform_dot(femm, ft.SysmatAssemblerGPU(result="device"), ft.NodalField(fens.xyz), u,
                       ft.DataCache(1.0))
    x0 = np.linspace(0, 1, M.shape[0])
    assert np.array_equal(ft.conjugategradient(M, np.ones_like(x0), x0, 0), x0)
    with pytest.raises(ValueError, match="Size mismatch"):
        ft.conjugategradient(M, np.ones(3), np.zeros(3), 5)
