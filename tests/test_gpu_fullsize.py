"""Full-size checks at the benchmark configurations, through properties that
do not need the oracle at that size: the CSR structure has exactly the
nonzero count of the configuration (pattern bit-exact), symmetric
stiffnesses are symmetric as bilinear forms, rigid-body motions are in the
kernel of the elasticity stiffness and constants in the kernel of the
diffusion stiffness, and the mixed-precision H20 matrix is within the mixed
bound of the FP64 one.  (The oracle checks the same kernels entry by entry on
smaller meshes.)"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _rigid_modes(xyz):
    """Three translations and three rotations as nodal displacement vectors
    (node-major, three DOFs per node)."""
    n = xyz.shape[0]
    c = xyz - xyz.mean(axis=0)
    modes = []
    for d in range(3):
        u = np.zeros((n, 3))
        u[:, d] = 1.0
        modes.append(u.ravel())
    for axis in range(3):
        w = np.zeros(3)
        w[axis] = 1.0
        modes.append(np.cross(w, c).ravel())
    return modes


def _kernel_residual(K, xyz, rng):
    """max over the rigid modes of |K u| / (|K x| |u| / |x|), x random."""
    x = rng.uniform(-1, 1, K.shape[0])
    scale = np.linalg.norm(K @ x) / np.linalg.norm(x)
    return max(np.linalg.norm(K @ u) / (scale * np.linalg.norm(u)) for u in _rigid_modes(xyz))


def _symmetry_gap(K, rng):
    x = rng.uniform(-1, 1, K.shape[0])
    y = rng.uniform(-1, 1, K.shape[0])
    a, b = y @ (K @ x), x @ (K @ y)
    return abs(a - b) / (np.linalg.norm(K @ x) * np.linalg.norm(y))


def test_t10_60_fp64_full_size(ft):
    """T10 60^3 elasticity, FP64 (the headline configuration): 1,296,000
    elements, 5,314,683 DOFs, 451,604,169 nonzeros."""
    fens, fes = ft.t10_elastic_mesh(n=60)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
    K = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(result="device"),
                               ft.NodalField(fens.xyz), u, ft.DeforModelRed3D,
                               ft.DataCache(ft.isotropic_D(210e9, 0.3)))
    assert fes.count() == 1_296_000 and K.shape == (5_314_683, 5_314_683)
    assert K.dm.nnz == 451_604_169
    rng = np.random.default_rng(1)
    assert _kernel_residual(K, fens.xyz, rng) <= 1e-9
    assert _symmetry_gap(K, rng) <= 1e-12


def test_h20_40_mixed_full_size(ft):
    """H20 40^3 elasticity with per-element (E, nu) and 1 % distorted
    elements: 64,000 elements, 811,923 DOFs, 136,823,049 nonzeros; the mixed
    matrix within the mixed gate of the FP64 one (every entry within 1e-6 of
    its row's largest, |dK x| within 1e-6 of |K x|), both annihilating rigid
    motions."""
    fens, fes, flagged = ft.h20_elastic_mesh(n=40)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 3)))
    rng = np.random.default_rng(4)
    cf = ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 0.5, fes.count()),
                                 rng.uniform(0.2, 0.35, fes.count()))
    geom = ft.NodalField(fens.xyz)
    K64 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(result="device"), geom, u,
                                 ft.DeforModelRed3D, cf)
    K32 = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="mixed", result="device"),
                                 geom, u, ft.DeforModelRed3D, cf)
    assert fes.count() == 64_000 and 600 <= len(flagged) <= 640  # 1 % chosen, a few refused
    assert K64.dm.nnz == 136_823_049 and K64.shape == (811_923, 811_923)
    x = rng.uniform(-1, 1, K64.shape[0])
    k64x = K64 @ x
    assert np.linalg.norm(K32 @ x - k64x) / np.linalg.norm(k64x) <= 1e-6
    v64, v32 = K64.values(), K32.values()
    assert np.abs(v32 - v64).max() <= 1e-6 * np.abs(v64).max()
    # the per-nonzero gate: |dK_ij| <= 1e-6 max_k |K_ik| in every row
    rowptr, _ = K64.dm.pattern()
    rowptr = np.asarray(rowptr, dtype=np.int64) - 1
    counts = np.diff(rowptr)
    full = counts > 0
    rowmax = np.zeros(len(counts))
    rowmax[full] = np.maximum.reduceat(np.abs(v64), rowptr[:-1][full])
    assert np.all(np.abs(v32 - v64) <= 1e-6 * np.repeat(rowmax, counts))
    assert _kernel_residual(K64, fens.xyz, rng) <= 1e-9
    assert _kernel_residual(K32, fens.xyz, rng) <= 1e-6
    assert _symmetry_gap(K64, rng) <= 1e-12


def test_h8_20_diffusion_full_size(ft):
    """H8 20^3 diffusion: 8,000 elements, 9,261 DOFs, 226,981 nonzeros;
    constants are in the kernel."""
    fens, fes = ft.h8_diffusion_mesh(n=20)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 1))))
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
    K = ft.bilform_diffusion(femm, ft.SysmatAssemblerGPU(result="device"),
                             ft.NodalField(fens.xyz), u, ft.DataCache(1.0))
    assert K.dm.nnz == 226_981
    ones = np.ones(K.shape[0])
    x = np.random.default_rng(2).uniform(-1, 1, K.shape[0])
    assert np.linalg.norm(K @ ones) <= 1e-12 * np.linalg.norm(K @ x) * np.sqrt(K.shape[0])
