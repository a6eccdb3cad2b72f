"""Batches (fegpu_batch_*): many assemblies of mixed element types and sizes
in one persistent launch, replayed as a CUDA graph.

Bar: every job's matrix equals the single-call FEGPU_MIXED result of the same
form with the FP32-pipe element tile bit for bit (same FP32 element
arithmetic, same element-order FP64 accumulation, whatever the schedule); the dot form, evaluated in FP64 by the
single call, agrees within the mixed-precision bound 1e-6 (normwise and
max-entry relative); and each job is within that bound of the FP64 result.
"""
import zlib

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED_TOL = 1e-6


@pytest.fixture(autouse=True)
def _fp32_pipe_single_calls(monkeypatch):
    """The persistent batch kernel forms element blocks on the FP32 pipe; the
    single-call references of these tests use the same tile (the single-call
    tensor-core blocks are checked against FP64 in test_gpu_parity)."""
    monkeypatch.setenv("FEGPU_MIXED_TC", "0")


def _field(ft, n, ndn):
    return ft.numberdofs(ft.NodalField(np.zeros((n, ndn))))


def _case(ft, name):
    """(form, femm, geom, u, coefficient, m) of one named job."""
    rng = np.random.default_rng(zlib.crc32(name.encode()))
    if name == "h8_diffusion":
        fens, fes = ft.h8_diffusion_mesh(n=5)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
        return "diffusion", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 1), \
            ft.DataCache(2.5), 3
    if name == "h20_elastic_per_element":
        fens, fes, _ = ft.h20_elastic_mesh(n=4, distort_fraction=0.05)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 3)))
        cf = ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 0.5, fes.count()),
                                     rng.uniform(0.2, 0.35, fes.count()))
        return "lin_elastic", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 3), cf, 3
    if name == "t4_elastic":
        fens, fes = ft.T4block(2.0, 1.0, 1.5, 4, 3, 3)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(1)))
        return "lin_elastic", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 3), \
            ft.DataCache(ft.isotropic_D(210e9, 0.3)), 3
    if name == "t10_diffusion_per_element":
        fens, fes = ft.t10_elastic_mesh(n=3)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
        return "diffusion", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 1), \
            ft.ElementwiseData(rng.uniform(0.5, 3.0, fes.count())), 3
    if name == "t10_elastic":
        fens, fes = ft.t10_elastic_mesh(n=4)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
        return "lin_elastic", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 3), \
            ft.DataCache(ft.isotropic_D(70e9, 0.33)), 3
    if name == "h20_diffusion_per_point":
        fens, fes = ft.H20block(1.0, 2.0, 1.0, 3, 2, 2)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 3)))
        cf = ft.DataCache(1.0, lambda c, X, t, fe, q: np.array(1.0 + X[0, 0] ** 2 + X[0, 2]))
        return "diffusion", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 1), cf, 3
    if name == "q4_diffusion_thickness":
        fens, fes = ft.Q4block(12.0, 1.1, 6, 4)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, 2), 0.32))
        return "diffusion", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 1), \
            ft.DataCache(1.3), 3
    if name.startswith("q4_dot"):
        fens, fes = ft.Q4block(2.0, 1.5, 5, 4)
        xyz = np.hstack([fens.xyz, rng.uniform(-0.05, 0.05, (fens.count(), 1))])
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, 2), 0.01))
        ndn, m = (3, 3) if name == "q4_dot3_m3" else (1, 2)
        cf = ft.DataCache(np.eye(ndn) * 7.8e3) if ndn == 3 else ft.DataCache(7.8e3)
        return "dot", femm, ft.NodalField(xyz), _field(ft, fens.count(), ndn), cf, m
    if name == "h8_dot3_matrix":
        fens, fes = ft.H8block(12.0, 1.1, 0.32, 4, 3, 2)
        femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(3, 2)))
        c = np.eye(3) * 1.7
        c[0, 1] = c[1, 0] = 0.2
        return "dot", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 3), \
            ft.DataCache(c), 3
    raise KeyError(name)


CASES = ["h8_diffusion", "h20_elastic_per_element", "t4_elastic", "t10_diffusion_per_element",
         "t10_elastic", "h20_diffusion_per_point", "q4_diffusion_thickness", "q4_dot3_m3",
         "q4_dot1_m2", "h8_dot3_matrix"]


def _single(ft, form, femm, geom, u, cf, m, precision):
    asm = ft.SysmatAssemblerGPU(precision=precision, result="device")
    if form == "diffusion":
        K = ft.bilform_diffusion(femm, asm, geom, u, cf)
    elif form == "lin_elastic":
        K = ft.bilform_lin_elastic(femm, asm, geom, u, ft.DeforModelRed3D, cf)
    else:
        K = ft.bilform_dot(femm, asm, geom, u, cf, m=m)
    return K.values()


def _near(v, ref, tol=MIXED_TOL):
    """max-entry and Frobenius relative errors within tol (same CSR order)."""
    assert np.abs(v - ref).max() <= tol * np.abs(ref).max()
    assert np.linalg.norm(v - ref) <= tol * np.linalg.norm(ref)


@pytest.fixture(scope="module")
def mixed_batch(ft):
    cases = [_case(ft, n) for n in CASES]
    b = ft.AssemblyBatch()
    mats = [b.add(form, femm, geom, u, cf, m=m) for form, femm, geom, u, cf, m in cases]
    b.run()
    return b, cases, mats


def test_batch_matches_single_calls(ft, mixed_batch):
    b, cases, mats = mixed_batch
    assert b.stats()["jobs"] == len(CASES)
    for name, (form, femm, geom, u, cf, m), M in zip(CASES, cases, mats):
        got = M.values()
        ref64 = _single(ft, form, femm, geom, u, cf, m, "fp64")
        if form == "dot":
            _near(got, ref64)
        else:
            ref = _single(ft, form, femm, geom, u, cf, m, "mixed")
            assert np.array_equal(got, ref), name
            _near(got, ref64)


def test_batch_job_alone_equals_job_in_mix(ft, mixed_batch):
    _, cases, mats = mixed_batch
    for i in (1, 4, 7):
        form, femm, geom, u, cf, m = cases[i]
        one = ft.AssemblyBatch()
        M = one.add(form, femm, geom, u, cf, m=m)
        one.run()
        assert np.array_equal(M.values(), mats[i].values()), CASES[i]


def test_batch_graph_replay_is_deterministic(ft, mixed_batch):
    b, _, mats = mixed_batch
    first = [M.values() for M in mats]
    for _ in range(3):
        b.run()
    for v, M in zip(first, mats):
        assert np.array_equal(v, M.values())


def test_batch_set_coef(ft):
    form, femm, geom, u, cf, m = _case(ft, "h20_elastic_per_element")
    b = ft.AssemblyBatch()
    M = b.add(form, femm, geom, u, cf, m=m)
    b.run()
    rng = np.random.default_rng(11)
    n = femm.integdomain.fes.count()
    cf2 = ft.IsotropicElementwise(rng.lognormal(np.log(200e9), 0.3, n), rng.uniform(0.25, 0.3, n))
    b.set_coef(M.job, cf2)
    b.run()
    assert np.array_equal(M.values(), _single(ft, form, femm, geom, u, cf2, m, "mixed"))


def test_batch_jobs_sharing_a_dofmap(ft):
    """Two matrices of one mesh and field in one batch (private block rings)."""
    form, femm, geom, u, cf, m = _case(ft, "t10_elastic")
    b = ft.AssemblyBatch()
    M1 = b.add(form, femm, geom, u, cf, m=m)
    cf2 = ft.DataCache(ft.isotropic_D(3.0e9, 0.45))
    M2 = b.add(form, femm, geom, u, cf2, m=m)
    b.run()
    assert np.array_equal(M1.values(), _single(ft, form, femm, geom, u, cf, m, "mixed"))
    assert np.array_equal(M2.values(), _single(ft, form, femm, geom, u, cf2, m, "mixed"))


def test_batch_autotuner_and_cache(ft, tmp_path, mixed_batch):
    _, cases, mats = mixed_batch
    b = ft.AssemblyBatch()
    out = [b.add(form, femm, geom, u, cf, m=m) for form, femm, geom, u, cf, m in cases[:5]]
    path = str(tmp_path / "tiles.txt")
    b.tune(path)
    lines = open(path).read().split("\n")
    kinds = {ln.split()[0] for ln in lines if ln.strip()}
    assert {"H8_diffusion", "H20_elasticity", "T4_elasticity", "T10_diffusion",
            "T10_elasticity"} <= kinds
    assert all(b.tile(j) >= 1 for j in range(5))
    b.run()
    for M, ref in zip(out, mats[:5]):
        assert np.array_equal(M.values(), ref.values())
    # a second batch reads the cache instead of timing again
    b2 = ft.AssemblyBatch()
    form, femm, geom, u, cf, m = cases[0]
    b2.add(form, femm, geom, u, cf, m=m)
    b2.tune(path)
    assert open(path).read().split("\n") == lines
    assert b2.tile(0) == b.tile(0)


def test_batch_rejects_unbatched_kinds(ft):
    FegpuError = ft.FegpuError
    fens, fes = ft.Q4block(1.0, 1.0, 2, 2)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.GaussRule(2, 2)))
    b = ft.AssemblyBatch()
    with pytest.raises(FegpuError, match="acceptable"):
        b.add("dot", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 1),
              ft.DataCache(1.0), m=1)
    with pytest.raises(FegpuError, match="3-D solids"):
        b.add("lin_elastic", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 3),
              ft.DataCache(ft.isotropic_D(1.0, 0.3)))
    with pytest.raises(ValueError):
        b.add("convection", femm, ft.NodalField(fens.xyz), _field(ft, fens.count(), 1),
              ft.DataCache(1.0))


def test_dependency_wait_runs_out_and_the_next_run_recovers(ft):
    """The failure path of the persistent kernel without a device fault: the
    completion of a job's first element stage is withheld (a counter nothing
    then raises), so the gather that depends on it waits until the wait limit
    (0.05 s here), the kernel skips the rest and ends, and the run reports
    FEGPU_ERR_DEVICE through the C ABI.  The same batch then runs cleanly at
    the default limit and its matrices equal those of the run before."""
    import time
    from importlib import import_module
    nat = import_module(ft.__name__ + "._native")
    b = ft.AssemblyBatch()
    mats = [b.add(*_case(ft, name)) for name in ("h20_elastic_per_element", "t10_elastic")]
    b.run()
    ref = [M.values() for M in mats]
    b.set_wait_limit(0.05)
    b.withhold(1)
    t0 = time.perf_counter()
    b.launch()
    with pytest.raises(nat.FegpuError, match="waited past its time limit"):
        b.wait()
    assert time.perf_counter() - t0 < 10.0
    b.withhold(-1)
    b.set_wait_limit(5.0)
    b.run()
    for M, r in zip(mats, ref):
        assert np.array_equal(M.values().view(np.int64), r.view(np.int64))
