"""The allocation-free entry point, fegpu_bilform_lin_elastic_noalloc.

It exists for callers that cannot allocate device memory once they are
running (a framework whose pool allocator has reserved the GPU, a time-step
loop that must not hit cudaMalloc's device-wide synchronisation): it runs the
mixed-precision elasticity assembly with its scratch in a static device array
of FEGPU_NOALLOC_SCRATCH_BYTES.  Here it is called through the C ABI, twice in
a row, and each result is checked against the regular entry point
(fegpu_bilform_lin_elastic with FEGPU_MIXED) on the same matrix, within the
FP64 parity bound of tests/test_gpu_parity.py.  This file sorts last so a run
that stops at its first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(v, ref):
    """|v - ref| <= 1e-12 |ref| + 1e-14 max|ref| (values in the same CSR order)."""
    bound = 1e-12 * np.abs(ref) + 1e-14 * np.abs(ref).max()
    return bool(np.all(np.abs(v - ref) <= bound))


@pytest.mark.parametrize("case", ["h20_per_element", "t10_constant"])
def test_noalloc_matches_regular_entry_point(ft, case):
    from importlib import import_module
    nat = import_module(ft.__name__ + "._native")
    L = nat.load()
    if case == "h20_per_element":
        fens, fes, _ = ft.h20_elastic_mesh(n=6, distort_fraction=0.05)
        rule = ft.GaussRule(3, 3)
        rng = np.random.default_rng(8)
        cf = ft.IsotropicElementwise(rng.lognormal(np.log(70e9), 0.5, fes.count()),
                                     rng.uniform(0.2, 0.35, fes.count()))
        data = np.ascontiguousarray(cf.lame)
        coef = nat.Coef(nat.COEF_ISO_LAME, 2, data.ctypes.data)
    else:
        fens, fes = ft.t10_elastic_mesh(n=5)
        rule = ft.TetRule(4)
        cf = ft.DataCache(ft.isotropic_D(210e9, 0.3))
        data = np.ascontiguousarray(ft.isotropic_D(210e9, 0.3).ravel())
        coef = nat.Coef(nat.COEF_CONST, 36, data.ctypes.data)
    femm = ft.FEMMBase(ft.IntegDomain(fes, rule))
    geom = ft.NodalField(fens.xyz)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    # the regular mixed-precision entry point (also builds the tables the
    # allocation-free one reads)
    K = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="mixed", result="device"),
                               geom, u, ft.DeforModelRed3D, cf)
    ref = K.values()
    for _ in range(2):
        st = L.fegpu_bilform_lin_elastic_noalloc(K.h, C.byref(coef))
        assert st == 0, L.fegpu_last_error().decode()
        got = K.values()
        assert _close(got, ref)


def test_noalloc_requires_the_tables(ft):
    """Without a prior regular mixed assembly the entry point refuses (it
    would otherwise have to allocate the node-to-element tables)."""
    from importlib import import_module
    nat = import_module(ft.__name__ + "._native")
    L = nat.load()
    fens, fes = ft.t10_elastic_mesh(n=3)
    femm = ft.FEMMBase(ft.IntegDomain(fes, ft.TetRule(4)))
    geom = ft.NodalField(fens.xyz)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    K = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(result="device"), geom, u,
                               ft.DeforModelRed3D, ft.DataCache(ft.isotropic_D(1.0, 0.3)))
    D = np.ascontiguousarray(ft.isotropic_D(1.0, 0.3).ravel())
    coef = nat.Coef(nat.COEF_CONST, 36, D.ctypes.data)
    st = L.fegpu_bilform_lin_elastic_noalloc(K.h, C.byref(coef))
    assert st == 4 and b"mixed-precision assembly" in L.fegpu_last_error()
