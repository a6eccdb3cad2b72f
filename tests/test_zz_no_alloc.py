"""The allocation-free entry point, fegpu_bilform_lin_elastic_noalloc.

It exists for callers that cannot allocate device memory once they are
running (a framework whose pool allocator has reserved the GPU, a time-step
loop that must not hit cudaMalloc's device-wide synchronisation): it runs the
mixed-precision elasticity assembly with its scratch in a static device array
of FEGPU_NOALLOC_SCRATCH_BYTES.  Here it is called through the C ABI, twice in
a row, and each result is checked against the regular entry point
(fegpu_bilform_lin_elastic with FEGPU_MIXED) on the same matrix, within the
FP64 parity bound of tests/test_gpu_parity.py.  The cases cover one chunk of
elements, several chunks (the ring reused across chunks), a mesh whose
scratch forces the chunk to be halved until it fits, and a per-element 6x6 D;
free device memory is the same before and after the calls (the array was
loaded when the context was created).  This file sorts last so a run that
stops at its first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _close(v, ref):
    """|v - ref| <= 1e-12 |ref| + 1e-14 max|ref| (values in the same CSR order)."""
    bound = 1e-12 * np.abs(ref) + 1e-14 * np.abs(ref).max()
    return bool(np.all(np.abs(v - ref) <= bound))


def nat_scratch_bytes():
    """FEGPU_NOALLOC_SCRATCH_BYTES of include/fegpu.h (64 MiB)."""
    return 64 * 1024 * 1024


def _free_bytes():
    import torch
    return torch.cuda.mem_get_info(0)[0]


def _case(ft, nat, case):
    rng = np.random.default_rng(8)
    if case in ("h20_per_element", "h20_multichunk", "h20_halving_per_element_D"):
        n = {"h20_per_element": 6, "h20_multichunk": 16, "h20_halving_per_element_D": 40}[case]
        fens, fes, _ = ft.h20_elastic_mesh(n=n, distort_fraction=0.05 if n < 40 else 0.01)
        rule = ft.GaussRule(3, 3)
        E = rng.lognormal(np.log(70e9), 0.5, fes.count())
        nu = rng.uniform(0.2, 0.35, fes.count())
        if case == "h20_halving_per_element_D":
            data = np.ascontiguousarray(
                np.stack([ft.isotropic_D(a, b) for a, b in zip(E, nu)]).reshape(-1, 36))
            cf = ft.ElementwiseData(data)
            coef = nat.Coef(nat.COEF_PER_ELEMENT, 36, data.ctypes.data)
        else:
            cf = ft.IsotropicElementwise(E, nu)
            data = np.ascontiguousarray(cf.lame)
            coef = nat.Coef(nat.COEF_ISO_LAME, 2, data.ctypes.data)
    else:
        fens, fes = ft.t10_elastic_mesh(n=5)
        rule = ft.TetRule(4)
        cf = ft.DataCache(ft.isotropic_D(210e9, 0.3))
        data = np.ascontiguousarray(ft.isotropic_D(210e9, 0.3).ravel())
        coef = nat.Coef(nat.COEF_CONST, 36, data.ctypes.data)
    return fens, fes, rule, cf, coef, data


@pytest.mark.parametrize("case", ["h20_per_element", "t10_constant", "h20_multichunk",
                                  "h20_halving_per_element_D"])
def test_noalloc_matches_regular_entry_point(ft, case):
    from importlib import import_module
    nat = import_module(ft.__name__ + "._native")
    L = nat.load()
    fens, fes, rule, cf, coef, data = _case(ft, nat, case)
    femm = ft.FEMMBase(ft.IntegDomain(fes, rule))
    geom = ft.NodalField(fens.xyz)
    u = ft.numberdofs(ft.NodalField(np.zeros((fens.count(), 3))))
    _free_bytes()  # the CUDA runtime of the measuring side is up before the first reading
    # the regular mixed-precision entry point (also builds the tables the
    # allocation-free one reads)
    K = ft.bilform_lin_elastic(femm, ft.SysmatAssemblerGPU(precision="mixed", result="device"),
                               geom, u, ft.DeforModelRed3D, cf)
    ref = K.values()
    free = [_free_bytes()]
    for _ in range(2):
        st = L.fegpu_bilform_lin_elastic_noalloc(K.h, C.byref(coef))
        assert st == 0, L.fegpu_last_error().decode()
        got = K.values()
        assert _close(got, ref)
        free.append(_free_bytes())
    # the static array was loaded with the context, not by the first call (the
    # first call may still load its gather kernel's code, a few MiB at most);
    # the second call changes nothing
    assert free[0] - free[1] < nat_scratch_bytes() // 4
    assert free[2] == free[1], "the allocation-free call changed the free device memory"


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
