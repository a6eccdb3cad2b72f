"""The C ABI: libfegpu.so loads and exports every function of include/fegpu.h
(no compute calls: no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    with open(os.path.join(ROOT, "include", "fegpu.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"^\s*(?:int|const char \*)\s*(fegpu_\w+)\s*\(", src, re.M)))


def test_header_declares_the_binding(ft):
    from importlib import import_module
    nat = import_module(ft.__name__ + "._native")
    assert sorted(nat.EXPORTS) == _declared()


def test_library_exports_every_symbol(ft):
    from importlib import import_module
    nat = import_module(ft.__name__ + "._native")
    if not os.path.exists(nat.LIBPATH):
        pytest.fail("libfegpu.so is not built (run __graft_entry__.build())")
    lib = ctypes.CDLL(nat.LIBPATH)
    missing = [s for s in _declared() if not hasattr(lib, s)]
    assert not missing, missing
    nat.load()


def test_last_error_is_a_string(ft):
    from importlib import import_module
    nat = import_module(ft.__name__ + "._native")
    L = nat.load()
    assert isinstance(L.fegpu_last_error(), bytes)


def test_argument_errors_without_gpu(ft):
    """Argument validation runs before any CUDA call."""
    from importlib import import_module
    nat = import_module(ft.__name__ + "._native")
    L = nat.load()
    h = ctypes.c_void_p()
    assert L.fegpu_context_create(-1, ctypes.byref(h)) != 0
    assert L.fegpu_assembler_create(None, 1, 3, 3, ctypes.byref(h)) != 0


def test_mesh_memory_estimate_without_gpu(ft):
    """fegpu_estimate_mesh_bytes (the serving loop's admission estimate) is
    host arithmetic: it grows with the mesh, with the DOFs per node and with
    the element's node count, rejects unknown element types and negative
    sizes, and its figure for the T10 60^3 configuration (1,296,000 elements,
    1,771,561 nodes, 3 DOFs per node, 451,604,169 stored values) covers at
    least the values (8 bytes each) and the column indices (4 bytes each)."""
    E60, N60 = 1_296_000, 1_771_561
    b = ft.estimate_mesh_bytes(4, E60, N60, 3)  # FEGPU_T10
    assert b >= 451_604_169 * 12
    assert b < 451_604_169 * 40
    assert ft.estimate_mesh_bytes(4, 2 * E60, 2 * N60, 3) > b
    assert ft.estimate_mesh_bytes(4, E60, N60, 1) < b
    assert ft.estimate_mesh_bytes(2, 64_000, 270_641, 3) > ft.estimate_mesh_bytes(1, 64_000, 68_921, 3)
    for bad in ((9, 10, 10, 1), (1, -1, 10, 1), (1, 10, 10, 4)):
        with pytest.raises(ft.FegpuError):
            ft.estimate_mesh_bytes(*bad)
