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
