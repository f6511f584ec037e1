"""CPU-only checks of the C ABI: the library loads and exports every symbol include/xrh.h declares."""
import ctypes
import os
import re

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB = os.path.join(REPO, "qodeapplications_gb300", "libxrh.so")


def declared_functions():
    names = set()
    for f in os.listdir(os.path.join(REPO, "include")):
        if f.endswith(".h"):
            txt = open(os.path.join(REPO, "include", f)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(xrh_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(LIB):
        from qodeapplications_gb300 import build
        build.build()
    return ctypes.CDLL(LIB)


def test_header_declares_entry_points():
    names = declared_functions()
    assert "xrh_gemm_fp64_grouped" in names and "xrh_density_accumulate" in names
    assert len(names) >= 9


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_functions() if not hasattr(lib, n)]
    assert not missing, missing


def test_status_strings_and_argument_checks(lib):
    lib.xrh_status_string.restype = ctypes.c_char_p
    assert lib.xrh_status_string(0) == b"ok"
    assert lib.xrh_abi_version() >= 1
    # argument validation happens before any device work: no GPU needed
    lib.xrh_couplings_count.restype = ctypes.c_int
    assert lib.xrh_couplings_count(0, 9, 0, None, 1, None, None, 0, None, None) == 1     # op length 0
    assert lib.xrh_couplings_count(2, 40, 0, None, 1, None, None, 0, None, None) == 1    # N > 64
    lib.xrh_gemm_fp64_grouped.restype = ctypes.c_int
    assert lib.xrh_gemm_fp64_grouped(None, 0, 0, None, None) == 0
    assert lib.xrh_gemm_fp64_grouped(None, 1, 4, None, None) == 1


def test_python_binding_declares_same_symbols():
    from qodeapplications_gb300 import _lib
    for n in declared_functions():
        assert n in _lib._SIGS, n
