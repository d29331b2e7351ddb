"""The C-ABI library loads on the CPU host and exports every symbol that
include/swampe_gb300.h declares (no compute calls: no GPU needed)."""
import ctypes
import re

from conftest import ROOT


def _declared():
    text = (ROOT / "include" / "swampe_gb300.h").read_text()
    return sorted(set(re.findall(r"\b(swp_[a-z_0-9]+)\s*\(", text)))


def test_header_declares_entry_points():
    names = _declared()
    assert "swp_forward" in names and "swp_adjoint_step" in names
    assert len(names) >= 10


def test_library_exports_all_declared_symbols():
    from my_swampe_gb300 import build, _lib

    build.build()
    lib = ctypes.CDLL(str(_lib.LIB_PATH))
    missing = [n for n in _declared() if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_lib.EXPORTS) <= set(_declared())


def test_plan_create_rejects_bad_arguments_without_gpu():
    from my_swampe_gb300 import _lib

    lib = _lib.load()
    plan = ctypes.c_void_p()
    Ms = (ctypes.c_int * 1)(42)
    Bs = (ctypes.c_int * 1)(1)
    assert lib.swp_plan_create(0, Ms, Bs, 0, ctypes.byref(plan)) == 1
    assert lib.swp_plan_create(1, Ms, Bs, 7, ctypes.byref(plan)) == 1
    assert lib.swp_plan_create(1, Ms, Bs, 0, None) == 1
