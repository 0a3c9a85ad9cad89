"""The C-ABI library: built in-tree, loadable, exports every declared entry
point (no compute calls; runs without a GPU)."""

import ctypes
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "martini_gb300.h")
LIB = os.path.join(ROOT, "martini_gb300", "libmartini_gb300.so")


def declared_functions():
    text = open(HEADER).read()
    return sorted(set(re.findall(r"^(?:const char\*|int|size_t|void)\s+(mg_\w+)\s*\(", text, re.M)))


def test_header_declares_entry_points():
    names = declared_functions()
    for n in ("mg_insert", "mg_plan", "mg_workspace_size", "mg_check", "mg_spectra", "mg_flux",
              "mg_version", "mg_last_error"):
        assert n in names


def test_library_exports_every_declared_symbol():
    if not os.path.exists(LIB):
        from martini_gb300 import build
        build.build()
    lib = ctypes.CDLL(LIB)
    for name in declared_functions():
        assert hasattr(lib, name), name
    lib.mg_version.restype = ctypes.c_char_p
    assert b"sm_103a" in lib.mg_version()


def test_python_binding_lists_all_exports():
    from martini_gb300 import _native
    assert sorted(_native.EXPORTS) == declared_functions()


def test_workspace_size_needs_no_gpu():
    from martini_gb300 import _native as N
    lib = N.load()
    p = N.Problem()
    p.n, p.nx, p.ny, p.nc = 1000, 64, 64, 32
    out = ctypes.c_size_t()
    assert lib.mg_workspace_size(ctypes.byref(p), 10_000, 4, ctypes.byref(out)) == 0
    base = ctypes.c_size_t()
    assert lib.mg_workspace_size(ctypes.byref(p), 0, 0, ctypes.byref(base)) == 0
    assert out.value >= base.value - 256 + 10_000 * 4 + 4 * 128 * 64 * 4
    p.nc = 0
    assert lib.mg_workspace_size(ctypes.byref(p), 0, 0, ctypes.byref(out)) == N.MG_ERR_INVALID_ARGUMENT
    assert b"invalid" in lib.mg_last_error()
