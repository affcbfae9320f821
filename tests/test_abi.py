"""The C-ABI library builds for sm_103a, loads, and exports every entry point
declared in include/*.h (no GPU needed: nothing here launches a kernel)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include"))) if f.endswith(".h")]


def declared_functions(path):
    text = open(path).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    names = set()
    for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][A-Za-z0-9_]*\s*\**\s+\**\s*([A-Za-z_][A-Za-z0-9_]*)\s*\(", text, flags=re.M):
        name = m.group(1)
        if name not in ("if", "for", "while", "return", "sizeof", "typedef"):
            names.add(name)
    return names


def test_headers_declare_entry_points():
    names = set()
    for h in HEADERS:
        names |= declared_functions(h)
    assert "qg_sv_anyCtrlOneTargDenseMatr" in names
    assert "applyHadamard" in names and "mixKrausMap" in names and "calcExpecPauliStr" in names
    assert len(names) > 100


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    missing = []
    for h in HEADERS:
        for name in sorted(declared_functions(h)):
            if not hasattr(lib, name):
                missing.append((os.path.basename(h), name))
    assert not missing, f"declared but not exported: {missing}"


def test_python_binding_covers_abi():
    from quest_gb300 import _lib
    names = set()
    for h in HEADERS:
        if h.endswith("quest_gb300.h"):
            names |= declared_functions(h)
    bound = set(_lib.ABI) | {"qg_get_last_error", "qg_get_error_string", "qg_get_version"}
    assert names <= bound, names - bound


def test_new_entry_points_validate_arguments_before_any_device_call(built_lib):
    # argument checks come before any CUDA call, so they hold without a GPU
    from quest_gb300._lib import lib
    L = lib()
    assert L.qg_set_l2_fetch_granularity(48) == -2
    assert L.qg_set_l2_fetch_granularity(-32) == -2
    assert L.qg_get_l2_fetch_granularity(None) == -2
    t = (ctypes.c_int * 5)(0, 1, 2, 3, 4)
    flag = ctypes.c_int(0)
    assert L.qg_tc_selftest_timeout(11, t, ctypes.byref(flag), None, None) == -2
    assert L.qg_tc_selftest_timeout(14, None, ctypes.byref(flag), None, None) == -2
