"""The C-ABI library loads and exports every entry point declared in include/obte.h (no GPU needed)."""
import ctypes
import os
import re

from openbte_gb300 import _lib

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for fn in os.listdir(os.path.join(ROOT, "include")):
        if fn.endswith(".h"):
            txt = open(os.path.join(ROOT, "include", fn)).read()
            txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
            names |= set(re.findall(r"\b(obte_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_all_declared_symbols():
    lib = _lib.load()
    missing = [n for n in sorted(declared_symbols()) if not hasattr(lib, n)]
    assert not missing, missing


def test_bindings_cover_header():
    bound = {s[0] for s in _lib.SIGNATURES}
    assert declared_symbols() <= bound, declared_symbols() - bound


def test_status_strings():
    lib = _lib.load()
    assert lib.obte_status_string(0) == b"OK"
    assert lib.obte_status_string(6) == b"CYCLE"
    assert lib.obte_status_string(99) == b"UNKNOWN"


def test_null_arguments_are_rejected_without_gpu():
    lib = _lib.load()
    assert lib.obte_bte_plan_create(None, None, None, ctypes.byref(ctypes.c_void_p())) == 1
    assert lib.obte_bte_solve(None, None, None, None, None, None, None, None) == 1
