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


def _pixel_problem(n, t, transmissions=True):
    """Host-only pieces of a transmission-interface pixel problem (PixelSolver's layout)."""
    from openbte_gb300.inverse import IsotropicMaterial, PixelSolver
    ps = PixelSolver(n, IsotropicMaterial.lognormal(4, 8), size=10.0)
    prob = ps._problem(t)
    if not transmissions:
        prob.side_transmission = None
    return ps, prob


def test_set_transmission_on_host_only_plan():
    """New transmissions on a host-only plan: accepted in (0, 1], rejected outside it and for plans created
    without transmissions; the sweep order does not change."""
    import numpy as np
    lib = _lib.load()
    n = 6
    rng = np.random.default_rng(3)
    ns = 2 * n * n
    t1 = np.ascontiguousarray(rng.uniform(0.1, 1.0, ns))
    ps, prob = _pixel_problem(n, t1)
    mat = ps.material.c_struct()
    h = ctypes.c_void_p()
    assert lib.obte_bte_plan_create(None, ctypes.byref(prob), ctypes.byref(mat), ctypes.byref(h)) == 0
    try:
        def order(q):
            o = np.zeros(n * n, dtype=np.int64)
            nl, nsl = ctypes.c_int64(), ctypes.c_int64()
            assert lib.obte_bte_schedule(h, q, o.ctypes.data_as(ctypes.POINTER(ctypes.c_int64)), None,
                                         ctypes.byref(nl), ctypes.byref(nsl)) == 0
            return o
        before = [order(q) for q in range(8)]
        nb = ctypes.c_int64(-1)
        for _ in range(2):
            t2 = np.ascontiguousarray(rng.uniform(0.1, 1.0, ns))
            assert lib.obte_bte_plan_set_transmission(h, t2.ctypes.data_as(ctypes.c_void_p), ctypes.byref(nb)) == 0
        assert nb.value == 0                      # host-only: nothing uploaded
        assert all(np.array_equal(order(q), b) for q, b in enumerate(before))
        # the coefficients equal those of a plan built with t2, bit for bit
        fresh = ctypes.c_void_p()
        _, prob_t2 = _pixel_problem(n, t2)
        assert lib.obte_bte_plan_create(None, ctypes.byref(prob_t2), ctypes.byref(mat), ctypes.byref(fresh)) == 0
        try:
            nf = 4
            for q in range(8):
                got = [np.zeros(n * n * nf), np.zeros(n * n), np.zeros(n * n)]
                want = [np.zeros(n * n * nf), np.zeros(n * n), np.zeros(n * n)]
                for hh, arr in ((h, got), (fresh, want)):
                    assert lib.obte_bte_schedule_coefficients(hh, q, *[a.ctypes.data_as(ctypes.c_void_p) for a in arr]) == 0
                for a, b in zip(got, want):
                    assert np.array_equal(a, b)
                assert np.abs(got[2]).max() > 0          # the periodic jump source is present
        finally:
            lib.obte_bte_plan_destroy(fresh)
        bad = t2.copy()
        bad[5] = 0.0
        assert lib.obte_bte_plan_set_transmission(h, bad.ctypes.data_as(ctypes.c_void_p), None) == 1
        assert lib.obte_bte_plan_set_transmission(h, None, None) == 1
    finally:
        lib.obte_bte_plan_destroy(h)
    ps2, prob2 = _pixel_problem(n, t1, transmissions=False)
    h2 = ctypes.c_void_p()
    assert lib.obte_bte_plan_create(None, ctypes.byref(prob2), ctypes.byref(mat), ctypes.byref(h2)) == 0
    try:
        assert lib.obte_bte_plan_set_transmission(h2, t1.ctypes.data_as(ctypes.c_void_p), None) == 1
    finally:
        lib.obte_bte_plan_destroy(h2)
