"""ctypes binding of the C ABI in include/obte.h (libobte_gb300.so).

This is the FFI layer a Python caller of the reference would add: plain
structs and pointers, no torch types. The library must be built
(``python -m openbte_gb300.build``); there is no CPU fallback and importing
the solver without it raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libobte_gb300.so")

OBTE_OK = 0
STATUS_NAMES = {0: "OK", 1: "BAD_ARG", 2: "OOM", 3: "ADMISSION_REJECTED", 4: "NOT_CONVERGED",
                5: "CUDA_ERROR", 6: "CYCLE", 7: "UNSUPPORTED", 8: "DEVICE_TIMEOUT"}
OBTE_ERR_BAD_ARG = 1
OBTE_ERR_ADMISSION = 3
OBTE_ERR_NOT_CONVERGED = 4
OBTE_ERR_UNSUPPORTED = 7
OBTE_ERR_DEVICE_TIMEOUT = 8

PRECISION = {"fp64": 0, "fp32_refine": 1, "fp32": 2, "df": 3}
CONTACT_NONE, CONTACT_PERIODIC, CONTACT_MIXED, CONTACT_NANOWIRE = 0, 1, 2, 3

p_i64 = C.POINTER(C.c_int64)
p_f64 = C.POINTER(C.c_double)


class Problem(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("n_elems", C.c_int64), ("n_sides", C.c_int64), ("elem_nv", C.c_int32),
        ("side_elem_map", p_i64), ("normal_areas", p_f64), ("elem_volumes", p_f64), ("side_areas", p_f64),
        ("n_internal", C.c_int64), ("internal", p_i64),
        ("n_periodic", C.c_int64), ("periodic_sides", p_i64), ("periodic_jump", p_f64),
        ("n_diffuse", C.c_int64), ("diffuse_sides", p_i64),
        ("n_mixed", C.c_int64), ("mixed_sides", p_i64), ("mixed_value", p_f64),
        ("contact_kind", C.c_int32), ("n_contact", C.c_int64), ("contact_sides", p_i64),
        ("contact_alpha", C.c_double), ("normalization", C.c_double), ("is_nanowire", C.c_int32),
        ("heat_source", p_f64), ("side_transmission", p_f64), ("reflect_internal", C.c_int32),
    ]


class MaterialC(C.Structure):
    _fields_ = [
        ("n_mfp", C.c_int32), ("n_dir", C.c_int32), ("dim_dir", C.c_int32), ("dim_sigma", C.c_int32),
        ("mfps", p_f64), ("vmfp", p_f64), ("sigma", p_f64), ("t_coeff", p_f64),
        ("heat_source_coeff", C.c_double),
    ]


class SolveOpts(C.Structure):
    _fields_ = [("precision", C.c_int32), ("rtol", C.c_double), ("max_sweeps", C.c_int32),
                ("restart", C.c_int32), ("refine_steps", C.c_int32), ("inner_rtol", C.c_double),
                ("warm_start", C.c_int32), ("precond", C.c_int32), ("dsa", C.c_int32)]


class SolveInfo(C.Structure):
    _fields_ = [("kappa_eff", C.c_double), ("n_sweeps", C.c_int32), ("n_sweeps_fp64", C.c_int32),
                ("residual", C.c_double), ("offset", C.c_double), ("converged", C.c_int32),
                ("n_sweeps_df", C.c_int32)]


class FourierProblem(C.Structure):
    _fields_ = [
        ("dim", C.c_int32), ("n_elems", C.c_int64), ("n_sides", C.c_int64), ("elem_nv", C.c_int32),
        ("side_elem_map", p_i64), ("normal_areas", p_f64), ("dists", p_f64), ("elem_volumes", p_f64),
        ("side_areas", p_f64), ("interp_weights", p_f64), ("gradient_weights", p_f64),
        ("elem_side_map", p_i64),
        ("n_internal", C.c_int64), ("internal", p_i64),
        ("n_periodic", C.c_int64), ("periodic_sides", p_i64), ("periodic_jump", p_f64),
        ("n_mixed", C.c_int64), ("mixed_sides", p_i64), ("mixed_value", p_f64), ("mixed_conductance", p_f64),
        ("contact_kind", C.c_int32), ("n_contact", C.c_int64), ("contact_sides", p_i64),
        ("contact_alpha", C.c_double), ("contact_conductance", C.c_double), ("normalization", C.c_double),
        ("kappa", p_f64), ("heat_source", p_f64), ("pin_elem", C.c_int32),
    ]


class FourierOpts(C.Structure):
    _fields_ = [("max_iter", C.c_int32), ("rtol", C.c_double), ("cg_rtol", C.c_double), ("cg_max_iter", C.c_int32)]


class FourierInfo(C.Structure):
    _fields_ = [("kappa", C.c_double), ("n_iter", C.c_int32), ("n_cg", C.c_int32)]


# (name, restype, argtypes) for every entry point declared in include/obte.h
SIGNATURES = [
    ("obte_context_create", C.c_int, [C.c_int, C.c_void_p, C.POINTER(C.c_void_p)]),
    ("obte_context_destroy", C.c_int, [C.c_void_p]),
    ("obte_context_set_stream", C.c_int, [C.c_void_p, C.c_void_p]),
    ("obte_status_string", C.c_char_p, [C.c_int]),
    ("obte_last_error", C.c_char_p, []),
    ("obte_launch_count", C.c_int64, []),
    ("obte_h2d_bytes", C.c_int64, []),
    ("obte_device_cache_trim", C.c_int, [p_i64]),
    ("obte_device_cache_bytes", C.c_int, [p_i64]),
    ("obte_bte_plan_create", C.c_int, [C.c_void_p, C.POINTER(Problem), C.POINTER(MaterialC), C.POINTER(C.c_void_p)]),
    ("obte_bte_plan_destroy", C.c_int, [C.c_void_p]),
    ("obte_bte_plan_set_transmission", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(C.c_int64)]),
    ("obte_bte_plan_set_stream", C.c_int, [C.c_void_p, C.c_void_p]),
    ("obte_bte_plan_footprint", C.c_int, [C.c_void_p, C.c_int32, C.c_int32, p_i64, p_i64]),
    ("obte_bte_plan_prepare", C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    ("obte_bte_solve", C.c_int, [C.c_void_p, C.POINTER(SolveOpts), C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p,
                                 C.c_void_p, C.POINTER(SolveInfo)]),
    ("obte_bte_sweep", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]),
    ("obte_bte_sweep_static", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32]),
    ("obte_bte_sweep_fields", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p]),
    ("obte_bte_plan_test_wait_timeout", C.c_int, [C.c_void_p, C.c_int32, C.c_int32]),
    ("obte_bte_kappa_gradient", C.c_int, [C.c_void_p, C.POINTER(SolveOpts), C.c_void_p, C.c_void_p,
                                          C.POINTER(SolveInfo)]),
    ("obte_bte_kappa_gradient_adjoint", C.c_int, [C.c_void_p, C.c_void_p, C.POINTER(SolveOpts), C.c_void_p,
                                                  C.c_void_p, C.POINTER(SolveInfo), C.POINTER(SolveInfo)]),
    ("obte_bte_state_layout", C.c_int, [C.c_void_p, p_i64, p_i64, p_i64]),
    ("obte_bte_precond_info", C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32),
                                        C.POINTER(C.c_double)]),
    ("obte_bte_precond_bytes", C.c_int, [C.c_void_p, p_i64, p_i64]),
    ("obte_bte_dsa_operator", C.c_int, [C.c_void_p, p_i64, C.c_void_p, C.c_void_p, C.c_void_p,
                                        C.POINTER(C.c_int32)]),
    ("obte_bte_schedule", C.c_int, [C.c_void_p, C.c_int32, p_i64, p_i64, p_i64, p_i64]),
    ("obte_bte_schedule_coefficients", C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("obte_bte_tables_digest", C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_uint64)]),
    ("obte_fourier_plan_create", C.c_int, [C.c_void_p, C.POINTER(FourierProblem), C.POINTER(C.c_void_p)]),
    ("obte_fourier_plan_destroy", C.c_int, [C.c_void_p]),
    ("obte_fourier_solve", C.c_int, [C.c_void_p, C.POINTER(FourierOpts), C.c_void_p, C.c_void_p,
                                     C.POINTER(FourierInfo)]),
]

_LIB = None


def load():
    """Load libobte_gb300.so, building it first if it is missing (nvcc required)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        from . import build as _build
        _build.build()
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libobte_gb300.so is not built (python -m openbte_gb300.build)")
    lib = C.CDLL(LIB_PATH)
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


class OBTEError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = status
        lib = _LIB
        detail = lib.obte_last_error().decode() if lib is not None else ""
        super().__init__(f"{what}: {STATUS_NAMES.get(status, status)}" + (f" ({detail})" if detail else ""))


class NotConverged(OBTEError):
    pass


class AdmissionRejected(OBTEError):
    pass


def check(status, what=""):
    if status == OBTE_OK:
        return
    if status == OBTE_ERR_NOT_CONVERGED:
        raise NotConverged(status, what)
    if status == OBTE_ERR_ADMISSION:
        raise AdmissionRejected(status, what)
    raise OBTEError(status, what)
