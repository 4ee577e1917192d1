"""ctypes binding of ``libatm_gb300.so`` (the C ABI in ``include/atm_gb300.h``).

There is no CPU fallback: if the library is missing or has no GPU, calls
raise ``AtmError``.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libatm_gb300.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_h = ctypes.c_void_p
_i = ctypes.c_int
_d = ctypes.c_double

# name -> (restype, argtypes); every entry point declared in atm_gb300.h
SIGNATURES = {
    "atm_last_error": (ctypes.c_char_p, []),
    "atm_version": (ctypes.c_char_p, []),
    "atm_ctx_create": (_i, [_i, _i, _i, _i, _dp, _i, _ip, _i, _ip, ctypes.POINTER(_h)]),
    "atm_check_mesh": (_i, [_i, _i, _i, ctypes.c_void_p, _i, ctypes.c_void_p, _i,
                           ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]),
    "atm_ctx_destroy": (_i, [_h]),
    "atm_upload_mesh": (_i, [_h, _i, _dp, _i, _ip, _i, _ip]),
    "atm_set_stream": (_i, [_h, ctypes.c_void_p]),
    "atm_synchronize": (_i, [_h]),
    "atm_stream_create": (_i, [ctypes.POINTER(ctypes.c_void_p)]),
    "atm_stream_destroy": (_i, [ctypes.c_void_p]),
    "atm_device_memory": (_i, [_dp, _dp]),
    "atm_n_scalar": (ctypes.c_long, [_h]),
    "atm_kernel_launches": (ctypes.c_long, []),
    "atm_probe_fma_peak": (_i, [_dp, _dp]),
    "atm_timing_enable": (_i, [_h, _i]),
    "atm_timing_read": (_i, [_h, _dp, ctypes.POINTER(ctypes.c_long), _dp, _dp, _i]),
    "atm_set_dt": (_i, [_h, _d]),
    "atm_set_mach": (_i, [_h, _d]),
    "atm_set_froude": (_i, [_h, _d]),
    "atm_set_hyperbolic_stage": (_i, [_h, _i]),
    "atm_set_ns_stage": (_i, [_h, _i]),
    "atm_set_rho_for_fixed": (_i, [_h, ctypes.c_void_p]),
    "atm_set_pres_fixed": (_i, [_h, ctypes.c_void_p]),
    "atm_set_u_fixed": (_i, [_h, ctypes.c_void_p]),
    "atm_vmult_rhs_rho_update": (_i, [_h, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), _i]),
    "atm_vmult_rhs_velocity_fixed": (_i, [_h, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), _i]),
    "atm_vmult_rhs_pressure": (_i, [_h, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), _i]),
    "atm_vmult_pressure": (_i, [_h, ctypes.c_void_p, ctypes.c_void_p]),
    "atm_vmult_enthalpy": (_i, [_h, ctypes.c_void_p, ctypes.c_void_p]),
    "atm_vmult": (_i, [_h, ctypes.c_void_p, ctypes.c_void_p]),
    "atm_schur_vmult_static_scratch": (_i, [_h, ctypes.c_void_p, ctypes.c_void_p]),
    "atm_diagonal_inverse": (_i, [_h, ctypes.c_void_p]),
    "atm_solve": (_i, [_h, ctypes.c_void_p, ctypes.c_void_p, _d, _i, _ip, _dp]),
    "atm_mg_add_level": (_i, [_h, _i, _i, _dp, _i, _ip, _i, _ip, _ip]),
    "atm_mg_set_smoother": (_i, [_h, _i, _d, _i, _i]),
    "atm_mg_vcycle": (_i, [_h, _i, ctypes.c_void_p, ctypes.c_void_p]),
    "atm_mg_set_graphs": (_i, [_h, _i]),
    "atm_set_autotune": (_i, [_h, _i]),
    "atm_autotune_table": (_i, [ctypes.POINTER(ctypes.c_int), _i]),
    "atm_mg_stats": (_i, [_h, ctypes.POINTER(ctypes.c_long)]),
    "atm_solve_fgmres": (_i, [_h, _i, ctypes.c_void_p, ctypes.c_void_p, _d, _i, _ip, _dp]),
    "atm_set_true_residual_check": (_i, [_h, _i]),
    "atm_solver_init": (_i, [_h, _d, _d, _d, _d, _i, _i]),
    "atm_solver_set_state": (_i, [_h, _dp, _dp, _dp]),
    "atm_solver_get_state": (_i, [_h, _dp, _dp, _dp]),
    "atm_solver_set_state_device": (_i, [_h, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "atm_solver_get_state_device": (_i, [_h, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "atm_solver_set_sponge": (_i, [_h, _dp, _d, _d]),
    "atm_solver_set_sponge_target": (_i, [_h, ctypes.c_void_p]),
    "atm_solver_set_clock": (_i, [_h, _d, ctypes.c_long]),
    "atm_solver_run": (_i, [_h, _i]),
    "atm_solver_set_continue_on_not_converged": (_i, [_h, _i]),
    "atm_solver_stats": (_i, [_h, _dp]),
    "atm3_ctx_create": (_i, [_i, _dp, _i, _ip, _ip, _i, _ip, ctypes.POINTER(_h)]),
    "atm3_ctx_destroy": (_i, [_h]),
    "atm3_set_params": (_i, [_h, _d, _d, _d]),
    "atm3_set_stage": (_i, [_h, _i, _i]),
    "atm3_set_frozen": (_i, [_h, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p]),
    "atm3_rhs": (_i, [_h, _i, ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), _i]),
    "atm3_apply": (_i, [_h, _i, ctypes.c_void_p, ctypes.c_void_p]),
    "atm3_solver_init": (_i, [_h, _d, _i, _i, _i]),
    "atm3_solver_set_state": (_i, [_h, _dp, _dp, _dp]),
    "atm3_solver_get_state": (_i, [_h, _dp, _dp, _dp]),
    "atm3_solver_run": (_i, [_h, _i]),
    "atm3_solver_stats": (_i, [_h, _dp]),
    "atm_set_members": (_i, [_h, _i, ctypes.POINTER(ctypes.c_int), _dp]),
    "atm_member_stats": (_i, [_h, _i, _dp]),
    "atm_solver_diagnostics": (_i, [_h, _dp]),
}

KERNEL_FAMILIES = ("rhs_rho", "rhs_vel", "rhs_pres", "B", "CD", "mass", "diag",
                   "block_inverse", "block_apply", "mg_level_apply", "mg_vcycle",
                   "pfix_prep")

STATUS = {0: "OK", 1: "BAD_ARG", 2: "NOT_CONVERGED", 3: "NONFINITE", 4: "OOM", 5: "TIMEOUT",
          6: "CUDA_ERROR", 7: "NOT_READY"}


class AtmError(RuntimeError):
    def __init__(self, code: int, where: str, msg: str):
        super().__init__(f"{where}: {STATUS.get(code, code)}: {msg}")
        self.code = code


_lib = None


def load(path: str = LIB_PATH):
    """Load the library (building it first if it is absent)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        from . import build as _build
        _build.build()
    L = ctypes.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def check(code: int, where: str) -> None:
    if code != 0:
        msg = load().atm_last_error().decode(errors="replace")
        raise AtmError(code, where, msg)


def call(name: str, *args) -> None:
    check(getattr(load(), name)(*args), name)


TUNE_FAMILIES = ("rhs_rho", "rhs_vel", "rhs_pres", "B", "CD")


def autotune_table():
    """Cells-per-block choices of the autotuner so far (this process)."""
    lib = load()
    n = lib.atm_autotune_table(None, 0)
    buf = (ctypes.c_int * (8 * max(n, 1)))()
    n = lib.atm_autotune_table(buf, n)
    rows = []
    for i in range(n):
        r = buf[8 * i: 8 * i + 8]
        rows.append({"family": TUNE_FAMILIES[r[1]], "degree": r[2], "mode": r[3],
                     "hanging": bool(r[4]), "bytes": r[5], "log2_cells": r[6],
                     "cells_per_block": r[7]})
    return rows
