"""ctypes loaders for the in-tree native libraries.

The solver library is required: when it is missing the loader raises instead
of falling back to any CPU path.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

from .build import OUT

_solver = None
_geom = None

c_int_p = ctypes.POINTER(ctypes.c_int)
c_i8_p = ctypes.POINTER(ctypes.c_int8)
c_i32_p = ctypes.POINTER(ctypes.c_int32)
c_double_p = ctypes.POINTER(ctypes.c_double)
c_void_pp = ctypes.POINTER(ctypes.c_void_p)

# exported names and argtypes of include/fsi_mg.h
SOLVER_SYMBOLS = {
    "fsi_mg_create": [ctypes.c_void_p, c_double_p, c_double_p, c_double_p, c_void_pp],
    "fsi_mg_set_geometry": [ctypes.c_void_p, c_i8_p, c_i8_p, c_i8_p, c_i8_p, c_i8_p, c_i8_p, c_i8_p, c_i8_p,
                            ctypes.c_int, c_i32_p, c_i32_p, c_i32_p, c_i32_p, c_i32_p, c_i32_p,
                            c_double_p, c_double_p, c_double_p],
    "fsi_mg_solve": [ctypes.c_void_p, c_double_p, c_double_p, c_double_p, c_int_p, c_double_p, c_int_p,
                     c_double_p],
    "fsi_mg_solve_device": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, c_int_p,
                            c_double_p, c_int_p, c_double_p],
    "fsi_mg_mg_solver": [ctypes.c_void_p, c_double_p, c_double_p, c_double_p],
    "fsi_mg_calc_residual": [ctypes.c_void_p, c_double_p, c_double_p, c_double_p, c_int_p],
    "fsi_mg_subtract_average": [ctypes.c_void_p, c_double_p],
    "fsi_mg_correct_pressure": [ctypes.c_void_p, c_double_p, c_double_p],
    "fsi_mg_get_pgrad": [ctypes.c_void_p, c_double_p],
    "fsi_mg_level_count": [ctypes.c_void_p, ctypes.c_int],
    "fsi_mg_level_size": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int],
    "fsi_mg_debug_level_op": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                              ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p],
    "fsi_mg_stats": [ctypes.c_void_p, c_double_p, ctypes.c_int],
    "fsi_mg_residual_history": [ctypes.c_void_p, c_double_p, ctypes.c_int],
    "fsi_mg_time_kernel": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p],
    "fsi_mg_line_timing": [ctypes.c_void_p, ctypes.c_int, c_double_p],
    "fsi_mg_set_fresh_cells": [ctypes.c_void_p, ctypes.c_void_p],
    "fsi_mg_subtract_average_noalloc": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                        ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                        ctypes.c_void_p],
    "fsi_mg_face_vel_rhs": [ctypes.c_void_p, ctypes.c_int, ctypes.c_double] + [ctypes.c_void_p] * 11 + [c_double_p],
    "fsi_mg_correct_vel": [ctypes.c_void_p, ctypes.c_double] + [ctypes.c_void_p] * 10,
    "fsi_mg_update_pressure": [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p],
    "fsi_mg_set_bc": [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                      ctypes.c_void_p, c_double_p],
    "fsi_mg_rhs_advec_diff": [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double, ctypes.c_void_p],
    "fsi_mg_rhs_adjust_bc": [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p],
    "fsi_mg_solve_ad": [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.c_void_p, ctypes.c_void_p,
                        ctypes.c_void_p, ctypes.c_void_p, c_int_p, c_double_p],
    "fsi_mg_set_velocity_ghosts": [ctypes.c_void_p, c_double_p, c_double_p, c_double_p, c_double_p,
                                   ctypes.c_double, ctypes.c_double],
    "fsi_mg_last_error": [],
    "fsi_mg_destroy": [ctypes.c_void_p],
}
SOLVER_RESTYPES = {"fsi_mg_last_error": ctypes.c_char_p, "fsi_mg_destroy": None}

GEOM_SYMBOLS = {
    "fsi_geom_icosphere": [ctypes.c_int, ctypes.c_double, ctypes.c_double, ctypes.c_double, ctypes.c_double,
                           c_double_p, ctypes.c_int, c_i32_p, ctypes.c_int, c_int_p, c_int_p],
    "fsi_geom_iblank": [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                        ctypes.c_int, c_double_p, ctypes.c_int, c_i32_p, c_i8_p],
    "fsi_geom_ghost_list": [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_i8_p, c_i8_p, ctypes.c_int,
                            c_i32_p, c_i32_p, c_i32_p],
    "fsi_geom_gcm_coeffs": [ctypes.c_int, ctypes.c_int, ctypes.c_int, c_double_p, c_double_p, c_double_p,
                            ctypes.c_int, c_double_p, ctypes.c_int, c_i32_p, ctypes.c_double, ctypes.c_int,
                            c_i32_p, c_i32_p, c_i32_p, c_i32_p, c_i32_p, c_i32_p, c_double_p, c_double_p,
                            c_double_p, c_double_p, c_double_p],
}
GEOM_RESTYPES = {"fsi_geom_iblank": ctypes.c_long}


def _bind(lib, table, restypes):
    for name, argtypes in table.items():
        fn = getattr(lib, name)
        fn.argtypes = argtypes
        fn.restype = restypes.get(name, ctypes.c_int)
    return lib


def solver_lib_path() -> Path:
    return OUT / "libfsi_mg.so"


def geom_lib_path() -> Path:
    return OUT / "libfsi_geom.so"


def solver():
    """Load the CUDA solver library (raises if it has not been built)."""
    global _solver
    if _solver is None:
        path = solver_lib_path()
        if not path.exists():
            raise RuntimeError(f"CUDA solver library missing: {path}; run flow_structure_interaction_fem_ibm_gb300.build")
        _solver = _bind(ctypes.CDLL(str(path)), SOLVER_SYMBOLS, SOLVER_RESTYPES)
    return _solver


def geometry():
    global _geom
    if _geom is None:
        path = geom_lib_path()
        if not path.exists():
            from .build import build_geometry
            build_geometry()
        _geom = _bind(ctypes.CDLL(str(path)), GEOM_SYMBOLS, GEOM_RESTYPES)
    return _geom


def ptr(a, ctype):
    """Pointer to the first element of a contiguous numpy array (or None)."""
    if a is None:
        return None
    return a.ctypes.data_as(ctypes.POINTER(ctype))
