"""ctypes binding of ``libtopomax_gb300.so`` (the C ABI in include/topomax_gb300.h).

The library is built in-tree by ``topomax_gb300.build``.  There is no CPU
implementation behind this module: if the library or a CUDA device is
missing, loading fails with an error.
"""
from __future__ import annotations

import ctypes
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libtopomax_gb300.so")

TOPO_OK = 0
TOPO_ERR_ARG = -1
TOPO_ERR_NOT_CONVERGED = -2
TOPO_ERR_TIMEOUT = -3
TOPO_ERR_NAN = -4
TOPO_ERR_CUDA = -5
TOPO_ERR_STATE = -6
TOPO_ERR_PROJECTION = -7

SIDE_LEFT, SIDE_RIGHT, SIDE_TOP, SIDE_BOTTOM = 1, 2, 4, 8
PREC_FP64, PREC_MIXED = 0, 1
SOLVE_WARM = 1

EXPORTED = [
    "topo_create", "topo_create_filter", "topo_destroy", "topo_last_error", "topo_sizes",
    "topo_set_penalization", "topo_set_iteration_limit", "topo_set_filter_warm_start", "topo_filter_apply", "topo_filter_solve", "topo_state_solve",
    "topo_compliance", "topo_sensitivity_rhs", "topo_sensitivity", "topo_emd_step",
    "topo_emd_finish", "topo_integrate", "topo_state_warm_start", "topo_apply_state", "topo_load_vector", "topo_time_operator",
    "topo_launch_count", "topo_kernel_clock", "topo_kernel_clock_report", "topo_march_tiles_report", "topo_sensitivity_rhs_noalloc", "topo_mass_apply",
    "topo_dem_create", "topo_dem_destroy", "topo_dem_last_error", "topo_dem_set_penalization",
    "topo_dem_set_external", "topo_dem_set_mask", "topo_dem_enforce", "topo_dem_energy",
    "topo_dem_energy_backward", "topo_dem_objective_gradient",
    "topo_density_filter_create", "topo_density_filter_destroy", "topo_density_filter_nnz",
    "topo_density_filter_apply",
    "topo_fluid_create", "topo_fluid_destroy", "topo_fluid_last_error", "topo_fluid_sizes",
    "topo_fluid_set_penalization", "topo_fluid_boundary_values", "topo_fluid_apply", "topo_fluid_state_solve",
    "topo_fluid_objective", "topo_fluid_gradient_rhs", "topo_fluid_gradient", "topo_fluid_launch_count",
]


class GridDesc(ctypes.Structure):
    _fields_ = [("width", ctypes.c_double), ("height", ctypes.c_double),
                ("nx", ctypes.c_int), ("ny", ctypes.c_int)]


class Material(ctypes.Structure):
    _fields_ = [("young_modulus", ctypes.c_double), ("poisson_ratio", ctypes.c_double),
                ("filter_radius", ctypes.c_double), ("penal_min", ctypes.c_double)]


class BCDesc(ctypes.Structure):
    _fields_ = [("fixed_sides", ctypes.c_int), ("n_fixed_points", ctypes.c_int),
                ("fixed_points", ctypes.POINTER(ctypes.c_double))]


class Traction(ctypes.Structure):
    _fields_ = [("side", ctypes.c_int), ("center", ctypes.c_double), ("length", ctypes.c_double),
                ("value_x", ctypes.c_double), ("value_y", ctypes.c_double)]


class LoadDesc(ctypes.Structure):
    _fields_ = [("has_body_force", ctypes.c_int), ("center_x", ctypes.c_double),
                ("center_y", ctypes.c_double), ("radius", ctypes.c_double),
                ("value_x", ctypes.c_double), ("value_y", ctypes.c_double),
                ("n_tractions", ctypes.c_int), ("tractions", ctypes.POINTER(Traction))]


class Flow(ctypes.Structure):
    _fields_ = [("side", ctypes.c_int), ("center", ctypes.c_double), ("length", ctypes.c_double),
                ("rate", ctypes.c_double)]


class DemDesc(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("dshape", ctypes.c_float * 32),
                ("detJ", ctypes.c_float), ("lame_lambda", ctypes.c_float), ("two_mu", ctypes.c_float)]


_lib = None
P = ctypes.c_void_p
D = ctypes.c_double
I = ctypes.c_int
PI = ctypes.POINTER(ctypes.c_int)
PD = ctypes.POINTER(ctypes.c_double)


def load_library(path: str | None = None) -> ctypes.CDLL:
    """Load the C-ABI library (no CUDA call is made)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} not found: build it with `python -m topomax_gb300.build` "
                          "(there is no CPU fallback)")
    lib = ctypes.CDLL(p)
    lib.topo_create.restype = P
    lib.topo_create.argtypes = [ctypes.POINTER(GridDesc), ctypes.POINTER(Material), ctypes.POINTER(BCDesc),
                                ctypes.POINTER(LoadDesc), I, PI]
    lib.topo_create_filter.restype = P
    lib.topo_create_filter.argtypes = [ctypes.POINTER(GridDesc), D, I, PI]
    lib.topo_destroy.restype = None
    lib.topo_destroy.argtypes = [P]
    lib.topo_last_error.restype = ctypes.c_char_p
    lib.topo_last_error.argtypes = [P]
    lib.topo_sizes.argtypes = [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    lib.topo_set_penalization.argtypes = [P, D]
    lib.topo_set_iteration_limit.argtypes = [P, I]
    lib.topo_set_filter_warm_start.argtypes = [P, I]
    lib.topo_filter_apply.argtypes = [P, P, P, D, PI, P]
    lib.topo_filter_solve.argtypes = [P, P, P, D, PI, P]
    lib.topo_state_solve.argtypes = [P, P, P, D, I, PI, P]
    lib.topo_compliance.argtypes = [P, P, P, P]
    lib.topo_sensitivity_rhs.argtypes = [P, P, P, P, P]
    lib.topo_sensitivity.argtypes = [P, P, P, P, D, PI, P]
    lib.topo_emd_step.argtypes = [P, P, P, D, D, P, PD, P]
    lib.topo_emd_finish.argtypes = [P, P, P, P, PD, P]
    lib.topo_integrate.argtypes = [P, P, P, P]
    lib.topo_state_warm_start.argtypes = [P, ctypes.POINTER(P), I, P, P]
    lib.topo_apply_state.argtypes = [P, P, P, P, P]
    lib.topo_load_vector.argtypes = [P, P, P]
    lib.topo_mass_apply.argtypes = [P, P, P, P]
    lib.topo_time_operator.argtypes = [P, PD, P]
    lib.topo_launch_count.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    lib.topo_kernel_clock.argtypes = [I]
    lib.topo_kernel_clock_report.restype = ctypes.c_int64
    lib.topo_kernel_clock_report.argtypes = [ctypes.c_char_p, ctypes.c_int64]
    lib.topo_march_tiles_report.restype = ctypes.c_int64
    lib.topo_march_tiles_report.argtypes = [ctypes.c_char_p, ctypes.c_int64]
    lib.topo_sensitivity_rhs_noalloc.argtypes = [ctypes.POINTER(GridDesc), D, D, D, D, P, P, P, P]
    lib.topo_dem_create.restype = P
    lib.topo_dem_create.argtypes = [ctypes.POINTER(DemDesc), PI]
    lib.topo_dem_destroy.restype = None
    lib.topo_dem_destroy.argtypes = [P]
    lib.topo_dem_last_error.restype = ctypes.c_char_p
    lib.topo_dem_last_error.argtypes = [P]
    lib.topo_dem_set_penalization.argtypes = [P, D]
    lib.topo_dem_set_external.argtypes = [P, P]
    lib.topo_dem_set_mask.argtypes = [P, P]
    lib.topo_dem_enforce.argtypes = [P, P, P, P]
    lib.topo_dem_energy.argtypes = [P, P, P, I, P, P]
    lib.topo_dem_energy_backward.argtypes = [P, P, P, I, P, P, P, P]
    lib.topo_dem_objective_gradient.argtypes = [P, P, P, P, P, P]
    lib.topo_density_filter_create.restype = P
    lib.topo_density_filter_create.argtypes = [I, I, D, D, D, PI]
    lib.topo_density_filter_destroy.restype = None
    lib.topo_density_filter_destroy.argtypes = [P]
    lib.topo_density_filter_nnz.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    lib.topo_density_filter_apply.argtypes = [P, P, P, I, P]
    lib.topo_fluid_create.restype = P
    lib.topo_fluid_create.argtypes = [ctypes.POINTER(GridDesc), D, ctypes.POINTER(Flow), I, PI]
    lib.topo_fluid_destroy.restype = None
    lib.topo_fluid_destroy.argtypes = [P]
    lib.topo_fluid_last_error.restype = ctypes.c_char_p
    lib.topo_fluid_last_error.argtypes = [P]
    lib.topo_fluid_sizes.argtypes = [P, ctypes.POINTER(ctypes.c_int64), ctypes.POINTER(ctypes.c_int64)]
    lib.topo_fluid_set_penalization.argtypes = [P, D]
    lib.topo_fluid_boundary_values.argtypes = [P, P, P]
    lib.topo_fluid_apply.argtypes = [P, P, P, P, I, P]
    lib.topo_fluid_state_solve.argtypes = [P, P, P, P, D, PI, P]
    lib.topo_fluid_objective.argtypes = [P, P, P, P, P]
    lib.topo_fluid_gradient_rhs.argtypes = [P, P, P, P, P]
    lib.topo_fluid_gradient.argtypes = [P, P, P, P, D, PI, P]
    lib.topo_fluid_launch_count.argtypes = [P, ctypes.POINTER(ctypes.c_int64)]
    no_int = ("topo_create", "topo_create_filter", "topo_destroy", "topo_last_error", "topo_dem_create",
              "topo_dem_destroy", "topo_dem_last_error", "topo_density_filter_create",
              "topo_density_filter_destroy", "topo_fluid_create", "topo_fluid_destroy", "topo_fluid_last_error")
    for name in EXPORTED:
        if name not in no_int:
            getattr(lib, name).restype = I
    if path is None:
        _lib = lib
    return lib


class TopoError(ValueError):
    """A failed C-ABI call (ValueError keeps the reference's exception type)."""

    def __init__(self, code: int, message: str):
        super().__init__(message)
        self.code = code


def check(rc: int, ctx) -> None:
    if rc == TOPO_OK:
        return
    lib = load_library()
    msg = lib.topo_last_error(ctx).decode() if ctx else ""
    if rc == TOPO_ERR_CUDA:
        raise RuntimeError(f"topomax_gb300 CUDA error: {msg}")
    raise TopoError(rc, msg or f"topomax_gb300 error {rc}")
