"""Solver parameters and reference constants.

The field set mirrors the reference's hot-path input flags (IBM/MAIN.F90
read_inputs: pp_solver_type/iRedBlack :476, omega :478, iterMax_Poisson and
restol_Poisson :480, mgcycle :483, iterFinest/iterCoarsest :485, mgLevels
:487, iterMax_ad/restol_ad :473, velocity and pressure BC types :415-449) and
is laid out exactly like ``fsi_mg_params`` in ``include/fsi_mg.h``.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

# IBM/AMODULES.F90:14-118
VISCOUS_FLOW, POTENTIAL_FLOW = 1, 2
BC_TYPE_DIRICHLET, BC_TYPE_ZERO_GRADIENT, BC_TYPE_PULSATILE_INFLOW, BC_TYPE_SYMMETRY = 1, 2, 3, 4
BC_TYPE_PERIODIC, BC_TYPE_USER_SPECIFIED, BC_TYPE_SHEAR = 5, 6, 7
PBC_DIRICHLET, PBC_NEUMANN = 1, 2
PP_SOLVER_TYPE_LSOR, PP_SOLVER_TYPE_MG = 1, 3
NO_INTERNAL_BOUNDARY, GCM_METHOD = 0, 2
DIM_2D, DIM_3D = 2, 3

PRECISION_FP64 = 0
PRECISION_MIXED = 1

# status codes returned by solve entry points (include/fsi_mg.h)
FSI_MG_CONVERGED = 0
FSI_MG_NOT_CONVERGED = 1
FSI_MG_GHOST_NOT_CONVERGED = 2


class FsiMgParams(ctypes.Structure):
    _fields_ = [
        ("ndim", ctypes.c_int),
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("pp_solver_type", ctypes.c_int),
        ("iRedBlack", ctypes.c_int),
        ("mgcycle", ctypes.c_int * 3),
        ("iterFinest", ctypes.c_int), ("iterCoarsest", ctypes.c_int),
        ("mgLevels", ctypes.c_int * 3),
        ("iterMax_Poisson", ctypes.c_int), ("iterMax_ad", ctypes.c_int),
        ("bc", ctypes.c_int * 6),
        ("pbc", ctypes.c_int * 6),
        ("internal_boundary_present", ctypes.c_int),
        ("boundary_formulation", ctypes.c_int),
        ("coarse_flag_mode", ctypes.c_int),
        ("precision_mode", ctypes.c_int),
        ("outer_krylov", ctypes.c_int),
        ("omega", ctypes.c_double),
        ("restol_Poisson", ctypes.c_double),
        ("restol_ad", ctypes.c_double),
        ("ppp", ctypes.c_double * 6),
        ("outflow_area", ctypes.c_double),
        ("alfa", ctypes.c_double),
    ]


@dataclass
class SolverParams:
    """Hot-path settings.  Defaults are the harness settings used for every
    configuration: MG (pp_solver_type 3), automatic V-cycle hierarchy,
    iterFinest 2, iterCoarsest 10, omega 1, probeLengthNormalized 2 (geometry),
    restol_ad 1e-13, iterMax_ad 200, all-Neumann pressure, no-slip walls."""

    ndim: int = DIM_3D
    nx: int = 17
    ny: int = 17
    nz: int = 17
    pp_solver_type: int = PP_SOLVER_TYPE_MG
    iRedBlack: int = 0
    mgcycle: tuple = (1, 1, 1)
    iterFinest: int = 2
    iterCoarsest: int = 10
    mgLevels: tuple = (0, 0, 0)
    iterMax_Poisson: int = 10000
    iterMax_ad: int = 200
    bc: tuple = (BC_TYPE_DIRICHLET,) * 6
    pbc: tuple = (PBC_NEUMANN,) * 6
    internal_boundary_present: int = 0
    boundary_formulation: int = NO_INTERNAL_BOUNDARY
    coarse_flag_mode: int = 0
    precision_mode: int = PRECISION_FP64
    outer_krylov: int = 0
    omega: float = 1.0
    restol_Poisson: float = 1e-8
    restol_ad: float = 1e-13
    ppp: tuple = (0.0,) * 6
    outflow_area: float = 1.0
    alfa: float = 0.0
    extra: dict = field(default_factory=dict)

    def to_c(self) -> FsiMgParams:
        p = FsiMgParams()
        for name, _ in FsiMgParams._fields_:
            val = getattr(self, name)
            if isinstance(val, (tuple, list)):
                arr = getattr(p, name)
                for i, v in enumerate(val):
                    arr[i] = v
            else:
                setattr(p, name, val)
        return p

    @property
    def cells(self):
        return (self.nx - 1, self.ny - 1, self.nz - 1)
