"""ctypes wrapper of the geometry oracle (TEST INFRASTRUCTURE ONLY).

geom_oracle.c restates, in the reference's loop order, how the reference
turns one closed triangulated body into the pressure solve's inputs:
determine_norm_dir_unstruc (IBM/BOUNDARY_SET_ARCLENGTH_NORM.F90:200-320),
set_iblank_canonical_body_fast with search_vertex_dotNorm
(IBM/BOUNDARY_IBLANK_FAST.F90:2-1024), the ghost list and image-point
coefficients of GCM_set_internal_boundary (IBM/GCM_SET_BOUNDARY.F90:2-494)
with GCM_calc_bodyIntercept_Unstruc
(IBM/GCM_INTERCEPT_KERNELS_UNSTRUC.F90:26-398).  The tests use it as the
checker of the product geometry (csrc/geometry.cpp); nothing in the package
imports it.

Parity pin: the reference cannot be compiled here (no Fortran compiler), so
this restatement is checked by what its rules imply on a closed convex body:
it classifies every cell centre farther than rounding from the surface as
the exact inside test does, and its intercepts lie on the surface
(tests/test_geometry_reference.py).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass

import numpy as np

from .oracle import HERE, build

LIB = HERE / "_build" / "liborgeom.so"
_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_i8 = ctypes.POINTER(ctypes.c_int8)
_i32 = ctypes.POINTER(ctypes.c_int32)


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists() or LIB.stat().st_mtime < (HERE / "geom_oracle.c").stat().st_mtime:
            build()
        L = ctypes.CDLL(str(LIB))
        L.og_orient_inward.argtypes = [ctypes.c_int, _dp, ctypes.c_int, _i32] + [ctypes.c_double] * 3
        L.og_orient_inward.restype = ctypes.c_int
        L.og_iblank.argtypes = [ctypes.c_int] * 3 + [_dp] * 3 + [ctypes.c_int, _dp, ctypes.c_int, _i32, _i8, _i8]
        L.og_iblank.restype = ctypes.c_long
        L.og_ghost_list.argtypes = [ctypes.c_int] * 3 + [_i8, _i8, ctypes.c_int] + [_i32] * 3
        L.og_ghost_list.restype = ctypes.c_int
        L.og_gcm.argtypes = ([ctypes.c_int] * 3 + [_dp] * 3 + [ctypes.c_int, _dp, ctypes.c_int, _i32, ctypes.c_double,
                             ctypes.c_int] + [_i32] * 6 + [_dp] * 5 + [_i32])
        L.og_gcm.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a, t=_dp):
    return a.ctypes.data_as(t)


@dataclass
class ReferenceGeometry:
    tris: np.ndarray          # (3 nt) element nodes in the reference's inward order
    flipped: bool             # whether the orientation step swapped nodes 2 and 3
    iblank: np.ndarray        # (nx+2, ny+2, nz+2) int8, Fortran order
    band: np.ndarray          # cells classified by the dot-normal test
    ghost: np.ndarray
    iG: np.ndarray
    jG: np.ndarray
    kG: np.ndarray
    iCI: np.ndarray
    jCI: np.ndarray
    kCI: np.ndarray
    coeffN: np.ndarray        # (8, nGhost)
    coeffD: np.ndarray
    probe: np.ndarray
    xBI: np.ndarray           # (3, nGhost)
    xIP: np.ndarray
    elem: np.ndarray          # closest element of each ghost (0-based)

    @property
    def nGhost(self) -> int:
        return int(self.iG.size)


def reference_geometry(nx, ny, nz, x, y, z, verts, tris, outside_point, probe_length_normalized=2.0):
    """The reference's inputs for one body: orientation, iblank, ghost list and
    image-point coefficients.  nx, ny, nz are node counts; x, y, z the node
    arrays with ghosts (0:n+1)."""
    L = lib()
    x, y, z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
    v = np.ascontiguousarray(verts, dtype=np.float64).ravel()
    t = np.ascontiguousarray(tris, dtype=np.int32).ravel().copy()
    nv, nt = v.size // 3, t.size // 3
    flipped = L.og_orient_inward(nv, _p(v), nt, _p(t, _i32), *map(float, outside_point))
    if flipped < 0:
        raise ValueError("orientation failed")
    sh = (nx + 2, ny + 2, nz + 2)
    ib = np.zeros(sh, np.int8, order="F")
    band = np.zeros(sh, np.int8, order="F")
    ns = L.og_iblank(nx, ny, nz, _p(x), _p(y), _p(z), nv, _p(v), nt, _p(t, _i32), _p(ib, _i8), _p(band, _i8))
    if ns < 0:
        raise RuntimeError("dot-normal search failed (no reference marker or a list overflow)")
    ghost = np.zeros(sh, np.int8, order="F")
    cap = int(ns) + 1
    iG, jG, kG = (np.zeros(cap, np.int32) for _ in range(3))
    n = L.og_ghost_list(nx, ny, nz, _p(ib, _i8), _p(ghost, _i8), cap, _p(iG, _i32), _p(jG, _i32), _p(kG, _i32))
    if n < 0:
        raise RuntimeError("ghost list capacity")
    iG, jG, kG = iG[:n].copy(), jG[:n].copy(), kG[:n].copy()
    iCI, jCI, kCI, elem = (np.zeros(n, np.int32) for _ in range(4))
    cN = np.zeros((8, n), order="F")
    cD = np.zeros((8, n), order="F")
    bi = np.zeros((3, n), order="F")
    ip = np.zeros((3, n), order="F")
    probe = np.zeros(n)
    rc = L.og_gcm(nx, ny, nz, _p(x), _p(y), _p(z), nv, _p(v), nt, _p(t, _i32), float(probe_length_normalized), n,
                  _p(iG, _i32), _p(jG, _i32), _p(kG, _i32), _p(iCI, _i32), _p(jCI, _i32), _p(kCI, _i32),
                  _p(cN), _p(cD), _p(probe), _p(bi), _p(ip), _p(elem, _i32))
    if rc != 0:
        raise RuntimeError(f"image-point search failed ({rc})")
    return ReferenceGeometry(tris=t, flipped=bool(flipped), iblank=ib, band=band, ghost=ghost, iG=iG, jG=jG, kG=kG,
                             iCI=iCI, jCI=jCI, kCI=kCI, coeffN=cN, coeffD=cD, probe=probe, xBI=bi, xIP=ip, elem=elem)
