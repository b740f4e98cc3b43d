"""Host-side interface to the GPU pressure-Poisson multigrid.

Mirrors the reference's operator interface for this path, one method per
reference routine, with the same argument meaning and the same status codes:

    MG_initial(...)            IBM/CORE_MG.F90:31          -> fsi_mg_create
    set_boundary(geometry)     IBM/BOUNDARY_SET.F90:8      -> fsi_mg_set_geometry
    solve_poisson(pPrime,nlu0) IBM/CORE_POISSON.F90:493    -> fsi_mg_solve / fsi_mg_solve_device
    MG_Solver(var, rr)         IBM/CORE_MG.F90:281         -> fsi_mg_mg_solver
    calc_residual(var, r)      IBM/CORE_POISSON.F90:1111   -> fsi_mg_calc_residual
    subtracting_average_pressure(p)  IBM/CORE_POISSON.F90:419
    GCM_correct_pressure(p)    IBM/CORE_POISSON.F90:1794

Arrays are numpy arrays in Fortran order over the reference's full range
(0:nx+1, 0:ny+1, 0:nz+1).  All compute runs in the CUDA library; there is no
CPU fallback -- a missing library or device raises.
"""
from __future__ import annotations

import ctypes
from typing import Optional

import numpy as np

from . import _native
from .params import FSI_MG_CONVERGED, SolverParams

_dp = ctypes.POINTER(ctypes.c_double)
_i8 = ctypes.POINTER(ctypes.c_int8)
_i32 = ctypes.POINTER(ctypes.c_int32)


class FsiMgError(RuntimeError):
    pass


class RhsAdFields(ctypes.Structure):
    """fsi_mg_rhs_ad_fields of include/fsi_mg.h (device pointers)."""
    _fields_ = [("u", ctypes.c_void_p), ("v", ctypes.c_void_p), ("w", ctypes.c_void_p),
                ("face_u", ctypes.c_void_p), ("face_v", ctypes.c_void_p), ("face_w", ctypes.c_void_p),
                ("bc", ctypes.c_void_p * 9), ("viscTot", ctypes.c_void_p), ("bcvisc", ctypes.c_void_p * 3),
                ("exp_weight", ctypes.c_void_p),
                ("nluOld", ctypes.c_void_p), ("nlvOld", ctypes.c_void_p), ("nlwOld", ctypes.c_void_p),
                ("p", ctypes.c_void_p),
                ("nlu", ctypes.c_void_p), ("nlv", ctypes.c_void_p), ("nlw", ctypes.c_void_p),
                ("reinv", ctypes.c_double)]


class BcValues(ctypes.Structure):
    """fsi_mg_bc_values of include/fsi_mg.h."""
    _fields_ = [("vel", (ctypes.c_double * 3) * 6), ("freq", (ctypes.c_double * 3) * 6),
                ("time", ctypes.c_double), ("tstart_gust", ctypes.c_double),
                ("xout", ctypes.c_double), ("yout", ctypes.c_double)]


def _p(a, t=_dp):
    if a is None:
        return None
    if not a.flags["F_CONTIGUOUS"] and a.ndim > 1:
        raise ValueError("arrays must be Fortran-contiguous")
    return a.ctypes.data_as(t)


def _check(rc: int):
    if rc < 0:
        raise FsiMgError(f"fsi_mg error {rc}: {_native.solver().fsi_mg_last_error().decode()}")
    return rc


class PoissonSolver:
    """One GPU solver context (the reference's MG module state for one grid)."""

    def __init__(self, params: SolverParams, x: np.ndarray, y: np.ndarray, z: np.ndarray):
        self.params = params
        self._cp = params.to_c()
        self.lib = _native.solver()
        h = ctypes.c_void_p()
        self._x, self._y, self._z = (np.ascontiguousarray(a, dtype=np.float64) for a in (x, y, z))
        _check(self.lib.fsi_mg_create(ctypes.byref(self._cp), _p(self._x), _p(self._y), _p(self._z), ctypes.byref(h)))
        self.h = h
        self.shape = (params.nx + 2, params.ny + 2, params.nz + 2)

    # -- MG_initial ------------------------------------------------------
    @classmethod
    def MG_initial(cls, params, x, y, z):
        return cls(params, x, y, z)

    def close(self):
        if getattr(self, "h", None):
            self.lib.fsi_mg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # -- set_boundary ----------------------------------------------------
    def set_boundary(self, geom):
        g = geom
        fl = [np.asfortranarray(a, dtype=np.int8) for a in g.flags]
        self._keep = (np.asfortranarray(g.iblank, dtype=np.int8), np.asfortranarray(g.ghost, dtype=np.int8), fl)
        ib, gm, fl = self._keep
        n = int(g.nGhost)
        arrs = [None] * 6
        coeff = probe = None
        if n > 0:
            arrs = [np.ascontiguousarray(a, dtype=np.int32) for a in (g.iG, g.jG, g.kG, g.iCI, g.jCI, g.kCI)]
            coeff = np.asfortranarray(g.coeff, dtype=np.float64)
            probe = np.ascontiguousarray(g.probe, dtype=np.float64)
        pg = None if g.pgrad is None else np.ascontiguousarray(g.pgrad, dtype=np.float64)
        self._keep2 = (arrs, coeff, probe, pg)
        _check(self.lib.fsi_mg_set_geometry(self.h, _p(ib, _i8), _p(gm, _i8), *[_p(a, _i8) for a in fl], n,
                                            *[_p(a, _i32) for a in arrs], _p(coeff), _p(probe), _p(pg)))
        return self

    # -- solve_poisson ---------------------------------------------------
    def solve_poisson(self, pPrime: np.ndarray, nlu0: np.ndarray, want_nlw0: bool = False):
        """In-place solve on host arrays.  Returns (status, iters, maxres, loc, compTime[, nlw0])."""
        assert pPrime.shape == self.shape and nlu0.shape == self.shape
        nlw0 = np.zeros(self.shape, order="F") if want_nlw0 else None
        it, mr, ct = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        loc = (ctypes.c_int * 3)()
        st = _check(self.lib.fsi_mg_solve(self.h, _p(pPrime), _p(np.asfortranarray(nlu0)), _p(nlw0), ctypes.byref(it),
                                          ctypes.byref(mr), loc, ctypes.byref(ct)))
        out = (st, it.value, mr.value, tuple(loc), ct.value)
        return out + ((nlw0,) if want_nlw0 else ())

    def solve_poisson_device(self, d_pPrime: int, d_nlu0: int, d_nlw0: Optional[int] = None):
        """Solve on device pointers (e.g. torch tensor .data_ptr()) of full-layout arrays."""
        it, mr, ct = ctypes.c_int(), ctypes.c_double(), ctypes.c_double()
        loc = (ctypes.c_int * 3)()
        st = _check(self.lib.fsi_mg_solve_device(self.h, ctypes.c_void_p(d_pPrime), ctypes.c_void_p(d_nlu0),
                                                 ctypes.c_void_p(d_nlw0) if d_nlw0 else None, ctypes.byref(it),
                                                 ctypes.byref(mr), loc, ctypes.byref(ct)))
        return st, it.value, mr.value, tuple(loc), ct.value

    # -- steps either side of the solve (device pointers, full layout) ----
    def face_vel_rhs(self, dt: float, d_u: int, d_v: int, d_w: int, d_face_u: int, d_face_v: int, d_face_w: int,
                     d_nlu0: int, d_bc=(None, None, None), frac_step_type: int = 0, d_p: Optional[int] = None):
        """face_vel + rhs_poisson (IBM/CORE_FRAC_STEP_ROUTINES.F90:6-240,
        IBM/CORE_POISSON.F90:123-417) on device arrays.  Returns sum nlu0 dV."""
        vp = lambda a: ctypes.c_void_p(a) if a else None
        total = ctypes.c_double()
        _check(self.lib.fsi_mg_face_vel_rhs(self.h, frac_step_type, float(dt), vp(d_u), vp(d_v), vp(d_w), vp(d_p),
                                            vp(d_bc[0]), vp(d_bc[1]), vp(d_bc[2]), vp(d_face_u), vp(d_face_v),
                                            vp(d_face_w), vp(d_nlu0), ctypes.byref(total)))
        return total.value

    def correct_vel(self, dt: float, d_pPrime: int, d_u: int, d_v: int, d_w: int, d_face_u: int, d_face_v: int,
                    d_face_w: int, d_bc=(None, None, None)):
        """correct_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:244-448) on device
        arrays (updated in place); the ghost-cell velocities once
        set_velocity_ghosts registered them.  Returns the status (2: the ghost
        velocities did not converge)."""
        vp = lambda a: ctypes.c_void_p(a) if a else None
        return _check(self.lib.fsi_mg_correct_vel(self.h, float(dt), vp(d_pPrime), vp(d_u), vp(d_v), vp(d_w),
                                                  vp(d_bc[0]), vp(d_bc[1]), vp(d_bc[2]), vp(d_face_u),
                                                  vp(d_face_v), vp(d_face_w)))

    def rhs_advec_diff(self, dt: float, vel, faces, visc, nl, nl_old=(None, None, None), bc=(None,) * 9,
                       bcvisc=(None,) * 3, exp_weight=None, p=None, advec_scheme: int = 2,
                       frac_step_type: int = 0):
        """rhs_advec_diff (IBM/CORE_RHS_AD.F90:13-585) on device pointers:
        vel = (u, v, w), faces, visc (viscTot), nl = (nlu, nlv, nlw) OUT,
        nl_old INOUT with AB2 (advec_scheme 1)."""
        f = RhsAdFields()
        f.u, f.v, f.w = vel
        f.face_u, f.face_v, f.face_w = faces
        for q in range(9):
            f.bc[q] = bc[q]
        f.viscTot = visc
        for q in range(3):
            f.bcvisc[q] = bcvisc[q]
        f.exp_weight = exp_weight
        f.nluOld, f.nlvOld, f.nlwOld = nl_old
        f.p = p
        f.nlu, f.nlv, f.nlw = nl
        _check(self.lib.fsi_mg_rhs_advec_diff(self.h, advec_scheme, frac_step_type, float(dt), ctypes.byref(f)))

    @staticmethod
    def _ad_fields(faces, visc, nl, bc=(None,) * 9, bcvisc=(None,) * 3, reinv=0.0):
        f = RhsAdFields()
        f.reinv = float(reinv)
        f.face_u, f.face_v, f.face_w = faces
        for q in range(9):
            f.bc[q] = bc[q]
        f.viscTot = visc
        for q in range(3):
            f.bcvisc[q] = bcvisc[q]
        f.nlu, f.nlv, f.nlw = nl
        return f

    def rhs_adjust_bc(self, dt: float, faces, visc, nl, bc=(None,) * 9, bcvisc=(None,) * 3, advec_scheme: int = 2):
        """rhs_adjust_bc (IBM/CORE_RHS_AD.F90:588-780) on device pointers; nl INOUT."""
        f = self._ad_fields(faces, visc, nl, bc, bcvisc)
        _check(self.lib.fsi_mg_rhs_adjust_bc(self.h, advec_scheme, float(dt), ctypes.byref(f)))

    def solve_ad(self, dt: float, faces, visc, vel, nl, bcvisc=(None,) * 3, advec_scheme: int = 2,
                 bc=(None,) * 9, reinv: float = 0.0):
        """solve_ad (IBM/CORE_SOLVE_AD.F90:12-267) on device pointers: vel =
        (u, v, w) INOUT, nl the right-hand sides.  With zero-gradient sides and
        a GCM body the faces, the zero-gradient planes of bc (all nine arrays)
        and nl are INOUT too (GCM_enforce_global_mass_consv with 1/Re = reinv);
        advec_scheme 3 (CRANK_NICOLSON2) rewrites the faces every iteration with
        face_vel of the current velocities (bc's normal components, 0 where NULL).
        Returns (status, iterations, maxres)."""
        f = self._ad_fields(faces, visc, nl, bc=bc, bcvisc=bcvisc, reinv=reinv)
        it, mr = ctypes.c_int(), ctypes.c_double()
        st = _check(self.lib.fsi_mg_solve_ad(self.h, advec_scheme, float(dt), ctypes.byref(f),
                                             *(ctypes.c_void_p(a) if a else None for a in vel), ctypes.byref(it),
                                             ctypes.byref(mr)))
        return st, it.value, mr.value

    def set_velocity_ghosts(self, coeffGCMD, bi=None, probe_length_normalized: float = 2.0):
        """Ghost-cell velocities for correct_vel (GCM_vel_set_bc_internal):
        coeffGCMD (8, nGhost) Fortran order, bi = (uBI, vBI, wBI) or None (body
        at rest); the weights follow probeLengthNormalized (IBM/MAIN.F90:913-914)."""
        bw = probe_length_normalized / (probe_length_normalized - 1.0)
        iw = 1.0 / (probe_length_normalized - 1.0)
        cd = None if coeffGCMD is None else np.asfortranarray(coeffGCMD, dtype=np.float64)
        u, v, w = (None, None, None) if bi is None else (np.ascontiguousarray(a, dtype=np.float64) for a in bi)
        _check(self.lib.fsi_mg_set_velocity_ghosts(self.h, _p(cd), _p(u), _p(v), _p(w), bw, iw))
        self._vg_keep = (cd, u, v, w)
        return self

    def set_bc(self, d_vel, d_bc9, values, freq=None, time: float = 0.0, tstart_gust: float = 0.0,
               xout: float = 1.0, yout: float = 1.0) -> float:
        """set_bc (IBM/CORE_SET_BC.F90:22-298, outer sides) with
        enforce_global_mass_consv and set_outer_ghost_vel on device arrays:
        d_vel = (u, v, w) INOUT, d_bc9 the nine boundary-value arrays in the
        order bcxu, bcyu, bczu, bcxv, ... (OUT on the planes); values / freq
        6 x 3 (side x1..z2, component u, v, w).  Returns correction_vel."""
        bv = BcValues()
        val = np.asarray(values, dtype=np.float64).reshape(6, 3)
        fr = np.zeros((6, 3)) if freq is None else np.asarray(freq, dtype=np.float64).reshape(6, 3)
        for s in range(6):
            for q in range(3):
                bv.vel[s][q] = float(val[s, q])
                bv.freq[s][q] = float(fr[s, q])
        bv.time, bv.tstart_gust, bv.xout, bv.yout = float(time), float(tstart_gust), float(xout), float(yout)
        bcs = (ctypes.c_void_p * 9)(*[ctypes.c_void_p(a) for a in d_bc9])
        corr = ctypes.c_double()
        _check(self.lib.fsi_mg_set_bc(self.h, ctypes.byref(bv), *(ctypes.c_void_p(a) for a in d_vel), bcs,
                                      ctypes.byref(corr)))
        return corr.value

    def update_pressure(self, d_pPrime: int, d_p: int, frac_step_type: int = 0):
        """update_pressure (IBM/CORE_FRAC_STEP_ROUTINES.F90:949-967) on device arrays."""
        _check(self.lib.fsi_mg_update_pressure(self.h, frac_step_type, ctypes.c_void_p(d_pPrime),
                                               ctypes.c_void_p(d_p)))

    # -- finer hooks -----------------------------------------------------
    def MG_Solver(self, var: np.ndarray, rr: np.ndarray) -> float:
        ct = ctypes.c_double()
        _check(self.lib.fsi_mg_mg_solver(self.h, _p(var), _p(np.asfortranarray(rr)), ctypes.byref(ct)))
        return ct.value

    def calc_residual(self, var, r):
        m = ctypes.c_double()
        loc = (ctypes.c_int * 3)()
        _check(self.lib.fsi_mg_calc_residual(self.h, _p(np.asfortranarray(var)), _p(np.asfortranarray(r)),
                                             ctypes.byref(m), loc))
        return m.value, tuple(loc)

    def set_fresh_cells(self, fresh_cell):
        """fresh_cell (int8, full layout) of a moving body for the mean removal;
        None turns it off (IBM/CORE_POISSON.F90:459-488)."""
        if fresh_cell is None:
            _check(self.lib.fsi_mg_set_fresh_cells(self.h, None))
        else:
            f = np.asfortranarray(fresh_cell, dtype=np.int8)
            if f.shape != self.shape:
                raise ValueError(f"fresh_cell has shape {f.shape}, expected {self.shape}")
            _check(self.lib.fsi_mg_set_fresh_cells(self.h, f.ctypes.data_as(ctypes.c_void_p)))
        return self

    def subtracting_average_pressure(self, p):
        _check(self.lib.fsi_mg_subtract_average(self.h, _p(p)))
        return p

    def GCM_correct_pressure(self, p, want_nlw0=False):
        nlw0 = np.zeros(self.shape, order="F") if want_nlw0 else None
        _check(self.lib.fsi_mg_correct_pressure(self.h, _p(p), _p(nlw0)))
        return (p, nlw0) if want_nlw0 else p

    def pgrad(self):
        from .problem import pgrad_size
        out = np.zeros(pgrad_size(self.params))
        _check(self.lib.fsi_mg_get_pgrad(self.h, _p(out)))
        return out

    def level_count(self, d):
        return _check(self.lib.fsi_mg_level_count(self.h, d))

    def level_size(self, d, n):
        return _check(self.lib.fsi_mg_level_size(self.h, d, n))

    def level_shape(self, d, n):
        p = self.params
        sh = [p.nx + 1, p.ny + 1, p.nz + 1]
        if n > 1:
            sh[d] = self.level_size(d, n) + 2
        return tuple(sh)

    def debug_op(self, op, d, n, a=None, b=None, c=None):
        def vp(x):
            return None if x is None else ctypes.c_void_p(x.ctypes.data)
        return _check(self.lib.fsi_mg_debug_level_op(self.h, op, d, n, vp(a), vp(b), vp(c)))

    def stats(self):
        out = np.zeros(8)
        _check(self.lib.fsi_mg_stats(self.h, _p(out), 8))
        return dict(iters=int(out[0]), maxres=out[1], seconds=out[2], ghost_sweeps=int(out[3]),
                    launches=int(out[4]), device_bytes=int(out[5]), wall_seconds=out[6], e2e_seconds=out[7])

    def residual_history(self):
        n = _check(self.lib.fsi_mg_residual_history(self.h, None, 0))
        out = np.zeros(max(n, 1))
        self.lib.fsi_mg_residual_history(self.h, _p(out), n)
        return out[:n]

    def time_kernel(self, which: int, precision: int, reps: int = 20):
        """Average device time (ms) of one kernel and its algorithmic bytes per launch."""
        ms, nb = ctypes.c_double(), ctypes.c_double()
        _check(self.lib.fsi_mg_time_kernel(self.h, which, precision, reps, ctypes.byref(ms), ctypes.byref(nb)))
        return ms.value, nb.value

    def line_timing(self, enable: int = -1):
        """Event timing of the level-1 line launches inside solves (enable 1:
        reset and start, 0: stop, -1: read).  Returns per precision the launch
        count, summed ms and algorithmic bytes per launch."""
        out = np.zeros(6)
        _check(self.lib.fsi_mg_line_timing(self.h, enable, _p(out)))
        return {"fp32": {"launches": int(out[0]), "ms": out[1], "alg_bytes": out[2]},
                "fp64": {"launches": int(out[3]), "ms": out[4], "alg_bytes": out[5]}}


def solve(problem, p0=None, **overrides):
    """Convenience: build a solver for ``problem``, solve from ``p0`` (zeros)."""
    params = problem.params
    for k, v in overrides.items():
        setattr(params, k, v)
    s = PoissonSolver(params, problem.x, problem.y, problem.z).set_boundary(problem.geom)
    p = np.zeros(problem.shape, order="F") if p0 is None else np.array(p0, order="F", copy=True)
    st, it, mr, loc, ct, nlw0 = s.solve_poisson(p, problem.nlu0, want_nlw0=True)
    res = dict(p=p, status=st, iters=it, maxres=mr, loc=loc, seconds=ct, nlw0=nlw0, stats=s.stats(),
               hist=s.residual_history())
    s.close()
    return res


__all__ = ["PoissonSolver", "FsiMgError", "solve", "FSI_MG_CONVERGED"]
