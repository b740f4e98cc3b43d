"""ctypes wrapper of the CPU oracle (TEST INFRASTRUCTURE ONLY).

The oracle is a plain-C FP64 restatement of the reference's pressure-Poisson
multigrid path (see mg_oracle.h).  Only the tests, the smoke check and the
CPU-baseline leg of the benchmark import this module, and only as the
checker; the product solver never calls it.

Parity pin: the reference cannot be built here (no Fortran compiler), so the
oracle is pinned by the reference's own known-answer test (Poisson_Tester,
IBM/CORE_POISSON.F90:1386-1790) and by internal cross-checks (MG against the
plain line-SOR path, tdma against a dense solve), all in tests/.
"""
from __future__ import annotations

import ctypes
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "_build" / "libmgoracle.so"

_lib = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_i8 = ctypes.POINTER(ctypes.c_int8)
_i32 = ctypes.POINTER(ctypes.c_int32)


def build():
    subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not LIB.exists() or LIB.stat().st_mtime < (HERE / "mg_oracle.c").stat().st_mtime:
            build()
        L = ctypes.CDLL(str(LIB))
        L.or_create.restype = ctypes.c_void_p
        L.or_create.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.or_destroy.argtypes = [ctypes.c_void_p]
        L.or_destroy.restype = None
        L.or_set_geometry.argtypes = [ctypes.c_void_p] + [_i8] * 8 + [ctypes.c_int] + [_i32] * 6 + [_dp] * 3
        L.or_solve.argtypes = [ctypes.c_void_p, _dp, _dp, _dp, _ip, _dp, _ip, _dp]
        L.or_mg_solver.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.or_calc_residual.argtypes = [ctypes.c_void_p, _dp, _dp, _ip]
        L.or_calc_residual.restype = ctypes.c_double
        L.or_subtract_average.argtypes = [ctypes.c_void_p, _dp]
        L.or_subtract_average.restype = None
        L.or_set_fresh.argtypes = [ctypes.c_void_p, _i8]
        L.or_set_fresh.restype = None
        L.or_gcm_correct_pressure.argtypes = [ctypes.c_void_p, _dp]
        L.or_gcm_correct_pressure.restype = None
        L.or_level_count.argtypes = [ctypes.c_void_p, ctypes.c_int]
        L.or_level_size.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int]
        L.or_level_metrics.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int] + [_dp] * 6
        L.or_level_metrics.restype = None
        L.or_coarse_iblank.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _i8]
        L.or_coarse_iblank.restype = None
        L.or_level_flags.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _i8]
        L.or_level_flags.restype = None
        for nm in ("or_itsolv_level",):
            getattr(L, nm).argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp]
            getattr(L, nm).restype = None
        L.or_residual_level.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp]
        L.or_residual_level.restype = None
        L.or_restrict_level.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp]
        L.or_restrict_level.restype = None
        L.or_prolong_level.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_int, _dp, _dp]
        L.or_prolong_level.restype = None
        L.or_ghost_update.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, ctypes.c_int, ctypes.c_int, _ip, _dp]
        L.or_ghost_update.restype = None
        L.or_tdma.argtypes = [_dp, _dp, _dp, _dp, _dp, ctypes.c_int, ctypes.c_int]
        L.or_tdma.restype = None
        L.or_outer_ghost.argtypes = [ctypes.c_void_p, _dp]
        L.or_outer_ghost.restype = None
        L.or_get_pgrad.argtypes = [ctypes.c_void_p, _dp]
        L.or_get_pgrad.restype = None
        L.or_face_vel.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double] + [_dp] * 10
        L.or_face_vel.restype = None
        L.or_rhs_poisson.argtypes = [ctypes.c_void_p, ctypes.c_double] + [_dp] * 4
        L.or_rhs_poisson.restype = ctypes.c_double
        L.or_correct_vel.argtypes = [ctypes.c_void_p, ctypes.c_double] + [_dp] * 10
        L.or_correct_vel.restype = None
        L.or_update_pressure.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp, _dp]
        L.or_update_pressure.restype = None
        L.or_set_bc.argtypes = ([ctypes.c_void_p, _dp, _dp] + [ctypes.c_double] * 4 + [_dp] * 3
                                + [ctypes.POINTER(_dp), _dp])
        L.or_set_bc.restype = ctypes.c_int
        L.or_set_vel_ghosts.argtypes = [ctypes.c_void_p] + [_dp] * 4 + [ctypes.c_double] * 2
        L.or_set_vel_ghosts.restype = None
        L.or_vel_ghost_iters.argtypes = [ctypes.c_void_p]
        L.or_rhs_advec_diff.argtypes = ([ctypes.c_void_p, ctypes.c_int, ctypes.c_int, ctypes.c_double] + [_dp] * 6
                                        + [ctypes.POINTER(_dp), _dp, ctypes.POINTER(_dp)] + [_dp] * 8)
        L.or_rhs_advec_diff.restype = None
        L.or_set_solve_ad.argtypes = [ctypes.c_void_p, ctypes.c_double, _dp, ctypes.POINTER(_dp)]
        L.or_set_solve_ad.restype = None
        L.or_rhs_adjust_bc.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.POINTER(_dp),
                                       ctypes.POINTER(_dp), _dp, _dp, _dp]
        L.or_rhs_adjust_bc.restype = None
        L.or_solve_ad.argtypes = ([ctypes.c_void_p, ctypes.c_int, ctypes.c_double, ctypes.POINTER(_dp)] + [_dp] * 6
                                  + [ctypes.POINTER(_dp), ctypes.c_double, ctypes.c_int, _dp])
        L.or_solve_ad.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a, t=_dp):
    return None if a is None else a.ctypes.data_as(t)


def tdma(a, b, c, r, n1, n2):
    u = np.zeros_like(r)
    lib().or_tdma(_p(a), _p(b), _p(c), _p(r), _p(u), n1, n2)
    return u


class Oracle:
    """One reference solver state (module variables of the reference)."""

    def __init__(self, problem, **overrides):
        self.problem = problem
        params = problem.params
        for k, v in overrides.items():
            setattr(params, k, v)
        self.params = params
        self._cp = params.to_c()
        L = lib()
        self.h = L.or_create(ctypes.byref(self._cp), _p(problem.x), _p(problem.y), _p(problem.z))
        if not self.h:
            raise ValueError("oracle rejected the parameters")
        g = problem.geom
        f = g.flags
        rc = L.or_set_geometry(self.h, _p(g.iblank, _i8), _p(g.ghost, _i8), *[_p(a, _i8) for a in f],
                               g.nGhost, _p(g.iG, _i32), _p(g.jG, _i32), _p(g.kG, _i32),
                               _p(g.iCI, _i32), _p(g.jCI, _i32), _p(g.kCI, _i32),
                               _p(g.coeff), _p(g.probe), _p(g.pgrad))
        if rc != 0:
            raise ValueError(f"oracle geometry rejected ({rc})")

    def close(self):
        if self.h:
            lib().or_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, p0=None):
        pr = self.problem
        p = np.zeros(pr.shape, order="F") if p0 is None else np.array(p0, order="F", copy=True)
        nlw0 = np.zeros(pr.shape, order="F")
        it, mr = ctypes.c_int(), ctypes.c_double()
        loc = (ctypes.c_int * 3)()
        hist = np.zeros(self.params.iterMax_Poisson + 1)
        st = lib().or_solve(self.h, _p(p), _p(pr.nlu0), _p(nlw0), ctypes.byref(it), ctypes.byref(mr), loc, _p(hist))
        return dict(p=p, nlw0=nlw0, status=st, iters=it.value, maxres=mr.value, loc=tuple(loc),
                    hist=hist[: it.value].copy())

    def mg_solver(self, var, rr):
        lib().or_mg_solver(self.h, _p(var), _p(rr))
        return var

    def calc_residual(self, var, r):
        loc = (ctypes.c_int * 3)()
        m = lib().or_calc_residual(self.h, _p(var), _p(r), loc)
        return m, tuple(loc)

    def set_fresh(self, fresh):
        """fresh_cell array (full layout, int8) used by subtract_average; None clears it."""
        if fresh is None:
            lib().or_set_fresh(self.h, None)
        else:
            self._fresh = np.asfortranarray(fresh, dtype=np.int8)
            lib().or_set_fresh(self.h, _p(self._fresh, _i8))
        return self

    def subtract_average(self, p):
        lib().or_subtract_average(self.h, _p(p))
        return p

    def correct_pressure(self, p):
        lib().or_gcm_correct_pressure(self.h, _p(p))
        return p

    def pgrad(self):
        from flow_structure_interaction_fem_ibm_gb300.problem import pgrad_size
        out = np.zeros(pgrad_size(self.params))
        lib().or_get_pgrad(self.h, _p(out))
        return out

    # ----- fractional-step routines either side of the solve -----
    def face_vel(self, dt, u, v, w, p=None, bc=(None, None, None), frac_step_type=0, faces=None):
        """face_vel; returns (face_u, face_v, face_w).  `faces` (three arrays,
        updated in place) keeps the caller's values outside the written faces."""
        sh = self.problem.shape
        fu, fv, fw = faces if faces is not None else (np.zeros(sh, order="F") for _ in range(3))
        lib().or_face_vel(self.h, frac_step_type, dt, _p(u), _p(v), _p(w), _p(p), _p(bc[0]), _p(bc[1]), _p(bc[2]),
                          _p(fu), _p(fv), _p(fw))
        return fu, fv, fw

    def rhs_poisson(self, dt, face_u, face_v, face_w):
        nlu0 = np.zeros(self.problem.shape, order="F")
        s = lib().or_rhs_poisson(self.h, dt, _p(face_u), _p(face_v), _p(face_w), _p(nlu0))
        return nlu0, s

    def correct_vel(self, dt, pPrime, u, v, w, face_u, face_v, face_w, bc=(None, None, None)):
        """In place on u, v, w and the faces."""
        lib().or_correct_vel(self.h, dt, _p(pPrime), _p(u), _p(v), _p(w), _p(bc[0]), _p(bc[1]), _p(bc[2]),
                             _p(face_u), _p(face_v), _p(face_w))

    def set_vel_ghosts(self, coeffD, bi=None, probe_length_normalized=2.0):
        """Ghost-cell velocities for correct_vel (weights of IBM/MAIN.F90:913-914)."""
        bw = probe_length_normalized / (probe_length_normalized - 1.0)
        iw = 1.0 / (probe_length_normalized - 1.0)
        self._vg = (None if coeffD is None else np.asfortranarray(coeffD, dtype=np.float64),) + \
            ((None, None, None) if bi is None else tuple(np.ascontiguousarray(a, dtype=np.float64) for a in bi))
        lib().or_set_vel_ghosts(self.h, *(_p(a) for a in self._vg), bw, iw)
        return self

    def vel_ghost_iters(self):
        return lib().or_vel_ghost_iters(self.h)

    def rhs_advec_diff(self, dt, u, v, w, faces, visc, nl_old, nl, bc9=(None,) * 9, bcvisc=(None,) * 3,
                       exp_weight=None, p=None, advec_scheme=2, frac_step_type=0):
        """rhs_advec_diff; nl_old (AB2 history) and nl (nlu, nlv, nlw) are
        updated in place.  advec_scheme 1 ADAMS_BASHFORTH2, 2/3 CRANK_NICOLSON."""
        b9 = (_dp * 9)(*[_p(a) for a in bc9])
        b3 = (_dp * 3)(*[_p(a) for a in bcvisc])
        lib().or_rhs_advec_diff(self.h, advec_scheme, frac_step_type, dt, _p(u), _p(v), _p(w), *(_p(a) for a in faces),
                                b9, _p(visc), b3, _p(exp_weight), *(_p(a) for a in nl_old), _p(p),
                                *(_p(a) for a in nl))
        return nl

    # ----- implicit momentum solve -----
    def set_solve_ad(self, dt, visc, bcvisc=(None,) * 3):
        lib().or_set_solve_ad(self.h, dt, _p(visc), (_dp * 3)(*[_p(a) for a in bcvisc]))

    def rhs_adjust_bc(self, dt, faces, nl, bc9=(None,) * 9, advec_scheme=2):
        lib().or_rhs_adjust_bc(self.h, advec_scheme, dt, (_dp * 3)(*[_p(a) for a in faces]),
                               (_dp * 9)(*[_p(a) for a in bc9]), *(_p(a) for a in nl))
        return nl

    def solve_ad(self, dt, faces, vel, nl, advec_scheme=2, order=0, bc9=None, reinv=0.0):
        """solve_ad on vel = (u, v, w) in place; returns (iterations, maxres).
        With zero-gradient sides and a GCM body each iteration also rewrites
        faces, the zero-gradient planes of bc9 and nl (GCM_enforce_global_mass_consv
        with 1/Re = reinv); with advec_scheme 3 (CRANK_NICOLSON2) each iteration
        rewrites faces with face_vel of the current velocities (bc9's normal
        components, or 0 without bc9)."""
        mr = ctypes.c_double()
        b9 = None if bc9 is None else (_dp * 9)(*[_p(a) for a in bc9])
        it = lib().or_solve_ad(self.h, advec_scheme, dt, (_dp * 3)(*[_p(a) for a in faces]), *(_p(a) for a in vel),
                               *(_p(a) for a in nl), b9, reinv, order, ctypes.byref(mr))
        if it < 0:
            raise ValueError("solve_ad: zero-gradient sides with a GCM body need bc9 and outflow_area > 0")
        return it, mr.value

    def set_bc(self, vel, bc9, values, freq=None, time=0.0, tstart_gust=0.0, xout=1.0, yout=1.0):
        """set_bc (outer sides), enforce_global_mass_consv and set_outer_ghost_vel;
        vel = (u, v, w) and the nine bc arrays updated in place; values and freq
        are 6 x 3 (side x1..z2, component u, v, w).  Returns correction_vel."""
        val = np.ascontiguousarray(values, dtype=np.float64).reshape(18)
        fr = np.zeros(18) if freq is None else np.ascontiguousarray(freq, dtype=np.float64).reshape(18)
        corr = ctypes.c_double()
        rc = lib().or_set_bc(self.h, _p(val), _p(fr), time, tstart_gust, xout, yout, *(_p(a) for a in vel),
                             (_dp * 9)(*[_p(a) for a in bc9]), ctypes.byref(corr))
        if rc != 0:
            raise ValueError("set_bc: unsupported boundary type")
        return corr.value

    def update_pressure(self, pPrime, p, frac_step_type=0):
        lib().or_update_pressure(self.h, frac_step_type, _p(pPrime), _p(p))
        return p

    # ----- per-level operators (kernel parity) -----
    def nlev(self, d):
        return lib().or_level_count(self.h, d)

    def level_size(self, d, n):
        return lib().or_level_size(self.h, d, n)

    def level_shape(self, d, n):
        """Shape of a level-n array of the d-cycle: (0:m+1) along d, (0:n) elsewhere."""
        p = self.params
        sh = [p.nx + 1, p.ny + 1, p.nz + 1]
        if n > 1:
            sh[d] = self.level_size(d, n) + 2
        return tuple(sh)

    def coarse_iblank(self, d, n):
        out = np.zeros(self.level_shape(d, n), np.int8, order="F")
        lib().or_coarse_iblank(self.h, d, n, _p(out, _i8))
        return out

    def level_flags(self, d, n):
        sh = self.problem.shape
        out = np.zeros((6,) + sh, np.int8)
        buf = np.zeros(6 * int(np.prod(sh)), np.int8)
        lib().or_level_flags(self.h, d, n, _p(buf, _i8))
        return [buf[s * buf.size // 6:(s + 1) * buf.size // 6].reshape(sh, order="F") for s in range(6)]

    def itsolv(self, d, n, var, r):
        lib().or_itsolv_level(self.h, d, n, _p(var), _p(r))
        return var

    def residual(self, d, n, var, r):
        res = np.zeros_like(var)
        lib().or_residual_level(self.h, d, n, _p(var), _p(r), _p(res))
        return res

    def restrict(self, d, n, res):
        out = np.zeros(self.level_shape(d, n + 1), order="F")
        lib().or_restrict_level(self.h, d, n, _p(res), _p(out))
        return out

    def prolong(self, d, n, phi):
        out = np.zeros(self.level_shape(d, n), order="F")
        lib().or_prolong_level(self.h, d, n, _p(phi), _p(out))
        return out

    def outer_ghost(self, var):
        lib().or_outer_ghost(self.h, _p(var))
        return var

    def ghost_update(self, var):
        it = ctypes.c_int()
        flag = ctypes.c_double()
        sh = var.shape
        lib().or_ghost_update(self.h, _p(var), sh[0] - 1, sh[1] - 1, sh[2] - 1, ctypes.byref(it), ctypes.byref(flag))
        return it.value, flag.value
