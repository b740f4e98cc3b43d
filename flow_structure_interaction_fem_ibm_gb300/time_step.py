"""The fractional time step on the GPU, in the reference's order
(time_step, IBM/CORE_TIME_STEP.F90:201-267, stationary body, NO_VAN_KAN):

    rhs_advec_diff -> set_bc -> rhs_adjust_bc -> solve_ad -> face_vel +
    rhs_poisson -> solve_poisson -> correct_vel -> update_pressure

Every field lives in HBM for the whole run (torch tensors used as device
buffers, (k, j, i)-contiguous, i.e. the reference's column-major
(0:nx+1, 0:ny+1, 0:nz+1) layout); each routine is one C-ABI call of the
native library, so nothing crosses PCIe inside a step except the solvers'
convergence scalars.  pPrime persists between steps (the pressure solve
starts from the previous step's correction, as the reference's module array
does), and so do the outflow pressure-gradient planes of the compatibility
correction.
"""
from __future__ import annotations

import time
from typing import Optional

import numpy as np

from .poisson import PoissonSolver


class FractionalStep:
    """Drives a Problem through fractional time steps on cuda:0.

    ``bc_values`` are the 6 x 3 outer boundary values of set_bc (side x1..z2,
    component u, v, w); ``reinv`` is 1/Re (viscTot = reinv everywhere, a
    laminar run); ``advec_scheme`` 1 ADAMS_BASHFORTH2, 2 CRANK_NICOLSON1 or
    3 CRANK_NICOLSON2 (face_vel re-evaluated inside the momentum iteration).
    The pressure solve uses the problem's solver parameters."""

    def __init__(self, problem, dt: float, reinv: float, bc_values, advec_scheme: int = 2,
                 bc_freq=None, tstart_gust: float = 0.0, pressure_guess: str = "previous"):
        import torch
        self.torch = torch
        if pressure_guess not in ("previous", "extrapolate"):
            raise ValueError("pressure_guess: 'previous' (the reference's) or 'extrapolate'")
        # the pressure solve starts from the previous step's pPrime, as the reference's module
        # array does, or from its linear extrapolation 2 p(n-1) - p(n-2) in time (the same
        # converged pressure, to the solver's tolerance, from a closer start)
        self.pressure_guess = pressure_guess
        self._p_prev = None
        self.pr = problem
        self.dt, self.reinv, self.scheme = float(dt), float(reinv), int(advec_scheme)
        self.values = np.asarray(bc_values, dtype=np.float64).reshape(6, 3)
        self.freq = None if bc_freq is None else np.asarray(bc_freq, dtype=np.float64).reshape(6, 3)
        self.tstart_gust = float(tstart_gust)
        p = problem.params
        if 2 in tuple(p.bc) and p.precision_mode != 1 and p.outer_krylov == 0:
            # zero-gradient outflow makes nlw0 non-zero; the plain stationary MG form keeps
            # the reference's smoother, which adds nlw instead, and stalls
            raise ValueError("zero-gradient outflow needs a pressure solve whose residual includes the outflow "
                             "term nlw0: the mixed form (precision_mode 1) or FGMRES (outer_krylov > 0)")
        self.xout = float(problem.x[p.nx] - problem.x[1])
        self.yout = float(problem.y[p.ny] - problem.y[1])
        self.s = PoissonSolver(p, problem.x, problem.y, problem.z).set_boundary(problem.geom)
        if problem.geom.nGhost:
            self.s.set_velocity_ghosts(problem.geom.coeffD, None)
        shape = tuple(reversed(problem.shape))
        z = lambda: torch.zeros(shape, dtype=torch.float64, device="cuda")
        self.vel = [z() for _ in range(3)]
        self.faces = [z() for _ in range(3)]
        self.bc = [z() for _ in range(9)]
        self.nl = [z() for _ in range(3)]
        self.nl_old = [z() for _ in range(3)]
        self.visc = torch.full(shape, self.reinv, dtype=torch.float64, device="cuda")
        self.pPrime, self.p, self.nlu0 = z(), z(), z()
        # the outflow boundary term of GCM_correct_pressure (IBM/CORE_POISSON.F90:1813-1821) of the
        # last solve: with zero-gradient outflow the corrected faces satisfy div(face) = -dt nlw0
        # in the outflow cell layer (the outflow faces keep their set_bc values), and
        # div(face) = 0 to the solver's residual everywhere else
        self.nlw0 = z()
        self.time = 0.0
        self.ntime = 0
        self.history = []

    # -- host <-> device ---------------------------------------------------
    def _dev(self, a):
        return self.torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).transpose())).cuda()

    @staticmethod
    def host(t):
        return np.asfortranarray(t.cpu().numpy().transpose())

    @staticmethod
    def _ptrs(ts):
        return [t.data_ptr() for t in ts]

    def start(self, u, v, w):
        """Initial velocities (full layout): set_bc, then face_vel for the
        face velocities the first step's advection uses."""
        for t, a in zip(self.vel, (u, v, w)):
            t.copy_(self._dev(a))
        # the library queues its work on its own stream, which does not wait for torch's
        self.torch.cuda.synchronize()
        vp = self._ptrs(self.vel)
        self.s.set_bc(vp, self._ptrs(self.bc), self.values, self.freq, self.time, self.tstart_gust, self.xout,
                      self.yout)
        self.s.face_vel_rhs(self.dt, *vp, *self._ptrs(self.faces), self.nlu0.data_ptr(), d_bc=self._normal_bc())
        return self

    def _normal_bc(self):
        return (self.bc[0].data_ptr(), self.bc[4].data_ptr(), self.bc[8].data_ptr())

    # -- one step ------------------------------------------------------------
    def step(self, timed: bool = False) -> dict:
        """One time step; returns the solvers' iteration counts and residuals
        (and, with ``timed``, the wall milliseconds of each stage)."""
        torch = self.torch
        s, dt = self.s, self.dt
        vp, fp, bp = self._ptrs(self.vel), self._ptrs(self.faces), self._ptrs(self.bc)
        nlp, vis = self._ptrs(self.nl), self.visc.data_ptr()
        bv = [vis] * 3
        ms = {}
        clock = [time.perf_counter()]

        def mark(name):
            if timed:
                torch.cuda.synchronize()
                now = time.perf_counter()
                ms[name] = 1e3 * (now - clock[0])
                clock[0] = now

        s.rhs_advec_diff(dt, vp, fp, vis, nlp, nl_old=self._ptrs(self.nl_old), bc=bp, bcvisc=bv,
                         advec_scheme=self.scheme)
        mark("rhs_advec_diff")
        self.time += dt
        corr = s.set_bc(vp, bp, self.values, self.freq, self.time, self.tstart_gust, self.xout, self.yout)
        mark("set_bc")
        s.rhs_adjust_bc(dt, fp, vis, nlp, bc=bp, bcvisc=bv, advec_scheme=self.scheme)
        mark("rhs_adjust_bc")
        st_ad, it_ad, mr_ad = s.solve_ad(dt, fp, vis, vp, nlp, bcvisc=bv, advec_scheme=self.scheme, bc=bp,
                                         reinv=self.reinv)
        mark("solve_ad")
        s.face_vel_rhs(dt, *vp, *fp, self.nlu0.data_ptr(), d_bc=self._normal_bc())
        mark("face_vel_rhs")
        if self.pressure_guess == "extrapolate":
            torch.cuda.synchronize()   # the library's stream wrote pPrime last step
            if self._p_prev is None:
                self._p_prev = self.pPrime.clone()
            else:
                cur = self.pPrime.clone()
                self.pPrime.mul_(2.0).sub_(self._p_prev)
                self._p_prev = cur
            torch.cuda.synchronize()   # before the library's stream reads it
        st, it, mr, _, _ = s.solve_poisson_device(self.pPrime.data_ptr(), self.nlu0.data_ptr(),
                                                  self.nlw0.data_ptr())
        mark("solve_poisson")
        st_cv = s.correct_vel(dt, self.pPrime.data_ptr(), *vp, *fp, d_bc=self._normal_bc())
        mark("correct_vel")
        s.update_pressure(self.pPrime.data_ptr(), self.p.data_ptr(), 0)
        mark("update_pressure")
        self.ntime += 1
        rec = dict(ntime=self.ntime, poisson_status=st, poisson_iters=it, poisson_maxres=mr, ad_status=st_ad,
                   ad_iters=it_ad, ad_maxres=mr_ad, ghost_status=st_cv, correction_vel=corr)
        if timed:
            rec["ms"] = ms
        self.history.append(rec)
        return rec

    def fields(self) -> dict:
        self.torch.cuda.synchronize()   # the library's stream has finished
        return dict(u=self.host(self.vel[0]), v=self.host(self.vel[1]), w=self.host(self.vel[2]),
                    faces=[self.host(t) for t in self.faces], p=self.host(self.p),
                    pPrime=self.host(self.pPrime), bc=[self.host(t) for t in self.bc])

    def close(self):
        self.s.close()
