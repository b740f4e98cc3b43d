"""Adjoint of the whole fractional time step (torch harness around the GPU
step), for rollouts such as the sphere-wake channel.

One step of ``time_step.FractionalStep`` (IBM/CORE_TIME_STEP.F90:201-267,
NO_VAN_KAN, Crank-Nicolson 1 / 2 or Adams-Bashforth, central or hybrid
advection, stationary body, laminar viscosity 1/Re) maps the state
S = (u, v, w, face_u, face_v, face_w, bc9[, nl_old with Adams-Bashforth]) to
the next one:

    nl   = rhs_advec_diff(vel, faces, bc9)          IBM/CORE_RHS_AD.F90:13-585
    vel1, bc1 = set_bc(vel, t + dt)                 IBM/CORE_SET_BC.F90:22-377,
                                                    IBM/CORE_SET_OUTER_GHOST.F90:1-63
    nl1  = rhs_adjust_bc(faces, bc1, nl)            IBM/CORE_RHS_AD.F90:588-780
    vel2, bc2 = solve_ad(vel1, nl1, bc1, faces)     IBM/CORE_SOLVE_AD.F90:12-267 (implicit)
    faces3 = face_vel(vel2, bc2); f = rhs_poisson   IBM/CORE_FRAC_STEP_ROUTINES.F90:6-240,
                                                    IBM/CORE_POISSON.F90:123-163
    p    = solve_poisson(f)                         the GPU multigrid (implicit)
    vel3, faces4 = correct_vel(p, vel2, faces3)     IBM/CORE_FRAC_STEP_ROUTINES.F90:244-448

Every explicit routine is restated here as differentiable FP64 torch
(``StepOperators``, checked against the oracle's literal loops), so torch
autograd supplies their transposes.  The two implicit solves are
``torch.autograd.Function``s: their forward runs the product (the C-ABI
solve_ad and pressure solve on device arrays) and their backward solves the
transposed linearised system:

* solve_ad with zero-gradient outflow and a GCM body ends every iteration
  with GCM_enforce_global_mass_consv (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:6-252),
  so its converged state X = (u, v, w, s) -- s the accumulated shift of the
  zero-gradient planes -- solves F(X, theta) = 0: the momentum rows formed
  with the faces face_vel(u, bc + s e) and the right-hand sides
  nl + T(bc) - T(bc + s e), the ghost-cell velocity rows
  (IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:126-247), u = 0 in dead cells and
  zero net face flux.  Backward: GMRES on J^T lambda = Xbar with J^T v a
  vector-Jacobian product of F, then thetabar = -(dF/dtheta)^T lambda.
* The pressure solve with zero-gradient outflow solves
  B p = A_eff p + n1 (phi . p) / outflow_area = f, phi = A_eff^T vol (the
  compatibility fixed point of GCM_enforce_p_compatibility,
  IBM/GCM_GLOBAL_MASS_CONSERVE.F90:260-394); backward: B^T z = E^T pbar by
  FGMRES preconditioned with one forward multigrid application, and
  fbar = z - w_B (1 . z) / (1 . w_B), w_B the left null vector of B.

``RolloutAdjoint`` runs the forward rollout on the product, keeps the state
every ``checkpoint_every`` steps, and in the backward pass recomputes each
segment's states and pulls the cotangent back step by step.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .adjoint import ProjectionOperators, _DeviceMG, fgmres, fortran_zeros, as_fortran
from .grid import Metrics
from .params import DIM_3D, GCM_METHOD

_INC = ((0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1))  # incI/J/K
BC_DIRICHLET, BC_ZERO_GRADIENT, BC_SYMMETRY = 1, 2, 4


class StepOperators:
    """Differentiable FP64 restatement of the explicit routines of one
    fractional step on one geometry (arrays indexed [i, j, k] over the full
    (0:nx+1, 0:ny+1, 0:nz+1) layout), plus the residuals of the two implicit
    solves.  Constant viscosity ``reinv`` (viscTot = bcvisc = 1/Re)."""

    def __init__(self, problem, dt: float, reinv: float, bc_values, device="cpu", advec_scheme: int = 2):
        p = problem.params
        if advec_scheme not in (1, 2, 3):
            raise ValueError("advec_scheme 1 (ADAMS_BASHFORTH2), 2 or 3 (CRANK_NICOLSON1 / 2)")
        if p.ndim != DIM_3D:
            raise ValueError("the step adjoint is 3D")
        for s, t in enumerate(p.bc):
            if t not in (BC_DIRICHLET, BC_ZERO_GRADIENT, BC_SYMMETRY):
                raise ValueError(f"velocity side {s}: type {t} is not restated (Dirichlet, zero gradient, symmetry)")
        self.pr = problem
        self.dev = torch.device(device)
        self.scheme = int(advec_scheme)
        self.dt, self.reinv = float(dt), float(reinv)
        # the implicit convective terms: Crank-Nicolson halves, Adams-Bashforth none
        self.half = 0.0 if self.scheme == 1 else 0.5 * self.dt
        # hybrid advection: second-order upwind faces blended in by alfa (IBM/MAIN.F90:649-652)
        self.alfa = float(p.alfa)
        self.hybrid = abs(self.alfa) > 1.0e-3
        self.values = np.asarray(bc_values, dtype=np.float64).reshape(6, 3)
        self.n = (p.nx - 1, p.ny - 1, p.nz - 1)
        self.shape = problem.shape
        self.bctype = tuple(int(t) for t in p.bc)
        self.zg = any(t == BC_ZERO_GRADIENT for t in self.bctype)
        self.gcm = p.boundary_formulation == GCM_METHOD
        self.mass_consv = self.zg and self.gcm
        self.area = float(p.outflow_area)
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64), device=self.dev)
        ms = [Metrics(problem.x), Metrics(problem.y), Metrics(problem.z)]
        self.fx = [T(m.fx) for m in ms]
        self.dxinv = [T(m.dxinv) for m in ms]
        self.dxcinv = [T(m.dxcinv) for m in ms]
        self.dx = [T(m.dx) for m in ms]
        g = problem.geom
        self.fl = [T(f) for f in g.flags]
        I = self.I = tuple(slice(1, m + 1) for m in self.n)
        ib = T(g.iblank)[I]
        gh = T(g.ghost)[I]
        self.fluid = 1.0 - ib                     # interior cells, [i, j, k] over 1..n
        self.ghostm = ib * gh
        self.dead = ib * (1.0 - gh)
        n0, n1, n2 = self.n
        self.vol = self.dx[0][1:n0 + 1][:, None, None] * self.dx[1][1:n1 + 1][None, :, None] \
            * self.dx[2][1:n2 + 1][None, None, :]
        self.face_area = [self.vol * self.col(self.dxinv[a], a) for a in range(3)]
        # set_solve_ad's implicit diffusion coefficients (IBM/CORE_SET_SOLVERS.F90:20-95)
        visc = torch.full(self.shape, self.reinv, dtype=torch.float64, device=self.dev)
        self.adm, self.adp, self.amd, self.apd, self.nuM, self.nuP = [], [], [], [], [], []
        for a in range(3):
            m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
            fxm, fxp = self.col(self.fx[a], a), self.col(self.fx[a], a, 1)
            nuP = (fxp * self.cells(visc, a, 1) + (1.0 - fxp) * self.cells(visc, a)) * (1 - pp) + self.reinv * pp
            nuM = (fxm * self.cells(visc, a) + (1.0 - fxm) * self.cells(visc, a, -1)) * (1 - m) + self.reinv * m
            self.nuM.append(nuM)
            self.nuP.append(nuP)
            tm = (self.col(self.dxcinv[a], a) * (1 - m) + self.col(self.dxinv[a], a) * m * 2.0) * self.col(self.dxinv[a], a)
            tp = (self.col(self.dxcinv[a], a, 1) * (1 - pp) + self.col(self.dxinv[a], a) * pp * 2.0) \
                * self.col(self.dxinv[a], a)
            self.adm.append(-(0.5 * self.dt * nuM) * tm)
            self.adp.append(-(0.5 * self.dt * nuP) * tp)
            # rhs_bc_terms of the outflow balance: constant reinv (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:90-252)
            self.amd.append(-(0.50 * self.dt * self.reinv) * tm)
            self.apd.append(-(0.50 * self.dt * self.reinv) * tp)
        self._ghost_setup()

    # --------------------------------------------------------- indexing --
    def cells(self, X, a: int, off: int = 0):
        """Interior cells of X shifted by `off` along axis a ([i, j, k] order)."""
        sl = list(self.I)
        sl[a] = slice(1 + off, self.n[a] + 1 + off)
        return X[tuple(sl)]

    def col(self, v, a: int, off: int = 0):
        """1-D metric v at t + off along axis a, shaped to broadcast over the interior."""
        shp = [1, 1, 1]
        shp[a] = -1
        return v[1 + off:self.n[a] + 1 + off].reshape(shp)

    def plane(self, X, a: int, i: int):
        """Plane i of axis a over the transverse range 0..n+1 that set_bc and
        zg_correct_planes loop over (the arrays carry one more layer)."""
        sl = [slice(0, m + 2) for m in self.n]
        sl[a] = i
        return X[tuple(sl)]

    def zeros(self):
        return torch.zeros(self.shape, dtype=torch.float64, device=self.dev)

    def put_interior(self, base, val):
        out = self.zeros() if base is None else base.clone()
        out[self.I] = val
        return out

    def _faces_along(self, a, F1n, Flast, base):
        """Full face array of axis a from faces 1..n (F1n) and face n+1 (Flast),
        other entries from base; dead-cell faces zeroed under GCM
        (GCM_set_face_vel_body, IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:387-423)."""
        F = torch.cat([F1n, Flast], dim=a)
        if self.gcm:
            dc = self.dead
            z1 = torch.zeros_like(dc.narrow(a, 0, 1))
            dm = torch.clamp(torch.cat([dc, z1], dim=a) + torch.cat([z1, dc], dim=a), max=1.0)
            F = F * (1.0 - dm)
        out = self.zeros() if base is None else base.clone()
        sl = list(self.I)
        sl[a] = slice(1, self.n[a] + 2)
        out[tuple(sl)] = F
        return out

    def _mask_faces(self, a, Fm, Flast, b):
        """The two mask loops of face_vel / correct_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:
        178-195, :425-441): face t takes bc(t) if ium(t), else bc(t-1) if
        iup(t-1), else its value; face n+1 bc(n) if iup(n)."""
        n = self.n[a]
        m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
        first = Fm.narrow(a, 0, 1) * (1 - m.narrow(a, 0, 1)) + b.narrow(a, 0, 1) * m.narrow(a, 0, 1)
        pprev, bprev = pp.narrow(a, 0, n - 1), b.narrow(a, 0, n - 1)
        mt, bt = m.narrow(a, 1, n - 1), b.narrow(a, 1, n - 1)
        mid = (Fm.narrow(a, 1, n - 1) * (1 - pprev) + bprev * pprev) * (1 - mt) + bt * mt
        pl, bl = pp.narrow(a, n - 1, 1), b.narrow(a, n - 1, 1)
        last = Flast * (1 - pl) + bl * pl
        return torch.cat([first, mid], dim=a), last

    # --------------------------------------------------------- face_vel --
    def face_vel(self, vel, bcn, base=None):
        """face_vel, NO_VAN_KAN (IBM/CORE_FRAC_STEP_ROUTINES.F90:6-240): faces of
        the interior transverse range; bcn = (bcxu, bcyv, bczw)."""
        out = []
        for a in range(3):
            U = vel[a]
            b = self.cells(bcn[a], a) if bcn[a] is not None else torch.zeros_like(self.fluid)
            m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
            fxm, fxp = self.col(self.fx[a], a), self.col(self.fx[a], a, 1)
            Uc, Um, Up = self.cells(U, a), self.cells(U, a, -1), self.cells(U, a, 1)
            vm = (fxm * Uc + (1.0 - fxm) * Um) * (1 - m) + b * m
            n = self.n[a]
            vp_last = ((fxp * Up + (1.0 - fxp) * Uc) * (1 - pp) + b * pp).narrow(a, n - 1, 1)
            F1n, Flast = self._mask_faces(a, vm, vp_last, b)
            out.append(self._faces_along(a, F1n, Flast, None if base is None else base[a]))
        return out

    def rhs_poisson(self, faces):
        """nlu0 = dtinv div(face) (1 - iblank) on the interior (IBM/CORE_POISSON.F90:273-285)."""
        d = 0.0
        for a in range(3):
            d = d + (self.cells(faces[a], a, 1) - self.cells(faces[a], a)) * self.col(self.dxinv[a], a)
        return self.put_interior(None, (1.0 / self.dt) * d * self.fluid)

    def massflux(self, faces):
        """Net face flux out of the fluid cells (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:30-48)."""
        t = 0.0
        for a in range(3):
            t = t + (self.cells(faces[a], a, 1) - self.cells(faces[a], a)) * self.face_area[a]
        return (t * self.fluid).sum()

    # --------------------------------------------------- rhs_advec_diff --
    def rhs_advec_diff(self, vel, faces, bc9, nl_old=None):
        """Right-hand sides on the interior (rhs_advec central branch,
        rhs_loadAB, rhs_diff): Crank-Nicolson nl = vel - dt/2 N(vel) +
        dt/2 D(vel); Adams-Bashforth nl = vel - dt (1.5 N(vel) - 0.5 N_old) +
        dt/2 D(vel), which also returns the new N_old = N(vel)."""
        out, new_old = [], []
        for q in range(3):
            U = vel[q]
            conv, diff = 0.0, 0.0
            for a in range(3):
                b = self.cells(bc9[3 * q + a], a)
                m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
                fxm, fxp = self.col(self.fx[a], a), self.col(self.fx[a], a, 1)
                Uc, Um, Up = self.cells(U, a), self.cells(U, a, -1), self.cells(U, a, 1)
                velp = (fxp * Up + (1.0 - fxp) * Uc) * (1 - pp) + b * pp
                velm = (fxm * Uc + (1.0 - fxm) * Um) * (1 - m) + b * m
                if self.hybrid:
                    velp, velm = self._hybrid_faces(U, a, velp, velm, b, m, pp, faces[a])
                conv = conv + (velp * self.cells(faces[a], a, 1) - velm * self.cells(faces[a], a)) \
                    * self.col(self.dxinv[a], a)
                dinv = self.col(self.dxinv[a], a)
                am = (self.col(self.dxcinv[a], a) * (1 - m) + dinv * m * 2.0) * dinv * self.nuM[a]
                ap = (self.col(self.dxcinv[a], a, 1) * (1 - pp) + dinv * pp * 2.0) * dinv * self.nuP[a]
                diff = diff + am * (Um * (1 - m) + b * m) - (am + ap) * Uc + ap * (Up * (1 - pp) + b * pp)
            if self.scheme == 1:
                load = 1.5 * conv - (1.5 - 1.0) * self.cells(nl_old[q], 0)
                new_old.append(self.put_interior(nl_old[q], conv))
            else:
                load = conv * 0.5
            nl = self.cells(U, 0) - self.dt * load + 0.5 * self.dt * diff
            out.append(self.put_interior(None, nl))
        return (out, new_old) if self.scheme == 1 else out

    def _hybrid_faces(self, U, a, vele, velw, b, m, pp, F):
        """The face values of rhs_advec's hybrid branch (IBM/CORE_RHS_AD.F90:150-382):
        (1 - alfa) central + alfa second-order upwind, the upwind side chosen by
        the sign of the face velocity, the first and last two cells of the axis
        (iumm / iupp) falling back to the central value; along x the plus-side
        value weights U(ipp) with edxWeightp1, as the reference writes it."""
        n = self.n[a]
        t = torch.arange(1, n + 1, device=self.dev)
        shp = [1, 1, 1]
        shp[a] = -1
        dinv = self.dxinv[a]
        d = lambda idx: dinv[idx].reshape(shp)
        imm = torch.clamp(t - 2, min=0)                 # i-2, or 0
        ipp = torch.clamp(t + 2, max=n + 1)             # i+2, or the node count
        tm, tp = t - 1, t + 1
        em1 = (d(tm) + 2.0 * d(t)) / (d(tm) + d(t))
        em2 = d(t) / (d(tm) + d(t))
        ep1 = (d(ipp) + 2.0 * d(tp)) / (d(ipp) + d(tp))
        ep2 = ep1 if a == 0 else d(tp) / (d(ipp) + d(tp))
        wm1 = (d(imm) + 2.0 * d(tm)) / (d(imm) + d(tm))
        wm2 = d(tm) / (d(imm) + d(tm))
        wp1 = (d(tp) + 2.0 * d(t)) / (d(tp) + d(t))
        wp2 = d(t) / (d(tp) + d(t))
        mm = ((t == 1) | (t == 2)).to(torch.float64).reshape(shp)
        pq = ((t == n) | (t == n - 1)).to(torch.float64).reshape(shp)
        sl = list(self.I)

        def along(idx):   # U at the cells idx along a, interior elsewhere
            sl2 = list(sl)
            sl2[a] = slice(None)
            return U[tuple(sl2)].index_select(a, idx)

        Uc, Um, Up = self.cells(U, a), self.cells(U, a, -1), self.cells(U, a, 1)
        Umm, Upp = along(imm), along(ipp)
        one = torch.ones_like(Uc)
        sp = torch.copysign(one, self.cells(F, a, 1))
        sm = torch.copysign(one, self.cells(F, a))
        vele_up = ((1.0 + sp) * (mm * vele + (1 - mm) * (em1 * Uc - em2 * Um))
                   + (1.0 - sp) * (pq * vele + (1 - pq) * (ep1 * Up - ep2 * Upp))) * 0.5 * (1 - pp) + b * pp
        velw_up = ((1.0 + sm) * (mm * velw + (1 - mm) * (wm1 * Um - wm2 * Umm))
                   + (1.0 - sm) * (pq * velw + (1 - pq) * (wp1 * Uc - wp2 * Up))) * 0.5 * (1 - m) + b * m
        al = self.alfa
        return (1.0 - al) * vele + al * vele_up, (1.0 - al) * velw + al * velw_up

    def rhs_adjust_bc(self, faces, bc9, nl):
        """Boundary values of flagged faces times the implicit coefficients move
        to the right-hand sides (IBM/CORE_RHS_AD.F90:588-780)."""
        h = self.half
        md, pd = [], []
        for a in range(3):
            m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
            fxm, fxp = self.col(self.fx[a], a), self.col(self.fx[a], a, 1)
            dinv = self.col(self.dxinv[a], a)
            md.append(self.adm[a] - h * self.cells(faces[a], a) * ((1.0 - fxm) * (1 - m) + m) * dinv)
            pd.append(self.adp[a] + h * self.cells(faces[a], a, 1) * (fxp * (1 - pp) + pp) * dinv)
        out = []
        for q in range(3):
            r = self.cells(nl[q], 0)
            for a in range(3):
                b = self.cells(bc9[3 * q + a], a)
                m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
                r = r - md[a] * b * m - pd[a] * b * pp
            out.append(self.put_interior(nl[q], r))
        return out

    def bc_terms(self, bc9):
        """sum_a amd bc m + apd bc p per component (rhs_bc_terms with reinv)."""
        out = []
        for q in range(3):
            t = 0.0
            for a in range(3):
                b = self.cells(bc9[3 * q + a], a)
                m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
                t = t + self.amd[a] * b * m + self.apd[a] * b * pp
            out.append(t)
        return out

    # ------------------------------------------------------------ solve_ad --
    def ad_rows(self, faces):
        """Row coefficients (am, ap per axis, sum of ac) of itsolv_ad / calc_residual_ad
        with the Crank-Nicolson convective terms (IBM/CORE_SOLVE_AD.F90:343-390)."""
        h = self.half
        am, ap, acs = [], [], 0.0
        for a in range(3):
            m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
            fxm, fxp = self.col(self.fx[a], a), self.col(self.fx[a], a, 1)
            dinv = self.col(self.dxinv[a], a)
            Fm, Fp = self.cells(faces[a], a), self.cells(faces[a], a, 1)
            am.append(self.adm[a] - h * Fm * (1.0 - fxm) * dinv)
            ap.append(self.adp[a] + h * Fp * fxp * dinv)
            acs = acs + (-(self.adm[a] + self.adp[a]) + h * (Fp * (1.0 - fxp) * (1 - pp) - Fm * fxm * (1 - m)) * dinv)
        return am, ap, acs

    def row_op(self, U, rows):
        am, ap, acs = rows
        r = self.cells(U, 0) * (1.0 + acs)
        for a in range(3):
            m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
            r = r + self.cells(U, a, -1) * am[a] * (1 - m) + self.cells(U, a, 1) * ap[a] * (1 - pp)
        return r

    def shift_zg(self, bc9, s):
        """bc9 with the normal component of every zero-gradient plane shifted by
        -s (minus sides) / +s (plus sides) (zg_correct_planes)."""
        out = list(bc9)
        for a in range(3):
            for side in (0, 1):
                if self.bctype[2 * a + side] != BC_ZERO_GRADIENT:
                    continue
                q = 4 * a
                b = out[q].clone()
                i = 1 if side == 0 else self.n[a]
                self.plane(b, a, i).add_(-s if side == 0 else s)
                out[q] = b
        return out

    def ad_system(self, U3, s, nl, bc9, faces_in):
        """F(X, theta) of the converged solve_ad: momentum rows of fluid cells,
        ghost-velocity rows, u = 0 in dead cells (interior arrays), and with the
        outflow balance the net face flux / outflow_area."""
        vel = [self.put_interior(None, U) for U in U3]
        if self.mass_consv:
            bcs = self.shift_zg(bc9, s)
            faces = self.face_vel(vel, (bcs[0], bcs[4], bcs[8]))
            t0, t1 = self.bc_terms(bc9), self.bc_terms(bcs)
            rhs = [self.cells(nl[q], 0) + t0[q] - t1[q] for q in range(3)]
            rs = self.massflux(faces) / self.area
        else:
            # CRANK_NICOLSON2 re-evaluates face_vel of the current velocities every iteration
            # (IBM/CORE_SOLVE_AD.F90:155-157); CRANK_NICOLSON1 keeps the step's faces
            faces = self.face_vel(vel, (bc9[0], bc9[4], bc9[8])) if self.scheme == 3 else faces_in
            rhs = [self.cells(nl[q], 0) for q in range(3)]
            rs = None
        rows = self.ad_rows(faces)
        out = []
        for q in range(3):
            r = self.fluid * (rhs[q] - self.row_op(vel[q], rows)) + self.dead * U3[q]
            if self.nG:
                r = r + self.ghost_residual(vel[q])
            out.append(r)
        return out, rs

    # --------------------------------------------------- ghost velocities --
    def _ghost_setup(self):
        """Ghost-cell velocity rows u_g = -iw sum_r coeffGCMD(r, g) u(stencil r) (body
        at rest, probeLengthNormalized 2: bw = 2, iw = 1) as flat gathers over the
        [i, j, k] C-order flattening of the full array."""
        g = self.pr.geom
        self.nG = int(g.nGhost) if self.gcm else 0
        if not self.nG:
            return
        sx, sy, sz = self.shape
        lin = lambda i, j, k: (i * sy + j) * sz + k
        self.iw = 1.0
        gflat = np.array([lin(g.iG[n], g.jG[n], g.kG[n]) for n in range(self.nG)], dtype=np.int64)
        rows, cols, vals = [], [], []
        for n in range(self.nG):
            for r, (a, b, c) in enumerate(_INC):
                ii, jj, kk = g.iCI[n] + a, g.jCI[n] + b, g.kCI[n] + c
                if (ii, jj, kk) == (g.iG[n], g.jG[n], g.kG[n]):
                    continue   # the intercept value (zero for a body at rest)
                rows.append(n); cols.append(lin(ii, jj, kk)); vals.append(float(g.coeffD[r, n]))
        L = lambda a: torch.as_tensor(np.asarray(a, dtype=np.int64), device=self.dev)
        self.g_flat = L(gflat)
        self.g_rows, self.g_cols = L(rows), L(cols)
        self.g_vals = torch.as_tensor(np.asarray(vals), device=self.dev)
        # interior positions of the ghosts
        self.g_int = L([((g.iG[n] - 1) * self.n[1] + (g.jG[n] - 1)) * self.n[2] + (g.kG[n] - 1)
                        for n in range(self.nG)])
        # ghost-ghost couplings for the fixed-point sweeps
        pos = {int(v): n for n, v in enumerate(gflat)}
        gg = [(r_, pos[int(c)], v) for r_, c, v in zip(rows, cols, vals) if int(c) in pos]
        self.gg_rows = L([t[0] for t in gg]); self.gg_cols = L([t[1] for t in gg])
        self.gg_vals = torch.as_tensor(np.asarray([t[2] for t in gg], dtype=np.float64), device=self.dev)
        self.g_sweeps = VelGhosts.calibrate(self, self.gg_rows, self.gg_cols, self.gg_vals)
        self.g_sweeps_T = VelGhosts.calibrate(self, self.gg_cols, self.gg_rows, self.gg_vals)

    def ghost_gather(self, U):
        """sum_r coeffGCMD(r, g) U(stencil r) for every ghost g (U a full array)."""
        Uf = U.reshape(-1)
        return torch.zeros(self.nG, dtype=U.dtype, device=self.dev).index_add(0, self.g_rows,
                                                                              self.g_vals * Uf[self.g_cols])

    def ghost_residual(self, U):
        """u_g + iw sum_r coeffGCMD u(stencil r) at the ghosts, as an interior array."""
        rg = U.reshape(-1)[self.g_flat] + self.iw * self.ghost_gather(U)
        return torch.zeros(self.fluid.numel(), dtype=U.dtype, device=self.dev).index_add(
            0, self.g_int, rg).reshape(self.fluid.shape)

    def vel_ghosts(self, vel):
        """Ghost-cell velocities of the corrected velocities (VelGhosts)."""
        if not self.nG:
            return list(vel)
        return list(VelGhosts.apply(self, *vel))

    # --------------------------------------------------------- correct_vel --
    def correct_vel(self, p, vel, faces, bcn):
        """correct_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:244-448): cell update of the
        fluid cells, ghost-cell velocities, face pressure correction and masks."""
        new = []
        for a in range(3):
            m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
            fxm, fxp = self.col(self.fx[a], a), self.col(self.fx[a], a, 1)
            Pc, Pm, Pp = self.cells(p, a), self.cells(p, a, -1), self.cells(p, a, 1)
            pe = (fxp * Pp + (1.0 - fxp) * Pc) * (1 - pp) + Pc * pp
            pw = (fxm * Pc + (1.0 - fxm) * Pm) * (1 - m) + Pc * m
            g = (pe - pw) * self.col(self.dxinv[a], a)
            new.append(self.put_interior(vel[a], self.cells(vel[a], 0) - self.dt * g * self.fluid))
        if self.gcm:
            new = self.vel_ghosts(new)
        fout = []
        for a in range(3):
            n = self.n[a]
            m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
            b = self.cells(bcn[a], a) if bcn[a] is not None else torch.zeros_like(self.fluid)
            Pc, Pm = self.cells(p, a), self.cells(p, a, -1)
            pgm = (Pc - Pm) * self.col(self.dxcinv[a], a)
            Fc = self.cells(faces[a], a) - self.dt * pgm * (1 - m)
            pgp_last = ((self.cells(p, a, 1) - Pc) * self.col(self.dxcinv[a], a, 1)).narrow(a, n - 1, 1)
            Flast = self.cells(faces[a], a, 1).narrow(a, n - 1, 1) - self.dt * pgp_last * (1 - pp.narrow(a, n - 1, 1))
            F1n, FL = self._mask_faces(a, Fc, Flast, b)
            fout.append(self._faces_along(a, F1n, FL, faces[a]))
        return new, fout

    # ----------------------------------------------------------- set_bc --
    def set_bc(self, vel, bc9, time: float):
        """set_bc's outer sides (Dirichlet, zero gradient, symmetry;
        IBM/CORE_SET_BC.F90:22-298), enforce_global_mass_consv (:304-377) and
        set_outer_ghost_vel (IBM/CORE_SET_OUTER_GHOST.F90:1-63).  Returns (vel, bc9)."""
        del time   # the restated side types do not depend on time
        bc = [b.clone() for b in bc9]
        for a in range(3):
            for side in (0, 1):
                s = 2 * a + side
                i = 1 if side == 0 else self.n[a]
                for q in range(3):
                    dst = self.plane(bc[3 * q + a], a, i)
                    t = self.bctype[s]
                    if t == BC_DIRICHLET:
                        dst.fill_(float(self.values[s, q]))
                    elif t == BC_ZERO_GRADIENT or (t == BC_SYMMETRY and q != a):
                        dst.copy_(self.plane(vel[q], a, i))
                    else:
                        dst.fill_(0.0)
        if self.zg:
            t = 0.0
            for a in range(3):
                b = self.cells(bc[4 * a], a)
                m, pp = self.cells(self.fl[2 * a], a), self.cells(self.fl[2 * a + 1], a)
                t = t + (b * pp - b * m) * self.face_area[a]
            massflux = (t * self.fluid).sum()
            bc = self.shift_zg(bc, -massflux / self.area)   # correction_vel
        out = [v.clone() for v in vel]
        for a in range(3):
            na = self.n[a]
            for q in range(3):
                va = out[q]
                ba = bc[3 * q + a]
                lo = 2.0 * self.plane(ba, a, 1) - self.plane(va, a, 1)
                hi = 2.0 * self.plane(ba, a, na) - self.plane(va, a, na)
                self.plane(va, a, 0).copy_(lo)
                self.plane(va, a, na + 1).copy_(hi)
        return out, bc


class VelGhosts(torch.autograd.Function):
    """Ghost-cell velocities u_g = -iw sum_r coeffGCMD u(stencil r) for u, v, w
    (GCM_vel_set_bc_internal at rest): the fixed point of the ghost rows,
    independent of the incoming ghost values; backward by the transposed
    fixed point.  Both run a sweep count fixed once per geometry (twice what
    a random right-hand side needs to change by less than 1e-16), so no
    sweep synchronises with the host."""

    SWEEPS_MAX = 5000

    @staticmethod
    def _sweep(ops, rhs, x, rows, cols, vals):
        return rhs - ops.iw * torch.zeros_like(rhs).index_add(0, rows, vals * x[cols])

    @staticmethod
    def calibrate(ops, rows, cols, vals):
        if rows.numel() == 0:
            return 1
        g = torch.Generator(device="cpu").manual_seed(7)
        rhs = torch.randn(ops.nG, dtype=torch.float64, generator=g).to(ops.dev)
        x = rhs
        for k in range(1, VelGhosts.SWEEPS_MAX + 1):
            xn = VelGhosts._sweep(ops, rhs, x, rows, cols, vals)
            d = float((xn - x).abs().max())
            x = xn
            if d <= 1e-16 * float(x.abs().max()):
                return 2 * k
        raise RuntimeError("ghost-cell velocity rows do not contract")

    @staticmethod
    def _fixed_point(ops, rhs, rows, cols, vals, sweeps):
        x = rhs
        for _ in range(sweeps):
            x = VelGhosts._sweep(ops, rhs, x, rows, cols, vals)
        return x

    @staticmethod
    def forward(ctx, ops, u, v, w):
        ctx.ops = ops
        outs = []
        for U in (u, v, w):
            Uc = U.detach().clone(memory_format=torch.contiguous_format)
            flat = Uc.reshape(-1)
            flat[ops.g_flat] = 0.0
            rhs = -ops.iw * ops.ghost_gather(Uc)   # contributions of the non-ghost stencil cells
            x = VelGhosts._fixed_point(ops, rhs, ops.gg_rows, ops.gg_cols, ops.gg_vals, ops.g_sweeps)
            flat[ops.g_flat] = x
            outs.append(Uc)
        return tuple(outs)

    @staticmethod
    def backward(ctx, gu, gv, gw):
        ops = ctx.ops
        res = []
        for G in (gu, gv, gw):
            if G is None:
                res.append(None)
                continue
            Gf = G.reshape(-1).clone()
            gG = Gf[ops.g_flat].clone()
            # (I + iw C_GG)^T y = gG
            y = VelGhosts._fixed_point(ops, gG, ops.gg_cols, ops.gg_rows, ops.gg_vals, ops.g_sweeps_T)
            Gf[ops.g_flat] = 0.0
            # u_G = -iw (C_GF u + C_GG u_G): cotangent -iw C_GF^T y on the non-ghost stencil cells
            contrib = torch.zeros_like(Gf).index_add(0, ops.g_cols, -ops.iw * ops.g_vals * y[ops.g_rows])
            contrib[ops.g_flat] = 0.0
            res.append((Gf + contrib).reshape(G.shape))
        return (None, *res)


# ------------------------------------------------------------------ GMRES --
def gmres_flat(matvec, b, rtol=1e-12, m=40, max_apps=2000, x0=None):
    """Restarted GMRES(m) on 1-D vectors (classical Gram-Schmidt twice), from
    x0 (or zero); the tolerance is relative to |b|.  Returns (x, applications,
    relative residual)."""
    beta0 = float(torch.linalg.vector_norm(b))
    x = torch.zeros_like(b) if x0 is None else x0.clone()
    if beta0 == 0.0:
        return torch.zeros_like(b), 0, 0.0
    N = b.numel()
    V = torch.empty((m + 1, N), dtype=b.dtype, device=b.device)
    apps, rel = 0, 1.0
    r = b.clone() if x0 is None else b - matvec(x)
    apps += 0 if x0 is None else 1
    while apps < max_apps:
        beta = float(torch.linalg.vector_norm(r))
        rel = beta / beta0
        if rel <= rtol:
            break
        V[0] = r / beta
        H = np.zeros((m + 1, m))
        g = np.zeros(m + 1)
        g[0] = beta
        cs, sn = np.zeros(m), np.zeros(m)
        k = 0
        for j in range(m):
            wv = matvec(V[j]).clone()
            apps += 1
            Vj = V[:j + 1]
            h1 = Vj @ wv
            wv -= Vj.T @ h1
            h2 = Vj @ wv
            wv -= Vj.T @ h2
            hn_d = torch.linalg.vector_norm(wv)
            hv = torch.cat([h1 + h2, hn_d.reshape(1)]).cpu().numpy()
            H[:j + 1, j] = hv[:j + 1]
            hn = float(hv[j + 1])
            H[j + 1, j] = hn
            for i in range(j):
                a_, b_ = H[i, j], H[i + 1, j]
                H[i, j], H[i + 1, j] = cs[i] * a_ + sn[i] * b_, -sn[i] * a_ + cs[i] * b_
            rr = math.hypot(H[j, j], H[j + 1, j])
            cs[j], sn[j] = (H[j, j] / rr, H[j + 1, j] / rr) if rr > 0 else (1.0, 0.0)
            H[j, j], H[j + 1, j] = rr, 0.0
            g[j + 1], g[j] = -sn[j] * g[j], cs[j] * g[j]
            k = j + 1
            if abs(g[j + 1]) <= 0.5 * rtol * beta0 or hn == 0.0 or apps >= max_apps:
                break
            V[j + 1] = wv / hn
        y = np.linalg.solve(np.triu(H[:k, :k]), g[:k])
        x += torch.as_tensor(y, dtype=b.dtype, device=b.device) @ V[:k]
        r = b - matvec(x)
        apps += 1
    return x, apps, rel


# --------------------------------------------------------------- backends --
# A backend runs the two implicit solves of a step: solve_ad(vel, nl, bc, faces)
# -> (vel, bc, info), pressure(nlu0) -> p (full array after correct_pressure) and
# mg_apply(r) -> one forward MG_Solver application; it has .device and .pPrime.
class DeviceBackend:
    """The implicit solves on the product (C ABI on device arrays): solve_ad and
    the pressure solve with the problem's solver parameters, and one FP64
    MG_Solver application for the transposed pressure solve."""

    device = torch.device("cuda")

    def __init__(self, problem, dt, reinv, advec_scheme=2, mixed_precondition=False, pressure_guess="previous"):
        from .poisson import PoissonSolver
        self.pr = problem
        self.pressure_guess = pressure_guess   # as FractionalStep: 'previous' or 'extrapolate'
        self.p_prev = None
        p = problem.params
        self.s = PoissonSolver(p, problem.x, problem.y, problem.z).set_boundary(problem.geom)
        if problem.geom.nGhost:
            self.s.set_velocity_ghosts(problem.geom.coeffD, None)
        self.mg = _DeviceMG(problem, self.device, mixed_precondition=mixed_precondition)
        shape = tuple(reversed(problem.shape))
        z = lambda: torch.zeros(shape, dtype=torch.float64, device=self.device)
        self.vel = [z() for _ in range(3)]
        self.nl = [z() for _ in range(3)]
        self.bc = [z() for _ in range(9)]
        self.faces = [z() for _ in range(3)]
        self.visc = torch.full(shape, float(reinv), dtype=torch.float64, device=self.device)
        self.pPrime, self.nlu0, self.nlw0 = z(), z(), z()
        self.dt, self.reinv, self.scheme = float(dt), float(reinv), int(advec_scheme)

    @staticmethod
    def _load(bufs, ts):
        for b, t in zip(bufs, ts):
            b.permute(2, 1, 0).copy_(t.detach())

    @staticmethod
    def _view(bufs):
        return [b.permute(2, 1, 0).clone() for b in bufs]

    def solve_ad(self, vel, nl, bc, faces):
        self._load(self.vel, vel); self._load(self.nl, nl); self._load(self.bc, bc); self._load(self.faces, faces)
        # the library's stream does not wait for torch's: the inputs must be complete
        torch.cuda.synchronize()
        P = lambda ts: [t.data_ptr() for t in ts]
        vis = self.visc.data_ptr()
        st, it, mr = self.s.solve_ad(self.dt, P(self.faces), vis, P(self.vel), P(self.nl), bcvisc=[vis] * 3,
                                     advec_scheme=self.scheme, bc=P(self.bc), reinv=self.reinv)
        torch.cuda.synchronize()
        if st != 0:
            raise RuntimeError(f"solve_ad status {st} (maxres {mr})")
        return self._view(self.vel), self._view(self.bc), (it, mr)

    def pressure(self, nlu0):
        self.nlu0.permute(2, 1, 0).copy_(nlu0.detach())
        if self.pressure_guess == "extrapolate":
            if self.p_prev is None:
                self.p_prev = self.pPrime.clone()
            else:
                cur = self.pPrime.clone()
                self.pPrime.mul_(2.0).sub_(self.p_prev)
                self.p_prev = cur
        torch.cuda.synchronize()
        st, it, mr, _, _ = self.s.solve_poisson_device(self.pPrime.data_ptr(), self.nlu0.data_ptr(),
                                                        self.nlw0.data_ptr())
        torch.cuda.synchronize()
        if st not in (0,):
            raise RuntimeError(f"pressure solve status {st} (maxres {mr})")
        return self.pPrime.permute(2, 1, 0).clone()

    def mg_apply(self, r):
        return self.mg.precondition(as_fortran(r))

    def close(self):
        self.s.close()
        self.mg.close()


# -------------------------------------------------------- implicit solves --
class _SolveAD(torch.autograd.Function):
    """solve_ad as a function of (vel, nl, bc, faces): forward by the backend,
    backward by the implicit-function theorem on StepOperators.ad_system."""

    @staticmethod
    def forward(ctx, sa, *args):
        vel, nl, bc, faces = args[0:3], args[3:6], args[6:15], args[15:18]
        if sa.replay:
            v2, b2, info = sa.replay.pop(0)
        else:
            v2, b2, info = sa.backend.solve_ad(vel, nl, bc, faces)
            if sa.record is not None:
                sa.record.append((v2, b2, info))
        sa.last_ad = info
        ops = sa.ops
        s = 0.0
        if ops.mass_consv:
            a, side = sa.zg_side
            i = 1 if side == 0 else ops.n[a]
            d = (ops.plane(b2[4 * a], a, i) - ops.plane(bc[4 * a].detach(), a, i))[1:-1, 1:-1]
            s = float(d.mean()) * (-1.0 if side == 0 else 1.0)
        ctx.sa, ctx.s = sa, s
        ctx.save_for_backward(*v2, *[t.detach() for t in args[3:18]])
        return (*v2, *b2)

    @staticmethod
    def backward(ctx, *g):
        sa, ops = ctx.sa, ctx.sa.ops
        saved = ctx.saved_tensors
        v2, nl, bc, faces = saved[0:3], saved[3:6], saved[6:15], saved[15:18]
        zero = lambda: torch.zeros(ops.shape, dtype=torch.float64, device=ops.dev)
        gv = [zero() if t is None else t for t in g[0:3]]
        gb = [zero() if t is None else t for t in g[3:12]]
        # interior cotangents of the solution; the outer layers pass through from vel
        Xbar = [ops.cells(t, 0) for t in gv]
        gvel_in = [t.clone() for t in gv]
        for t in gvel_in:
            t[ops.I] = 0.0
        sbar = torch.zeros((), dtype=torch.float64, device=ops.dev)
        if ops.mass_consv:
            for a in range(3):
                for side in (0, 1):
                    if ops.bctype[2 * a + side] == BC_ZERO_GRADIENT:
                        i = 1 if side == 0 else ops.n[a]
                        sbar = sbar + ops.plane(gb[4 * a], a, i).sum() * (-1.0 if side == 0 else 1.0)
        t0 = _sync_time(ops.dev)
        with torch.enable_grad():
            X = [ops.cells(t, 0).detach().clone().requires_grad_(True) for t in v2]
            s = torch.tensor(ctx.s, dtype=torch.float64, device=ops.dev, requires_grad=True)
            th = [t.detach().clone().requires_grad_(True) for t in (*nl, *bc, *faces)]
            JT, outs, split = _ad_vjp(sa, ops, X, s, th)
            rs = outs[3] if len(outs) > 3 else None

            rhs = torch.cat([t.reshape(-1) for t in Xbar] + ([sbar.reshape(1)] if rs is not None else []))
            x0 = sa._guess(sa._lam_hist, rhs.shape) if sa.warm_start else None
            lam, apps, rel = gmres_flat(JT, rhs, rtol=sa.rtol_ad, x0=x0)
            sa._lam_hist = [lam] + sa._lam_hist[:1]
            sa.stats["ad_transposed_applications"] = sa.stats.get("ad_transposed_applications", 0) + apps
            sa.stats["ad_transposed_rel_residual"] = max(sa.stats.get("ad_transposed_rel_residual", 0.0), rel)
            gth = torch.autograd.grad(outs, th, grad_outputs=split(lam), allow_unused=True)
        gth = [zero() if t is None else -t for t in gth]
        sa.stats["ad_transposed_s"] = sa.stats.get("ad_transposed_s", 0.0) + _sync_time(ops.dev) - t0
        gnl, gbc, gfaces = gth[0:3], gth[3:12], gth[12:15]
        gbc = [a + b for a, b in zip(gb, gbc)]
        return (None, *gvel_in, *gnl, *gbc, *gfaces)


def _ad_vjp(sa, ops, X, s, th):
    """F of solve_ad at (X, s, theta) and its vector-Jacobian product in X.
    On the GPU the product is one CUDA graph (the forward and the warm-up run
    on a side stream, so that autograd issues the backward kernels there, and
    the capture records them): a GMRES iteration then costs one replay instead
    of launching the backward pass's kernels one by one from Python.  Returns
    (JT, outs, split)."""
    side = None
    if ops.dev.type == "cuda" and sa.graph_vjp:
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
    ctxm = torch.cuda.stream(side) if side is not None else _nullcontext()
    with ctxm:
        r, rs = ops.ad_system(X, s, th[0:3], th[3:12], th[12:15])
        outs = list(r) + ([rs] if rs is not None else [])
    xs = X + ([s] if rs is not None else [])
    sizes = [t.numel() for t in outs]

    def split(v):
        parts, o = [], 0
        for t, sz in zip(outs, sizes):
            parts.append(v[o:o + sz].reshape(t.shape))
            o += sz
        return parts

    def eager(v):
        gr = torch.autograd.grad(outs, xs, grad_outputs=split(v), retain_graph=True)
        return torch.cat([t.reshape(-1) for t in gr])

    if side is None:
        return eager, outs, split
    try:
        with torch.cuda.stream(side):
            static_v = [torch.zeros_like(t) for t in outs]
            for _ in range(2):
                torch.autograd.grad(outs, xs, grad_outputs=static_v, retain_graph=True)
            graph = torch.cuda.CUDAGraph()
            with torch.cuda.graph(graph, stream=side):
                static_g = torch.autograd.grad(outs, xs, grad_outputs=static_v, retain_graph=True)
                static_out = torch.cat([t.reshape(-1) for t in static_g])
        torch.cuda.current_stream().wait_stream(side)
    except RuntimeError as e:   # capture refused: the eager product
        torch.cuda.current_stream().wait_stream(side)
        sa.stats["vjp_graph_error"] = str(e)[:200]
        return eager, outs, split
    sa.stats["vjp_graph"] = True

    def graphed(v):
        for dst, src in zip(static_v, split(v)):
            dst.copy_(src)
        graph.replay()
        return static_out.clone()

    graphed.graph = graph
    return graphed, outs, split


class _nullcontext:
    def __enter__(self):
        return None

    def __exit__(self, *a):
        return False


class _Pressure(torch.autograd.Function):
    """The pressure solve B p = f (p with ghost and outer values): forward by
    the backend, backward B^T z = E^T pbar and fbar = P_B^T z."""

    @staticmethod
    def forward(ctx, sa, nlu0):
        ctx.sa = sa
        if sa.replay:
            return sa.replay.pop(0)
        p = sa.backend.pressure(nlu0)
        if sa.record is not None:
            sa.record.append(p)
        return p

    @staticmethod
    def backward(ctx, gp):
        sa = ctx.sa
        t0 = _sync_time(sa.ops.dev)
        s = sa.pops.extend_T(as_fortran(gp))
        z = sa.solve_BT(s, z0=sa._guess(sa._z_hist, s.shape) if sa.warm_start else None)
        sa._z_hist = [z] + sa._z_hist[:1]
        one = sa.pops.fluid
        w = sa.left_null()
        zhat = (z - w * (float((one * z).sum()) / float((one * w).sum()))) * one
        sa.stats["p_transposed_s"] = sa.stats.get("p_transposed_s", 0.0) + _sync_time(sa.ops.dev) - t0
        return None, zhat.contiguous()


class StepAdjoint:
    """One fractional step as a torch graph (explicit routines restated,
    implicit solves by the backend) and the transposed pressure operator."""

    def __init__(self, problem, dt, reinv, bc_values, backend, advec_scheme=2):
        self.pr = problem
        self.backend = backend
        dev = backend.device
        self.ops = StepOperators(problem, dt, reinv, bc_values, device=dev, advec_scheme=advec_scheme)
        self.pops = ProjectionOperators(problem, dev)
        self.dt = float(dt)
        self.rtol_ad, self.rtol_p = 1e-12, 1e-11
        self.stats = {}
        self.last_ad = None
        # record: the implicit solves' outputs of a step are appended here;
        # replay: a recorded list is consumed instead of solving again
        self.record, self.replay = None, None
        # warm starts of the transposed solves from the previous step's solutions
        self.warm_start = False
        self._lam_hist, self._z_hist = [], []   # the last two solutions, latest first
        self._bt = None
        # the GMRES matrix-vector product of the transposed solve_ad system as one CUDA graph
        self.graph_vjp = True
        ops = self.ops
        self.zg_side = None
        for s, t in enumerate(ops.bctype):
            if t == BC_ZERO_GRADIENT:
                self.zg_side = (s // 2, s % 2)
                break
        # n1: the outflow term of a unit shift of the zero-gradient planes (-1 minus, +1 plus)
        n1 = ops.zeros()
        acc = 0.0
        for a in range(3):
            for side in (0, 1):
                if ops.bctype[2 * a + side] == BC_ZERO_GRADIENT:
                    acc = acc - ops.col(ops.dxinv[a], a) * ops.cells(ops.fl[2 * a + side], a)
        # the compatibility fixed point of GCM_correct_pressure (zero-gradient sides with GCM)
        self.rank1 = ops.zg and ops.gcm
        if self.rank1:
            n1[ops.I] = acc * ops.fluid
        self.n1 = as_fortran(n1)
        self.area = ops.area
        self._w = None

    @staticmethod
    def _guess(hist, shape):
        """Start of a transposed solve: the linear extrapolation of the two
        previous steps' solutions (the previous one alone after one step)."""
        h = [t for t in hist if t.shape == shape]
        if not h:
            return None
        return 2.0 * h[0] - h[1] if len(h) > 1 else h[0]

    # pressure operator B = A_eff + n1 (vol^T A_eff) / area and its transpose
    def apply_B(self, pf):
        Ap = self.pops.apply_eff(pf)
        if not self.rank1:
            return Ap
        return Ap + self.n1 * (float((self.pops.vol * Ap).sum()) / self.area)

    def _apply_BT_eager(self, z):
        if not self.rank1:
            return self.pops.apply_eff_T(z)
        return self.pops.apply_eff_T(z + self.pops.vol * ((self.n1 * z).sum() / self.area))

    def apply_BT(self, z):
        """B^T z.  On the GPU one CUDA graph replay: the ghost-row sweeps of the
        extension's transpose alone are a few hundred small kernels, which
        launched one by one from Python would bound the transposed solve."""
        if self.ops.dev.type != "cuda" or not self.graph_vjp:
            return self._apply_BT_eager(z)
        if self._bt is None:
            zin = fortran_zeros(self.ops.shape, self.ops.dev)
            side = torch.cuda.Stream()
            side.wait_stream(torch.cuda.current_stream())
            try:
                with torch.cuda.stream(side):
                    for _ in range(2):
                        self._apply_BT_eager(zin)
                    g = torch.cuda.CUDAGraph()
                    with torch.cuda.graph(g, stream=side):
                        zout = self._apply_BT_eager(zin)
                torch.cuda.current_stream().wait_stream(side)
                self._bt = (g, zin, zout)
            except RuntimeError as e:   # capture refused: eager from now on
                torch.cuda.current_stream().wait_stream(side)
                self.stats["apply_BT_graph_error"] = str(e)[:200]
                self._bt = False
        if self._bt is False:
            return self._apply_BT_eager(z)
        g, zin, zout = self._bt
        zin.copy_(z)
        g.replay()
        return zout.clone()

    def _precond(self, v):
        vol = self.pops.vol
        vinv = torch.where(vol > 0, 1.0 / torch.where(vol > 0, vol, torch.ones_like(vol)), torch.zeros_like(vol))
        return vol * (as_fortran(self.backend.mg_apply(as_fortran(vinv * v))) * self.pops.fluid)

    def solve_BT(self, s, rtol=None, z0=None):
        """B^T z = s by FGMRES(60), from z0 (or zero); rtol relative to |s|."""
        rtol = self.rtol_p if rtol is None else rtol
        s = s * self.pops.fluid
        if z0 is None:
            z, apps, rel = fgmres(self.apply_BT, self._precond, s, None, rtol=rtol, m=60)
        else:
            r0 = s - self.apply_BT(z0)
            ns, nr = float(torch.linalg.vector_norm(s)), float(torch.linalg.vector_norm(r0))
            if nr <= rtol * ns:
                z, apps, rel = z0, 1, nr / max(ns, 1e-300)
            else:
                dz, apps, rel = fgmres(self.apply_BT, self._precond, r0, None, rtol=rtol * ns / nr, m=60)
                z, apps, rel = z0 + dz, apps + 1, rel * nr / max(ns, 1e-300)
        self.stats["p_transposed_applications"] = self.stats.get("p_transposed_applications", 0) + apps
        self.stats["p_transposed_rel_residual"] = max(self.stats.get("p_transposed_rel_residual", 0.0), rel)
        return z

    def left_null(self):
        """w_B with w_B^T B = 0, w_B . 1_F = fluid volume."""
        if self._w is None:
            v1 = self.pops.vol.clone()
            d = self.solve_BT(-self.apply_BT(v1), rtol=1e-13)
            w = (v1 + d) * self.pops.fluid
            self._w = w * (float(self.pops.vol.sum()) / float(w.sum()))
        return self._w

    # ---------------------------------------------------------------- step --
    def step(self, vel, faces, bc, *rest, time=0.0):
        """One step as a torch graph: returns the state after the step, (vel,
        faces, bc), with Adams-Bashforth (vel, faces, bc, nl_old) (rest =
        (nl_old,): the previous step's convective terms)."""
        ops = self.ops
        if ops.scheme == 1:
            nl, nl_old = ops.rhs_advec_diff(vel, faces, bc, rest[0])
        else:
            nl = ops.rhs_advec_diff(vel, faces, bc)
        vel1, bc1 = ops.set_bc(vel, bc, time + self.dt)
        nl1 = ops.rhs_adjust_bc(faces, bc1, nl)
        out = _SolveAD.apply(self, *vel1, *nl1, *bc1, *faces)
        vel2, bc2 = list(out[0:3]), list(out[3:12])
        bn = (bc2[0], bc2[4], bc2[8])
        faces3 = ops.face_vel(vel2, bn, base=faces)
        nlu0 = ops.rhs_poisson(faces3)
        p = _Pressure.apply(self, nlu0)
        vel3, faces4 = ops.correct_vel(p, vel2, faces3, bn)
        return (vel3, faces4, bc2, nl_old) if ops.scheme == 1 else (vel3, faces4, bc2)

    def step_recorded(self, state, time=0.0):
        """One step without a graph; returns (next state, the recorded
        outputs of its implicit solves) for step_vjp's replay."""
        self.record, self.replay = [], None
        try:
            with torch.no_grad():
                out = self.step(*state, time=time)
            return out, self.record
        finally:
            self.record = None

    def step_vjp(self, state, cot, time=0.0, replay=None):
        """(state cotangent before the step) for the cotangent `cot` of the
        state after it; state = (vel3, faces3, bc9) lists.  With `replay`
        (from step_recorded on the same state) the implicit solves are not
        run again."""
        self.replay = list(replay) if replay else None
        try:
            return self._step_vjp(state, cot, time)
        finally:
            self.replay = None

    def _step_vjp(self, state, cot, time=0.0):
        groups = [[t.detach().clone().requires_grad_(True) for t in grp] for grp in state]
        with torch.enable_grad():
            out = self.step(*groups, time=time)
            flat_out = [t for grp in out for t in grp]
            flat_cot = [t for grp in cot for t in grp]
            keep = [(o, c) for o, c in zip(flat_out, flat_cot) if c is not None]
            inputs = [t for grp in groups for t in grp]
            gr = torch.autograd.grad([o for o, _ in keep], inputs, grad_outputs=[c for _, c in keep],
                                     allow_unused=True)
        z = lambda t: torch.zeros(self.ops.shape, dtype=torch.float64, device=self.ops.dev) if t is None else t
        gr = [z(t) for t in gr]
        res, o = [], 0
        for grp in groups:
            res.append(gr[o:o + len(grp)])
            o += len(grp)
        return tuple(res)


def wake_plane_loss(problem, u, x_plane: float, device=None):
    """Mean streamwise velocity over the fluid cells of the cell plane whose
    centres lie nearest x = x_plane; returns (loss, plane index)."""
    m = Metrics(problem.x)
    n0 = problem.params.nx - 1
    i = int(np.argmin(np.abs(m.xc[1:n0 + 1] - x_plane))) + 1
    p = problem.params
    fl = torch.as_tensor(np.ascontiguousarray(1.0 - problem.geom.iblank[i, 1:p.ny, 1:p.nz], dtype=np.float64),
                         device=u.device if device is None else device)
    return (u[i, 1:p.ny, 1:p.nz] * fl).sum() / fl.sum(), i


# ---------------------------------------------------------------- rollout --
class RolloutAdjoint:
    """Forward rollout on the product (``time_step.FractionalStep``) with the
    state (u, v, w, faces, bc9, pPrime) kept every ``checkpoint_every`` steps
    over the last ``adjoint_steps`` steps; ``gradient`` recomputes each
    segment's states from its checkpoint (the step graph without gradients,
    implicit solves on the product, their outputs kept) and pulls the
    cotangent of the final state back one step at a time through
    ``StepAdjoint.step_vjp`` with those solves replayed.  The result is
    dL/d(state) at step ``steps - adjoint_steps``."""

    def __init__(self, problem, dt, reinv, bc_values, advec_scheme=2, rtol_ad=1e-12, rtol_p=1e-11,
                 mixed_precondition=False, warm_start=True, pressure_guess="previous"):
        from .time_step import FractionalStep
        self.pr, self.dt, self.reinv, self.scheme = problem, float(dt), float(reinv), int(advec_scheme)
        self.values = np.asarray(bc_values, dtype=np.float64).reshape(6, 3)
        self.fs = FractionalStep(problem, dt, reinv, self.values, advec_scheme=advec_scheme,
                                 pressure_guess=pressure_guess)
        self.backend = DeviceBackend(problem, dt, reinv, advec_scheme, mixed_precondition=mixed_precondition,
                                     pressure_guess=pressure_guess)
        self.sa = StepAdjoint(problem, dt, reinv, self.values, self.backend, advec_scheme)
        self.sa.rtol_ad, self.sa.rtol_p = float(rtol_ad), float(rtol_p)
        self.sa.warm_start = bool(warm_start)
        self.checkpoints = {}
        self.times = {}

    def _save(self):
        fs = self.fs
        torch.cuda.synchronize()   # the product's stream has finished the step
        cl = lambda ts: [t.permute(2, 1, 0).clone() for t in ts]
        return dict(vel=cl(fs.vel), faces=cl(fs.faces), bc=cl(fs.bc), nl_old=cl(fs.nl_old), pPrime=fs.pPrime.clone(),
                    time=fs.time, ntime=fs.ntime, p_prev=None if fs._p_prev is None else fs._p_prev.clone())

    def _load(self, st):
        fs = self.fs
        for dst, grp in ((fs.vel, st["vel"]), (fs.faces, st["faces"]), (fs.bc, st["bc"]), (fs.nl_old, st["nl_old"])):
            for b, t in zip(dst, grp):
                b.permute(2, 1, 0).copy_(t)
        fs.pPrime.copy_(st["pPrime"])
        fs._p_prev = None if st.get("p_prev") is None else st["p_prev"].clone()
        fs.time, fs.ntime = st["time"], st["ntime"]
        torch.cuda.synchronize()   # before the product's stream reads them

    def _state(self, st):
        """The step graph's state from a saved state."""
        S = (st["vel"], st["faces"], st["bc"])
        return S + (st["nl_old"],) if self.scheme == 1 else S

    def forward(self, u0, v0, w0, steps: int, adjoint_steps: int, checkpoint_every: int, warmup: int = 0):
        """Runs `steps` product steps from (u0, v0, w0); returns the final state.
        times["forward_s"] covers the steps after the first `warmup`;
        records holds the solvers' record of every step."""
        if not 0 < adjoint_steps <= steps:
            raise ValueError("0 < adjoint_steps <= steps")
        self.steps, self.adj, self.every = steps, adjoint_steps, max(1, int(checkpoint_every))
        self.first = steps - adjoint_steps
        self.checkpoints.clear()
        self.records = []
        self.fs.start(u0, v0, w0)
        torch.cuda.synchronize()
        t0 = time_now()
        for n in range(steps):
            if n == warmup:
                torch.cuda.synchronize()
                t0 = time_now()
            if n >= self.first and (n - self.first) % self.every == 0:
                self.checkpoints[n] = self._save()
            rec = self.fs.step()
            self.records.append(rec)
            if rec["ad_status"] != 0 or rec["poisson_status"] != 0 or rec["ghost_status"] != 0:
                raise RuntimeError(f"forward step {n}: {rec}")
        torch.cuda.synchronize()
        self.times["forward_s"] = time_now() - t0
        self.times["forward_steps"] = steps - min(warmup, steps)
        self.final = self._save()
        return self.final

    def rerun(self, state, steps: int):
        """The product's rollout of `steps` steps from a state (a checkpoint
        dict, possibly perturbed); returns the final velocities ([i, j, k])."""
        self._load(state)
        for _ in range(steps):
            rec = self.fs.step()
            if rec["ad_status"] != 0 or rec["poisson_status"] != 0:
                raise RuntimeError(f"rerun step: {rec}")
        torch.cuda.synchronize()
        return [t.permute(2, 1, 0) for t in self.fs.vel]

    def gradient(self, loss_fn):
        """dL/d(state at step steps - adjoint_steps) for L = loss_fn(vel) of the
        final velocities ([i, j, k] tensors); returns (L, cotangent state)."""
        torch.cuda.synchronize()
        t0 = time_now()
        self.sa.left_null()   # once per geometry (the first call solves for it)
        torch.cuda.synchronize()
        self.times["left_null_s"] = time_now() - t0
        vel = [t.detach().clone().requires_grad_(True) for t in self.final["vel"]]
        with torch.enable_grad():
            L = loss_fn(vel)
            gv = torch.autograd.grad(L, vel, allow_unused=True)
        sh = self.sa.ops.shape
        z = lambda: torch.zeros(sh, dtype=torch.float64, device=self.sa.ops.dev)
        cot = ([z() if g is None else g for g in gv], [z(), z(), z()], [z() for _ in range(9)])
        if self.scheme == 1:   # Adams-Bashforth carries the convective terms of the last step
            cot = cot + ([z(), z(), z()],)
        starts = sorted(self.checkpoints)
        recompute = 0.0
        for c in reversed(starts):
            end = min(c + self.every, self.steps)
            # recompute the segment's states from its checkpoint (the step graph without
            # gradients, implicit solves on the product), keeping each step's solves
            tr = time_now()
            ck = self.checkpoints[c]
            self.backend.pPrime.copy_(ck["pPrime"])
            self.backend.p_prev = None if ck.get("p_prev") is None else ck["p_prev"].clone()
            torch.cuda.synchronize()
            S, t = self._state(ck), ck["time"]
            seg = []
            for n in range(c, end):
                S1, rec = self.sa.step_recorded(S, time=t)
                seg.append((S, rec, t))
                S, t = S1, t + self.dt
            torch.cuda.synchronize()
            recompute += time_now() - tr
            for S, rec, t in reversed(seg):
                cot = self.sa.step_vjp(S, cot, time=t, replay=rec)
        torch.cuda.synchronize()
        self.times["adjoint_s"] = time_now() - t0
        self.times["recompute_s"] = recompute
        return float(L.detach()), cot

    def close(self):
        self.fs.close()
        self.backend.close()


def time_now():
    import time
    return time.perf_counter()


def _sync_time(dev):
    if dev.type == "cuda":
        torch.cuda.synchronize()
    return time_now()
