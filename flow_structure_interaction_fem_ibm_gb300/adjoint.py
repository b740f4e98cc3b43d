"""Projection step and its hand-written adjoint (torch harness around the
GPU multigrid).

The projection step of the fractional-step method, for dt = 1, stationary
walls with zero velocity, the plain (non Van Kan) face interpolation and no
pressure-oscillation cure:

    f  = D F u*                       face_vel (IBM/CORE_FRAC_STEP_ROUTINES.F90:80-109)
                                      + rhs_poisson (IBM/CORE_POISSON.F90:155-163)
    A_eff p = P f                     solve_poisson (the GPU multigrid of this package)
    u  = u* - G E p                   correct_vel cell-centre update
                                      (IBM/CORE_FRAC_STEP_ROUTINES.F90:244-370)

u* = (u, v, w) are cell-centred arrays over (0:nx+1, 0:ny+1, 0:nz+1); p lives on
the fluid cells F; E extends it to the ghost cells through the ghost-row fixed
point p_g = sum_r coeffGCMN(r,g) p(stencil r) (uNormal = 0; boundary cells never
enter because the outer faces are flagged); A_eff p = [A E p]_F is the
7-point operator of calc_residual applied to the extended pressure.  With
ghost rows A_eff is singular (constants) but not symmetric: its left null
vector w is not the cell-volume vector, so P f = f - 1_F (w.f)/(w.1_F) makes
the right-hand side consistent.

Adjoint (lambda = dL/du):   dL/du* = lambda - (D F)^T zhat,
    A_eff^T zhat = E^T G^T lambda,   1_F . zhat = 0.
The right-hand side is consistent because G E 1 = 0, and the normalisation
picks P^T z out of the solutions z + a w.  A_eff^T = V A_FF V^-1 + (ghost
coupling), V the fluid cell volumes (V A_FF is symmetric), so the transposed
system is solved by FGMRES preconditioned with V M V^-1, M one application of
the forward multigrid (MG_Solver): a multigrid solve on the transposed
ghost-cell operator.  The left null vector w comes from the same solver:
w = V 1 + d with A_eff^T d = -A_eff^T V 1.

Everything here is FP64 torch on the solver's device, the ghost-row
elimination included (fixed-point sweeps over the ghost-ghost couplings).
"""
from __future__ import annotations

import copy
import ctypes
import math
from typing import Optional

import numpy as np
import scipy.sparse as sp
import torch

from .grid import Metrics
from .params import DIM_3D, PRECISION_FP64

_INC = ((0, 0, 0), (0, 1, 0), (1, 1, 0), (1, 0, 0), (0, 0, 1), (0, 1, 1), (1, 1, 1), (1, 0, 1))  # incI/J/K


def fortran_zeros(shape, device):
    """FP64 tensor indexed [i, j, k] whose memory is Fortran-ordered."""
    return torch.zeros(tuple(reversed(shape)), dtype=torch.float64, device=device).permute(2, 1, 0)


def as_fortran(t):
    return t.permute(2, 1, 0).contiguous().permute(2, 1, 0)


class ProjectionOperators:
    """Linear pieces of the projection step on one geometry, with their
    hand-written transposes."""

    def __init__(self, problem, device="cpu"):
        self.pr = problem
        p = problem.params
        self.dev = torch.device(device)
        self.shape = problem.shape
        self.three_d = p.ndim == DIM_3D
        self.n = (p.nx - 1, p.ny - 1, p.nz - 1)
        mx, my, mz = Metrics(problem.x), Metrics(problem.y), Metrics(problem.z)
        t = lambda a: torch.as_tensor(np.asarray(a, dtype=np.float64), device=self.dev)
        self.fx, self.fy, self.fz = t(mx.fx), t(my.fx), t(mz.fx)
        self.dxinv, self.dyinv, self.dzinv = t(mx.dxinv), t(my.dxinv), t(mz.dxinv)
        self.dxcinv, self.dycinv, self.dzcinv = t(mx.dxcinv), t(my.dxcinv), t(mz.dxcinv)
        self.dx, self.dy, self.dz = t(mx.dx), t(my.dx), t(mz.dx)
        n0, n1, n2 = self.n
        I, J, K = self.IJK = (slice(1, n0 + 1), slice(1, n1 + 1), slice(1, n2 + 1))
        g = problem.geom
        self.mask = t(1.0 - g.iblank[I, J, K])                     # 1 on fluid interior cells
        self.flags = [t(f[I, J, K]) for f in g.flags]              # ium, iup, jum, jup, kum, kup
        self.fluid = fortran_zeros(self.shape, self.dev)
        self.fluid[I, J, K] = self.mask
        self.vol = fortran_zeros(self.shape, self.dev)
        self.vol[I, J, K] = (self.dx[I][:, None, None] * self.dy[J][None, :, None] * self.dz[K][None, None, :]
                             * self.mask)
        # 7-point coefficients of calc_residual (IBM/CORE_POISSON.F90:1111-1222)
        ium, iup, jum, jup, kum, kup = self.flags
        d2 = 1.0 if self.three_d else 0.0
        self.bmx = (self.dxcinv[1:n0 + 1] * self.dxinv[1:n0 + 1])[:, None, None] * (1 - ium)
        self.bpx = (self.dxcinv[2:n0 + 2] * self.dxinv[1:n0 + 1])[:, None, None] * (1 - iup)
        self.bmy = (self.dycinv[1:n1 + 1] * self.dyinv[1:n1 + 1])[None, :, None] * (1 - jum)
        self.bpy = (self.dycinv[2:n1 + 2] * self.dyinv[1:n1 + 1])[None, :, None] * (1 - jup)
        self.bmz = (self.dzcinv[1:n2 + 1] * self.dzinv[1:n2 + 1])[None, None, :] * (1 - kum) * d2
        self.bpz = (self.dzcinv[2:n2 + 2] * self.dzinv[1:n2 + 1])[None, None, :] * (1 - kup) * d2
        self.bc = -(self.bmx + self.bpx) - (self.bmy + self.bpy) - (self.bmz + self.bpz)
        self._ghost_setup()

    # ------------------------------------------------------------ ghosts --
    def _ghost_setup(self):
        """Ghost rows p_g = sum_r C(g, r) p(stencil r) as sparse matrices over
        the flattened full array (Fortran order): C_GF (ghost x cells, stencil
        cells that are not ghosts) and C_GG (ghost x ghost)."""
        g = self.pr.geom
        nG = g.nGhost
        self.nG = nG
        sx, sy = self.shape[0], self.shape[1]
        lin = lambda i, j, k: i + sx * (j + sy * k)
        if nG == 0:
            self.gidx = torch.zeros(0, dtype=torch.long, device=self.dev)
            return
        gi = np.array([lin(g.iG[n], g.jG[n], g.kG[n]) for n in range(nG)], dtype=np.int64)
        num = {int(v): n for n, v in enumerate(gi)}
        rows_f, cols_f, vals_f, rows_g, cols_g, vals_g = [], [], [], [], [], []
        for n in range(nG):
            for r, (a, b, c) in enumerate(_INC):
                ii, jj, kk = g.iCI[n] + a, g.jCI[n] + b, g.kCI[n] + c
                if (ii, jj, kk) == (g.iG[n], g.jG[n], g.kG[n]):
                    continue   # the ghost's own entry carries uNormal = 0
                cval = float(g.coeff[r, n])
                e = lin(ii, jj, kk)
                if e in num:
                    rows_g.append(n); cols_g.append(num[e]); vals_g.append(cval)
                else:
                    rows_f.append(n); cols_f.append(e); vals_f.append(cval)
        ntot = int(np.prod(self.shape))
        self.C_GF = sp.csr_matrix((vals_f, (rows_f, cols_f)), shape=(nG, ntot))
        self.C_GG = sp.csr_matrix((vals_g, (rows_g, cols_g)), shape=(nG, nG))
        self.gidx_np = gi
        self.gidx = torch.as_tensor(gi, device=self.dev)
        # ghost elimination p_G = (I - C_GG)^-1 C_GF p (extend) and its transpose
        # (extend_T): C_GF, C_GF^T, C_GG and C_GG^T as padded-row gathers on the
        # device; (I - C_GG)^-1 by the fixed-point sweeps x <- r + C_GG x that the
        # forward ghost rows use (the ghost-ghost couplings contract), with a
        # sweep count fixed once here so that no call synchronises
        self._gCGF = self._padded(self.C_GF)
        CT = self.C_GF.T.tocsr()
        rows = np.nonzero(np.diff(CT.indptr))[0]            # stencil cells that receive cotangents
        self._ct_rows = torch.as_tensor(rows, device=self.dev)
        self._gCGFT = self._padded(CT[rows])
        self._gCGG = self._padded(self.C_GG)
        self._gCGGT = self._padded(self.C_GG.T.tocsr())
        self._ghost_sweeps = max(self._sweeps_to_converge(False), self._sweeps_to_converge(True))

    GHOST_RTOL = 1e-16    # relative change at which the calibration sweeps stop
    GHOST_MAX = 5000      # calibration cap; not converging by then is an error

    def _sweeps_to_converge(self, transpose):
        """Twice the sweeps a random right-hand side needs until the largest
        change is below GHOST_RTOL of the largest value."""
        if self.C_GG.nnz == 0:
            return 1
        pad = self._gCGGT if transpose else self._gCGG
        g = torch.Generator(device="cpu").manual_seed(7)
        r = torch.randn(self.nG, dtype=torch.float64, generator=g).to(self.dev)
        x = r.clone()
        for k in range(1, self.GHOST_MAX + 1):
            xn = r + self._gather_mv(pad, x)
            d = float((xn - x).abs().max())
            x = xn
            if d <= self.GHOST_RTOL * float(x.abs().max()):
                return 2 * k
        raise RuntimeError("ghost-row couplings do not contract: (I - C_GG) sweeps did not converge")

    def _ghost_solve(self, r, transpose):
        """(I - C_GG)^-1 r, or its transpose."""
        if self.C_GG.nnz == 0:
            return r
        pad = self._gCGGT if transpose else self._gCGG
        x = r
        for _ in range(self._ghost_sweeps):
            x = r + self._gather_mv(pad, x)
        return x

    def _padded(self, S):
        """Sparse rows as (cols, vals) padded to the longest row, for a
        deterministic gather-and-sum product on the device."""
        S = S.tocsr()
        nr = S.shape[0]
        width = max(1, int(np.diff(S.indptr).max())) if nr else 1
        cols = np.zeros((nr, width), dtype=np.int64)
        vals = np.zeros((nr, width))
        for r in range(nr):
            a, b = S.indptr[r], S.indptr[r + 1]
            cols[r, :b - a] = S.indices[a:b]
            vals[r, :b - a] = S.data[a:b]
        return torch.as_tensor(cols, device=self.dev), torch.as_tensor(vals, device=self.dev)

    @staticmethod
    def _gather_mv(pad, v):
        cols, vals = pad
        return (vals * v[cols]).sum(dim=1)

    def _flat(self, x):
        """Fortran-order flat view (copy) of a full array as numpy."""
        return x.permute(2, 1, 0).reshape(-1).cpu().numpy()

    def extend(self, pf):
        """E: fluid pressure -> full array with ghost values from the ghost rows."""
        out = as_fortran(pf * self.fluid)
        if self.nG == 0:
            return out
        flat = out.permute(2, 1, 0).reshape(-1)
        flat[self.gidx] = self._ghost_solve(self._gather_mv(self._gCGF, flat), False)
        return out

    def extend_T(self, y):
        """E^T: full-array cotangent -> fluid cells (ghost cotangents pushed back
        through the transposed ghost rows)."""
        out = as_fortran(y * self.fluid)
        if self.nG == 0:
            return out
        q = self._ghost_solve(y.permute(2, 1, 0).reshape(-1)[self.gidx], True)
        flat = out.permute(2, 1, 0).reshape(-1)
        flat[self._ct_rows] += self._gather_mv(self._gCGFT, q)
        return out * self.fluid

    # ------------------------------------------------- divergence (D F) --
    def div(self, u, v, w):
        """nlu0 = div(face velocity) (1 - iblank), face velocities by face_vel
        with zero velocity on flagged faces."""
        n0, n1, n2 = self.n
        I, J, K = self.IJK
        ium, iup, jum, jup, kum, kup = self.flags
        fx, fy, fz = self.fx, self.fy, self.fz
        X = lambda a, b: a[b][:, None, None]
        Y = lambda a, b: a[b][None, :, None]
        Z = lambda a, b: a[b][None, None, :]
        s2, s1, s0 = slice(2, n0 + 2), slice(1, n0 + 1), slice(0, n0)
        fu_p = (X(fx, s2) * u[2:n0 + 2, J, K] + (1 - X(fx, s2)) * u[I, J, K]) * (1 - iup)
        fu_m = (X(fx, s1) * u[I, J, K] + (1 - X(fx, s1)) * u[0:n0, J, K]) * (1 - ium)
        t2, t1 = slice(2, n1 + 2), slice(1, n1 + 1)
        fv_p = (Y(fy, t2) * v[I, 2:n1 + 2, K] + (1 - Y(fy, t2)) * v[I, J, K]) * (1 - jup)
        fv_m = (Y(fy, t1) * v[I, J, K] + (1 - Y(fy, t1)) * v[I, 0:n1, K]) * (1 - jum)
        d = (fu_p - fu_m) * X(self.dxinv, s1) + (fv_p - fv_m) * Y(self.dyinv, t1)
        if self.three_d:
            r2, r1 = slice(2, n2 + 2), slice(1, n2 + 1)
            fw_p = (Z(fz, r2) * w[I, J, 2:n2 + 2] + (1 - Z(fz, r2)) * w[I, J, K]) * (1 - kup)
            fw_m = (Z(fz, r1) * w[I, J, K] + (1 - Z(fz, r1)) * w[I, J, 0:n2]) * (1 - kum)
            d = d + (fw_p - fw_m) * Z(self.dzinv, r1)
        out = fortran_zeros(self.shape, self.dev)
        out[I, J, K] = d * self.mask
        return out

    def div_T(self, z):
        """(D F)^T: cotangent on the right-hand side -> cotangents of u, v, w."""
        n0, n1, n2 = self.n
        I, J, K = self.IJK
        ium, iup, jum, jup, kum, kup = self.flags
        fx, fy, fz = self.fx, self.fy, self.fz
        uT, vT, wT = (fortran_zeros(self.shape, self.dev) for _ in range(3))
        zi = z[I, J, K] * self.mask
        a = zi * self.dxinv[1:n0 + 1][:, None, None]
        fxp, fxm = fx[2:n0 + 2][:, None, None], fx[1:n0 + 1][:, None, None]
        uT[2:n0 + 2, J, K] += a * (1 - iup) * fxp
        uT[I, J, K] += a * (1 - iup) * (1 - fxp) - a * (1 - ium) * fxm
        uT[0:n0, J, K] -= a * (1 - ium) * (1 - fxm)
        b = zi * self.dyinv[1:n1 + 1][None, :, None]
        fyp, fym = fy[2:n1 + 2][None, :, None], fy[1:n1 + 1][None, :, None]
        vT[I, 2:n1 + 2, K] += b * (1 - jup) * fyp
        vT[I, J, K] += b * (1 - jup) * (1 - fyp) - b * (1 - jum) * fym
        vT[I, 0:n1, K] -= b * (1 - jum) * (1 - fym)
        if self.three_d:
            c = zi * self.dzinv[1:n2 + 1][None, None, :]
            fzp, fzm = fz[2:n2 + 2][None, None, :], fz[1:n2 + 1][None, None, :]
            wT[I, J, 2:n2 + 2] += c * (1 - kup) * fzp
            wT[I, J, K] += c * (1 - kup) * (1 - fzp) - c * (1 - kum) * fzm
            wT[I, J, 0:n2] -= c * (1 - kum) * (1 - fzm)
        return uT, vT, wT

    # ------------------------------------------------------ gradient (G) --
    def grad(self, p):
        """Cell-centre pressure gradient of correct_vel on fluid interior
        cells (face pressures by interpolation, the cell's own pressure on
        flagged faces), zero elsewhere."""
        n0, n1, n2 = self.n
        I, J, K = self.IJK
        ium, iup, jum, jup, kum, kup = self.flags
        fxp, fxm = self.fx[2:n0 + 2][:, None, None], self.fx[1:n0 + 1][:, None, None]
        pc = p[I, J, K]
        pe = (fxp * p[2:n0 + 2, J, K] + (1 - fxp) * pc) * (1 - iup) + pc * iup
        pw = (fxm * pc + (1 - fxm) * p[0:n0, J, K]) * (1 - ium) + pc * ium
        fyp, fym = self.fy[2:n1 + 2][None, :, None], self.fy[1:n1 + 1][None, :, None]
        pn = (fyp * p[I, 2:n1 + 2, K] + (1 - fyp) * pc) * (1 - jup) + pc * jup
        ps = (fym * pc + (1 - fym) * p[I, 0:n1, K]) * (1 - jum) + pc * jum
        gx, gy, gz = (fortran_zeros(self.shape, self.dev) for _ in range(3))
        gx[I, J, K] = (pe - pw) * self.dxinv[1:n0 + 1][:, None, None] * self.mask
        gy[I, J, K] = (pn - ps) * self.dyinv[1:n1 + 1][None, :, None] * self.mask
        if self.three_d:
            fzp, fzm = self.fz[2:n2 + 2][None, None, :], self.fz[1:n2 + 1][None, None, :]
            pf = (fzp * p[I, J, 2:n2 + 2] + (1 - fzp) * pc) * (1 - kup) + pc * kup
            pb = (fzm * pc + (1 - fzm) * p[I, J, 0:n2]) * (1 - kum) + pc * kum
            gz[I, J, K] = (pf - pb) * self.dzinv[1:n2 + 1][None, None, :] * self.mask
        return gx, gy, gz

    def grad_T(self, lx, ly, lz):
        """G^T: cotangents of the corrected velocity -> cotangent of p (full array)."""
        n0, n1, n2 = self.n
        I, J, K = self.IJK
        ium, iup, jum, jup, kum, kup = self.flags
        out = fortran_zeros(self.shape, self.dev)
        b = lx[I, J, K] * self.mask * self.dxinv[1:n0 + 1][:, None, None]
        fxp, fxm = self.fx[2:n0 + 2][:, None, None], self.fx[1:n0 + 1][:, None, None]
        out[2:n0 + 2, J, K] += b * (1 - iup) * fxp
        out[I, J, K] += b * ((1 - iup) * (1 - fxp) + iup) - b * ((1 - ium) * fxm + ium)
        out[0:n0, J, K] -= b * (1 - ium) * (1 - fxm)
        c = ly[I, J, K] * self.mask * self.dyinv[1:n1 + 1][None, :, None]
        fyp, fym = self.fy[2:n1 + 2][None, :, None], self.fy[1:n1 + 1][None, :, None]
        out[I, 2:n1 + 2, K] += c * (1 - jup) * fyp
        out[I, J, K] += c * ((1 - jup) * (1 - fyp) + jup) - c * ((1 - jum) * fym + jum)
        out[I, 0:n1, K] -= c * (1 - jum) * (1 - fym)
        if self.three_d:
            d = lz[I, J, K] * self.mask * self.dzinv[1:n2 + 1][None, None, :]
            fzp, fzm = self.fz[2:n2 + 2][None, None, :], self.fz[1:n2 + 1][None, None, :]
            out[I, J, 2:n2 + 2] += d * (1 - kup) * fzp
            out[I, J, K] += d * ((1 - kup) * (1 - fzp) + kup) - d * ((1 - kum) * fzm + kum)
            out[I, J, 0:n2] -= d * (1 - kum) * (1 - fzm)
        return out

    # ----------------------------------------------- pressure operator A --
    def apply_full(self, p):
        """A p on fluid interior cells (p a full array, ghosts included)."""
        n0, n1, n2 = self.n
        I, J, K = self.IJK
        out = fortran_zeros(self.shape, self.dev)
        out[I, J, K] = (p[I, J, K] * self.bc + p[0:n0, J, K] * self.bmx + p[2:n0 + 2, J, K] * self.bpx
                        + p[I, 0:n1, K] * self.bmy + p[I, 2:n1 + 2, K] * self.bpy
                        + p[I, J, 0:n2] * self.bmz + p[I, J, 2:n2 + 2] * self.bpz) * self.mask
        return out

    def apply_full_T(self, z):
        """A^T z for z on fluid interior cells: a full array (fluid and ghost entries)."""
        n0, n1, n2 = self.n
        I, J, K = self.IJK
        zi = z[I, J, K] * self.mask
        out = fortran_zeros(self.shape, self.dev)
        out[I, J, K] += zi * self.bc
        out[0:n0, J, K] += zi * self.bmx
        out[2:n0 + 2, J, K] += zi * self.bpx
        out[I, 0:n1, K] += zi * self.bmy
        out[I, 2:n1 + 2, K] += zi * self.bpy
        out[I, J, 0:n2] += zi * self.bmz
        out[I, J, 2:n2 + 2] += zi * self.bpz
        return out

    def apply_eff(self, pf):
        return self.apply_full(self.extend(pf))

    def apply_eff_T(self, z):
        return self.extend_T(self.apply_full_T(z))

    def dot(self, a, b):
        return float((a * b).sum())


# ---------------------------------------------------------------- solves --
class _DeviceMG:
    """Forward multigrid on device buffers through the C ABI: full solves
    (FGMRES(m) around MG_Solver, FP64) and single MG_Solver applications (the
    preconditioner of the transposed solve)."""

    def __init__(self, problem, device, mixed_precondition: bool = False):
        from .poisson import PoissonSolver
        self.ops_shape = problem.shape
        self.dev = device
        base = copy.deepcopy(problem.params)
        base.precision_mode = PRECISION_FP64
        one = copy.deepcopy(base)
        one.outer_krylov, one.iterMax_Poisson, one.restol_Poisson = 0, 1, 0.0
        if mixed_precondition:   # one FP32 MG_Solver application inside the FP64 residual
            one.precision_mode = 1
        self.s_one = PoissonSolver(one, problem.x, problem.y, problem.z).set_boundary(problem.geom)
        self.base = base
        self.problem = problem
        self.p = fortran_zeros(problem.shape, device)
        self.b = fortran_zeros(problem.shape, device)
        self._full = {}

    def _solver(self, restol, krylov, iters):
        from .poisson import PoissonSolver
        key = (restol, krylov, iters)
        if key not in self._full:
            q = copy.deepcopy(self.base)
            q.outer_krylov, q.restol_Poisson, q.iterMax_Poisson = krylov, restol, iters
            self._full[key] = PoissonSolver(q, self.problem.x, self.problem.y, self.problem.z).set_boundary(
                self.problem.geom)
        return self._full[key]

    def precondition(self, r):
        """One MG_Solver application from zero on rhs r (fluid values)."""
        self.b.copy_(r)
        self.p.zero_()
        torch.cuda.synchronize()
        self.s_one.solve_poisson_device(self.p.data_ptr(), self.b.data_ptr())
        return self.p.clone()

    def solve(self, f, rtol=1e-12, krylov=30, iters=400):
        """Full solve A_eff p = f (f consistent); returns p with ghost values.
        The right-hand side is scaled to unit max-norm so that one handle per
        (rtol, krylov, iters) serves every call (the problem is linear)."""
        scale = float(f.abs().max())
        if scale == 0.0:
            return torch.zeros_like(self.p), 0, 0, 0.0
        self.b.copy_(f / scale)
        self.p.zero_()
        s = self._solver(rtol, krylov, iters)
        torch.cuda.synchronize()
        st, it, mr, loc, _ = s.solve_poisson_device(self.p.data_ptr(), self.b.data_ptr())
        return self.p * scale, st, it, mr * scale

    def close(self):
        self.s_one.close()
        for s in self._full.values():
            s.close()


def _flat_view(x):
    """1-D view (or copy) of a full array in Fortran order."""
    return x.permute(2, 1, 0).reshape(-1)


def fgmres(apply_op, precond, rhs, dot, rtol=1e-12, m=40, max_apps=400):
    """Right-preconditioned FGMRES on full arrays: the basis is kept as the
    rows of one matrix, so classical Gram-Schmidt (twice) is two matrix-vector
    products per pass and one host transfer per iteration.  Returns (x,
    applications, final relative 2-norm residual)."""
    shape = rhs.shape
    dev = rhs.device
    N = rhs.numel()
    unflat = lambda v: v.reshape(tuple(reversed(shape))).permute(2, 1, 0)
    b = _flat_view(rhs).clone()
    beta0 = float(torch.linalg.vector_norm(b))
    x = torch.zeros(N, dtype=torch.float64, device=dev)
    if beta0 == 0.0:
        return unflat(x), 0, 0.0
    V = torch.empty((m + 1, N), dtype=torch.float64, device=dev)
    Z = torch.empty((m, N), dtype=torch.float64, device=dev)
    apps = 0
    r = b
    rel = 1.0
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
            Z[j] = _flat_view(precond(unflat(V[j])))
            wv = _flat_view(apply_op(unflat(Z[j]))).clone()
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
        x += torch.as_tensor(y, device=dev) @ Z[:k]
        r = b - _flat_view(apply_op(unflat(x)))
    return unflat(x), apps, rel


class Projection:
    """The projection step of one geometry on the GPU: forward map, left null
    vector, transposed solve and gradient."""

    def __init__(self, problem, device="cuda"):
        self.ops = ProjectionOperators(problem, device)
        self.mg = _DeviceMG(problem, self.ops.dev)
        self.pr = problem
        o = self.ops
        self.vol = o.vol
        self.volinv = torch.where(o.vol > 0, 1.0 / torch.where(o.vol > 0, o.vol, torch.ones_like(o.vol)),
                                  torch.zeros_like(o.vol))
        self.stats = {}
        self.w = self._left_null()

    def _precond_T(self, v):
        """V M V^-1: forward multigrid conjugated by the fluid cell volumes."""
        return self.vol * (self.mg.precondition(self.volinv * v) * self.ops.fluid)

    def solve_T(self, s, rtol=1e-10):
        """A_eff^T z = s (s orthogonal to 1_F); returns one solution."""
        z, apps, rel = fgmres(self.ops.apply_eff_T, self._precond_T, s * self.ops.fluid, self.ops.dot,
                              rtol=rtol, m=60)
        self.stats["transposed_applications"] = apps
        self.stats["transposed_rel_residual"] = rel
        return z

    def _left_null(self):
        """w with w^T A_eff = 0, scaled so that w . 1_F = volume of the fluid."""
        v1 = self.vol.clone()
        d = self.solve_T(-self.ops.apply_eff_T(v1), rtol=1e-13)
        w = (v1 + d) * self.ops.fluid
        return w * (float(self.vol.sum()) / float(w.sum()))

    def compatible(self, f):
        """P f = f - 1_F (w.f)/(w.1_F)."""
        one = self.ops.fluid
        return f - one * (self.ops.dot(self.w, f) / self.ops.dot(self.w, one))

    def pressure(self, f, rtol=1e-12):
        p, st, it, mr = self.mg.solve(self.compatible(f), rtol=rtol)
        self.stats["forward_applications"] = it
        self.stats["forward_status"] = st
        return p

    def forward(self, u, v, w, rtol=1e-12):
        f = self.ops.div(u, v, w)
        p = self.pressure(f, rtol)
        gx, gy, gz = self.ops.grad(p)
        return u - gx, v - gy, w - gz, p

    def backward(self, lu, lv, lw, rtol=1e-10):
        """dL/du* for cotangents (lu, lv, lw) of the corrected velocity; rtol is
        the relative 2-norm residual of the transposed solve."""
        o = self.ops
        s = o.extend_T(o.grad_T(lu, lv, lw))
        z = self.solve_T(s, rtol)
        one = o.fluid
        zhat = (z - self.w * (o.dot(one, z) / o.dot(one, self.w))) * one
        du, dv, dw = o.div_T(zhat)
        return lu - du, lv - dv, lw - dw

    def close(self):
        self.mg.close()


class ProjectionStep(torch.autograd.Function):
    """torch.autograd.Function around the GPU projection step: forward through
    the multigrid solve, backward through the hand-written adjoint."""

    @staticmethod
    def forward(ctx, u, v, w, proj: Projection, rtol: float = 1e-12, rtol_T: float = 1e-10):
        ctx.proj, ctx.rtol = proj, rtol_T
        un, vn, wn, _ = proj.forward(u.detach(), v.detach(), w.detach(), rtol)
        return un, vn, wn

    @staticmethod
    def backward(ctx, gu, gv, gw):
        z = ctx.proj.ops.fluid
        gu, gv, gw = (torch.zeros_like(z) if g is None else g for g in (gu, gv, gw))
        du, dv, dw = ctx.proj.backward(gu, gv, gw, ctx.rtol)
        return du, dv, dw, None, None, None


def box_kinetic_energy(problem, u, v, w, box=((0.6, 0.9), (0.35, 0.65), (0.35, 0.65))):
    """1/2 sum |u|^2 vol over the cells whose centres lie in the box."""
    mx, my, mz = Metrics(problem.x), Metrics(problem.y), Metrics(problem.z)
    dev = u.device
    sel = lambda m, lo, hi: torch.as_tensor(((m.xc >= lo) & (m.xc <= hi)).astype(np.float64), device=dev)
    cx, cy, cz = sel(mx, *box[0]), sel(my, *box[1]), sel(mz, *box[2])
    vol = torch.as_tensor(mx.dx, device=dev)[:, None, None] * torch.as_tensor(my.dx, device=dev)[None, :, None] \
        * torch.as_tensor(mz.dx, device=dev)[None, None, :]
    wgt = cx[:, None, None] * cy[None, :, None] * cz[None, None, :] * vol
    return 0.5 * (wgt * (u * u + v * v + w * w)).sum()


def rollout(u, v, w, proj: Projection, steps: int, forcing=None, checkpoint_every: int = 0):
    """`steps` projection steps u <- Proj(u + forcing); with checkpoint_every = k
    only every k-th step's input is kept and the others are recomputed in the
    backward pass (torch.utils.checkpoint over segments of k steps)."""
    from torch.utils.checkpoint import checkpoint

    def segment(a, b, c, n):
        for _ in range(n):
            if forcing is not None:
                a, b, c = a + forcing[0], b + forcing[1], c + forcing[2]
            a, b, c = ProjectionStep.apply(a, b, c, proj)
        return a, b, c

    if checkpoint_every <= 0:
        return segment(u, v, w, steps)
    done = 0
    while done < steps:
        n = min(checkpoint_every, steps - done)
        u, v, w = checkpoint(segment, u, v, w, n, use_reentrant=False)
        done += n
    return u, v, w
