"""The implicit solves of a fractional step on the oracle, as a backend of
step_adjoint.StepAdjoint (test infrastructure: the CPU checks of the step
adjoint run the oracle's solve_ad and pressure solve where the product runs
its C-ABI solves)."""
import copy

import numpy as np
import torch

from oracle.oracle import Oracle


class OracleBackend:
    """The implicit solves on the oracle (CPU; test infrastructure): solve_ad
    with the outflow balance, and the pressure through the LSOR branch of
    solve_poisson, whose smoother adds the outflow term nlw0."""

    device = torch.device("cpu")

    def __init__(self, problem, dt, reinv, advec_scheme=2):
        pr = copy.deepcopy(problem)
        pr.params.pp_solver_type = 1
        self.pr = pr
        self.o = Oracle(pr)
        if pr.geom.nGhost:
            self.o.set_vel_ghosts(pr.geom.coeffD, None)
        sh = pr.shape
        self.visc = np.full(sh, reinv, order="F")
        self.o.set_solve_ad(dt, self.visc, (self.visc,) * 3)
        self.dt, self.reinv, self.scheme = dt, reinv, advec_scheme
        self.pPrime = np.zeros(sh, order="F")

    @staticmethod
    def _np(t):
        return np.asfortranarray(t.detach().cpu().numpy())

    def solve_ad(self, vel, nl, bc, faces):
        v = [self._np(t) for t in vel]
        n = [self._np(t) for t in nl]
        b = [self._np(t) for t in bc]
        f = [self._np(t) for t in faces]
        it, mr = self.o.solve_ad(self.dt, f, v, n, advec_scheme=self.scheme, bc9=b, reinv=self.reinv)
        T = lambda a: torch.as_tensor(np.ascontiguousarray(a))
        return [T(a) for a in v], [T(a) for a in b], (it, mr)

    def pressure(self, nlu0):
        self.pr.nlu0 = self._np(nlu0)
        sol = self.o.solve(self.pPrime)
        if sol["status"] not in (0,):
            raise RuntimeError(f"oracle pressure solve status {sol['status']}")
        self.pPrime = sol["p"]
        return torch.as_tensor(np.ascontiguousarray(sol["p"]))

    def mg_apply(self, r):
        var = np.zeros(self.pr.shape, order="F")
        self.o.mg_solver(var, self._np(r))
        return torch.as_tensor(np.ascontiguousarray(var))

    def close(self):
        self.o.close()
