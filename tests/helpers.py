"""Shared test helpers: problem builders with discretely compatible RHS."""
from __future__ import annotations

import functools

import numpy as np

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from oracle.oracle import Oracle


def oracle_stagnated(problem):
    """Stalled oracle pressure for the compatibility shift (one solve from zero,
    run to the plateau)."""
    def run(f):
        q = P.Problem(problem.params, problem.x, problem.y, problem.z, problem.geom, f, problem.name)

        def solve_from_zero(rhs, iters):
            q.nlu0 = rhs
            o = Oracle(q, iterMax_Poisson=iters, restol_Poisson=0.0, iRedBlack=0, coarse_flag_mode=0)
            r = o.solve()
            o.close()
            return r["p"], r["hist"]

        saved = (problem.params.iterMax_Poisson, problem.params.restol_Poisson, problem.params.iRedBlack,
                 problem.params.coarse_flag_mode)
        p = P.stall_until_plateau(solve_from_zero, f)
        (problem.params.iterMax_Poisson, problem.params.restol_Poisson, problem.params.iRedBlack,
         problem.params.coarse_flag_mode) = saved
        return p
    return run


@functools.lru_cache(maxsize=None)
def _sphere_cached(n, stretch, seed):
    pr = P.sphere(n, seed=seed, stretch=stretch)
    P.make_compatible(pr, oracle_stagnated(pr))
    return pr


def sphere_problem(n=16, stretch=1.5, seed=2, **kw):
    """Compatible-RHS sphere problem (fresh params/arrays each call)."""
    base = _sphere_cached(n, stretch, seed)
    import copy
    pr = copy.deepcopy(base)
    for k, v in kw.items():
        setattr(pr.params, k, v)
    return pr


def rel_l2_mean_free(a, b, mask, vol):
    """Relative L2 distance of two pressures after removing each one's
    volume-weighted mean over ``mask`` (the Neumann constant)."""
    w = vol * mask
    am = (a * w).sum() / w.sum()
    bm = (b * w).sum() / w.sum()
    da = (a - am) * mask
    db = (b - bm) * mask
    return float(np.sqrt(((da - db) ** 2 * vol).sum() / max((db ** 2 * vol).sum(), 1e-300)))


def interior(problem):
    p = problem.params
    return (slice(1, p.nx), slice(1, p.ny), slice(1, p.nz))


def cell_volumes(problem):
    from flow_structure_interaction_fem_ibm_gb300.grid import Metrics
    p = problem.params
    mx, my, mz = Metrics(problem.x), Metrics(problem.y), Metrics(problem.z)
    return (mx.dx[1:p.nx, None, None] * my.dx[None, 1:p.ny, None] * mz.dx[None, None, 1:p.nz])
