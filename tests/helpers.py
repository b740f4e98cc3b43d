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


def fresh_shell(problem):
    """Fresh-cell mask of a moving body for tests: the interior fluid cells with
    a ghost cell among their six face neighbours (a one-cell shell around the
    body, so fresh cells also neighbour each other)."""
    ib, gh = problem.geom.iblank, problem.geom.ghost
    fresh = np.zeros_like(ib, dtype=np.int8)
    nx, ny, nz = problem.params.nx, problem.params.ny, problem.params.nz
    three_d = problem.params.ndim == 3
    ks = range(1, nz) if three_d else [1]
    for k in ks:
        for j in range(1, ny):
            for i in range(1, nx):
                if ib[i, j, k] != 0:
                    continue
                nb = [gh[i - 1, j, k], gh[i + 1, j, k], gh[i, j - 1, k], gh[i, j + 1, k]]
                if three_d:
                    nb += [gh[i, j, k - 1], gh[i, j, k + 1]]
                if any(v == 1 for v in nb):
                    fresh[i, j, k] = 1
    return fresh


def fresh_reference(problem, p, fresh):
    """Fresh-cell step of subtracting_average_pressure restated with numpy
    loops (IBM/CORE_POISSON.F90:459-488), applied to p in place."""
    ib = problem.geom.iblank
    nx, ny, nz = problem.params.nx, problem.params.ny, problem.params.nz
    three_d = problem.params.ndim == 3
    for k in range(1, nz):
        for j in range(1, ny):
            for i in range(1, nx):
                if fresh[i, j, k] != 1:
                    continue
                cnt, s = 0, 0.0
                for kk in (range(k - 1, k + 2) if three_d else [k]):
                    for jj in range(j - 1, j + 2):
                        for ii in range(i - 1, i + 2):
                            if ib[ii, jj, kk] != 1 and fresh[ii, jj, kk] != 1:
                                cnt += 1
                                s = s + p[ii, jj, kk]
                p[i, j, k] = s / cnt
    return p


# ------------------------------------------------- fractional-step cases ----
def baffle_problem(cells=(12, 10, 14), stretch=1.5, seed=3):
    """3D box without a body, stretched grid, with two interior walls: an x-face
    baffle (iup(i0,...) = ium(i0+1,...) = 1) and a y-face baffle, each set from
    both sides as set_iup would for a thin body."""
    import numpy as np
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    p = P.default_params(3, *cells, body=False)
    kind = "uniform" if stretch is None else "tanh"
    x, y, z = P.make_grid(p.nx, p.ny, p.nz, kind, beta=stretch or 1.5)
    geom = P.empty_geometry(p)
    ium, iup, jum, jup = geom.flags[:4]
    i0, j0 = cells[0] // 2, cells[1] // 2
    iup[i0, 3:cells[1] - 2, 4:cells[2] - 3] = 1
    ium[i0 + 1, 3:cells[1] - 2, 4:cells[2] - 3] = 1
    jup[2:cells[0] - 3, j0, 2:cells[2] - 5] = 1
    jum[2:cells[0] - 3, j0 + 1, 2:cells[2] - 5] = 1
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = P.full_shape(p)
    u, v, w = (np.asfortranarray(rng.standard_normal(sh)) for _ in range(3))
    nlu0 = P.face_divergence(p, x, y, z, u, v, w, geom.iblank, geom.flags)
    P.remove_fluid_mean(p, x, y, z, nlu0, geom.iblank)
    return P.Problem(p, x, y, z, geom, nlu0, name=f"baffle_{cells[0]}x{cells[1]}x{cells[2]}")


def unpaired_flags_problem(cells=(10, 12, 9), seed=5, density=0.2):
    """3D stretched box without a body whose interior face flags are set at
    random and independently on the two sides of a face (iup(i) without
    ium(i+1) and so on), so that every branch of the reference's face masks is
    taken.  The outer faces keep set_outer_iup's flags."""
    import numpy as np
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    p = P.default_params(3, *cells, body=False)
    x, y, z = P.make_grid(p.nx, p.ny, p.nz, "tanh", beta=1.5)
    geom = P.empty_geometry(p)
    rng = np.random.Generator(np.random.PCG64(seed))
    n = cells
    for q, fl in enumerate(geom.flags):
        ax, hi = q // 2, q % 2
        sl = [slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1)]
        # interior faces only: skip the outer face of this side
        sl[ax] = slice(1, n[ax]) if hi else slice(2, n[ax] + 1)
        view = fl[tuple(sl)]
        view |= (rng.random(view.shape) < density).astype(np.int8)
    sh = P.full_shape(p)
    u, v, w = (np.asfortranarray(rng.standard_normal(sh)) for _ in range(3))
    nlu0 = P.face_divergence(p, x, y, z, u, v, w, geom.iblank, geom.flags)
    return P.Problem(p, x, y, z, geom, nlu0, name=f"unpaired_{n[0]}x{n[1]}x{n[2]}")


def step_cases():
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    return [
        ("sphere16_tanh", lambda: sphere_problem(16, stretch=1.5)),
        ("box2d_24", lambda: P.box2d(24, seed=9)),
        ("baffle_12x10x14", lambda: baffle_problem()),
        ("unpaired_10x12x9", lambda: unpaired_flags_problem()),
    ]


def step_fields(problem, seed, with_bc=True):
    """Seeded cell velocities, pressures, boundary face velocities and prior
    face arrays (full layout) for the fractional-step routines."""
    import numpy as np
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = problem.shape
    r = lambda: np.asfortranarray(rng.standard_normal(sh))
    f = dict(u=r(), v=r(), w=r(), p=r(), pPrime=r(), faces=[r(), r(), r()])
    f["bc"] = [r(), r(), r()] if with_bc else [None, None, None]
    if problem.params.ndim == 2:
        f["w"][...] = 0.0
    return f


SET_BC_TYPES = {
    # velocity BC types x1, x2, y1, y2, z1, z2 (1 Dirichlet, 2 zero gradient,
    # 3 pulsatile, 4 symmetry, 7 shear)
    "dirichlet": (1, 1, 1, 1, 1, 1),
    "channel": (1, 2, 4, 4, 4, 4),
    "mixed": (3, 2, 7, 4, 2, 7),
    "shear_x": (7, 2, 4, 4, 4, 4),
    "gust_on": (1, 3, 1, 1, 1, 1),
    "gust_off": (1, 3, 1, 1, 1, 1),
    "unpaired_zg": (2, 2, 1, 1, 1, 1),
    "sphere_channel": (1, 2, 4, 4, 4, 4),
    "box2d_channel": (1, 2, 4, 4, 4, 4),
}


def set_bc_case(name, seed=17):
    """A problem with the velocity BC types of SET_BC_TYPES[name] (outflow_area
    from set_outflow_area) and seeded inputs of set_bc: cell velocities, prior
    contents of the nine bc arrays, side values and frequencies, time."""
    import numpy as np
    from flow_structure_interaction_fem_ibm_gb300 import problem as P
    if name == "unpaired_zg":
        pr = unpaired_flags_problem()
    elif name == "sphere_channel":
        pr = sphere_problem(16, stretch=1.5)
    elif name == "box2d_channel":
        pr = P.box2d(24, seed=9)
    else:
        pr = baffle_problem(cells=(10, 12, 9))
    p = pr.params
    p.bc = SET_BC_TYPES[name]
    p.outflow_area = P.outflow_area(p, pr.x, pr.y, pr.z, pr.geom.iblank) if 2 in p.bc else 1.0
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = pr.shape
    r = lambda: np.asfortranarray(rng.standard_normal(sh))
    f = dict(vel=[r(), r(), r()], bc9=[r() for _ in range(9)], val=rng.standard_normal((6, 3)),
             freq=rng.uniform(0.5, 3.0, (6, 3)), time=0.37, tstart_gust=0.5 if name == "gust_off" else 0.2,
             xout=float(pr.x[p.nx] - pr.x[1]), yout=float(pr.y[p.ny] - pr.y[1]))
    return pr, f
