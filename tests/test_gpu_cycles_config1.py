"""GPU parity for the W- and F-cycle schedules and for the 2D 128^2
all-Neumann workload (the reference's CPU case), through the C ABI.

W and F cycles (mgCycle 2 and 3, IBM/CORE_MG.F90:1239-1663 with the GMM/WF
toggling at :1307-1308,1381) and the MG_Solv_z quirk (the z cycle picks its
schedule from mgCycleX, :515) are compared with the oracle:
* one MG_Solver call from a random iterate, oracle in the GPU's line order:
  1e-10 relative;
* whole solves in the GPU's order: the same iteration count and pressure;
* converged pressure against the oracle in the reference's own order at a
  tight tolerance: 1e-10 relative L2.

The 2D 128^2 box (seeded N(0,1) cell velocities, face_vel divergence, mean
removed) at tolerance 1e-8: the GPU repeats the oracle's iteration in the
GPU's line order (same count, 1e-11), and is as close to the reference-order
oracle as that oracle run is.  Two correct solvers that differ only in their
line order stop at different points of the residual ball: the oracle against
itself, reference order against the GPU's order, differs by 7.4e-7 at 1e-8,
1.5e-9 at 1e-10 and 1.8e-11 at 1e-12.  So the 1e-10 bar on the converged
pressure applies at the tight tolerance, where it is checked too.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver, solve
from oracle.oracle import Oracle
from tests.helpers import cell_volumes, interior, rel_l2_mean_free, sphere_problem

pytestmark = pytest.mark.gpu

CYCLES = [(2, 2, 2), (3, 3, 3), (2, 1, 3), (3, 2, 1), (1, 3, 2)]


def _cases():
    return [("sphere16_tanh", lambda **kw: sphere_problem(16, stretch=1.5, **kw)),
            ("box2d_32", lambda **kw: P.box2d(32, seed=9, **kw))]


def _mask_vol(pr):
    I = interior(pr)
    return 1.0 - pr.geom.iblank[I], cell_volumes(pr), I


def _rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.mark.parametrize("cyc", CYCLES, ids=lambda c: "cycle%d%d%d" % c)
@pytest.mark.parametrize("name,make", _cases(), ids=[c[0] for c in _cases()])
def test_mg_solver_one_call_w_f_cycles(name, make, cyc, gpu_built):
    pr = make(mgcycle=cyc, iRedBlack=3, coarse_flag_mode=1)
    o = Oracle(pr)
    g = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        rng = np.random.default_rng(8)
        p = np.asfortranarray(rng.standard_normal(pr.shape))
        o.subtract_average(p)
        ref = o.mg_solver(p.copy(order="F"), pr.nlu0)
        got = p.copy(order="F")
        g.MG_Solver(got, pr.nlu0)
        I = tuple(slice(0, m) for m in (pr.params.nx + 1, pr.params.ny + 1, pr.params.nz + 1))
        assert _rel(got[I], ref[I]) < 1e-10
    finally:
        g.close()
        o.close()


@pytest.mark.parametrize("cyc", CYCLES[:3], ids=lambda c: "cycle%d%d%d" % c)
@pytest.mark.parametrize("name,make", _cases(), ids=[c[0] for c in _cases()])
def test_w_f_cycle_solves(name, make, cyc, gpu_built):
    pr = make()
    m, v, I = _mask_vol(pr)
    # whole solve in the GPU's order: the same iteration
    tol = 1e-10 * abs(pr.nlu0).max()
    ref = Oracle(make(restol_Poisson=tol, mgcycle=cyc, iRedBlack=3, coarse_flag_mode=1)).solve()
    got = solve(make(restol_Poisson=tol, mgcycle=cyc))
    assert ref["status"] == 0 and got["status"] == 0
    assert got["iters"] == ref["iters"]
    assert rel_l2_mean_free(got["p"][I], ref["p"][I], m, v) < 1e-11
    # converged pressure against the reference's own line order
    tight = 1e-12 * abs(pr.nlu0).max()
    ref0 = Oracle(make(restol_Poisson=tight, mgcycle=cyc, iRedBlack=0)).solve()
    got0 = solve(make(restol_Poisson=tight, mgcycle=cyc))
    assert ref0["status"] == 0 and got0["status"] == 0
    assert rel_l2_mean_free(got0["p"][I], ref0["p"][I], m, v) <= 1e-10


def _config1(**kw):
    return P.box2d(128, seed=1, **kw)


def test_config1_box2d_128_at_tolerance_1e8(gpu_built):
    pr = _config1()
    m, v, I = _mask_vol(pr)
    tol = 1e-8 * abs(pr.nlu0).max()
    gpu_order = Oracle(_config1(restol_Poisson=tol, iRedBlack=3, coarse_flag_mode=1)).solve()
    ref_order = Oracle(_config1(restol_Poisson=tol, iRedBlack=0)).solve()
    got = solve(_config1(restol_Poisson=tol))
    assert got["status"] == 0 and got["maxres"] <= tol
    assert got["iters"] == gpu_order["iters"]
    assert rel_l2_mean_free(got["p"][I], gpu_order["p"][I], m, v) < 1e-11
    # as close to the reference-order run as the oracle's own GPU-order run is
    own = rel_l2_mean_free(gpu_order["p"][I], ref_order["p"][I], m, v)
    err = rel_l2_mean_free(got["p"][I], ref_order["p"][I], m, v)
    assert own < 2e-6
    assert abs(err - own) <= 1e-9, (err, own)


def test_config1_box2d_128_converged(gpu_built):
    pr = _config1()
    m, v, I = _mask_vol(pr)
    tight = 1e-12 * abs(pr.nlu0).max()
    ref = Oracle(_config1(restol_Poisson=tight, iRedBlack=0)).solve()
    for kw in ({}, {"outer_krylov": 30}):
        got = solve(_config1(restol_Poisson=tight, **kw))
        assert got["status"] == 0
        assert rel_l2_mean_free(got["p"][I], ref["p"][I], m, v) <= 1e-10


def test_config1_mixed_precision_error(gpu_built):
    """Mixed form (FP32 cycle in FP64 refinement, stationary and FGMRES) at
    1e-10 against the FP64 oracle solved tight: <= 1e-8.  (At 1e-8 the 2D
    residual ball alone holds pressures 7e-7 apart, as the FP64 oracle in the
    GPU's order shows, so the precision comparison is made at 1e-10, where
    that FP64 run is 1.2e-9 from the tight solution.)"""
    pr = _config1()
    m, v, I = _mask_vol(pr)
    ref = Oracle(_config1(restol_Poisson=1e-13 * abs(pr.nlu0).max(), iRedBlack=0)).solve()
    for kw in ({}, {"outer_krylov": 30}):
        got = solve(_config1(restol_Poisson=1e-10 * abs(pr.nlu0).max(), precision_mode=1, **kw))
        assert got["status"] == 0
        assert rel_l2_mean_free(got["p"][I], ref["p"][I], m, v) <= 1e-8


@pytest.mark.parametrize("cyc", [(1, 1, 1), (3, 3, 3)], ids=["V", "F"])
@pytest.mark.parametrize("counts", [(1, 10), (1, 4), (3, 2)], ids=lambda c: "finest%d_coarsest%d" % c)
def test_mg_solver_one_call_smoothing_counts(counts, cyc, gpu_built):
    """iterFinest / iterCoarsest (IBM/CORE_MG.F90:1148-1153, read at IBM/MAIN.F90:485):
    one MG_Solver call equals the oracle's with the same counts."""
    fin, coa = counts
    pr = sphere_problem(16, stretch=1.5, mgcycle=cyc, iRedBlack=3, coarse_flag_mode=1, iterFinest=fin,
                        iterCoarsest=coa)
    o = Oracle(pr)
    g = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        rng = np.random.default_rng(8)
        p = np.asfortranarray(rng.standard_normal(pr.shape))
        o.subtract_average(p)
        ref = o.mg_solver(p.copy(order="F"), pr.nlu0)
        got = p.copy(order="F")
        g.MG_Solver(got, pr.nlu0)
        I = tuple(slice(0, m) for m in (pr.params.nx + 1, pr.params.ny + 1, pr.params.nz + 1))
        assert _rel(got[I], ref[I]) < 1e-10
    finally:
        g.close()
        o.close()


@pytest.mark.parametrize("omega", [0.8, 1.3])
def test_mg_solver_one_call_relaxation(omega, gpu_built):
    """The line-SOR relaxation var (1 - omega) + omega sol (IBM/CORE_MG.F90:2008,
    read at IBM/MAIN.F90:478): one MG_Solver call against the oracle's."""
    pr = sphere_problem(16, stretch=1.5, iRedBlack=3, coarse_flag_mode=1, omega=omega)
    o = Oracle(pr)
    g = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        rng = np.random.default_rng(8)
        p = np.asfortranarray(rng.standard_normal(pr.shape))
        o.subtract_average(p)
        ref = o.mg_solver(p.copy(order="F"), pr.nlu0)
        got = p.copy(order="F")
        g.MG_Solver(got, pr.nlu0)
        I = tuple(slice(0, m) for m in (pr.params.nx + 1, pr.params.ny + 1, pr.params.nz + 1))
        assert _rel(got[I], ref[I]) < 1e-10
    finally:
        g.close()
        o.close()
