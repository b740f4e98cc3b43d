"""Several fractional time steps of the sphere channel (Dirichlet inflow,
zero-gradient outflow with the outflow mass balance, symmetry sides, GCM
ghost-cell sphere) through FractionalStep on the GPU against the oracle's
chain in the reference's order (IBM/CORE_TIME_STEP.F90:201-267) with one
oracle context, so that the outflow pressure-gradient planes of the
compatibility correction persist between steps on both sides.

Zero-gradient outflow makes nlw0 (the outflow pressure-gradient term of
GCM_correct_pressure) non-zero.  The reference's MG smoother adds nlw
instead, so its stationary MG iteration converges to a system without
nlw0 while calc_residual measures the one with it, and stalls.  The
pressure solve here is the mixed form's stationary outer iteration, a
defect correction on b - A p + nlw0, or FGMRES(30).  FGMRES runs in FP64
or mixed and applies the operator of the compatibility fixed point:
A p + (phi . p / outflow_area) n1.  Its reference is the reference's LSOR branch of
solve_poisson, whose smoother adds nlw0 (the oracle with pp_solver_type
1).  Both solve the consistent system.  Both iterative solves run to tight
tolerances; after three steps the velocities, faces, boundary values and
pressure (up to its constant) agree to 1e-7."""
import copy

import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from oracle.oracle import Oracle

DT, REINV, STEPS = 0.005, 1.0 / 300.0, 3
INFLOW = np.array([[1.0, 0.0, 0.0]] + [[0.0, 0.0, 0.0]] * 5)


def small_channel():
    pr = P.channel((24, 16, 16))
    p = pr.params
    p.restol_ad, p.iterMax_ad = 1e-13, 500
    p.restol_Poisson, p.iterMax_Poisson = 1e-9, 5000
    p.precision_mode, p.outer_krylov = 1, 0
    return pr


def initial_velocity(pr, seed=5):
    """Uniform inflow plus a small seeded perturbation, zero inside the body."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = pr.shape
    fluid = 1.0 - pr.geom.iblank
    u = np.asfortranarray((1.0 + 0.05 * rng.standard_normal(sh)) * fluid)
    v = np.asfortranarray(0.05 * rng.standard_normal(sh) * fluid)
    w = np.asfortranarray(0.05 * rng.standard_normal(sh) * fluid)
    return u, v, w


def oracle_rollout(pr, u0, v0, w0, steps, scheme):
    pr = copy.deepcopy(pr)
    pr.params.pp_solver_type = 1   # the LSOR branch of solve_poisson (its smoother adds nlw0)
    o = Oracle(pr)
    try:
        o.set_vel_ghosts(pr.geom.coeffD, None)
        u, v, w = (a.copy(order="F") for a in (u0, v0, w0))
        sh = pr.shape
        bc9 = [np.zeros(sh, order="F") for _ in range(9)]
        o.set_bc([u, v, w], bc9, INFLOW, time=0.0)
        bn = (bc9[0], bc9[4], bc9[8])
        faces = list(o.face_vel(DT, u, v, w, bc=bn))
        visc = np.full(sh, REINV, order="F")
        old = [np.zeros(sh, order="F") for _ in range(3)]
        nl = [np.zeros(sh, order="F") for _ in range(3)]
        pPrime = np.zeros(sh, order="F")
        p = np.zeros(sh, order="F")
        t = 0.0
        iters = []
        for _ in range(steps):
            o.rhs_advec_diff(DT, u, v, w, faces, visc, old, nl, bc9=bc9, bcvisc=(visc,) * 3, advec_scheme=scheme)
            t += DT
            o.set_bc([u, v, w], bc9, INFLOW, time=t)
            o.set_solve_ad(DT, visc, (visc,) * 3)
            o.rhs_adjust_bc(DT, faces, nl, bc9=bc9, advec_scheme=scheme)
            it_ad, mr_ad = o.solve_ad(DT, faces, [u, v, w], nl, advec_scheme=scheme, bc9=bc9, reinv=REINV)
            o.face_vel(DT, u, v, w, bc=bn, faces=faces)
            nlu0, _ = o.rhs_poisson(DT, *faces)
            pr.nlu0 = nlu0
            sol = o.solve(pPrime)
            pPrime = sol["p"]
            o.correct_vel(DT, pPrime, u, v, w, *faces, bc=bn)
            p = o.update_pressure(pPrime, p, 0)
            iters.append((it_ad, mr_ad, sol["status"], sol["iters"], sol["maxres"]))
        return dict(u=u, v=v, w=w, faces=faces, bc9=bc9, p=p, iters=iters)
    finally:
        o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("solver", [(1, 0), (1, 30), (0, 30)], ids=["mixed_stationary", "mixed_fgmres30",
                                                                    "fp64_fgmres30"])
@pytest.mark.parametrize("scheme", [1, 2, 3], ids=["ab2", "cn", "cn2"])
def test_gpu_channel_rollout_matches_oracle(gpu_built, scheme, solver):
    from flow_structure_interaction_fem_ibm_gb300.time_step import FractionalStep
    pr = small_channel()
    pr.params.precision_mode, pr.params.outer_krylov = solver
    u0, v0, w0 = initial_velocity(pr)
    ref = oracle_rollout(pr, u0, v0, w0, STEPS, scheme)
    for it_ad, mr_ad, st, it, mr in ref["iters"]:
        assert mr_ad <= 1e-13 and st == 0
    fs = FractionalStep(pr, DT, REINV, INFLOW, advec_scheme=scheme).start(u0, v0, w0)
    try:
        for _ in range(STEPS):
            rec = fs.step()
            assert rec["ad_status"] == 0 and rec["poisson_status"] == 0 and rec["ghost_status"] == 0
        got = fs.fields()
    finally:
        fs.close()
    n = pr.params
    I = (slice(1, n.nx), slice(1, n.ny), slice(1, n.nz))
    tol = 1e-7
    for k in "uvw":
        a, b = got[k][I], ref[k][I]
        assert np.abs(a - b).max() <= tol * max(1.0, np.abs(b).max()), k
    for q, (a, b) in enumerate(zip(got["faces"], ref["faces"])):
        assert np.abs(a - b).max() <= tol * max(1.0, np.abs(b).max()), ("face", q)
    for q, (a, b) in enumerate(zip(got["bc"], ref["bc9"])):
        assert np.abs(a - b).max() <= tol * max(1.0, np.abs(b).max()), ("bc", q)
    fl = (1 - pr.geom.iblank[I]).astype(bool)
    g, r = got["p"][I][fl], ref["p"][I][fl]
    assert np.abs((g - g.mean()) - (r - r.mean())).max() <= tol * max(1.0, np.abs(r).max())


@pytest.mark.gpu
def test_extrapolated_pressure_start_gives_the_same_rollout(gpu_built):
    """pressure_guess='extrapolate' only moves the pressure solve's starting
    guess (2 p(n-1) - p(n-2)): after several steps the fields agree with the
    reference's start from p(n-1) to the solvers' tolerances."""
    from flow_structure_interaction_fem_ibm_gb300.time_step import FractionalStep
    pr = small_channel()
    pr.params.precision_mode, pr.params.outer_krylov = 1, 30
    u0, v0, w0 = initial_velocity(pr)
    out = {}
    for guess in ("previous", "extrapolate"):
        fs = FractionalStep(pr, DT, REINV, INFLOW, pressure_guess=guess).start(u0, v0, w0)
        try:
            for _ in range(5):
                rec = fs.step()
                assert rec["ad_status"] == 0 and rec["poisson_status"] == 0
            out[guess] = fs.fields()
        finally:
            fs.close()
    n = pr.params
    I = (slice(1, n.nx), slice(1, n.ny), slice(1, n.nz))
    for k in "uvw":
        a, b = out["extrapolate"][k][I], out["previous"][k][I]
        assert np.abs(a - b).max() <= 1e-7 * max(1.0, np.abs(b).max()), k
