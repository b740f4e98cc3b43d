"""Zero-gradient outflow with a GCM body in solve_ad: every iteration ends
with GCM_enforce_global_mass_consv (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:6-252),
which re-evaluates face_vel into the step's faces, removes the boundary terms
of the right-hand sides, corrects the zero-gradient planes by -massflux /
outflow_area and puts the terms back.

CPU: the oracle's literal restatement converges and leaves the faces of the
converged velocities without net flux out of the fluid cells.  The pressure
solve's compatibility shift of the outflow planes is linear in p and
balances the flux in one application; the FGMRES operator with zero-gradient
outflow is built on those two facts.  GPU: the
converged velocities, the faces, the nine bc arrays and the right-hand sides
agree with the oracle's reference-order solve to 1e-9.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.grid import Metrics
from oracle.oracle import Oracle
from tests.helpers import sphere_problem, step_fields

NU, DT = 0.02, 0.01
INFLOW = np.array([[1.0, 0.0, 0.0]] + [[0.0, 0.0, 0.0]] * 5)


def _channel_sphere():
    pr = sphere_problem(16, stretch=1.5)
    p = pr.params
    p.bc = (1, 2, 4, 4, 4, 4)
    p.outflow_area = P.outflow_area(p, pr.x, pr.y, pr.z, pr.geom.iblank)
    p.restol_ad, p.iterMax_ad = 1e-12, 500
    return pr


def net_flux(pr, faces):
    """(net face flux out of the fluid cells, gross x flux) of face arrays."""
    mx, my, mz = Metrics(pr.x), Metrics(pr.y), Metrics(pr.z)
    p = pr.params
    I, J, K = slice(1, p.nx), slice(1, p.ny), slice(1, p.nz)
    fu, fv, fw = faces
    dx, dy, dz = mx.dx[I][:, None, None], my.dx[J][None, :, None], mz.dx[K][None, None, :]
    t = ((fu[2:p.nx + 1, J, K] - fu[I, J, K]) * dy * dz + (fv[I, 2:p.ny + 1, K] - fv[I, J, K]) * dx * dz
         + (fw[I, J, 2:p.nz + 1] - fw[I, J, K]) * dx * dy) * (1 - pr.geom.iblank[I, J, K])
    return float(t.sum()), float(np.abs(fu[I, J, K] * dy * dz).sum())


def oracle_inputs(pr, scheme, seed=21):
    """set_bc, face_vel, rhs_advec_diff and rhs_adjust_bc of a step on the
    oracle: the inputs of solve_ad (velocities, faces, bc arrays, right-hand sides)."""
    f = step_fields(pr, seed, with_bc=False)
    f["u"] += 1.0
    visc = np.full(pr.shape, NU, order="F")
    o = Oracle(pr)
    try:
        o.set_vel_ghosts(pr.geom.coeffD, None)
        u, v, w = (f[k].copy(order="F") for k in "uvw")
        bc9 = [np.zeros(pr.shape, order="F") for _ in range(9)]
        o.set_bc([u, v, w], bc9, INFLOW)
        faces = list(o.face_vel(DT, u, v, w, bc=(bc9[0], bc9[4], bc9[8])))
        old = [np.zeros(pr.shape, order="F") for _ in range(3)]
        nl = [np.zeros(pr.shape, order="F") for _ in range(3)]
        o.rhs_advec_diff(DT, u, v, w, faces, visc, old, nl, bc9=bc9, bcvisc=(visc,) * 3, advec_scheme=scheme)
        o.set_solve_ad(DT, visc, (visc,) * 3)
        o.rhs_adjust_bc(DT, faces, nl, bc9=bc9, advec_scheme=scheme)
    finally:
        o.close()
    return dict(vel=[u, v, w], faces=faces, bc9=bc9, nl=nl, visc=visc)


def oracle_solve_ad(pr, inp, scheme):
    o = Oracle(pr)
    try:
        o.set_vel_ghosts(pr.geom.coeffD, None)
        o.set_solve_ad(DT, inp["visc"], (inp["visc"],) * 3)
        vel = [a.copy(order="F") for a in inp["vel"]]
        faces = [a.copy(order="F") for a in inp["faces"]]
        bc9 = [a.copy(order="F") for a in inp["bc9"]]
        nl = [a.copy(order="F") for a in inp["nl"]]
        it, mr = o.solve_ad(DT, faces, vel, nl, advec_scheme=scheme, bc9=bc9, reinv=NU)
        final = o.face_vel(DT, *vel, bc=(bc9[0], bc9[4], bc9[8]))
    finally:
        o.close()
    return dict(vel=vel, faces=faces, bc9=bc9, nl=nl, it=it, mr=mr, final_faces=final)


@pytest.mark.parametrize("scheme", [1, 2, 3], ids=["ab2", "cn", "cn2"])
def test_oracle_outflow_balance_in_solve_ad(scheme):
    pr = _channel_sphere()
    inp = oracle_inputs(pr, scheme)
    before, gross = net_flux(pr, inp["faces"])
    assert abs(before) > 1e-4 * gross           # the inflow and the outflow planes do not balance yet
    out = oracle_solve_ad(pr, inp, scheme)
    assert out["mr"] <= 1e-12 and out["it"] > 1
    # the corrected outflow planes moved and the converged faces carry no net flux
    assert np.abs(out["bc9"][0] - inp["bc9"][0]).max() > 1e-6
    for faces in (out["faces"], out["final_faces"]):
        m, gross = net_flux(pr, faces)
        assert abs(m) <= 1e-12 * gross


def test_oracle_solve_ad_refuses_outflow_balance_without_bc():
    pr = _channel_sphere()
    inp = oracle_inputs(pr, 2)
    o = Oracle(pr)
    try:
        o.set_solve_ad(DT, inp["visc"], (inp["visc"],) * 3)
        with pytest.raises(ValueError):
            o.solve_ad(DT, inp["faces"], inp["vel"], inp["nl"], advec_scheme=2)
    finally:
        o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [1, 2, 3], ids=["ab2", "cn", "cn2"])
def test_gpu_outflow_balance_in_solve_ad_matches_oracle(gpu_built, scheme):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver
    pr = _channel_sphere()
    inp = oracle_inputs(pr, scheme)
    ref = oracle_solve_ad(pr, inp, scheme)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.transpose())).cuda()
    host = lambda t: np.asfortranarray(t.cpu().numpy().transpose())
    s = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        s.set_velocity_ghosts(pr.geom.coeffD, None)
        dvel = [dev(a) for a in inp["vel"]]
        dfaces = [dev(a) for a in inp["faces"]]
        dbc = [dev(a) for a in inp["bc9"]]
        dnl = [dev(a) for a in inp["nl"]]
        dvisc = dev(inp["visc"])
        st, it, mr = s.solve_ad(DT, [t.data_ptr() for t in dfaces], dvisc.data_ptr(), [t.data_ptr() for t in dvel],
                                [t.data_ptr() for t in dnl], bcvisc=[dvisc.data_ptr()] * 3, advec_scheme=scheme,
                                bc=[t.data_ptr() for t in dbc], reinv=NU)
        assert st == 0 and mr <= 1e-12
        I = (slice(1, pr.params.nx), slice(1, pr.params.ny), slice(1, pr.params.nz))
        for name, got, want in (("vel", dvel, ref["vel"]), ("faces", dfaces, ref["faces"]),
                                ("bc", dbc, ref["bc9"]), ("nl", dnl, ref["nl"])):
            for q, (a, b) in enumerate(zip(got, want)):
                h = host(a)
                if name in ("vel", "nl"):
                    h, b = h[I], b[I]
                err = float(np.abs(h - b).max())
                assert err <= 1e-9 * max(1.0, float(np.abs(b).max())), (name, q, err)
        m, gross = net_flux(pr, [host(t) for t in dfaces])
        assert abs(m) <= 1e-11 * gross
    finally:
        s.close()


def _compat_shift(pr, p):
    """The outflow planes' shift of one GCM_correct_pressure on p (fresh oracle,
    planes starting at zero), and the p it leaves (ghost layers updated)."""
    o = Oracle(pr)
    try:
        q = o.correct_pressure(np.array(p, order="F", copy=True))
        return o.pgrad(), q, o
    except Exception:
        o.close()
        raise


def test_compatibility_shift_is_linear_in_p_and_balances_the_flux():
    """The two facts behind the FGMRES operator with zero-gradient outflow
    (IBM/GCM_GLOBAL_MASS_CONSERVE.F90:260-394): the shift of the outflow
    planes is a linear function of p (with planes starting at zero,
    shift(p1 + p2) = shift(p1) + shift(p2)); and after one correction the
    pressure-gradient flux balances, so a second correction with the same p
    leaves the planes where they are."""
    pr = sphere_problem(12, stretch=None, bc=(1, 2, 1, 1, 1, 1), outflow_area=1.0)
    rng = np.random.default_rng(11)
    p1 = np.asfortranarray(rng.standard_normal(pr.shape))
    p2 = np.asfortranarray(rng.standard_normal(pr.shape))
    g1, _, o1 = _compat_shift(pr, p1)
    g2, _, o2 = _compat_shift(pr, p2)
    g12, q12, o12 = _compat_shift(pr, p1 + p2)
    try:
        assert np.abs(g12).max() > 1e-3                 # the planes moved
        np.testing.assert_allclose(g12, g1 + g2, rtol=0, atol=1e-12 * np.abs(g12).max())
        o12.correct_pressure(q12)                        # same p, planes already balanced
        np.testing.assert_allclose(o12.pgrad(), g12, rtol=0, atol=1e-12 * np.abs(g12).max())
    finally:
        for o in (o1, o2, o12):
            o.close()
