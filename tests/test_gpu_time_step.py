"""One whole fractional time step on the GPU against the oracle, in the
reference's order (IBM/CORE_TIME_STEP.F90:201-267): rhs_advec_diff ->
rhs_adjust_bc -> solve_ad -> face_vel + rhs_poisson -> solve_poisson ->
correct_vel -> update_pressure, every field on the device through the C ABI,
the oracle in the reference's own line orders.  Both iterative solves run to
tight tolerances, so the two steps agree to the solver tolerance; the
corrected faces are divergence-free on both sides."""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from oracle.oracle import Oracle
from tests.helpers import step_fields

pytestmark = pytest.mark.gpu


def _box():
    p = P.default_params(3, 12, 10, 14, body=False)
    p.restol_ad, p.iterMax_ad = 1e-12, 500
    p.iterMax_Poisson = 500
    x, y, z = P.make_grid(p.nx, p.ny, p.nz, "tanh", beta=1.5)
    return P.Problem(p, x, y, z, P.empty_geometry(p), np.zeros(P.full_shape(p), order="F"), name="box_step")


@pytest.mark.parametrize("scheme", [1, 2], ids=["ab2", "cn"])
def test_whole_time_step_matches_oracle(gpu_built, scheme):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver
    pr = _box()
    f = step_fields(pr, 7, with_bc=False)
    dt, nu = 0.01, 0.02
    visc = np.full(pr.shape, nu, order="F")
    o = Oracle(pr)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.transpose())).cuda()
    host = lambda t: np.asfortranarray(t.cpu().numpy().transpose())
    n = pr.params
    I = (slice(1, n.nx), slice(1, n.ny), slice(1, n.nz))
    # the previous step's faces: face_vel of the starting velocity
    faces0 = o.face_vel(dt, f["u"], f["v"], f["w"])
    # ---- oracle step
    u, v, w = (f[k].copy(order="F") for k in "uvw")
    faces = [a.copy(order="F") for a in faces0]
    old = [np.zeros(pr.shape, order="F") for _ in range(3)]
    nl = [np.zeros(pr.shape, order="F") for _ in range(3)]
    o.rhs_advec_diff(dt, u, v, w, faces, visc, old, nl, bcvisc=(visc,) * 3, advec_scheme=scheme)
    o.set_solve_ad(dt, visc, (visc,) * 3)
    o.rhs_adjust_bc(dt, faces, nl, advec_scheme=scheme)
    it_ad, mr_ad = o.solve_ad(dt, faces, [u, v, w], nl, advec_scheme=scheme)
    faces = list(o.face_vel(dt, u, v, w))
    nlu0, _ = o.rhs_poisson(dt, *faces)
    restol = 1e-11 * float(np.abs(nlu0).max())
    pr.params.restol_Poisson = restol
    pr.nlu0 = nlu0
    sol = Oracle(pr).solve()
    assert sol["status"] == 0 and mr_ad <= 1e-12
    pp = sol["p"]
    o.correct_vel(dt, pp, u, v, w, *faces)
    p_ref = o.update_pressure(pp, np.zeros(pr.shape, order="F"), 0)
    div_ref, _ = o.rhs_poisson(dt, *faces)
    assert np.abs(div_ref).max() <= 10 * restol
    # ---- GPU step (same parameters, restol set before the handle is made)
    s = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        du, dv, dw = (dev(f[k]) for k in "uvw")
        dfaces = [dev(a) for a in faces0]
        dvisc = dev(visc)
        dold = [dev(np.zeros(pr.shape, order="F")) for _ in range(3)]
        dnl = [dev(np.zeros(pr.shape, order="F")) for _ in range(3)]
        vp = [t.data_ptr() for t in (du, dv, dw)]
        fp = [t.data_ptr() for t in dfaces]
        nlp = [t.data_ptr() for t in dnl]
        bv = [dvisc.data_ptr()] * 3
        s.rhs_advec_diff(dt, vp, fp, dvisc.data_ptr(), nlp, nl_old=[t.data_ptr() for t in dold], bcvisc=bv,
                         advec_scheme=scheme)
        s.rhs_adjust_bc(dt, fp, dvisc.data_ptr(), nlp, bcvisc=bv, advec_scheme=scheme)
        st_ad, _, mr_g = s.solve_ad(dt, fp, dvisc.data_ptr(), vp, nlp, bcvisc=bv, advec_scheme=scheme)
        assert st_ad == 0 and mr_g <= 1e-12
        dnlu0, dpp, dp = (dev(np.zeros(pr.shape, order="F")) for _ in range(3))
        s.face_vel_rhs(dt, *vp, *fp, dnlu0.data_ptr())
        st, it, mr, _, _ = s.solve_poisson_device(dpp.data_ptr(), dnlu0.data_ptr())
        assert st == 0 and mr <= restol
        s.correct_vel(dt, dpp.data_ptr(), *vp, *fp)
        s.update_pressure(dpp.data_ptr(), dp.data_ptr(), 0)
        # velocities and faces agree to the solvers' tolerance; pressures up to the Neumann constant
        for a, b in zip((du, dv, dw), (u, v, w)):
            assert np.abs(host(a)[I] - b[I]).max() <= 1e-8 * max(1.0, np.abs(b).max())
        for a, b in zip(dfaces, faces):
            assert np.abs(host(a) - b).max() <= 1e-8 * max(1.0, np.abs(b).max())
        g = host(dp)[I]
        r = p_ref[I]
        assert np.abs((g - g.mean()) - (r - r.mean())).max() <= 1e-8 * max(1.0, np.abs(r).max())
        div_gpu, _ = o.rhs_poisson(dt, *(host(t) for t in dfaces))
        assert np.abs(div_gpu).max() <= 10 * restol
    finally:
        s.close()
        o.close()


def _channel():
    """Channel box without a body: Dirichlet inflow x1 (u = 1), zero-gradient
    outflow x2, symmetry sides (the outer sides of a channel run)."""
    p = P.default_params(3, 16, 8, 10, body=False)
    p.bc = (1, 2, 4, 4, 4, 4)
    p.restol_ad, p.iterMax_ad = 1e-12, 500
    p.iterMax_Poisson = 2000
    x, y, z = P.make_grid(p.nx, p.ny, p.nz, "tanh", beta=1.5)
    geom = P.empty_geometry(p)
    p.outflow_area = P.outflow_area(p, x, y, z, geom.iblank)
    return P.Problem(p, x, y, z, geom, np.zeros(P.full_shape(p), order="F"), name="channel_step")


CHANNEL_VALUES = np.array([[1.0, 0.0, 0.0]] + [[0.0, 0.0, 0.0]] * 5)


def oracle_channel_step(pr, f, dt, visc, scheme):
    """The oracle's step: set_bc of the previous step, then rhs_advec_diff ->
    set_bc -> rhs_adjust_bc -> solve_ad -> face_vel -> rhs_poisson -> solve ->
    correct_vel -> update_pressure.  Returns the fields and the solve's tolerance."""
    o = Oracle(pr)
    try:
        u, v, w = (f[k].copy(order="F") for k in "uvw")
        bc9 = [np.zeros(pr.shape, order="F") for _ in range(9)]
        o.set_bc([u, v, w], bc9, CHANNEL_VALUES, time=0.0)
        faces = list(o.face_vel(dt, u, v, w, bc=(bc9[0], bc9[4], bc9[8])))
        old = [np.zeros(pr.shape, order="F") for _ in range(3)]
        nl = [np.zeros(pr.shape, order="F") for _ in range(3)]
        o.rhs_advec_diff(dt, u, v, w, faces, visc, old, nl, bc9=bc9, bcvisc=(visc,) * 3, advec_scheme=scheme)
        corr = o.set_bc([u, v, w], bc9, CHANNEL_VALUES, time=dt)
        o.set_solve_ad(dt, visc, (visc,) * 3)
        o.rhs_adjust_bc(dt, faces, nl, bc9=bc9, advec_scheme=scheme)
        it_ad, mr_ad = o.solve_ad(dt, faces, [u, v, w], nl, advec_scheme=scheme, bc9=bc9)
        bcn = (bc9[0], bc9[4], bc9[8])
        faces = list(o.face_vel(dt, u, v, w, bc=bcn))
        nlu0, _ = o.rhs_poisson(dt, *faces)
        restol = 1e-10 * float(np.abs(nlu0).max())
        pr.params.restol_Poisson = restol
        pr.nlu0 = nlu0
        so = Oracle(pr)
        sol = so.solve()
        so.close()
        pp = sol["p"]
        o.correct_vel(dt, pp, u, v, w, *faces, bc=bcn)
        p_ref = o.update_pressure(pp, np.zeros(pr.shape, order="F"), 0)
        return dict(u=u, v=v, w=w, faces=faces, p=p_ref, bc9=bc9, corr=corr, restol=restol, sol=sol,
                    mr_ad=mr_ad)
    finally:
        o.close()


@pytest.mark.parametrize("scheme", [1, 2, 3], ids=["ab2", "cn", "cn2"])
def test_channel_time_step_with_set_bc_matches_oracle(gpu_built, scheme):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver
    pr = _channel()
    f = step_fields(pr, 11, with_bc=False)
    f["u"] += 1.0
    dt, nu = 0.01, 0.02
    visc = np.full(pr.shape, nu, order="F")
    ref = oracle_channel_step(pr, f, dt, visc, scheme)
    assert ref["sol"]["status"] == 0 and ref["mr_ad"] <= 1e-12 and ref["corr"] != 0.0
    restol = ref["restol"]
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.transpose())).cuda()
    host = lambda t: np.asfortranarray(t.cpu().numpy().transpose())
    n = pr.params
    I = (slice(1, n.nx), slice(1, n.ny), slice(1, n.nz))
    s = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        du, dv, dw = (dev(f[k]) for k in "uvw")
        vp = [t.data_ptr() for t in (du, dv, dw)]
        dbc = [dev(np.zeros(pr.shape, order="F")) for _ in range(9)]
        bp = [t.data_ptr() for t in dbc]
        bn = (bp[0], bp[4], bp[8])
        s.set_bc(vp, bp, CHANNEL_VALUES, time=0.0)
        dfaces = [dev(np.zeros(pr.shape, order="F")) for _ in range(3)]
        fp = [t.data_ptr() for t in dfaces]
        dscratch = dev(np.zeros(pr.shape, order="F"))
        s.face_vel_rhs(dt, *vp, *fp, dscratch.data_ptr(), d_bc=bn)
        dvisc = dev(visc)
        dold = [dev(np.zeros(pr.shape, order="F")) for _ in range(3)]
        dnl = [dev(np.zeros(pr.shape, order="F")) for _ in range(3)]
        nlp = [t.data_ptr() for t in dnl]
        bv = [dvisc.data_ptr()] * 3
        s.rhs_advec_diff(dt, vp, fp, dvisc.data_ptr(), nlp, nl_old=[t.data_ptr() for t in dold], bc=bp, bcvisc=bv,
                         advec_scheme=scheme)
        corr = s.set_bc(vp, bp, CHANNEL_VALUES, time=dt)
        assert abs(corr - ref["corr"]) <= 1e-12 * abs(ref["corr"])
        s.rhs_adjust_bc(dt, fp, dvisc.data_ptr(), nlp, bc=bp, bcvisc=bv, advec_scheme=scheme)
        st_ad, _, mr_g = s.solve_ad(dt, fp, dvisc.data_ptr(), vp, nlp, bcvisc=bv, advec_scheme=scheme, bc=bp)
        assert st_ad == 0 and mr_g <= 1e-12
        dnlu0, dpp, dp = (dev(np.zeros(pr.shape, order="F")) for _ in range(3))
        s.face_vel_rhs(dt, *vp, *fp, dnlu0.data_ptr(), d_bc=bn)
        st, it, mr, _, _ = s.solve_poisson_device(dpp.data_ptr(), dnlu0.data_ptr())
        assert st == 0 and mr <= restol
        s.correct_vel(dt, dpp.data_ptr(), *vp, *fp, d_bc=bn)
        s.update_pressure(dpp.data_ptr(), dp.data_ptr(), 0)
        for a, b in zip((du, dv, dw), (ref["u"], ref["v"], ref["w"])):
            assert np.abs(host(a)[I] - b[I]).max() <= 1e-8 * max(1.0, np.abs(b).max())
        for a, b in zip(dfaces, ref["faces"]):
            assert np.abs(host(a) - b).max() <= 1e-8 * max(1.0, np.abs(b).max())
        for a, b in zip(dbc, ref["bc9"]):
            assert np.abs(host(a) - b).max() <= 1e-8 * max(1.0, np.abs(b).max())
        g = host(dp)[I]
        r = ref["p"][I]
        assert np.abs((g - g.mean()) - (r - r.mean())).max() <= 1e-8 * max(1.0, np.abs(r).max())
    finally:
        s.close()
