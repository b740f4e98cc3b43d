"""Implicit momentum solve (set_solve_ad, rhs_adjust_bc, solve_ad of
IBM/CORE_SET_SOLVERS.F90:20-95, IBM/CORE_RHS_AD.F90:588-780,
IBM/CORE_SOLVE_AD.F90:12-907).

CPU: the oracle's literal line Gauss-Seidel restatement is pinned by an
independent vectorised restatement of the discrete operator (the converged
velocity satisfies it to the tolerance), by the identity case (no viscosity,
no convection) and by the agreement of the reference's lexicographic line
order with the red-black order the GPU uses.  GPU: one red-black iteration
matches the oracle in the same order to 1e-12, and converged solutions match
the oracle's reference-order solution.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from oracle.oracle import Oracle
from tests.helpers import baffle_problem, sphere_problem, step_fields


def _operator(pr, dt, nu, faces, var, half_dt):
    """A_ad var over the interior (vectorised restatement, constant viscosity,
    no bc viscosity): per axis the implicit diffusion coefficient
    -(dt/2 nu) (dcinv(i) or 2 dinv(i) on flagged faces) dinv(i), plus the
    Crank-Nicolson convective terms."""
    n = [pr.params.nx - 1, pr.params.ny - 1, pr.params.nz - 1]
    I = tuple(slice(1, m + 1) for m in n)
    out = var[I].copy()
    diag = np.zeros_like(out)
    ms = [P.Metrics(c) for c in (pr.x, pr.y, pr.z)]
    for a in range(3 if pr.params.ndim == 3 else 2):
        m = ms[a]
        sh = [1, 1, 1]; sh[a] = n[a]
        dinv = m.dxinv[1:n[a] + 1].reshape(sh)
        dcm = m.dxcinv[1:n[a] + 1].reshape(sh)
        dcp = m.dxcinv[2:n[a] + 2].reshape(sh)
        fxm = m.fx[1:n[a] + 1].reshape(sh)
        fxp = m.fx[2:n[a] + 2].reshape(sh)
        fm = pr.geom.flags[2 * a][I].astype(float)
        fp = pr.geom.flags[2 * a + 1][I].astype(float)
        am = -(0.5 * dt * nu) * ((dcm * (1 - fm) + dinv * fm * 2.0) * dinv)
        ap = -(0.5 * dt * nu) * ((dcp * (1 - fp) + dinv * fp * 2.0) * dinv)
        ac = -(am + ap)
        lo = [slice(1, m_ + 1) for m_ in n]; hi = [slice(1, m_ + 1) for m_ in n]
        lo[a] = slice(0, n[a]); hi[a] = slice(2, n[a] + 2)
        lo, hi = tuple(lo), tuple(hi)
        hi_face = [slice(1, m_ + 1) for m_ in n]; hi_face[a] = slice(2, n[a] + 2)
        F0, F1 = faces[a][I], faces[a][tuple(hi_face)]
        am = am - half_dt * F0 * (1 - fxm) * dinv
        ap = ap + half_dt * F1 * fxp * dinv
        ac = ac + half_dt * (F1 * (1 - fxp) * (1 - fp) - F0 * fxm * (1 - fm)) * dinv
        diag += ac
        out += var[lo] * am * (1 - fm) + var[hi] * ap * (1 - fp)
    out += var[I] * diag
    return out * (1 - pr.geom.iblank[I])


def _box(n=(9, 8, 7)):
    p = P.default_params(3, *n, body=False)
    p.restol_ad, p.iterMax_ad = 1e-12, 500
    x, y, z = P.make_grid(p.nx, p.ny, p.nz, "tanh", beta=1.5)
    return P.Problem(p, x, y, z, P.empty_geometry(p), np.zeros(P.full_shape(p), order="F"), name="box_ad")


@pytest.mark.parametrize("scheme", [1, 2], ids=["ab2", "cn"])
def test_solve_ad_converges_to_the_discrete_operator(scheme):
    pr = _box()
    f = step_fields(pr, 5)
    dt, nu = 0.05, 0.02
    visc = np.full(pr.shape, nu, order="F")
    faces = [0.5 * a for a in f["faces"]]
    o = Oracle(pr)
    try:
        o.set_solve_ad(dt, visc, bcvisc=(visc, visc, visc))   # the wall viscosity is the fluid's
        vel = [a.copy(order="F") for a in (f["u"], f["v"], f["w"])]
        rhs = [f["pPrime"], f["p"], f["u"]]
        it, mr = o.solve_ad(dt, faces, vel, rhs, advec_scheme=scheme)
        assert 1 < it < 500 and mr <= 1e-12
        half_dt = 0.0 if scheme == 1 else 0.5 * dt
        n = pr.params
        I = (slice(1, n.nx), slice(1, n.ny), slice(1, n.nz))
        for q in range(3):
            res = rhs[q][I] - _operator(pr, dt, nu, faces, vel[q], half_dt)
            assert np.abs(res).max() <= 1e-11
        # the red-black line order reaches the same solution
        vel2 = [a.copy(order="F") for a in (f["u"], f["v"], f["w"])]
        o.solve_ad(dt, faces, vel2, rhs, advec_scheme=scheme, order=1)
        for a, b in zip(vel, vel2):
            assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(a).max())
    finally:
        o.close()


def test_crank_nicolson2_converges_with_the_faces_of_its_velocities():
    """CRANK_NICOLSON2 (IBM/CORE_SOLVE_AD.F90:155-157) re-evaluates face_vel of
    the current velocities after every set of sweeps: at convergence the faces
    are face_vel of the returned velocities and those velocities satisfy the
    momentum rows formed with them."""
    pr = _box()
    f = step_fields(pr, 5)
    dt, nu = 0.05, 0.02
    visc = np.full(pr.shape, nu, order="F")
    faces = [0.5 * a for a in f["faces"]]
    o = Oracle(pr)
    try:
        o.set_solve_ad(dt, visc, bcvisc=(visc, visc, visc))
        vel = [a.copy(order="F") for a in (f["u"], f["v"], f["w"])]
        rhs = [f["pPrime"], f["p"], f["u"]]
        start = [a.copy(order="F") for a in faces]
        it, mr = o.solve_ad(dt, faces, vel, rhs, advec_scheme=3)
        assert 1 < it < 500 and mr <= 1e-12
        assert max(np.abs(a - b).max() for a, b in zip(faces, start)) > 1e-3   # the faces moved
        again = o.face_vel(dt, *vel, faces=[a.copy(order="F") for a in faces])
        for a, b in zip(faces, again):
            assert np.array_equal(a, b)
        n = pr.params
        I = (slice(1, n.nx), slice(1, n.ny), slice(1, n.nz))
        for q in range(3):
            res = rhs[q][I] - _operator(pr, dt, nu, faces, vel[q], 0.5 * dt)
            assert np.abs(res).max() <= 1e-11
        # the red-black line order reaches the same fixed point
        vel2 = [a.copy(order="F") for a in (f["u"], f["v"], f["w"])]
        faces2 = [0.5 * a for a in f["faces"]]
        o.solve_ad(dt, faces2, vel2, rhs, advec_scheme=3, order=1)
        for a, b in zip(vel, vel2):
            assert np.abs(a - b).max() <= 1e-10 * max(1.0, np.abs(a).max())
    finally:
        o.close()


def test_solve_ad_identity_without_viscosity_or_convection():
    pr = _box()
    f = step_fields(pr, 6)
    o = Oracle(pr)
    try:
        o.set_solve_ad(0.1, np.zeros(pr.shape, order="F"))
        vel = [np.zeros(pr.shape, order="F") for _ in range(3)]
        rhs = [f["u"], f["v"], f["w"]]
        o.solve_ad(0.1, [np.zeros(pr.shape, order="F")] * 3, vel, rhs, advec_scheme=1)
        n = pr.params
        I = (slice(1, n.nx), slice(1, n.ny), slice(1, n.nz))
        for a, b in zip(vel, rhs):
            assert np.array_equal(a[I], b[I])
    finally:
        o.close()


# ----------------------------------------------------------------- GPU --
def _gpu_cases():
    from tests.helpers import unpaired_flags_problem
    return [("box_9x8x7", _box), ("box2d_24", lambda: P.box2d(24, seed=9)),
            ("unpaired_10x12x9", lambda: unpaired_flags_problem()),
            ("sphere16_tanh", lambda: sphere_problem(16, stretch=1.5))]


def _setup(pr, seed):
    f = step_fields(pr, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 7))
    f["visc"] = np.asfortranarray(0.01 + 0.01 * rng.random(pr.shape))
    f["bcvisc"] = [np.asfortranarray(0.01 + 0.01 * rng.random(pr.shape)) for _ in range(3)]
    f["rhs"] = [np.asfortranarray(rng.standard_normal(pr.shape)) for _ in range(3)]
    f["faces"] = [0.3 * a for a in f["faces"]]
    if pr.params.ndim == 2:
        f["faces"][2][...] = 0.0
    return f


@pytest.mark.gpu
@pytest.mark.parametrize("case", _gpu_cases(), ids=lambda c: c[0])
@pytest.mark.parametrize("scheme", [1, 2, 3], ids=["ab2", "cn", "cn2"])
@pytest.mark.parametrize("mode", ["one_iteration", "converged"])
def test_gpu_solve_ad_matches_oracle(gpu_built, case, scheme, mode):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver
    pr = case[1]()
    pr.params.restol_ad = 1e-12
    pr.params.iterMax_ad = 1 if mode == "one_iteration" else 500
    f = _setup(pr, 90 + scheme)
    dt = 0.05
    g = pr.geom
    o = Oracle(pr)
    s = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.transpose())).cuda()
    host = lambda t: np.asfortranarray(t.cpu().numpy().transpose())
    try:
        if g.nGhost:
            bi = [0.05 * np.ones(g.nGhost) for _ in range(3)]
            o.set_vel_ghosts(g.coeffD, bi)
            s.set_velocity_ghosts(g.coeffD, bi)
        o.set_solve_ad(dt, f["visc"], f["bcvisc"])
        vel = [f[k].copy(order="F") for k in "uvw"]
        faces = [a.copy(order="F") for a in f["faces"]]   # CRANK_NICOLSON2 rewrites them
        order = 1 if mode == "one_iteration" else 0
        it_ref, mr_ref = o.solve_ad(dt, faces, vel, f["rhs"], advec_scheme=scheme, order=order)
        dvel = [dev(f[k]) for k in "uvw"]
        dfaces = [dev(a) for a in f["faces"]]
        drhs = [dev(a) for a in f["rhs"]]
        dvisc = dev(f["visc"])
        dbcv = [dev(a) for a in f["bcvisc"]]
        st, it, mr = s.solve_ad(dt, [t.data_ptr() for t in dfaces], dvisc.data_ptr(), [t.data_ptr() for t in dvel],
                                [t.data_ptr() for t in drhs], bcvisc=[t.data_ptr() for t in dbcv],
                                advec_scheme=scheme)
        ncomp = 3 if pr.params.ndim == 3 else 2
        keep = np.ones(pr.shape, bool)
        if mode == "one_iteration":
            assert it == it_ref == 1
            tol = 1e-12
            # with iterMax_ad = 1 the ghost velocities get one Jacobi (GPU) or one
            # Gauss-Seidel (reference) sweep, which differ; every other cell agrees
            keep = ~g.ghost.astype(bool)
        else:
            assert st == 0 and mr <= 1e-12 and mr_ref <= 1e-12
            tol = 1e-9
        for q in range(ncomp):
            got = host(dvel[q])
            err = np.abs(got - vel[q])[keep].max()
            assert err <= tol * max(1.0, np.abs(vel[q]).max()), (q, err)
        if scheme == 3 and mode == "converged":   # the faces of the converged velocities
            for q in range(3):
                err = np.abs(host(dfaces[q]) - faces[q]).max()
                assert err <= tol * max(1.0, np.abs(faces[q]).max()), ("face", q, err)
    finally:
        s.close()
        o.close()


@pytest.mark.gpu
@pytest.mark.parametrize("case", _gpu_cases()[:3], ids=lambda c: c[0])
@pytest.mark.parametrize("scheme", [1, 2], ids=["ab2", "cn"])
def test_gpu_rhs_adjust_bc_matches_oracle(gpu_built, case, scheme):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver
    pr = case[1]()
    f = _setup(pr, 95 + scheme)
    rng = np.random.Generator(np.random.PCG64(3))
    bc9 = [np.asfortranarray(rng.standard_normal(pr.shape)) for _ in range(9)]
    dt = 0.05
    o = Oracle(pr)
    s = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    dev = lambda a: torch.from_numpy(np.ascontiguousarray(a.transpose())).cuda()
    host = lambda t: np.asfortranarray(t.cpu().numpy().transpose())
    try:
        o.set_solve_ad(dt, f["visc"], f["bcvisc"])
        nl = [a.copy(order="F") for a in f["rhs"]]
        o.rhs_adjust_bc(dt, f["faces"], nl, bc9=bc9, advec_scheme=scheme)
        dnl = [dev(a) for a in f["rhs"]]
        keep = [dev(a) for a in f["faces"]] + [dev(f["visc"])] + [dev(a) for a in bc9] + [dev(a) for a in f["bcvisc"]]
        s.rhs_adjust_bc(dt, [t.data_ptr() for t in keep[:3]], keep[3].data_ptr(), [t.data_ptr() for t in dnl],
                        bc=[t.data_ptr() for t in keep[4:13]], bcvisc=[t.data_ptr() for t in keep[13:16]],
                        advec_scheme=scheme)
        for a, b in zip(dnl, nl):
            got = host(a)
            assert np.abs(got - b).max() <= 1e-12 * max(1.0, np.abs(b).max())
    finally:
        s.close()
        o.close()
