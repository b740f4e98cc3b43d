"""Momentum right-hand side (rhs_advec_diff, IBM/CORE_RHS_AD.F90:13-585).

CPU: the oracle's literal-loop restatement is pinned by the central scheme's
exact answers on a uniform grid (advection of a linear field by uniform face
velocities, diffusion of linear and quadratic fields), by the
Adams-Bashforth history, and for the hybrid scheme (alfa) by the same
linear-field answers and by a vectorised numpy restatement.  GPU:
fsi_mg_rhs_advec_diff matches the oracle on whole arrays (1e-12 relative;
FMA contraction on the GPU) for both advection schemes, both
fractional-step types, with and without boundary arrays and variable
viscosity, central and hybrid, in 3D and 2D.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from oracle.oracle import Oracle
from tests.helpers import baffle_problem, sphere_problem, step_fields, unpaired_flags_problem


def _uniform_box(n=10):
    p = P.default_params(3, n, n, n, body=False)
    x, y, z = P.make_grid(p.nx, p.ny, p.nz, "uniform")
    geom = P.empty_geometry(p)
    return P.Problem(p, x, y, z, geom, np.zeros(P.full_shape(p), order="F"), name="box_uniform")


def _cells(pr):
    mx, my, mz = (P.Metrics(c) for c in (pr.x, pr.y, pr.z))
    return np.meshgrid(mx.xc, my.xc, mz.xc, indexing="ij")


def _zeros(pr, k=1):
    out = [np.zeros(pr.shape, order="F") for _ in range(k)]
    return out if k > 1 else out[0]


def test_central_scheme_known_answers():
    pr = _uniform_box(10)
    X, Y, Z = _cells(pr)
    dt, nu = 0.01, 0.3
    a, b, c = 0.7, -0.4, 0.25
    faces = [np.full(pr.shape, a, order="F"), np.full(pr.shape, b, order="F"), np.full(pr.shape, c, order="F")]
    u = np.asfortranarray(2.0 * X + 1.0)          # linear: advected at rate a*2, no diffusion
    v = np.asfortranarray(Y * Y)                  # quadratic: diffusion 2 nu, advection b*2y (central exact)
    w = np.asfortranarray(np.ones(pr.shape))      # constant: nothing
    visc = np.full(pr.shape, nu, order="F")
    o = Oracle(pr)
    try:
        nl = o.rhs_advec_diff(dt, u, v, w, faces, visc, _zeros(pr, 3), _zeros(pr, 3), advec_scheme=2)
        I = (slice(2, 10), slice(2, 10), slice(2, 10))   # away from the walls
        assert np.allclose(nl[0][I], (u - dt * 0.5 * (a * 2.0))[I], rtol=0, atol=1e-13)
        assert np.allclose(nl[1][I], (v - dt * 0.5 * (b * 2.0 * Y) + 0.5 * dt * 2.0 * nu)[I], rtol=0, atol=1e-12)
        assert np.allclose(nl[2][I], w[I], rtol=0, atol=1e-14)
        # Adams-Bashforth: nl = 1.5 N - 0.5 N_old, history updated
        old = [np.full(pr.shape, 0.2, order="F") for _ in range(3)]
        nl2 = o.rhs_advec_diff(dt, u, v, w, faces, visc, old, _zeros(pr, 3), advec_scheme=1)
        assert np.allclose(old[0][I], a * 2.0, atol=1e-12)
        assert np.allclose(nl2[0][I], (u - dt * (1.5 * a * 2.0 - 0.5 * 0.2))[I], atol=1e-13)
    finally:
        o.close()


def _cases():
    return [("sphere16_tanh", lambda: sphere_problem(16, stretch=1.5)),
            ("box2d_24", lambda: P.box2d(24, seed=9)),
            ("unpaired_10x12x9", lambda: unpaired_flags_problem())]


def _fields(pr, seed):
    f = step_fields(pr, seed)
    rng = np.random.Generator(np.random.PCG64(seed + 100))
    r = lambda: np.asfortranarray(rng.standard_normal(pr.shape))
    f["visc"] = np.asfortranarray(0.01 + 0.005 * rng.random(pr.shape))
    f["bc9"] = [r() for _ in range(9)]
    f["bcvisc"] = [np.asfortranarray(0.02 * rng.random(pr.shape)) for _ in range(3)]
    f["ew"] = np.asfortranarray(np.where(rng.random(pr.shape) < 0.1, 1.0, 1.5))
    f["old"] = [r() for _ in range(3)]
    f["nl0"] = [r() for _ in range(3)]
    return f


@pytest.mark.gpu
@pytest.mark.parametrize("case", _cases(), ids=lambda c: c[0])
@pytest.mark.parametrize("scheme", [1, 2], ids=["ab2", "cn"])
@pytest.mark.parametrize("frac", [0, 1], ids=["no_van_kan", "van_kan"])
@pytest.mark.parametrize("with_bc", [False, True], ids=["bc0", "bc"])
@pytest.mark.parametrize("alfa", [0.0, 0.65], ids=["central", "hybrid"])
def test_gpu_rhs_advec_diff_matches_oracle(gpu_built, case, scheme, frac, with_bc, alfa):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver
    pr = case[1]()
    pr.params.alfa = alfa
    f = _fields(pr, 81 + scheme + 2 * frac)
    bc9 = f["bc9"] if with_bc else [None] * 9
    bcv = f["bcvisc"] if with_bc else [None] * 3
    ew = f["ew"] if with_bc else None
    dt = 0.02
    o = Oracle(pr)
    s = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    dev = lambda a: None if a is None else torch.from_numpy(np.ascontiguousarray(a.transpose())).cuda()
    host = lambda t: np.asfortranarray(t.cpu().numpy().transpose())
    ptr = lambda t: None if t is None else t.data_ptr()
    try:
        old = [a.copy(order="F") for a in f["old"]]
        nl = [a.copy(order="F") for a in f["nl0"]]
        o.rhs_advec_diff(dt, f["u"], f["v"], f["w"], f["faces"], f["visc"], old, nl, bc9=bc9, bcvisc=bcv,
                         exp_weight=ew, p=f["p"], advec_scheme=scheme, frac_step_type=frac)
        d = {k: dev(f[k]) for k in ("u", "v", "w", "p", "visc")}
        dfaces = [dev(a) for a in f["faces"]]
        dbc = [dev(a) for a in bc9]
        dbcv = [dev(a) for a in bcv]
        dew = dev(ew)
        dold = [dev(a) for a in f["old"]]
        dnl = [dev(a) for a in f["nl0"]]
        s.rhs_advec_diff(dt, [ptr(d[k]) for k in "uvw"], [ptr(t) for t in dfaces], ptr(d["visc"]),
                         [ptr(t) for t in dnl], nl_old=[ptr(t) for t in dold], bc=[ptr(t) for t in dbc],
                         bcvisc=[ptr(t) for t in dbcv], exp_weight=ptr(dew), p=ptr(d["p"]), advec_scheme=scheme,
                         frac_step_type=frac)
        for a, b in zip(dnl + dold, nl + old):
            got = host(a)
            assert np.abs(got - b).max() <= 1e-12 * max(np.abs(b).max(), 1.0)
    finally:
        s.close()
        o.close()


# --------------------------------------------------------------- hybrid ----
def _hybrid_advection(pr, vel, faces, bcs, alfa):
    """rhs_advec with the hybrid scheme (IBM/CORE_RHS_AD.F90:150-382), written
    with numpy over whole arrays, independently of the oracle's loops: the
    interior advection term of one velocity component."""
    prm = pr.params
    n = (prm.nx - 1, prm.ny - 1, prm.nz - 1)
    nd = 3 if prm.ndim == 3 else 2
    ms = [P.Metrics(c) for c in (pr.x, pr.y, pr.z)]
    fl = pr.geom.flags
    I = (slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1))
    total = None
    for a in range(nd):
        nc, nn = n[a], n[a] + 1
        idx = np.arange(1, nc + 1)
        sh = [1, 1, 1]
        sh[a] = nc
        col = lambda arr1d, ind: arr1d[ind].reshape(sh)

        def tk(arr, ind):
            out = np.take(arr, ind, axis=a)
            sl = [slice(1, n[0] + 1), slice(1, n[1] + 1), slice(1, n[2] + 1)]
            sl[a] = slice(None)
            return out[tuple(sl)]
        fx, dinv = ms[a].fx, ms[a].dxinv
        gx = 1.0 - fx
        imm, ipp = np.maximum(idx - 2, 0), np.minimum(idx + 2, nn)
        v_i, v_im, v_ip, v_imm, v_ipp = (tk(vel, q) for q in (idx, idx - 1, idx + 1, imm, ipp))
        F0, F1 = tk(faces[a], idx), tk(faces[a], idx + 1)
        fm, fp = fl[2 * a][I], fl[2 * a + 1][I]
        bc = bcs[a][I]
        ve = (col(fx, idx + 1) * v_ip + col(gx, idx + 1) * v_i) * (1 - fp) + bc * fp
        vw = (col(fx, idx) * v_i + col(gx, idx) * v_im) * (1 - fm) + bc * fm
        s0, s1 = np.copysign(1.0, F0), np.copysign(1.0, F1)
        d = lambda q: col(dinv, q)
        em1 = (d(idx - 1) + 2.0 * d(idx)) / (d(idx - 1) + d(idx))
        em2 = d(idx) / (d(idx - 1) + d(idx))
        ep1 = (d(ipp) + 2.0 * d(idx + 1)) / (d(ipp) + d(idx + 1))
        ep2 = d(idx + 1) / (d(ipp) + d(idx + 1))
        wm1 = (d(imm) + 2.0 * d(idx - 1)) / (d(imm) + d(idx - 1))
        wm2 = d(idx - 1) / (d(imm) + d(idx - 1))
        wp1 = (d(idx + 1) + 2.0 * d(idx)) / (d(idx + 1) + d(idx))
        wp2 = d(idx) / (d(idx + 1) + d(idx))
        mm = ((idx == 1) | (idx == 2)).astype(float).reshape(sh)
        pp = ((idx == nc) | (idx == nc - 1)).astype(float).reshape(sh)
        q2 = ep1 if a == 0 else ep2   # the x direction weights vel(ipp) with edxWeightp1 (:203-205)
        ve_up = ((1.0 + s1) * (mm * ve + (1 - mm) * (em1 * v_i - em2 * v_im))
                 + (1.0 - s1) * (pp * ve + (1 - pp) * (ep1 * v_ip - q2 * v_ipp))) * 0.5 * (1 - fp) + bc * fp
        vw_up = ((1.0 + s0) * (mm * vw + (1 - mm) * (wm1 * v_im - wm2 * v_imm))
                 + (1.0 - s0) * (pp * vw + (1 - pp) * (wp1 * v_i - wp2 * v_ip))) * 0.5 * (1 - fm) + bc * fm
        term = (((1.0 - alfa) * ve + alfa * ve_up) * F1 - ((1.0 - alfa) * vw + alfa * vw_up) * F0) * d(idx)
        total = term if total is None else total + term
    return total


def test_hybrid_upwind_known_answer():
    """Second-order upwind face values are exact for a linear field on a
    uniform grid, so away from the walls (where iumm/iupp switch back to the
    central faces) the hybrid term equals the central one, for either sign of
    the y and z face velocities and for positive x face velocities.  For a
    negative x face velocity the reference weights vel(ipp) with
    edxWeightp1 (IBM/CORE_RHS_AD.F90:203-205, where y and z use their p2
    weights), so the east face value is 1.5 (v(i+1) - v(i+2)) on a uniform
    grid: the restatement keeps that."""
    pr = _uniform_box(12)
    X, Y, Z = _cells(pr)
    h = 1.0 / 12
    I = (slice(3, 11), slice(3, 11), slice(3, 11))

    def advection(field, faces, alfa, comp):
        pr.params.alfa = alfa
        o = Oracle(pr)
        try:
            old = _zeros(pr, 3)
            o.rhs_advec_diff(0.01, field, field, field, faces, np.zeros(pr.shape, order="F"), old, _zeros(pr, 3),
                             advec_scheme=1)
            return old[comp]
        finally:
            o.close()
    try:
        for axis, field in ((0, 2.0 * X + 1.0), (1, 2.0 * Y + 1.0), (2, 2.0 * Z + 1.0)):
            field = np.asfortranarray(field)
            for sgn in (1.0, -1.0):
                faces = [np.full(pr.shape, 0.0, order="F") for _ in range(3)]
                faces[axis][...] = sgn * 0.7
                central = advection(field, faces, 0.0, 0)
                hybrid = advection(field, faces, 1.0, 0)
                assert np.allclose(central[I], sgn * 0.7 * 2.0, rtol=0, atol=1e-12)
                if axis == 0 and sgn < 0:
                    # east face 1.5 (v(i+1) - v(i+2)) = -3h; west face exact (v(i) + v(i+1)) / 2
                    west = 2.0 * (X - 0.5 * h) + 1.0
                    quirk = (-3.0 * h * (-0.7) - west * (-0.7)) / h
                    assert np.allclose(hybrid[I], quirk[I], rtol=0, atol=1e-11)
                else:
                    assert np.allclose(hybrid[I], central[I], rtol=0, atol=1e-12)
    finally:
        pr.params.alfa = 0.0


@pytest.mark.parametrize("alfa", [0.0, 0.65, 1.0])
def test_hybrid_upwind_matches_vectorised_restatement(alfa):
    """The oracle's literal loops against the numpy restatement on a stretched
    box with random velocities, signed faces and boundary values (the
    Adams-Bashforth history array returns the advection term exactly)."""
    pr = P.box3d((10, 12, 9), seed=4, stretch=1.5)
    pr.params.alfa = alfa
    rng = np.random.Generator(np.random.PCG64(33))
    r = lambda: np.asfortranarray(rng.standard_normal(pr.shape))
    vel = [r() for _ in range(3)]
    faces = [r() for _ in range(3)]
    bc9 = [r() for _ in range(9)]
    o = Oracle(pr)
    try:
        old = _zeros(pr, 3)
        o.rhs_advec_diff(0.01, *vel, faces, np.zeros(pr.shape, order="F"), old, _zeros(pr, 3), bc9=bc9,
                         advec_scheme=1)
    finally:
        o.close()
    prm = pr.params
    I = (slice(1, prm.nx), slice(1, prm.ny), slice(1, prm.nz))
    for q in range(3):
        ref = _hybrid_advection(pr, vel[q], faces, bc9[3 * q:3 * q + 3], alfa)
        assert np.abs(old[q][I] - ref).max() <= 1e-12 * np.abs(ref).max()
