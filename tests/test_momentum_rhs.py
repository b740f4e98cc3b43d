"""Momentum right-hand side (rhs_advec_diff, IBM/CORE_RHS_AD.F90:13-585).

CPU: the oracle's literal-loop restatement is pinned by the central scheme's
exact answers on a uniform grid (advection of a linear field by uniform face
velocities, diffusion of linear and quadratic fields) and by the
Adams-Bashforth history.  GPU: fsi_mg_rhs_advec_diff matches the oracle on
whole arrays (1e-12 relative; FMA contraction on the GPU) for both
advection schemes, both fractional-step types, with and without boundary
arrays and variable viscosity, in 3D and 2D.
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
def test_gpu_rhs_advec_diff_matches_oracle(gpu_built, case, scheme, frac, with_bc):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver
    pr = case[1]()
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
