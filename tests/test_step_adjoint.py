"""Adjoint of the whole fractional step (step_adjoint.py) on the CPU.

The differentiable restatement of the explicit routines is pinned by the
oracle's literal loops (set_bc with the outflow correction and the outer
ghost layers, face_vel, rhs_advec_diff, rhs_adjust_bc, rhs_poisson,
correct_vel with the ghost-cell velocities) on a channel with a ghost-cell
sphere and zero-gradient outflow.  The implicit systems whose transposes the
backward pass solves vanish at the oracle's converged solutions: solve_ad
with the outflow balance inside its iteration (X = (u, v, w, s)), and the
pressure's compatibility fixed point B p = f.  The adjoint of two whole steps
(oracle backend) matches FP64 central differences in directions of the
velocities, the faces and the boundary values.
"""
import numpy as np
import pytest
import torch

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.step_adjoint import StepAdjoint, StepOperators, VelGhosts, wake_plane_loss
from oracle.oracle import Oracle
from tests.step_adjoint_oracle import OracleBackend

DT, NU = 0.005, 1.0 / 300.0
INFLOW = np.array([[1.0, 0.0, 0.0]] + [[0.0, 0.0, 0.0]] * 5)
T = lambda a: torch.as_tensor(np.ascontiguousarray(a, dtype=np.float64))
N = lambda t: np.asfortranarray(t.detach().numpy())


def _channel():
    pr = P.channel((16, 12, 12))
    p = pr.params
    p.restol_ad, p.iterMax_ad = 1e-14, 1000
    p.restol_Poisson, p.iterMax_Poisson = 1e-12, 20000
    return pr


def _velocity(pr, seed=5):
    rng = np.random.default_rng(seed)
    sh = pr.shape
    fl = 1.0 - pr.geom.iblank
    u = np.asfortranarray((1.0 + 0.05 * rng.standard_normal(sh)) * fl)
    v = np.asfortranarray(0.05 * rng.standard_normal(sh) * fl)
    w = np.asfortranarray(0.05 * rng.standard_normal(sh) * fl)
    return u, v, w


def _close(a, b, tol):
    return float(np.abs(a - b).max()) <= tol * max(1.0, float(np.abs(b).max()))


def test_explicit_routines_match_the_oracle():
    pr = _channel()
    assert pr.geom.nGhost > 0
    ops = StepOperators(pr, DT, NU, INFLOW)
    rng = np.random.default_rng(1)
    sh = pr.shape
    r = lambda: np.asfortranarray(rng.standard_normal(sh))
    o = Oracle(pr)
    try:
        o.set_vel_ghosts(pr.geom.coeffD, None)
        u, v, w = r(), r(), r()
        bc9 = [r() for _ in range(9)]
        vt, bt = ops.set_bc([T(u), T(v), T(w)], [T(b) for b in bc9], 0.0)
        corr = o.set_bc([u, v, w], bc9, INFLOW, time=0.0)
        assert corr != 0.0
        for a, b in zip(vt, (u, v, w)):
            assert _close(N(a), b, 1e-14)
        for a, b in zip(bt, bc9):
            assert _close(N(a), b, 1e-14)
        bn = (bc9[0], bc9[4], bc9[8])
        base = [r() for _ in range(3)]
        ft = ops.face_vel([T(u), T(v), T(w)], [T(b) for b in bn], base=[T(a) for a in base])
        fo = o.face_vel(DT, u, v, w, bc=bn, faces=[a.copy(order="F") for a in base])
        for a, b in zip(ft, fo):
            assert np.array_equal(N(a), b)
        faces = [a.copy(order="F") for a in fo]
        visc = np.full(sh, NU, order="F")
        nl = [np.zeros(sh, order="F") for _ in range(3)]
        o.rhs_advec_diff(DT, u, v, w, faces, visc, [np.zeros(sh, order="F") for _ in range(3)], nl, bc9=bc9,
                         bcvisc=(visc,) * 3, advec_scheme=2)
        nlt = ops.rhs_advec_diff([T(u), T(v), T(w)], [T(a) for a in faces], [T(b) for b in bc9])
        I = ops.I
        for a, b in zip(nlt, nl):
            assert _close(N(a)[I], b[I], 1e-14)
        o.set_solve_ad(DT, visc, (visc,) * 3)
        nl2 = [a.copy(order="F") for a in nl]
        o.rhs_adjust_bc(DT, faces, nl2, bc9=bc9, advec_scheme=2)
        nlt2 = ops.rhs_adjust_bc([T(a) for a in faces], [T(b) for b in bc9], [T(a) for a in nl])
        for a, b in zip(nlt2, nl2):
            assert _close(N(a)[I], b[I], 1e-14)
        nlu0, _ = o.rhs_poisson(DT, *faces)
        assert _close(N(ops.rhs_poisson([T(a) for a in faces])), nlu0, 1e-14)
        pp = r()
        u2, v2, w2 = (a.copy(order="F") for a in (u, v, w))
        fc = [a.copy(order="F") for a in faces]
        o.correct_vel(DT, pp, u2, v2, w2, *fc, bc=bn)
        vt, ftc = ops.correct_vel(T(pp), [T(u), T(v), T(w)], [T(a) for a in faces], [T(b) for b in bn])
        for a, b in zip(vt, (u2, v2, w2)):
            assert _close(N(a), b, 1e-13)
        for a, b in zip(ftc, fc):
            assert _close(N(a), b, 1e-13)
    finally:
        o.close()


def _solve_ad_inputs(pr, o):
    u, v, w = _velocity(pr)
    sh = pr.shape
    bc9 = [np.zeros(sh, order="F") for _ in range(9)]
    o.set_bc([u, v, w], bc9, INFLOW, time=0.0)
    faces = list(o.face_vel(DT, u, v, w, bc=(bc9[0], bc9[4], bc9[8])))
    visc = np.full(sh, NU, order="F")
    nl = [np.zeros(sh, order="F") for _ in range(3)]
    o.rhs_advec_diff(DT, u, v, w, faces, visc, [np.zeros(sh, order="F") for _ in range(3)], nl, bc9=bc9,
                     bcvisc=(visc,) * 3, advec_scheme=2)
    o.set_bc([u, v, w], bc9, INFLOW, time=DT)
    o.set_solve_ad(DT, visc, (visc,) * 3)
    o.rhs_adjust_bc(DT, faces, nl, bc9=bc9, advec_scheme=2)
    return [u, v, w], faces, nl, bc9


def test_solve_ad_system_vanishes_at_the_oracle_solution():
    pr = _channel()
    ops = StepOperators(pr, DT, NU, INFLOW)
    o = Oracle(pr)
    try:
        o.set_vel_ghosts(pr.geom.coeffD, None)
        vel, faces, nl, bc9 = _solve_ad_inputs(pr, o)
        nl_in = [a.copy(order="F") for a in nl]
        bc_in = [a.copy(order="F") for a in bc9]
        f_in = [a.copy(order="F") for a in faces]
        it, mr = o.solve_ad(DT, faces, vel, nl, advec_scheme=2, bc9=bc9, reinv=NU)
        assert mr <= 1e-14
        n0 = ops.n[0]
        shift = bc9[0][n0, 1:-2, 1:-2] - bc_in[0][n0, 1:-2, 1:-2]
        s = float(shift.mean())
        assert abs(s) > 1e-6 and float(np.abs(shift - s).max()) <= 1e-14
        r, rs = ops.ad_system([T(a)[ops.I] for a in vel], torch.tensor(s, dtype=torch.float64),
                              [T(a) for a in nl_in], [T(b) for b in bc_in], [T(a) for a in f_in])
        for x in r:
            assert float(x.abs().max()) <= 1e-13
        assert abs(float(rs)) <= 1e-13
        # the converged faces are face_vel of the converged velocities with the shifted planes
        ft = ops.face_vel([T(a) for a in vel], (T(bc9[0]), T(bc9[4]), T(bc9[8])))
        for a, b in zip(ft, faces):
            assert _close(N(a)[ops.I], b[ops.I], 1e-14)
    finally:
        o.close()


def test_pressure_fixed_point_and_left_null_vector():
    pr = _channel()
    be = OracleBackend(pr, DT, NU)
    sa = StepAdjoint(pr, DT, NU, INFLOW, be)
    try:
        o = be.o
        vel, faces, nl, bc9 = _solve_ad_inputs(pr, o)
        o.solve_ad(DT, faces, vel, nl, advec_scheme=2, bc9=bc9, reinv=NU)
        o.face_vel(DT, *vel, bc=(bc9[0], bc9[4], bc9[8]), faces=faces)
        nlu0, _ = o.rhs_poisson(DT, *faces)
        p = be.pressure(T(nlu0))
        pf = p * sa.pops.fluid
        res = (sa.apply_B(pf) - T(nlu0) * sa.pops.fluid)
        assert float(res.abs().max()) <= 1e-10 * float(np.abs(nlu0).max())
        # the outflow term is active: without it the residual is not small
        assert float((sa.pops.apply_eff(pf) - T(nlu0) * sa.pops.fluid).abs().max()) > 1e-6
        w = sa.left_null()
        g = torch.Generator().manual_seed(3)
        x = torch.randn(pr.shape, dtype=torch.float64, generator=g) * sa.pops.fluid
        Bx = sa.apply_B(x)
        assert abs(float((w * Bx).sum())) <= 1e-10 * float((w.abs() * Bx.abs()).sum())
        # transposed operator: dot-product test
        y = torch.randn(pr.shape, dtype=torch.float64, generator=g) * sa.pops.fluid
        lhs, rhs = float((y * sa.apply_B(x)).sum()), float((sa.apply_BT(y) * x).sum())
        assert abs(lhs - rhs) <= 1e-11 * abs(lhs)
    finally:
        be.close()


def test_ghost_velocity_map_transpose():
    pr = _channel()
    ops = StepOperators(pr, DT, NU, INFLOW)
    g = torch.Generator().manual_seed(4)
    x = [torch.randn(pr.shape, dtype=torch.float64, generator=g).requires_grad_(True) for _ in range(3)]
    y = [torch.randn(pr.shape, dtype=torch.float64, generator=g) for _ in range(3)]
    out = VelGhosts.apply(ops, *x)
    # the ghost values are a linear map of the others; the ghost inputs do not matter
    gx = torch.autograd.grad(out, x, grad_outputs=y)
    lhs = sum(float((a * b.detach()).sum()) for a, b in zip(y, out))
    rhs = sum(float((a * b.detach()).sum()) for a, b in zip(gx, x))
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    for t in gx:
        assert float(t.reshape(-1)[ops.g_flat].abs().max()) == 0.0
    # the ghost rows hold after the map
    for t in out:
        assert float(ops.ghost_residual(t.detach()).abs().max()) <= 1e-14


@pytest.mark.parametrize("part", ["velocity", "faces", "bc", "velocity_warm_start"])
def test_two_step_adjoint_matches_central_differences(part):
    pr = _channel()
    be = OracleBackend(pr, DT, NU)
    sa = StepAdjoint(pr, DT, NU, INFLOW, be)
    if part == "velocity_warm_start":   # transposed solves started from the later step's solutions
        sa.warm_start, part = True, "velocity"
    ops = sa.ops
    sh = pr.shape
    try:
        u, v, w = _velocity(pr)
        vel, bc = ops.set_bc([T(u), T(v), T(w)], [torch.zeros(sh, dtype=torch.float64) for _ in range(9)], 0.0)
        faces = ops.face_vel(vel, (bc[0], bc[4], bc[8]))
        S0 = (vel, faces, bc)
        steps = 2

        def run(S):
            be.pPrime[...] = 0.0
            with torch.no_grad():
                for n in range(steps):
                    S = sa.step(*S, time=n * DT)
            return S

        loss = lambda S: float(wake_plane_loss(pr, S[0][0], 3.0)[0])
        states, S = [S0], S0
        be.pPrime[...] = 0.0
        with torch.no_grad():
            for n in range(steps - 1):
                S = sa.step(*S, time=n * DT)
                states.append(S)
            Sf = sa.step(*S, time=(steps - 1) * DT)
        uf = Sf[0][0].clone().requires_grad_(True)
        with torch.enable_grad():
            gu = torch.autograd.grad(wake_plane_loss(pr, uf, 3.0)[0], uf)[0]
        z = lambda: torch.zeros(sh, dtype=torch.float64)
        cot = ([gu, z(), z()], [z(), z(), z()], [z() for _ in range(9)])
        for n in reversed(range(steps)):
            be.pPrime[...] = 0.0
            cot = sa.step_vjp(states[n], cot, time=n * DT)
        rng = np.random.default_rng(11)
        inner = torch.zeros(sh, dtype=torch.float64)
        inner[ops.I] = 1.0
        k = {"velocity": 0, "faces": 1, "bc": 2}[part]
        d = [T(rng.standard_normal(sh)) * inner for _ in S0[k]]
        if part == "velocity":
            d = [t * T(1.0 - pr.geom.iblank) for t in d]
        adj = sum(float((a * b).sum()) for a, b in zip(cot[k], d))
        h = 1e-5

        def moved(sgn):
            grp = [a + sgn * h * b for a, b in zip(S0[k], d)]
            return tuple(grp if i == k else S0[i] for i in range(3))

        fd = (loss(run(moved(1.0))) - loss(run(moved(-1.0)))) / (2 * h)
        assert abs(fd) > 1e-6
        # FD noise of the iterative solves (about 1e-11 absolute at h = 1e-5) bounds the
        # agreement for the weak boundary-value direction
        assert abs(fd - adj) <= 1e-7 * abs(fd) + 1e-11, (fd, adj)
        assert sa.stats["ad_transposed_rel_residual"] <= 1e-12
    finally:
        be.close()


def test_replayed_solves_give_the_same_cotangent():
    """step_vjp with the implicit solves recorded by step_recorded (the
    rollout's recompute pass) equals step_vjp solving them again."""
    pr = _channel()
    be = OracleBackend(pr, DT, NU)
    sa = StepAdjoint(pr, DT, NU, INFLOW, be)
    sh = pr.shape
    try:
        u, v, w = _velocity(pr)
        vel, bc = sa.ops.set_bc([T(u), T(v), T(w)], [torch.zeros(sh, dtype=torch.float64) for _ in range(9)], 0.0)
        S0 = (vel, sa.ops.face_vel(vel, (bc[0], bc[4], bc[8])), bc)
        be.pPrime[...] = 0.0
        S1, rec = sa.step_recorded(S0)
        assert len(rec) == 2
        g = torch.Generator().manual_seed(2)
        cot = tuple([torch.randn(sh, dtype=torch.float64, generator=g) for _ in grp] for grp in S1)
        a = sa.step_vjp(S0, cot, replay=rec)
        be.pPrime[...] = 0.0
        b = sa.step_vjp(S0, cot)
        for ga, gb in zip(a, b):
            for x, y in zip(ga, gb):
                assert float((x - y).abs().max()) <= 1e-12 * max(1.0, float(y.abs().max()))
    finally:
        be.close()


def _box_channel():
    """Channel box without a body (Dirichlet inflow, zero-gradient outflow,
    symmetry sides): solve_ad has no outflow balance, and CRANK_NICOLSON2
    re-evaluates the faces inside its iteration."""
    p = P.default_params(3, 12, 8, 8, body=False)
    p.bc = (1, 2, 4, 4, 4, 4)
    p.restol_ad, p.iterMax_ad = 1e-14, 1000
    p.restol_Poisson, p.iterMax_Poisson = 1e-12, 20000
    x, y, z = P.make_grid(p.nx, p.ny, p.nz, "tanh", beta=1.5)
    geom = P.empty_geometry(p)
    p.outflow_area = P.outflow_area(p, x, y, z, geom.iblank)
    return P.Problem(p, x, y, z, geom, np.zeros(P.full_shape(p), order="F"), name="box_channel")


@pytest.mark.parametrize("scheme", [2, 3], ids=["cn", "cn2"])
def test_two_step_adjoint_without_a_body(scheme):
    pr = _box_channel()
    be = OracleBackend(pr, DT, NU, advec_scheme=scheme)
    sa = StepAdjoint(pr, DT, NU, INFLOW, be, advec_scheme=scheme)
    assert not sa.ops.mass_consv and not sa.rank1
    sh = pr.shape
    try:
        u, v, w = _velocity(pr)
        vel, bc = sa.ops.set_bc([T(u), T(v), T(w)], [torch.zeros(sh, dtype=torch.float64) for _ in range(9)], 0.0)
        S0 = (vel, sa.ops.face_vel(vel, (bc[0], bc[4], bc[8])), bc)

        def run(S):
            be.pPrime[...] = 0.0
            with torch.no_grad():
                for n in range(2):
                    S = sa.step(*S, time=n * DT)
            return S

        be.pPrime[...] = 0.0
        with torch.no_grad():
            S1 = sa.step(*S0)
            S2 = sa.step(*S1, time=DT)
        uf = S2[0][0].clone().requires_grad_(True)
        with torch.enable_grad():
            gu = torch.autograd.grad(wake_plane_loss(pr, uf, 0.6)[0], uf)[0]
        z = lambda: torch.zeros(sh, dtype=torch.float64)
        cot = ([gu, z(), z()], [z(), z(), z()], [z() for _ in range(9)])
        for S, t in ((S1, DT), (S0, 0.0)):
            be.pPrime[...] = 0.0
            cot = sa.step_vjp(S, cot, time=t)
        rng = np.random.default_rng(13)
        inner = torch.zeros(sh, dtype=torch.float64)
        inner[sa.ops.I] = 1.0
        d = [T(rng.standard_normal(sh)) * inner for _ in range(3)]
        adj = sum(float((a * b).sum()) for a, b in zip(cot[0], d))
        h = 1e-5
        Lp = float(wake_plane_loss(pr, run(([a + h * b for a, b in zip(S0[0], d)], S0[1], S0[2]))[0][0], 0.6)[0])
        Lm = float(wake_plane_loss(pr, run(([a - h * b for a, b in zip(S0[0], d)], S0[1], S0[2]))[0][0], 0.6)[0])
        fd = (Lp - Lm) / (2 * h)
        assert abs(fd) > 1e-6
        assert abs(fd - adj) <= 1e-7 * abs(fd) + 1e-11, (fd, adj)
    finally:
        be.close()


def test_adams_bashforth_right_hand_side_matches_the_oracle():
    """rhs_advec_diff with ADAMS_BASHFORTH2 (rhs_loadAB, IBM/CORE_RHS_AD.F90:385-430):
    nl and the updated history nl_old against the oracle's loops."""
    pr = _channel()
    ops = StepOperators(pr, DT, NU, INFLOW, advec_scheme=1)
    rng = np.random.default_rng(21)
    sh = pr.shape
    r = lambda: np.asfortranarray(rng.standard_normal(sh))
    o = Oracle(pr)
    try:
        u, v, w = r(), r(), r()
        faces = [r(), r(), r()]
        bc9 = [r() for _ in range(9)]
        old = [r(), r(), r()]
        visc = np.full(sh, NU, order="F")
        nl = [np.zeros(sh, order="F") for _ in range(3)]
        old_o = [a.copy(order="F") for a in old]
        o.rhs_advec_diff(DT, u, v, w, faces, visc, old_o, nl, bc9=bc9, bcvisc=(visc,) * 3, advec_scheme=1)
        nlt, oldt = ops.rhs_advec_diff([T(u), T(v), T(w)], [T(a) for a in faces], [T(b) for b in bc9],
                                       [T(a) for a in old])
        for a, b in zip(nlt, nl):
            assert _close(N(a)[ops.I], b[ops.I], 1e-14)
        for a, b in zip(oldt, old_o):
            assert _close(N(a), b, 1e-14)
    finally:
        o.close()


def test_two_step_adjoint_adams_bashforth():
    """ADAMS_BASHFORTH2 carries the convective terms of the last step: the
    state gains nl_old, and the adjoint of two steps matches central
    differences in the velocity and in that history."""
    pr = _channel()
    be = OracleBackend(pr, DT, NU, advec_scheme=1)
    sa = StepAdjoint(pr, DT, NU, INFLOW, be, advec_scheme=1)
    sh = pr.shape
    try:
        u, v, w = _velocity(pr)
        vel, bc = sa.ops.set_bc([T(u), T(v), T(w)], [torch.zeros(sh, dtype=torch.float64) for _ in range(9)], 0.0)
        rng = np.random.default_rng(4)
        old = [T(0.1 * rng.standard_normal(sh)) for _ in range(3)]
        S0 = (vel, sa.ops.face_vel(vel, (bc[0], bc[4], bc[8])), bc, old)

        def run(S):
            be.pPrime[...] = 0.0
            with torch.no_grad():
                for n in range(2):
                    S = sa.step(*S, time=n * DT)
            return S

        be.pPrime[...] = 0.0
        with torch.no_grad():
            S1 = sa.step(*S0)
            S2 = sa.step(*S1, time=DT)
        uf = S2[0][0].clone().requires_grad_(True)
        with torch.enable_grad():
            gu = torch.autograd.grad(wake_plane_loss(pr, uf, 3.0)[0], uf)[0]
        z = lambda: torch.zeros(sh, dtype=torch.float64)
        cot = ([gu, z(), z()], [z(), z(), z()], [z() for _ in range(9)], [z(), z(), z()])
        for S, t in ((S1, DT), (S0, 0.0)):
            be.pPrime[...] = 0.0
            cot = sa.step_vjp(S, cot, time=t)
        inner = torch.zeros(sh, dtype=torch.float64)
        inner[sa.ops.I] = 1.0
        for k in (0, 3):
            d = [T(rng.standard_normal(sh)) * inner for _ in range(3)]
            adj = sum(float((a * b).sum()) for a, b in zip(cot[k], d))
            h = 1e-5

            def moved(sgn):
                return tuple([a + sgn * h * b for a, b in zip(S0[k], d)] if i == k else S0[i] for i in range(4))

            fd = (float(wake_plane_loss(pr, run(moved(1.0))[0][0], 3.0)[0])
                  - float(wake_plane_loss(pr, run(moved(-1.0))[0][0], 3.0)[0])) / (2 * h)
            assert abs(fd) > 1e-7
            assert abs(fd - adj) <= 1e-7 * abs(fd) + 1e-11, (k, fd, adj)
    finally:
        be.close()


def test_hybrid_right_hand_side_matches_the_oracle():
    """rhs_advec_diff with the hybrid blend (alfa 0.65, IBM/CORE_RHS_AD.F90:150-382,
    x-direction edxWeightp1 weight included) against the oracle's loops, with face
    velocities of both signs."""
    pr = _channel()
    pr.params.alfa = 0.65
    ops = StepOperators(pr, DT, NU, INFLOW)
    assert ops.hybrid
    rng = np.random.default_rng(23)
    sh = pr.shape
    r = lambda: np.asfortranarray(rng.standard_normal(sh))
    o = Oracle(pr)
    try:
        u, v, w = r(), r(), r()
        faces = [r(), r(), r()]
        bc9 = [r() for _ in range(9)]
        visc = np.full(sh, NU, order="F")
        nl = [np.zeros(sh, order="F") for _ in range(3)]
        o.rhs_advec_diff(DT, u, v, w, faces, visc, [np.zeros(sh, order="F") for _ in range(3)], nl, bc9=bc9,
                         bcvisc=(visc,) * 3, advec_scheme=2)
        nlt = ops.rhs_advec_diff([T(u), T(v), T(w)], [T(a) for a in faces], [T(b) for b in bc9])
        for a, b in zip(nlt, nl):
            assert _close(N(a)[ops.I], b[ops.I], 1e-13)
        # the blend is active: the central restatement differs
        pr.params.alfa = 0.0
        central = StepOperators(pr, DT, NU, INFLOW).rhs_advec_diff([T(u), T(v), T(w)], [T(a) for a in faces],
                                                                   [T(b) for b in bc9])
        assert max(float((a - c).abs().max()) for a, c in zip(nlt, central)) > 1e-4
    finally:
        o.close()


def test_two_step_adjoint_hybrid():
    pr = _channel()
    pr.params.alfa = 0.5
    be = OracleBackend(pr, DT, NU)
    sa = StepAdjoint(pr, DT, NU, INFLOW, be)
    sh = pr.shape
    try:
        u, v, w = _velocity(pr)
        vel, bc = sa.ops.set_bc([T(u), T(v), T(w)], [torch.zeros(sh, dtype=torch.float64) for _ in range(9)], 0.0)
        S0 = (vel, sa.ops.face_vel(vel, (bc[0], bc[4], bc[8])), bc)

        def run(S):
            be.pPrime[...] = 0.0
            with torch.no_grad():
                for n in range(2):
                    S = sa.step(*S, time=n * DT)
            return S

        be.pPrime[...] = 0.0
        with torch.no_grad():
            S1 = sa.step(*S0)
            S2 = sa.step(*S1, time=DT)
        uf = S2[0][0].clone().requires_grad_(True)
        with torch.enable_grad():
            gu = torch.autograd.grad(wake_plane_loss(pr, uf, 3.0)[0], uf)[0]
        z = lambda: torch.zeros(sh, dtype=torch.float64)
        cot = ([gu, z(), z()], [z(), z(), z()], [z() for _ in range(9)])
        for S, t in ((S1, DT), (S0, 0.0)):
            be.pPrime[...] = 0.0
            cot = sa.step_vjp(S, cot, time=t)
        rng = np.random.default_rng(6)
        inner = torch.zeros(sh, dtype=torch.float64)
        inner[sa.ops.I] = 1.0
        d = [T(rng.standard_normal(sh)) * inner * T(1.0 - pr.geom.iblank) for _ in range(3)]
        adj = sum(float((a * b).sum()) for a, b in zip(cot[0], d))
        h = 1e-6
        Lp = float(wake_plane_loss(pr, run(([a + h * b for a, b in zip(S0[0], d)], S0[1], S0[2]))[0][0], 3.0)[0])
        Lm = float(wake_plane_loss(pr, run(([a - h * b for a, b in zip(S0[0], d)], S0[1], S0[2]))[0][0], 3.0)[0])
        fd = (Lp - Lm) / (2 * h)
        assert abs(fd) > 1e-6
        assert abs(fd - adj) <= 1e-6 * abs(fd) + 1e-10, (fd, adj)
    finally:
        be.close()
