"""Adjoint of the fractional-step rollout on the GPU (step_adjoint.py).

The torch step graph (restated explicit routines, the product's solve_ad and
pressure solve through the C ABI) reproduces the product step
(time_step.FractionalStep) on the sphere channel with zero-gradient outflow;
the checkpointed rollout adjoint matches FP64 central differences of the
product's own rollout.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P

DT, REINV = 0.005, 1.0 / 300.0
INFLOW = np.array([[1.0, 0.0, 0.0]] + [[0.0, 0.0, 0.0]] * 5)


def _channel():
    pr = P.channel((24, 16, 16))
    p = pr.params
    p.restol_ad, p.iterMax_ad = 1e-13, 500
    p.precision_mode, p.outer_krylov = 0, 30          # FP64 FGMRES(30) pressure
    p.restol_Poisson, p.iterMax_Poisson = 1e-10, 2000
    return pr


def _velocity(pr, seed=5):
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = pr.shape
    fl = 1.0 - pr.geom.iblank
    u = np.asfortranarray((1.0 + 0.05 * rng.standard_normal(sh)) * fl)
    v = np.asfortranarray(0.05 * rng.standard_normal(sh) * fl)
    w = np.asfortranarray(0.05 * rng.standard_normal(sh) * fl)
    return u, v, w


@pytest.mark.gpu
def test_torch_step_matches_the_product_step(gpu_built):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.step_adjoint import DeviceBackend, StepAdjoint
    from flow_structure_interaction_fem_ibm_gb300.time_step import FractionalStep
    pr = _channel()
    fs = FractionalStep(pr, DT, REINV, INFLOW).start(*_velocity(pr))
    be = DeviceBackend(pr, DT, REINV)
    sa = StepAdjoint(pr, DT, REINV, INFLOW, be)
    try:
        for _ in range(2):
            fs.step()
        view = lambda ts: [t.permute(2, 1, 0).clone() for t in ts]
        S0 = (view(fs.vel), view(fs.faces), view(fs.bc))
        be.pPrime.copy_(fs.pPrime)
        rec = fs.step()
        assert rec["ad_status"] == 0 and rec["poisson_status"] == 0
        with torch.no_grad():
            vel, faces, bc = sa.step(*S0)
        I = sa.ops.I
        for a, b in zip(vel, view(fs.vel)):
            err = float((a[I] - b[I]).abs().max())
            assert err <= 1e-10 * max(1.0, float(b[I].abs().max())), err
        for a, b in zip(faces, view(fs.faces)):
            err = float((a - b).abs().max())
            assert err <= 1e-10 * max(1.0, float(b.abs().max())), err
        for a, b in zip(bc, view(fs.bc)):
            err = float((a - b).abs().max())
            assert err <= 1e-10 * max(1.0, float(b.abs().max())), err
    finally:
        fs.close()
        be.close()


@pytest.mark.gpu
@pytest.mark.parametrize("scheme", [2, 1], ids=["cn", "ab2"])
def test_rollout_adjoint_matches_central_differences(gpu_built, scheme):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.step_adjoint import RolloutAdjoint, wake_plane_loss
    pr = _channel()
    ra = RolloutAdjoint(pr, DT, REINV, INFLOW, advec_scheme=scheme)
    steps, adj, every = 6, 4, 2
    try:
        ra.forward(*_velocity(pr), steps=steps, adjoint_steps=adj, checkpoint_every=every)
        loss_fn = lambda vel: wake_plane_loss(pr, vel[0], 3.0)[0]
        L, cot = ra.gradient(loss_fn)
        first = steps - adj
        base = ra.checkpoints[first]
        g = torch.Generator(device="cpu").manual_seed(9)
        fl = torch.as_tensor(np.ascontiguousarray(1.0 - pr.geom.iblank), device="cuda")
        inner = torch.zeros(pr.shape, dtype=torch.float64, device="cuda")
        inner[ra.sa.ops.I] = 1.0
        for trial in range(2):
            d = [torch.randn(pr.shape, dtype=torch.float64, generator=g).cuda() * fl * inner for _ in range(3)]
            adj_dot = sum(float((a * b).sum()) for a, b in zip(cot[0], d))
            h = 1e-4

            def run(sgn):
                st = dict(base)
                st["vel"] = [a + sgn * h * b for a, b in zip(base["vel"], d)]
                return float(loss_fn(ra.rerun(st, adj)))   # the product's rollout from the moved state

            fd = (run(1.0) - run(-1.0)) / (2 * h)
            assert abs(fd) > 1e-5
            assert abs(fd - adj_dot) <= 1e-6 * abs(fd), (trial, fd, adj_dot)
        assert ra.sa.stats["ad_transposed_rel_residual"] <= 1e-12
    finally:
        ra.close()
