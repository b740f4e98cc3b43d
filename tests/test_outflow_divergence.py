"""Where the corrected faces of a channel step are not divergence-free, and why.

With a zero-gradient outflow side, GCM_correct_pressure adds the outflow
pressure-gradient planes to the Poisson rows of the last cell layer as nlw0
(IBM/CORE_POISSON.F90:1794-1823), while correct_vel leaves the outflow faces at
the values set_bc gave them (IBM/CORE_FRAC_STEP_ROUTINES.F90:244-448: a face
takes bc where its flag is set).  So after the projection

    div(face) = -dt nlw0            in the outflow cell layer,
    div(face) = O(dt * residual)    everywhere else,

which is the reference's own behaviour: the oracle's chain in the
reference's order shows it, and the GPU's FractionalStep reproduces it.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300.grid import Metrics
from oracle.oracle import Oracle
from tests.test_gpu_rollout import DT, initial_velocity, oracle_rollout, small_channel


def _div(pr, fu, fv, fw):
    n = pr.params
    nx, ny, nz = n.nx - 1, n.ny - 1, n.nz - 1
    mx, my, mz = Metrics(pr.x), Metrics(pr.y), Metrics(pr.z)
    I, J, K = slice(1, nx + 1), slice(1, ny + 1), slice(1, nz + 1)
    d = ((fu[2:nx + 2, J, K] - fu[I, J, K]) * mx.dxinv[I, None, None]
         + (fv[I, 2:ny + 2, K] - fv[I, J, K]) * my.dxinv[None, J, None]
         + (fw[I, J, 2:nz + 2] - fw[I, J, K]) * mz.dxinv[None, None, K])
    return d * (1 - pr.geom.iblank[I, J, K]), (I, J, K)


def test_oracle_chain_divergence_is_the_outflow_term():
    pr = small_channel()
    u0, v0, w0 = initial_velocity(pr)
    cap = {}
    orig = Oracle.solve

    def solve_capture(self, p0=None):
        r = orig(self, p0)
        cap["nlw0"] = r["nlw0"]
        return r

    Oracle.solve = solve_capture
    try:
        ref = oracle_rollout(pr, u0, v0, w0, 2, 2)
    finally:
        Oracle.solve = orig
    div, (I, J, K) = _div(pr, *ref["faces"])
    nlw0 = cap["nlw0"][I, J, K] * (1 - pr.geom.iblank[I, J, K])
    assert np.abs(div[:-1]).max() < 1e-10            # inside: the projection's residual
    assert np.abs(div[-1]).max() > 1e-6              # the outflow layer is not divergence-free
    assert np.abs(div + DT * nlw0).max() < 1e-10     # ... and carries exactly -dt nlw0
    assert np.count_nonzero(nlw0[:-1]) == 0


@pytest.mark.gpu
def test_gpu_rollout_divergence_is_the_outflow_term(gpu_built):
    import torch
    from flow_structure_interaction_fem_ibm_gb300.time_step import FractionalStep
    from tests.test_gpu_rollout import INFLOW, REINV
    pr = small_channel()
    pr.params.precision_mode, pr.params.outer_krylov = 1, 30
    u0, v0, w0 = initial_velocity(pr)
    fs = FractionalStep(pr, DT, REINV, INFLOW, advec_scheme=2).start(u0, v0, w0)
    try:
        for _ in range(2):
            rec = fs.step()
            assert rec["poisson_status"] == 0 and rec["ad_status"] == 0
        got = fs.fields()
        nlw0 = fs.host(fs.nlw0)
        torch.cuda.synchronize()
    finally:
        fs.close()
    div, (I, J, K) = _div(pr, *got["faces"])
    nlw0 = nlw0[I, J, K] * (1 - pr.geom.iblank[I, J, K])
    assert np.abs(div[:-1]).max() < 1e-8
    assert np.abs(div[-1]).max() > 1e-6
    assert np.abs(div + DT * nlw0).max() < 1e-8
