"""GPU parity of fsi_mg_set_bc (set_bc's outer sides, enforce_global_mass_consv
and set_outer_ghost_vel; IBM/CORE_SET_BC.F90:22-377,
IBM/CORE_SET_OUTER_GHOST.F90:1-63) with the oracle, through the C ABI on
device arrays.

Whole arrays are compared (u, v, w and the nine bc arrays), so entries the
routine must not touch are checked too.  Without zero-gradient sides every
value is a copy, a product or 2 b - u and must match bit for bit; with them the
mass-flux sum runs in another order on the GPU (CTA partial sums), so the
corrected planes and the ghost layers built from them agree to 1e-12 of the
largest value.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300.poisson import FsiMgError, PoissonSolver
from oracle.oracle import Oracle
from tests.helpers import SET_BC_TYPES, set_bc_case

pytestmark = pytest.mark.gpu

ZG = 2


def _dev(a):
    import torch
    return torch.from_numpy(np.ascontiguousarray(np.asarray(a, dtype=np.float64).transpose())).cuda()


def _host(t):
    return np.asfortranarray(t.cpu().numpy().transpose())


def _run_both(pr, f):
    o = Oracle(pr)
    g = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        vel = [a.copy(order="F") for a in f["vel"]]
        bc9 = [a.copy(order="F") for a in f["bc9"]]
        c_or = o.set_bc(vel, bc9, f["val"], f["freq"], f["time"], f["tstart_gust"], f["xout"], f["yout"])
        dvel = [_dev(a) for a in f["vel"]]
        dbc = [_dev(a) for a in f["bc9"]]
        c_gpu = g.set_bc([t.data_ptr() for t in dvel], [t.data_ptr() for t in dbc], f["val"], f["freq"], f["time"],
                         f["tstart_gust"], f["xout"], f["yout"])
        return (vel + bc9, c_or), ([_host(t) for t in dvel + dbc], c_gpu)
    finally:
        g.close()
        o.close()


@pytest.mark.parametrize("case", sorted(SET_BC_TYPES))
def test_set_bc_matches_oracle(gpu_built, case):
    pr, f = set_bc_case(case)
    (ref, c_or), (out, c_gpu) = _run_both(pr, f)
    names = ["u", "v", "w", "bcxu", "bcyu", "bczu", "bcxv", "bcyv", "bczv", "bcxw", "bcyw", "bczw"]
    if ZG in pr.params.bc:
        assert c_or != 0.0
        assert abs(c_gpu - c_or) <= 1e-12 * abs(c_or)
        for nm, a, b in zip(names, out, ref):
            tol = 1e-12 * max(1.0, float(np.abs(b).max()))
            assert float(np.abs(a - b).max()) <= tol, nm
    else:
        assert c_gpu == 0.0 and c_or == 0.0
        for nm, a, b in zip(names, out, ref):
            np.testing.assert_array_equal(a, b, err_msg=nm)


def test_set_bc_rejects_user_specified(gpu_built):
    """User-specified (Blasius) sides are refused before any launch: the arrays stay as they were."""
    pr, f = set_bc_case("channel")
    dvel = [_dev(a) for a in f["vel"]]
    dbc = [_dev(a) for a in f["bc9"]]
    before = [t.clone() for t in dvel + dbc]
    pr.params.bc = (6, 2, 4, 4, 4, 4)
    g = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        with pytest.raises(FsiMgError, match="user-specified"):
            g.set_bc([t.data_ptr() for t in dvel], [t.data_ptr() for t in dbc], f["val"])
    finally:
        g.close()
    for t, b in zip(dvel + dbc, before):
        assert bool((t == b).all())
