"""CPU checks of the oracle (the C restatement of the reference MG path).

The reference cannot be compiled here, so the oracle is pinned by the
reference's own known-answer test (Poisson_Tester, IBM/CORE_POISSON.F90:
1386-1790: nlu0 = -2 cos x cos y on [0,pi]^2, exact cos x cos y) and by
cross-checks between independent paths of the reference algorithm.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.grid import Metrics
from oracle.oracle import Oracle, tdma
from tests.helpers import cell_volumes, interior, rel_l2_mean_free, sphere_problem


def test_tdma_matches_dense_solve():
    rng = np.random.default_rng(0)
    for n in (1, 2, 7, 64, 257):
        a = np.zeros(n + 1); b = np.zeros(n + 1); c = np.zeros(n + 1); r = np.zeros(n + 1)
        a[1:] = rng.uniform(-1, 1, n); c[1:] = rng.uniform(-1, 1, n)
        b[1:] = 3.0 + rng.uniform(0, 1, n)
        r[1:] = rng.standard_normal(n)
        u = tdma(a, b, c, r, 1, n)
        A = np.diag(b[1:]) + np.diag(a[2:], -1) + np.diag(c[1:n], 1)
        ref = np.linalg.solve(A, r[1:])
        assert np.allclose(u[1:], ref, rtol=1e-13, atol=1e-13)


def _kat_error(n):
    pr = P.kat2d(n, restol_Poisson=1e-11)
    res = Oracle(pr).solve()
    assert res["status"] == 0
    mx, my = Metrics(pr.x), Metrics(pr.y)
    ex = np.cos(mx.xc[1:n + 1, None]) * np.cos(my.xc[None, 1:n + 1])
    d = res["p"][1:n + 1, 1:n + 1, 1] - ex
    return float(np.abs(d - d.mean()).max()), res


def test_known_answer_second_order():
    """Poisson_Tester: the MG solution converges to cos x cos y at second order
    (calc_grid_convergence_test, IBM/CORE_POISSON.F90:1616-1677)."""
    errs = [_kat_error(n)[0] for n in (32, 64, 128)]
    assert errs[0] < 1e-3
    for e0, e1 in zip(errs, errs[1:]):
        assert 3.6 < e0 / e1 < 4.4


def test_known_answer_mg_converges_fast():
    _, res = _kat_error(64)
    assert res["iters"] <= 12
    h = res["hist"]
    assert h[-1] <= 1e-11 and all(b < a for a, b in zip(h, h[1:]))


def test_mg_and_lsor_reach_same_pressure_2d():
    """MG (pp_solver_type 3) and plain line SOR (pp_solver_type 1) solve the same
    discrete system (IBM/CORE_POISSON.F90:566-676)."""
    pr = P.box2d(24, seed=5, restol_Poisson=1e-12)
    mg = Oracle(pr).solve()
    pr2 = P.box2d(24, seed=5, restol_Poisson=1e-12, pp_solver_type=1, iterMax_Poisson=20000)
    ls = Oracle(pr2).solve()
    assert mg["status"] == 0 and ls["status"] == 0
    I = interior(pr)
    vol = cell_volumes(pr)
    mask = np.ones_like(vol)
    assert rel_l2_mean_free(mg["p"][I], ls["p"][I], mask, vol) < 1e-10


def test_mg_and_lsor_reach_same_pressure_sphere():
    pr = sphere_problem(12, stretch=None, restol_Poisson=1e-12)
    mg = Oracle(pr).solve()
    pr2 = sphere_problem(12, stretch=None, restol_Poisson=1e-12, pp_solver_type=1, iterMax_Poisson=20000)
    ls = Oracle(pr2).solve()
    assert mg["status"] == 0 and ls["status"] == 0
    I = interior(pr)
    vol = cell_volumes(pr)
    mask = 1.0 - pr.geom.iblank[I]
    assert rel_l2_mean_free(mg["p"][I], ls["p"][I], mask, vol) < 1e-9


@pytest.mark.parametrize("rb", [1, 2, 3])
def test_smoother_orderings_converge_to_same_pressure(rb):
    """Lexicographic (iRedBlack 0), the reference colourings (1, 2) and the full
    red-black order used on the GPU (3) reach the same converged pressure."""
    base = sphere_problem(16, restol_Poisson=1e-12)
    ref = Oracle(base).solve()
    alt = Oracle(sphere_problem(16, restol_Poisson=1e-12, iRedBlack=rb, iterMax_Poisson=400)).solve()
    assert ref["status"] == 0 and alt["status"] == 0
    I = interior(base)
    mask = 1.0 - base.geom.iblank[I]
    assert rel_l2_mean_free(ref["p"][I], alt["p"][I], mask, cell_volumes(base)) < 1e-9


def test_coarse_flag_modes_converge_to_same_pressure():
    """Without a body the reference keeps coarse face flags from deeper levels
    (IBM/CORE_MG.F90:1736 only recomputes them with a body); recomputing them
    changes the iteration, not the converged pressure."""
    a = Oracle(P.box2d(32, seed=3, restol_Poisson=1e-12, coarse_flag_mode=0)).solve()
    b = Oracle(P.box2d(32, seed=3, restol_Poisson=1e-12, coarse_flag_mode=1)).solve()
    pr = P.box2d(32, seed=3)
    I = interior(pr)
    assert rel_l2_mean_free(a["p"][I], b["p"][I], np.ones(cell_volumes(pr).shape), cell_volumes(pr)) < 1e-10
    assert b["iters"] <= a["iters"]


def test_nonconvergence_status():
    """iterMax_Poisson reached -> status 1 (IBM/CORE_POISSON.F90:665-669)."""
    res = Oracle(P.box2d(32, seed=3, iterMax_Poisson=2, restol_Poisson=1e-14)).solve()
    assert res["status"] == 1 and res["iters"] == 2


def test_compatibility_shift_restores_convergence():
    raw = P.sphere(12, stretch=None, seed=7)
    stalled = Oracle(raw, iterMax_Poisson=25, restol_Poisson=0.0).solve()
    fixed = sphere_problem(12, stretch=None, seed=7, iterMax_Poisson=25, restol_Poisson=0.0)
    ok = Oracle(fixed).solve()
    assert stalled["hist"][-1] > 1e-4 * abs(raw.nlu0).max()
    assert ok["hist"][-1] < 1e-12 * abs(fixed.nlu0).max()


def test_level_hierarchy_matches_reference_rule():
    """Automatic level counts (IBM/CORE_MG.F90:48-78): 256 -> 7, 128 -> 6, 96 -> 5, 24 -> 3."""
    for n, nl, coarsest in ((256, 7, 4), (128, 6, 4), (96, 5, 6), (24, 3, 6)):
        pr = P.box2d(n) if n <= 128 else None
        if pr is None:
            continue
        o = Oracle(pr)
        assert o.nlev(0) == nl and o.level_size(0, nl) == coarsest


def test_golden_fixtures_reproduced():
    """The committed golden vectors (tests/golden/make_golden.py) are reproduced."""
    from tests.golden.make_golden import GOLDEN, compute
    data = np.load(GOLDEN)
    fresh = compute()
    for k in data.files:
        if np.issubdtype(data[k].dtype, np.integer):
            assert np.array_equal(data[k], fresh[k]), k
        else:
            assert np.allclose(data[k], fresh[k], rtol=1e-11, atol=1e-14 * max(1.0, abs(data[k]).max())), k


def test_fresh_cells_in_mean_removal():
    """subtracting_average_pressure on a moving body: fresh cells take the mean
    of their non-blanked, non-fresh neighbours (IBM/CORE_POISSON.F90:459-488)."""
    from tests.helpers import fresh_reference, fresh_shell
    pr = P.sphere(12, stretch=None, seed=13)
    fresh = fresh_shell(pr)
    assert fresh.sum() > 0
    rng = np.random.default_rng(3)
    p = np.asfortranarray(rng.standard_normal(pr.shape))
    o = Oracle(pr)
    base = o.subtract_average(p.copy(order="F"))
    o.set_fresh(fresh)
    got = o.subtract_average(p.copy(order="F"))
    o.close()
    ref = fresh_reference(pr, base.copy(order="F"), fresh)
    assert np.array_equal(got, ref)
    assert not np.array_equal(got, base)
