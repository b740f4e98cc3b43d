"""Kernel-level parity of the CUDA library against the oracle, one reference
operator at a time, through the C ABI (fsi_mg_debug_level_op).

Integer outputs (coarse iblank, face flags) must be bit-exact.  FP64 outputs
of one operator application must agree to 1e-12 relative (the GPU contracts
multiply-adds into FMAs; the oracle does not).  The oracle runs with the GPU's
smoother order (full red-black, iRedBlack = 3) and fresh coarse face flags.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.poisson import PoissonSolver
from oracle.oracle import Oracle
from tests.helpers import sphere_problem

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def cases():
    return [
        ("sphere16_tanh", lambda: sphere_problem(16, stretch=1.5)),
        ("sphere12_unif", lambda: sphere_problem(12, stretch=None)),
        ("box2d_32", lambda: P.box2d(32, seed=9)),
        # long lines: the warp-partition smoother with 2, 4 and 8 rows per lane
        ("box2d_256", lambda: P.box2d(256, seed=9)),
        ("sphere_48x80x160", lambda: P.sphere((48, 80, 160), seed=5, stretch=1.5)),
        # cubic: coarsest levels with two long directions of equal length (S = 2)
        ("sphere48_tanh", lambda: P.sphere(48, seed=6, stretch=1.5)),
        # 256-cell x- and z-lines: the pipelined FP32 sweep in those directions
        ("sphere_256x20x256", lambda: P.sphere((256, 20, 256), seed=7, stretch=1.5)),
        # full 64-cell y-lines and 32-cell z-lines over 64 x-cells (lines of exactly 32 S cells in
        # every direction of a 3D grid)
        ("sphere_64x64x32", lambda: P.sphere((64, 64, 32), seed=8, stretch=1.5)),
    ]


@pytest.fixture(params=cases(), ids=lambda c: c[0])
def pair(request, gpu_built):
    pr = request.param[1]()
    pr.params.iRedBlack = 3
    pr.params.coarse_flag_mode = 1
    o = Oracle(pr)
    g = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    yield pr, o, g
    g.close()
    o.close()


def levels(o, nd):
    for d in range(nd):
        for n in range(1, o.nlev(d) + 1):
            yield d, n


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def test_hierarchy_sizes(pair):
    pr, o, g = pair
    nd = pr.params.ndim
    for d in range(nd):
        assert g.level_count(d) == o.nlev(d)
        for n in range(1, o.nlev(d) + 1):
            assert g.level_size(d, n) == o.level_size(d, n)


def test_coarse_iblank_bit_exact(pair):
    pr, o, g = pair
    for d, n in levels(o, pr.params.ndim):
        if n == 1:
            continue
        ref = o.coarse_iblank(d, n)
        got = np.zeros(ref.shape, np.int8, order="F")
        g.debug_op(3, d, n, got)
        assert np.array_equal(got, ref), (d, n)


def test_face_flags_bit_exact(pair):
    pr, o, g = pair
    sh = pr.shape
    for d, n in levels(o, pr.params.ndim):
        ref = o.level_flags(d, n)
        buf = np.zeros(6 * int(np.prod(sh)), np.int8)
        g.debug_op(4, d, n, buf)
        got = [buf[s * buf.size // 6:(s + 1) * buf.size // 6].reshape(sh, order="F") for s in range(6)]
        m = list(o.level_shape(d, n))
        sl = tuple(slice(1, mm - 1) for mm in m)
        for s in range(6):
            if pr.params.ndim == 2 and s >= 4:
                continue
            assert np.array_equal(got[s][sl], ref[s][sl]), (d, n, s)


def test_line_smoother_sweep(pair):
    """One MG_itsolv (x, y, z line sweeps, red then black) at every level."""
    pr, o, g = pair
    rng = np.random.default_rng(1)
    for d, n in levels(o, pr.params.ndim):
        sh = o.level_shape(d, n)
        v0 = np.asfortranarray(rng.standard_normal(sh))
        r = np.asfortranarray(rng.standard_normal(sh))
        ref = o.itsolv(d, n, v0.copy(order="F"), r)
        got = v0.copy(order="F")
        g.debug_op(0, d, n, got, r)
        assert rel(got, ref) < RTOL, (d, n, rel(got, ref))


def test_line_smoother_sweep_partition_fp64(pair):
    """The same sweep through the warp-per-line partition solver in FP64 (a
    mixed-form handle keeps no factored FP64 tables, so its FP64 sweeps take
    that kernel): 1e-12 against the oracle."""
    pr, o, g = pair
    import copy
    q = copy.deepcopy(pr.params)
    q.precision_mode = 1
    gm = PoissonSolver(q, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        rng = np.random.default_rng(11)
        for d, n in levels(o, pr.params.ndim):
            sh = o.level_shape(d, n)
            v0 = np.asfortranarray(rng.standard_normal(sh))
            r = np.asfortranarray(rng.standard_normal(sh))
            ref = o.itsolv(d, n, v0.copy(order="F"), r)
            got = v0.copy(order="F")
            gm.debug_op(0, d, n, got, r)
            assert rel(got, ref) < RTOL, (d, n, rel(got, ref))
    finally:
        gm.close()


def test_line_smoother_sweep_fp32(pair):
    """One MG_itsolv of the mixed form's FP32 smoother at every level against
    the FP64 oracle on the same FP32-rounded inputs: the sweep's rounding
    only (2e-5 relative to the largest value)."""
    pr, o, g = pair
    rng = np.random.default_rng(12)
    for d, n in levels(o, pr.params.ndim):
        sh = o.level_shape(d, n)
        v0 = np.asfortranarray(rng.standard_normal(sh).astype(np.float32).astype(np.float64))
        r = np.asfortranarray(rng.standard_normal(sh).astype(np.float32).astype(np.float64))
        ref = o.itsolv(d, n, v0.copy(order="F"), r)
        got = v0.copy(order="F")
        g.debug_op(7, d, n, got, r)
        assert rel(got, ref) < 2e-5, (d, n, rel(got, ref))


def test_residual_restriction(pair):
    pr, o, g = pair
    rng = np.random.default_rng(2)
    for d, n in levels(o, pr.params.ndim):
        if n == o.nlev(d):
            continue
        sh = o.level_shape(d, n)
        v = np.asfortranarray(rng.standard_normal(sh))
        r = np.asfortranarray(rng.standard_normal(sh))
        ref = o.restrict(d, n, o.residual(d, n, v, r))
        got = np.zeros(ref.shape, order="F")
        g.debug_op(1, d, n, v, r, got)
        sl = tuple(slice(1, m - 1) for m in ref.shape)
        assert rel(got[sl], ref[sl]) < RTOL, (d, n)


def test_prolongation_correction(pair):
    pr, o, g = pair
    rng = np.random.default_rng(3)
    for d, n in levels(o, pr.params.ndim):
        if n == o.nlev(d):
            continue
        phi = np.asfortranarray(rng.standard_normal(o.level_shape(d, n + 1)))
        v = np.asfortranarray(rng.standard_normal(o.level_shape(d, n)))
        corr = o.prolong(d, n, phi)
        ib = o.coarse_iblank(d, n) if n > 1 else pr.geom.iblank[:pr.params.nx + 1, :pr.params.ny + 1, :pr.params.nz + 1]
        ref = v + corr * (1 - ib)
        got = v.copy(order="F")
        g.debug_op(2, d, n, phi, got)
        sl = tuple(slice(1, m - 1) for m in ref.shape)
        assert rel(got[sl], ref[sl]) < RTOL, (d, n)


def test_outer_ghost_layer(pair):
    pr, o, g = pair
    rng = np.random.default_rng(4)
    sh = o.level_shape(0, 1)
    v = np.asfortranarray(rng.standard_normal(sh))
    ref = o.outer_ghost(v.copy(order="F"))
    got = v.copy(order="F")
    g.debug_op(6, 0, 1, got)
    assert np.array_equal(got, ref)


def test_ghost_rows_fixed_point(pair):
    """Jacobi on the GPU and Gauss-Seidel in the reference converge to the same
    ghost values within restol_ad."""
    pr, o, g = pair
    if pr.geom.nGhost == 0:
        pytest.skip("no body")
    rng = np.random.default_rng(5)
    sh = o.level_shape(0, 1)
    v = np.asfortranarray(rng.standard_normal(sh))
    ref = v.copy(order="F")
    o.ghost_update(ref)
    got = v.copy(order="F")
    iters = np.zeros(1, np.int32)
    g.debug_op(5, 0, 1, got, iters)
    assert iters[0] >= 1
    assert np.abs(got - ref).max() < 1e-11


def test_calc_residual_and_location(pair):
    pr, o, g = pair
    rng = np.random.default_rng(6)
    p = np.asfortranarray(rng.standard_normal(pr.shape))
    m_ref, loc_ref = o.calc_residual(p, pr.nlu0)
    m, loc = g.calc_residual(p, pr.nlu0)
    assert abs(m - m_ref) <= 1e-12 * m_ref
    assert loc == loc_ref


def test_subtract_average(pair):
    pr, o, g = pair
    rng = np.random.default_rng(7)
    p = np.asfortranarray(rng.standard_normal(pr.shape))
    ref = o.subtract_average(p.copy(order="F"))
    got = g.subtracting_average_pressure(p.copy(order="F"))
    assert np.abs(got - ref).max() < 1e-13


def test_mg_solver_one_cycle(pair):
    """One full MG_Solver call (x, y, z semi-coarsening cycles) from a random
    iterate: same schedule, same red-black order -> same iterate."""
    pr, o, g = pair
    rng = np.random.default_rng(8)
    p = np.asfortranarray(rng.standard_normal(pr.shape))
    o.subtract_average(p)
    ref = o.mg_solver(p.copy(order="F"), pr.nlu0)
    got = p.copy(order="F")
    g.MG_Solver(got, pr.nlu0)
    I = tuple(slice(0, m) for m in (pr.params.nx + 1, pr.params.ny + 1, pr.params.nz + 1))
    assert rel(got[I], ref[I]) < 1e-10


def test_subtract_average_fresh_cells(pair):
    """Mean removal with the fresh cells of a moving body, GPU vs oracle."""
    from tests.helpers import fresh_shell
    pr, o, g = pair
    if pr.geom.nGhost == 0:
        pytest.skip("no body")
    fresh = fresh_shell(pr)
    rng = np.random.default_rng(17)
    p = np.asfortranarray(rng.standard_normal(pr.shape))
    o.set_fresh(fresh)
    g.set_fresh_cells(fresh)
    try:
        ref = o.subtract_average(p.copy(order="F"))
        got = g.subtracting_average_pressure(p.copy(order="F"))
        assert np.abs(got - ref).max() < 1e-13
    finally:
        o.set_fresh(None)
        g.set_fresh_cells(None)


@pytest.mark.parametrize("omega", [0.8, 1.3])
def test_line_smoother_sweeps_with_relaxation(omega, gpu_built):
    """One MG_itsolv at every level with omega != 1 (the relaxed store
    var (1 - omega) + omega sol of the line kernels): FP64 within 1e-12 and the
    FP32 smoother within its rounding of the FP64 oracle."""
    pr = P.sphere((64, 64, 32), seed=8, stretch=1.5)
    pr.params.iRedBlack, pr.params.coarse_flag_mode, pr.params.omega = 3, 1, omega
    o = Oracle(pr)
    g = PoissonSolver(pr.params, pr.x, pr.y, pr.z).set_boundary(pr.geom)
    try:
        rng = np.random.default_rng(14)
        for d, n in levels(o, pr.params.ndim):
            sh = o.level_shape(d, n)
            v0 = np.asfortranarray(rng.standard_normal(sh).astype(np.float32).astype(np.float64))
            r = np.asfortranarray(rng.standard_normal(sh).astype(np.float32).astype(np.float64))
            ref = o.itsolv(d, n, v0.copy(order="F"), r)
            for op, tol in ((0, RTOL), (7, 2e-5)):
                got = v0.copy(order="F")
                g.debug_op(op, d, n, got, r)
                assert rel(got, ref) < tol, (op, d, n, rel(got, ref))
    finally:
        g.close()
        o.close()
