"""Known-answer checks of the oracle in 3D, on stretched grids and with a
ghost-cell body: the cases the reference's own Poisson_Tester
(IBM/CORE_POISSON.F90:1386-1790, 2D, uniform, no body) does not reach.

* Stretched metrics: on [0,1]^3 tanh-stretched toward the centre (beta 1.5,
  the workloads' grid), all-Neumann, nlu0 = -3 pi^2 cos(pi x) cos(pi y)
  cos(pi z) at the cell centres.  The exact answer is cos cos cos (zero normal
  derivative on every wall), and the MG solution must converge to it at second
  order, as Poisson_Tester's calc_grid_convergence_test checks in 2D
  (IBM/CORE_POISSON.F90:1616-1677).  A wrong metric product (dcinv, dinv of
  IBM/CORE_MG.F90:148-266, 1950-1962) or a wrong finest-level boundary row
  breaks the order or the limit.
* Ghost-cell rows: for the angular field p = (x - c)_1 / |x - c| around the
  sphere's centre c, the normal derivative vanishes on the sphere, and the
  ghost, its body intercept and its image point lie on one ray from c.  So the
  Neumann ghost rows (IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:250-384 with the
  coeffGCMN of IBM/GCM_SET_BOUNDARY.F90:307-494) must return p at the ghost
  centre up to the interpolation error of the rows: measured on the tanh
  grid, the rms error over the ghosts falls 2.7x and 3.0x per halving of h
  (16 -> 32 -> 64 cells), the max error 2.1x and 2.0x (first order in the
  max norm: the rows couple ghosts to ghosts, which spreads the trilinear
  error).
* Constant and linear fields through the whole solve: nlu0 = A p for a field p
  built independently of the oracle's operator (the reference's 7-point
  stencil with face flags, written out here in numpy) is solved back to p.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.grid import Metrics, make_grid
from oracle.oracle import Oracle


def _cos3d(n, stretch=1.5):
    p = P.default_params(3, n, n, n, body=False, restol_Poisson=1e-11)
    x, y, z = make_grid(p.nx, p.ny, p.nz, "tanh", beta=stretch)
    geom = P.empty_geometry(p)
    mx, my, mz = Metrics(x), Metrics(y), Metrics(z)
    X, Y, Z = np.meshgrid(mx.xc[1:n + 1], my.xc[1:n + 1], mz.xc[1:n + 1], indexing="ij")
    exact = np.cos(np.pi * X) * np.cos(np.pi * Y) * np.cos(np.pi * Z)
    nlu0 = np.zeros(P.full_shape(p), order="F")
    nlu0[1:n + 1, 1:n + 1, 1:n + 1] = -3.0 * np.pi ** 2 * exact
    # the discrete sum of the sampled source is not exactly zero: remove its
    # volume-weighted mean (the Neumann problem's compatibility condition)
    P.remove_fluid_mean(p, x, y, z, nlu0, geom.iblank)
    vol = mx.dx[1:n + 1, None, None] * my.dx[None, 1:n + 1, None] * mz.dx[None, None, 1:n + 1]
    return P.Problem(p, x, y, z, geom, nlu0, name=f"cos3d_{n}"), exact, vol


def _cos3d_error(n):
    pr, exact, vol = _cos3d(n)
    pr.params.restol_Poisson = 1e-11 * float(np.abs(pr.nlu0).max())
    o = Oracle(pr)
    res = o.solve()
    o.close()
    assert res["status"] == 0
    d = res["p"][1:n + 1, 1:n + 1, 1:n + 1] - exact
    d -= (d * vol).sum() / vol.sum()
    return float(np.sqrt((d ** 2 * vol).sum() / vol.sum()))


def test_stretched_3d_known_answer_second_order():
    """Measured: volume-weighted L2 errors 8.07e-3, 2.40e-3, 6.44e-4 at 16^3,
    32^3, 64^3 (ratios 3.36 and 3.74, approaching 4 from below as the
    stretched grid resolves the field)."""
    e16, e32, e64 = (_cos3d_error(n) for n in (16, 32, 64))
    assert e16 < 2e-2
    assert 3.0 < e16 / e32 < 4.5, (e16, e32)
    assert 3.5 < e32 / e64 < 4.3, (e32, e64)
    assert e32 / e64 > e16 / e32


def _angular_ghost_error(n):
    pr = P.sphere(n, seed=2, stretch=1.5)
    g = pr.geom
    o = Oracle(pr, restol_ad=1e-14, iterMax_ad=500)
    mx, my, mz = Metrics(pr.x), Metrics(pr.y), Metrics(pr.z)
    X, Y, Z = np.meshgrid(mx.xc, my.xc, mz.xc, indexing="ij")
    r = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2)
    field = (X - 0.5) / r
    v = np.asfortranarray(field[: pr.params.nx + 1, : pr.params.ny + 1, : pr.params.nz + 1])
    got = v.copy(order="F")
    got[g.iG, g.jG, g.kG] = 0.0   # the ghost values come from the rows alone
    o.ghost_update(got)
    o.close()
    err = np.abs(got[g.iG, g.jG, g.kG] - v[g.iG, g.jG, g.kG])
    return float(err.max()), float(np.sqrt((err ** 2).mean())), g.nGhost


def test_ghost_rows_reproduce_a_field_with_zero_normal_derivative():
    m16, r16, n16 = _angular_ghost_error(16)
    m32, r32, n32 = _angular_ghost_error(32)
    m64, r64, n64 = _angular_ghost_error(64)
    assert n16 < n32 < n64
    assert m16 < 0.02
    for (ma, ra), (mb, rb) in (((m16, r16), (m32, r32)), ((m32, r32), (m64, r64))):
        assert mb < ma / 1.8, (ma, mb)   # at least first order in the max norm
        assert rb < ra / 2.5, (ra, rb)   # better than order 1.3 in rms


def _stencil_apply(pr, p):
    """nlu0 = A p on fluid cells, the 7-point operator of MG_Residual
    (IBM/CORE_MG.F90:2316-2375) with the face flags of the geometry, written
    independently of the oracle."""
    prm = pr.params
    n0, n1, n2 = prm.nx - 1, prm.ny - 1, prm.nz - 1
    ms = [Metrics(c) for c in (pr.x, pr.y, pr.z)]
    fm, fp = pr.geom.flags[0::2], pr.geom.flags[1::2]   # ium, iup, jum, jup, kum, kup
    out = np.zeros(pr.shape, order="F")
    I = (slice(1, n0 + 1), slice(1, n1 + 1), slice(1, n2 + 1))
    nd = 3 if prm.ndim == 3 else 2
    acc = np.zeros((n0, n1, n2))
    for a in range(nd):
        m = ms[a]
        n = (n0, n1, n2)[a]
        sh = [1, 1, 1]; sh[a] = n
        cm = (m.dxcinv[1:n + 1] * m.dxinv[1:n + 1]).reshape(sh)
        cp = (m.dxcinv[2:n + 2] * m.dxinv[1:n + 1]).reshape(sh)
        lo = [slice(1, n0 + 1), slice(1, n1 + 1), slice(1, n2 + 1)]
        up, dn = list(lo), list(lo)
        up[a] = slice(2, n + 2); dn[a] = slice(0, n)
        am = cm * (1 - fm[a][I])
        ap = cp * (1 - fp[a][I])
        acc += ap * (p[tuple(up)] - p[I]) + am * (p[tuple(dn)] - p[I])
    out[I] = acc * (1 - pr.geom.iblank[I])
    return out


@pytest.mark.parametrize("kind", ["constant", "bilinear"])
def test_solve_recovers_a_manufactured_field(kind):
    """f = A p computed here, then solved by the oracle from p = 0, gives back
    p up to the Neumann constant (constant p: f = 0; bilinear p: a non-trivial
    right-hand side, compatible by construction because the Neumann faces
    carry no flux, whose solution is known without the oracle)."""
    pr = P.box3d((10, 12, 14), seed=3, stretch=1.5)
    prm = pr.params
    n0, n1, n2 = prm.nx - 1, prm.ny - 1, prm.nz - 1
    mx, my, mz = Metrics(pr.x), Metrics(pr.y), Metrics(pr.z)
    X, Y, Z = np.meshgrid(mx.xc, my.xc, mz.xc, indexing="ij")
    if kind == "constant":
        p = np.full(pr.shape, 2.5)
    else:
        p = 1.0 + 0.3 * X - 0.7 * Y + 0.2 * Z + 0.5 * X * Y
    p = np.asfortranarray(p)
    # Neumann outer ghost layer (set_outer_ghost_pres, IBM/CORE_SET_OUTER_GHOST.F90:66-213)
    p[0], p[n0 + 1] = p[1], p[n0]
    p[:, 0], p[:, n1 + 1] = p[:, 1], p[:, n1]
    p[:, :, 0], p[:, :, n2 + 1] = p[:, :, 1], p[:, :, n2]
    f = _stencil_apply(pr, p)
    pr.nlu0 = f
    prm.restol_Poisson = 1e-13 * max(float(np.abs(f).max()), 1.0)
    prm.iterMax_Poisson = 400
    res = Oracle(pr).solve()
    I = (slice(1, n0 + 1), slice(1, n1 + 1), slice(1, n2 + 1))
    vol = mx.dx[1:n0 + 1, None, None] * my.dx[None, 1:n1 + 1, None] * mz.dx[None, None, 1:n2 + 1]
    a = res["p"][I] - (res["p"][I] * vol).sum() / vol.sum()
    b = p[I] - (p[I] * vol).sum() / vol.sum()
    assert res["status"] == 0
    assert np.abs(a - b).max() <= 1e-9 * max(np.abs(b).max(), 1.0)
