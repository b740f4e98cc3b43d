"""CPU pins of the oracle's set_bc (IBM/CORE_SET_BC.F90:22-377 with
IBM/CORE_SET_OUTER_GHOST.F90:1-63).

* An independent vectorised restatement in numpy gives the same planes,
  ghost layers and correction (the mass-flux sum runs in another order:
  1e-12 relative).
* With set_outflow_area's area and only outer face flags, the corrected
  boundary values carry zero net mass flux (global mass conservation).
* The ghost layers put the boundary value at the face: (u(0) + u(1)) / 2 =
  bcxu(1), and so on.
* A side type the restatement does not cover (user-specified) is refused.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.grid import Metrics
from oracle.oracle import Oracle
from tests.helpers import set_bc_case

ZG = 2


def numpy_set_bc(pr, vel, bc9, val, freq, time, tstart_gust, xout, yout):
    """Vectorised set_bc + enforce_global_mass_consv + set_outer_ghost_vel."""
    p = pr.params
    nx, ny, nz = p.nx, p.ny, p.nz
    nc = (nx - 1, ny - 1, nz - 1)
    pi = 4.0 * np.arctan(1.0)
    xs = (pr.x, pr.y)
    for s in range(6):
        a, hi = s // 2, s % 2
        idx = [slice(0, nx + 1), slice(0, ny + 1), slice(0, nz + 1)]
        idx[a] = nc[a] if hi else 1
        idx = tuple(idx)
        t = p.bc[s]
        for q in range(3):
            out = bc9[3 * q + a]
            cell = vel[q][idx]
            if t == 1:
                out[idx] = val[s, q]
            elif t == ZG:
                out[idx] = cell
            elif t == 3:
                v = val[s, q] * np.sin(2.0 * pi * freq[s, q] * time)
                if s == 1 and q == 0:
                    v = val[s, q] * abs(np.sin(2.0 * pi * freq[s, q] * time)) if time > tstart_gust else 0.0
                out[idx] = v
            elif t == 4:
                out[idx] = 0.0 if q == a else cell
            elif t == 7:
                if q != a:
                    out[idx] = val[s, q]
                elif a == 1:
                    out[idx] = val[s, q] * xs[0][0:nx + 1][:, None] / xout
                else:
                    shape = (ny + 1, 1) if a == 0 else (1, ny + 1)
                    out[idx] = val[s, q] * xs[1][0:ny + 1].reshape(shape) / yout
    corr = 0.0
    if ZG in p.bc:
        mx, my, mz = Metrics(pr.x), Metrics(pr.y), Metrics(pr.z)
        I, J, K = slice(1, nc[0] + 1), slice(1, nc[1] + 1), slice(1, nc[2] + 1)
        dx, dy, dz = mx.dx[I][:, None, None], my.dx[J][None, :, None], mz.dx[K][None, None, :]
        ium, iup, jum, jup, kum, kup = (f[I, J, K].astype(np.float64) for f in pr.geom.flags)
        bu, bv, bw = bc9[0][I, J, K], bc9[4][I, J, K], bc9[8][I, J, K]
        m = (-bu * ium * dy * dz + bu * iup * dy * dz - bv * jum * dx * dz + bv * jup * dx * dz
             - bw * kum * dx * dy + bw * kup * dx * dy) * (1 - pr.geom.iblank[I, J, K])
        corr = -float(m.sum()) / p.outflow_area
        for s in range(6):
            if p.bc[s] != ZG:
                continue
            a, hi = s // 2, s % 2
            idx = [slice(0, nx + 1), slice(0, ny + 1), slice(0, nz + 1)]
            idx[a] = nc[a] if hi else 1
            bc9[4 * a][tuple(idx)] += corr if hi else -corr
    for a, n in enumerate((nx, ny, nz)):
        def sl(i):
            idx = [slice(0, nx + 1), slice(0, ny + 1), slice(0, nz + 1)]
            idx[a] = i
            return tuple(idx)
        for q in range(3):
            vel[q][sl(0)] = 2.0 * bc9[3 * q + a][sl(1)] - vel[q][sl(1)]
            vel[q][sl(n)] = 2.0 * bc9[3 * q + a][sl(n - 1)] - vel[q][sl(n - 1)]
    return corr


CASES = ["dirichlet", "channel", "mixed", "shear_x", "gust_on", "gust_off", "unpaired_zg", "sphere_channel",
         "box2d_channel"]


def boundary_massflux(pr, bc9):
    mx, my, mz = Metrics(pr.x), Metrics(pr.y), Metrics(pr.z)
    p = pr.params
    I, J, K = slice(1, p.nx), slice(1, p.ny), slice(1, p.nz)
    dx, dy, dz = mx.dx[I][:, None, None], my.dx[J][None, :, None], mz.dx[K][None, None, :]
    ium, iup, jum, jup, kum, kup = (f[I, J, K].astype(np.float64) for f in pr.geom.flags)
    bu, bv, bw = bc9[0][I, J, K], bc9[4][I, J, K], bc9[8][I, J, K]
    m = ((iup - ium) * bu * dy * dz + (jup - jum) * bv * dx * dz + (kup - kum) * bw * dx * dy) \
        * (1 - pr.geom.iblank[I, J, K])
    return float(m.sum()), float(np.abs(m).sum())


@pytest.mark.parametrize("case", CASES)
def test_oracle_matches_numpy(case):
    pr, f = set_bc_case(case)
    o = Oracle(pr)
    try:
        vel = [a.copy(order="F") for a in f["vel"]]
        bc9 = [a.copy(order="F") for a in f["bc9"]]
        c_or = o.set_bc(vel, bc9, f["val"], f["freq"], f["time"], f["tstart_gust"], f["xout"], f["yout"])
    finally:
        o.close()
    vel_np = [a.copy(order="F") for a in f["vel"]]
    bc9_np = [a.copy(order="F") for a in f["bc9"]]
    c_np = numpy_set_bc(pr, vel_np, bc9_np, f["val"], f["freq"], f["time"], f["tstart_gust"], f["xout"], f["yout"])
    assert abs(c_or - c_np) <= 1e-12 * max(1.0, abs(c_np))
    for a, b in zip(vel + bc9, vel_np + bc9_np):
        np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 * max(1.0, float(np.abs(b).max())))
    if ZG not in pr.params.bc:
        for a, b in zip(vel + bc9, vel_np + bc9_np):
            np.testing.assert_array_equal(a, b)


@pytest.mark.parametrize("case", ["channel", "mixed", "sphere_channel", "box2d_channel"])
def test_outflow_correction_conserves_mass(case):
    pr, f = set_bc_case(case)
    o = Oracle(pr)
    try:
        vel = [a.copy(order="F") for a in f["vel"]]
        bc9 = [a.copy(order="F") for a in f["bc9"]]
        corr = o.set_bc(vel, bc9, f["val"], f["freq"], f["time"], f["tstart_gust"], f["xout"], f["yout"])
    finally:
        o.close()
    # the uncorrected flux (zero-gradient planes back to their cell values) is not zero ...
    raw = [a.copy(order="F") for a in bc9]
    nc = (pr.params.nx - 1, pr.params.ny - 1, pr.params.nz - 1)
    for s in range(6):
        if pr.params.bc[s] == ZG:
            a, hi = s // 2, s % 2
            idx = [slice(None)] * 3
            idx[a] = nc[a] if hi else 1
            raw[4 * a][tuple(idx)] -= corr if hi else -corr
    m_raw, scale = boundary_massflux(pr, raw)
    assert abs(m_raw) > 1e-6 * scale
    assert corr != 0.0
    # ... and the corrected one is
    m, scale = boundary_massflux(pr, bc9)
    assert abs(m) <= 1e-13 * scale


@pytest.mark.parametrize("case", ["channel", "mixed", "box2d_channel"])
def test_ghost_layers_put_the_boundary_value_on_the_face(case):
    pr, f = set_bc_case(case)
    o = Oracle(pr)
    try:
        vel = [a.copy(order="F") for a in f["vel"]]
        bc9 = [a.copy(order="F") for a in f["bc9"]]
        o.set_bc(vel, bc9, f["val"], f["freq"], f["time"], f["tstart_gust"], f["xout"], f["yout"])
    finally:
        o.close()
    p = pr.params
    n = (p.nx, p.ny, p.nz)
    # interior rows of each plane: the later axes' ghost phases rewrite the ghost rows
    I = [slice(1, p.nx), slice(1, p.ny), slice(1, p.nz)]
    for a in range(3):
        for q in range(3):
            lo = list(I); lo[a] = 0
            l1 = list(I); l1[a] = 1
            hi = list(I); hi[a] = n[a]
            h1 = list(I); h1[a] = n[a] - 1
            u, b = vel[q], bc9[3 * q + a]
            np.testing.assert_allclose(0.5 * (u[tuple(lo)] + u[tuple(l1)]), b[tuple(l1)], rtol=0, atol=1e-14 * 8)
            np.testing.assert_allclose(0.5 * (u[tuple(hi)] + u[tuple(h1)]), b[tuple(h1)], rtol=0, atol=1e-14 * 8)


def test_user_specified_refused():
    pr, f = set_bc_case("dirichlet")
    pr.params.bc = (6, 2, 1, 1, 1, 1)
    o = Oracle(pr)
    try:
        with pytest.raises(ValueError):
            o.set_bc([a.copy(order="F") for a in f["vel"]], [a.copy(order="F") for a in f["bc9"]], f["val"])
    finally:
        o.close()


def test_outflow_area_matches_reference_formula():
    pr, _ = set_bc_case("sphere_channel")
    p = pr.params
    mx, my, mz = Metrics(pr.x), Metrics(pr.y), Metrics(pr.z)
    nxc = p.nx - 1
    area_right = sum(my.dx[j] * mz.dx[k] * (1 - pr.geom.iblank[nxc, j, k])
                     for j in range(1, p.ny) for k in range(1, p.nz))
    assert abs(P.outflow_area(p, pr.x, pr.y, pr.z, pr.geom.iblank) - area_right) <= 1e-14 * area_right


def test_fractional_step_refuses_outflow_with_the_plain_stationary_solve():
    """Zero-gradient outflow with the plain stationary MG form would stall (the
    reference's MG smoother adds nlw, not the outflow term nlw0); FractionalStep
    refuses it before it touches the device."""
    pytest.importorskip("torch")
    from flow_structure_interaction_fem_ibm_gb300.time_step import FractionalStep
    pr = P.channel((24, 16, 16))
    pr.params.precision_mode, pr.params.outer_krylov = 0, 0
    with pytest.raises(ValueError, match="nlw0"):
        FractionalStep(pr, 0.005, 1.0 / 300.0, np.zeros((6, 3)))


def test_channel_builder():
    """The sphere-wake channel: 192 x 128 x 128 cells on [0,6] x [0,4]^2, inflow,
    zero-gradient outflow and symmetry sides, outflow_area the 4 x 4 outflow
    plane (the sphere of diameter 1 at (1.5, 2, 2) does not reach it)."""
    pr = P.channel()
    p = pr.params
    assert (p.nx, p.ny, p.nz) == (193, 129, 129)
    assert tuple(p.bc) == P.CHANNEL_BC
    assert abs(p.outflow_area - 16.0) <= 1e-12
    assert abs(pr.x[p.nx] - 6.0) <= 1e-12 and abs(pr.y[p.ny] - 4.0) <= 1e-12
    g = pr.geom
    assert g.nGhost > 0 and int(g.iblank.sum()) > 0
    # every blanked cell lies inside the sphere's bounding box
    ii, jj, kk = np.nonzero(g.iblank)
    xc = 0.5 * (pr.x[ii] + pr.x[ii + 1])
    assert xc.min() > 0.9 and xc.max() < 2.1
