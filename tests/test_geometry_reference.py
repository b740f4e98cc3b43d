"""The product geometry (csrc/geometry.cpp, through problem.body_geometry)
against the geometry oracle (oracle/geom_oracle.c), which restates the
reference's own rules in its loop order: inward element normals
(IBM/BOUNDARY_SET_ARCLENGTH_NORM.F90:69-165, 200-320), iblank by the band and
dot-normal fill (IBM/BOUNDARY_IBLANK_FAST.F90:2-1024), the ghost list and
image-point coefficients (IBM/GCM_SET_BOUNDARY.F90:2-494) with its body
intercepts (IBM/GCM_INTERCEPT_KERNELS_UNSTRUC.F90:26-398).

On every sphere workload of the benchmarks and on a non-convex torus,
iblank, the ghost list, the body intercepts, image points, probe lengths and
stencil cells are identical bit for bit.  The interpolation weights differ only by the rounding of the
reference's global-coordinate Vandermonde systems (the product solves the
same systems in stencil-local coordinates): at most 2.2e-8 at 256^3, where
the reference-order weights of a constant miss 1 by 4e-8 and the product's
by 1e-15.
"""
import numpy as np
import pytest

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.grid import Metrics, make_grid
from oracle.geom import lib, reference_geometry

INC = np.array([[0, 0, 0], [0, 1, 0], [1, 1, 0], [1, 0, 0], [0, 0, 1], [0, 1, 1], [1, 1, 1], [1, 0, 1]])

# cells, grid, lengths, sphere centre, radius, weight tolerance
CASES = {
    "sphere_32_tanh": ((32, 32, 32), "tanh", (1, 1, 1), (0.5, 0.5, 0.5), 0.15, 1e-10),
    "sphere_64_tanh": ((64, 64, 64), "tanh", (1, 1, 1), (0.5, 0.5, 0.5), 0.15, 1e-9),
    "channel_24x16x16": ((24, 16, 16), "uniform", (6, 4, 4), (1.5, 2, 2), 0.5, 1e-11),
    "sphere_128_tanh": ((128, 128, 128), "tanh", (1, 1, 1), (0.5, 0.5, 0.5), 0.15, 1e-8),
    "sphere_256_tanh": ((256, 256, 256), "tanh", (1, 1, 1), (0.5, 0.5, 0.5), 0.15, 5e-8),
    "channel_192x128x128": ((192, 128, 128), "uniform", (6, 4, 4), (1.5, 2, 2), 0.5, 1e-9),
}


def _both(cells, kind, lengths, centre, radius, tris_inward=False):
    p = P.default_params(3, *cells, body=True)
    x, y, z = make_grid(p.nx, p.ny, p.nz, kind, beta=1.5, lengths=lengths)
    v, t = P.icosphere(4, radius, centre)
    if tris_inward:
        t = t.reshape(-1, 3)[:, [0, 2, 1]].ravel().copy()
    g = P.body_geometry(p, x, y, z, v, t)
    outside = np.asarray(centre) + 2.0 * np.asarray(lengths, dtype=float)
    r = reference_geometry(p.nx, p.ny, p.nz, x, y, z, v, t, outside)
    return p, (x, y, z), (v, t), g, r


def _self_rows(g):
    m = np.zeros((8, g.nGhost), bool)
    for n in range(g.nGhost):
        cells = np.array([g.iCI[n], g.jCI[n], g.kCI[n]]) + INC
        m[:, n] = (cells == [g.iG[n], g.jG[n], g.kG[n]]).all(axis=1)
    return m


@pytest.mark.parametrize("case", list(CASES))
def test_product_geometry_is_the_reference_geometry(case):
    cells, kind, lengths, centre, radius, wtol = CASES[case]
    p, _, _, g, r = _both(cells, kind, lengths, centre, radius)
    I = (slice(1, p.nx), slice(1, p.ny), slice(1, p.nz))
    assert r.flipped                                  # the icosphere is written outward
    assert np.array_equal(g.iblank[I], r.iblank[I])
    assert np.array_equal(g.ghost[I], r.ghost[I])
    assert g.nGhost == r.nGhost > 0
    for a, b in ((g.iG, r.iG), (g.jG, r.jG), (g.kG, r.kG), (g.iCI, r.iCI), (g.jCI, r.jCI), (g.kCI, r.kCI)):
        assert np.array_equal(a, b)
    assert np.array_equal(g.xBI, r.xBI)
    assert np.array_equal(g.xIP, r.xIP)
    assert np.array_equal(g.probe, r.probe)
    # weights: the ghost's own row multiplies uNormal = 0 (IBM/GCM_GHOSTCELL_VEL_UPDATE_UNSTRUC.F90:
    # 250-384) and is left out; the others agree to the reference's rounding
    own = _self_rows(g)
    assert np.abs(g.coeff[~own] - r.coeffN[~own]).max() <= wtol
    assert np.abs(g.coeffD - r.coeffD).max() <= 2 * wtol
    # a constant is reproduced to rounding by the product's weights
    ones = np.where(own, 0.0, g.coeff).sum(axis=0)
    assert np.abs(ones - 1.0).max() <= 1e-13


def _torus(R=0.25, r=0.1, nu=64, nv=24, centre=(0.5, 0.5, 0.5), tilt=0.3):
    """A closed torus about a tilted axis, written outward: a non-convex body."""
    u = 2 * np.pi * np.arange(nu) / nu
    w = 2 * np.pi * np.arange(nv) / nv
    U, W = np.meshgrid(u, w, indexing="ij")
    pts = np.stack([((R + r * np.cos(W)) * np.cos(U)).ravel(), ((R + r * np.cos(W)) * np.sin(U)).ravel(),
                    (r * np.sin(W)).ravel()], 1)
    c, s_ = np.cos(tilt), np.sin(tilt)
    pts = pts @ np.array([[1, 0, 0], [0, c, -s_], [0, s_, c]]).T + np.asarray(centre)
    at = lambda a, b: (a % nu) * nv + (b % nv)
    tris = []
    for a in range(nu):
        for b in range(nv):
            tris += [(at(a, b), at(a + 1, b), at(a + 1, b + 1)), (at(a, b), at(a + 1, b + 1), at(a, b + 1))]
    T = np.array(tris, np.int32)
    if np.einsum("ij,ij->i", pts[T[:, 0]], np.cross(pts[T[:, 1]], pts[T[:, 2]])).sum() < 0:
        T = T[:, [0, 2, 1]]
    return pts.ravel().copy(), T.ravel().copy()


def test_product_geometry_is_the_reference_geometry_on_a_torus():
    """A non-convex body on a stretched 96^3 grid.  Here the dot-normal rule
    leaves 4 cell centres fluid that lie inside the surface (winding number 1,
    3-4% of a cell from it); the product reproduces that too."""
    p = P.default_params(3, 96, 96, 96, body=True)
    x, y, z = make_grid(p.nx, p.ny, p.nz, "tanh", beta=1.5)
    v, t = _torus()
    g = P.body_geometry(p, x, y, z, v, t)
    r = reference_geometry(p.nx, p.ny, p.nz, x, y, z, v, t, (3.0, 3.0, 3.0))
    assert np.array_equal(g.iblank, r.iblank) and int(g.iblank.sum()) == 108992
    assert np.array_equal(g.iG, r.iG) and np.array_equal(g.jG, r.jG) and np.array_equal(g.kG, r.kG)
    assert np.array_equal(g.xBI, r.xBI) and np.array_equal(g.xIP, r.xIP)
    own = _self_rows(g)
    assert np.abs(g.coeff[~own] - r.coeffN[~own]).max() <= 1e-9


def test_product_geometry_does_not_depend_on_the_surface_orientation():
    cells, kind, lengths, centre, radius, _ = CASES["sphere_32_tanh"]
    _, _, _, g_out, _ = _both(cells, kind, lengths, centre, radius)
    _, _, _, g_in, r_in = _both(cells, kind, lengths, centre, radius, tris_inward=True)
    assert not r_in.flipped
    assert np.array_equal(g_out.iblank, g_in.iblank)
    assert np.array_equal(g_out.xBI, g_in.xBI) and np.array_equal(g_out.coeff, g_in.coeff)


def test_oracle_classifies_the_sphere_and_lands_on_its_surface():
    """What the reference's rules must give on a closed convex body: every
    cell centre inside the icosphere's inradius is solid and every one outside
    the sphere is fluid, the band covers the surface, and each body intercept
    lies on the plane of its element, between the inradius and the sphere."""
    cells, kind, lengths, centre, radius, _ = CASES["sphere_64_tanh"]
    p, (x, y, z), (v, t), _, r = _both(cells, kind, lengths, centre, radius)
    mx, my, mz = Metrics(x), Metrics(y), Metrics(z)
    n = cells[0]
    X, Y, Z = np.meshgrid(mx.xc[1:n + 1], my.xc[1:n + 1], mz.xc[1:n + 1], indexing="ij")
    rad = np.sqrt((X - 0.5) ** 2 + (Y - 0.5) ** 2 + (Z - 0.5) ** 2)
    V = v.reshape(-1, 3)
    T = r.tris.reshape(-1, 3)
    N = np.cross(V[T[:, 1]] - V[T[:, 0]], V[T[:, 2]] - V[T[:, 1]])
    N /= np.linalg.norm(N, axis=1)[:, None]
    inradius = np.einsum("ij,ij->i", -N, V[T[:, 0]] - 0.5).min()   # nearest face plane to the centre
    assert 0.998 * radius < inradius < radius
    ib = r.iblank[1:n + 1, 1:n + 1, 1:n + 1]
    assert (ib[rad < inradius * (1 - 1e-12)] == 1).all() and (ib[rad > radius] == 0).all()
    band = r.band[1:n + 1, 1:n + 1, 1:n + 1].astype(bool)
    assert band[np.abs(rad - radius) < 0.5 * np.diff(mx.x).min()].all()
    for k in range(r.nGhost):
        e = T[r.elem[k]]
        nrm = np.cross(V[e[1]] - V[e[0]], V[e[2]] - V[e[1]])
        nrm /= np.linalg.norm(nrm)
        assert abs(nrm @ (r.xBI[:, k] - V[e[0]])) <= 1e-15
        assert nrm @ (0.5 - V[e[0]]) > 0                  # the normals point into the body
        assert inradius * (1 - 1e-14) <= np.linalg.norm(r.xBI[:, k] - 0.5) <= radius * (1 + 1e-14)


def test_oracle_orientation_step():
    """determine_norm_dir_unstruc: an outward surface is reordered, an inward
    one is left alone."""
    import ctypes
    v, t = P.icosphere(2, 0.3, (0.5, 0.5, 0.5))
    L = lib()
    dp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int32)
    t1 = t.copy()
    assert L.og_orient_inward(v.size // 3, v.ctypes.data_as(dp), t1.size // 3, t1.ctypes.data_as(ip), 2.0, 2.0, 2.0) == 1
    assert np.array_equal(t1.reshape(-1, 3), t.reshape(-1, 3)[:, [0, 2, 1]])
    assert L.og_orient_inward(v.size // 3, v.ctypes.data_as(dp), t1.size // 3, t1.ctypes.data_as(ip), 2.0, 2.0, 2.0) == 0


def _custom(n, centre, radius):
    p = P.default_params(3, n, n, n, body=True)
    x, y, z = make_grid(p.nx, p.ny, p.nz, "uniform")
    v, t = P.icosphere(3, radius, centre)
    g = P.body_geometry(p, x, y, z, v, t)
    r = reference_geometry(p.nx, p.ny, p.nz, x, y, z, v, t, (3.0, 3.0, 3.0))
    return p, g, r


def test_isolated_solid_cell_is_removed():
    """find_isolatedIblank (IBM/BOUNDARY_SET.F90:440-499): a body that
    encloses a single cell centre leaves no solid cell."""
    h = 1.0 / 16
    p, g, r = _custom(16, (7.5 * h, 7.5 * h, 7.5 * h), 0.3 * h)
    assert int(r.band.sum()) > 0
    assert int(g.iblank.sum()) == 0 and int(r.iblank.sum()) == 0
    assert g.nGhost == 0


def test_one_cell_gap_at_the_outer_wall_is_closed():
    """fill_cell (IBM/SSM_SET_BC.F90:1425-1511): a fluid cell between the body
    and the flagged outer face turns solid, in the product as in the oracle."""
    h = 1.0 / 16
    p, g, r = _custom(16, (12.0 * h, 8.0 * h, 8.0 * h), 2.75 * h)
    I = (slice(1, p.nx), slice(1, p.ny), slice(1, p.nz))
    assert np.array_equal(g.iblank[I], r.iblank[I])
    nxc = p.nx - 1
    closed = (g.iblank[nxc] == 1) & (g.iblank[nxc - 1] == 1)
    assert closed.any()                          # the gap cells on the axis lines closed
    assert (g.iblank[nxc][g.iblank[nxc - 1] == 0] == 0).all()
    assert g.nGhost == r.nGhost and np.array_equal(g.xBI, r.xBI)
