"""Host geometry producer: icosphere, iblank, ghost list and image-point
coefficients (restating IBM/GCM_SET_BOUNDARY.F90 for an unstructured body)."""
import numpy as np

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.grid import Metrics, make_grid
from flow_structure_interaction_fem_ibm_gb300.params import SolverParams


def test_icosphere_counts_and_radius():
    v, t = P.icosphere(4, 0.15, (0.5, 0.5, 0.5))
    assert v.size // 3 == 2562 and t.size // 3 == 5120
    r = np.linalg.norm(v.reshape(-1, 3) - 0.5, axis=1)
    assert np.allclose(r, 0.15, rtol=1e-12)
    V = v.reshape(-1, 3); T = t.reshape(-1, 3)
    n = np.cross(V[T[:, 1]] - V[T[:, 0]], V[T[:, 2]] - V[T[:, 0]])
    c = V[T].mean(axis=1) - 0.5
    assert (np.einsum("ij,ij->i", n, c) > 0).all()   # outward


def _geom(n=32, stretch=1.5):
    p = SolverParams(ndim=3, nx=n + 1, ny=n + 1, nz=n + 1, internal_boundary_present=1, boundary_formulation=2)
    x, y, z = make_grid(p.nx, p.ny, p.nz, "tanh" if stretch else "uniform", beta=stretch or 1.5)
    v, t = P.icosphere(4, 0.15, (0.5, 0.5, 0.5))
    return p, x, y, z, P.body_geometry(p, x, y, z, v, t), v, t


def test_iblank_matches_sphere_away_from_surface():
    p, x, y, z, g, _, _ = _geom(32)
    mx, my, mz = Metrics(x), Metrics(y), Metrics(z)
    n = 32
    X, Y, Z = np.meshgrid(mx.xc[1:n + 1], my.xc[1:n + 1], mz.xc[1:n + 1], indexing="ij")
    r = np.sqrt((X - .5) ** 2 + (Y - .5) ** 2 + (Z - .5) ** 2)
    ib = g.iblank[1:n + 1, 1:n + 1, 1:n + 1]
    assert (ib[r < 0.15 * 0.995] == 1).all()
    assert (ib[r > 0.15] == 0).all()
    assert g.iblank[0].sum() == 0 and g.iblank[:, :, n + 1].sum() == 0


def test_ghost_marks_rule_and_order():
    p, x, y, z, g, _, _ = _geom(24, None)
    ib = g.iblank.astype(int)
    n = 24
    expect = []
    for k in range(1, n + 1):
        for j in range(1, n + 1):
            for i in range(1, n + 1):
                if ib[i, j, k] != 1:
                    continue
                nb = [ib[max(i - 1, 1), j, k], ib[min(i + 1, n), j, k], ib[i, max(j - 1, 1), k],
                      ib[i, min(j + 1, n), k], ib[i, j, max(k - 1, 1)], ib[i, j, min(k + 1, n)]]
                if min(nb) == 0:
                    expect.append((i, j, k))
    got = list(zip(g.iG.tolist(), g.jG.tolist(), g.kG.tolist()))
    assert got == expect
    assert int(g.ghost.sum()) == len(expect)


def test_image_point_coefficients_reproduce_trilinear_fields():
    """coeffGCMN interpolates any trilinear field exactly at the image point
    (IBM/GCM_SET_BOUNDARY.F90:307-494); when the ghost itself is in the stencil
    its row carries the Neumann condition, so the other weights sum to 1."""
    p, x, y, z, g, _, _ = _geom(24, 1.5)
    mx, my, mz = Metrics(x), Metrics(y), Metrics(z)
    inc = np.array([[0, 0, 0], [0, 1, 0], [1, 1, 0], [1, 0, 0], [0, 0, 1], [0, 1, 1], [1, 1, 1], [1, 0, 1]])
    assert g.nGhost > 50
    for n in range(g.nGhost):
        cells = np.array([g.iCI[n], g.jCI[n], g.kCI[n]]) + inc
        selfrow = [(c == [g.iG[n], g.jG[n], g.kG[n]]).all() for c in cells]
        w = g.coeff[:, n]
        others = ~np.array(selfrow)
        assert abs(w[others].sum() - 1.0) < 1e-12   # constants reproduced: the Neumann operator stays singular
        assert g.probe[n] > 0
    assert np.isfinite(g.coeff).all()
