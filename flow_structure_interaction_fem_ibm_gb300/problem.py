"""Problem assembly: grid, boundary flags, immersed body and right-hand side.

This is the host-side data a Fortran caller holds in its modules before it
calls ``solve_poisson`` (IBM/CORE_POISSON.F90:493): node arrays, the INTEGER(1)
flag arrays iblank / ghostCellMark / ium..kup over (0:nx+1,0:ny+1,0:nz+1), the
ghost list with coeffGCMN(8,nGhost) and probeLength, the boundary pressure
gradients pgrad*, and nlu0.  All 3D arrays are numpy arrays in Fortran order.

Workloads (seeded synthetic inputs; the reference ships no input decks):
  * ``box2d``   -- 2D uniform grid, all-Neumann, no body, RHS = divergence of an
                   i.i.d. N(0,1) cell velocity field, mean removed.
  * ``sphere``  -- 3D grid (uniform or tanh-stretched toward the centre) with a
                   stationary sphere (4x-subdivided icosphere, ghost-cell
                   Neumann body); RHS = divergence of a Gaussian random field
                   band-limited to |k| <= 8, mean removed over fluid cells.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _native
from .grid import Metrics, make_grid
from .params import (BC_TYPE_DIRICHLET, BC_TYPE_ZERO_GRADIENT, DIM_2D, DIM_3D, GCM_METHOD, NO_INTERNAL_BOUNDARY,
                     SolverParams)


def full_shape(p: SolverParams):
    return (p.nx + 2, p.ny + 2, p.nz + 2)


@dataclass
class Geometry:
    iblank: np.ndarray
    ghost: np.ndarray
    flags: list                      # [ium, iup, jum, jup, kum, kup]
    nGhost: int = 0
    iG: Optional[np.ndarray] = None
    jG: Optional[np.ndarray] = None
    kG: Optional[np.ndarray] = None
    iCI: Optional[np.ndarray] = None
    jCI: Optional[np.ndarray] = None
    kCI: Optional[np.ndarray] = None
    coeff: Optional[np.ndarray] = None       # coeffGCMN (8, nGhost) Fortran order
    probe: Optional[np.ndarray] = None
    pgrad: Optional[np.ndarray] = None       # 6 boundary planes packed
    coeffD: Optional[np.ndarray] = None      # coeffGCMD (8, nGhost): Dirichlet weights of the ghost velocity
    xBI: Optional[np.ndarray] = None         # (3, nGhost) body intercepts
    xIP: Optional[np.ndarray] = None         # (3, nGhost) image points


@dataclass
class Problem:
    params: SolverParams
    x: np.ndarray
    y: np.ndarray
    z: np.ndarray
    geom: Geometry
    nlu0: np.ndarray
    name: str = ""

    @property
    def shape(self):
        return full_shape(self.params)


def outer_flags(p: SolverParams):
    """set_outer_iup (IBM/BOUNDARY_SET.F90:54-80): ium(1,:,:) = iup(nxc,:,:) = 1
    etc.  In 2D the k flags stay 0."""
    sh = full_shape(p)
    fl = [np.zeros(sh, dtype=np.int8, order="F") for _ in range(6)]
    nxc, nyc, nzc = p.nx - 1, p.ny - 1, p.nz - 1
    fl[0][1, 1:p.ny + 1, 1:p.nz + 1] = 1
    fl[1][nxc, 1:p.ny + 1, 1:p.nz + 1] = 1
    fl[2][1:p.nx + 1, 1, 1:p.nz + 1] = 1
    fl[3][1:p.nx + 1, nyc, 1:p.nz + 1] = 1
    if p.ndim == DIM_3D:
        fl[4][1:p.nx + 1, 1:p.ny + 1, 1] = 1
        fl[5][1:p.nx + 1, 1:p.ny + 1, nzc] = 1
    return fl


def pgrad_size(p: SolverParams) -> int:
    nx2, ny2, nz2 = full_shape(p)
    return 2 * ny2 * nz2 + 2 * nx2 * nz2 + 2 * nx2 * ny2


def empty_geometry(p: SolverParams) -> Geometry:
    sh = full_shape(p)
    return Geometry(iblank=np.zeros(sh, np.int8, order="F"), ghost=np.zeros(sh, np.int8, order="F"),
                    flags=outer_flags(p), nGhost=0, pgrad=np.zeros(pgrad_size(p)))


def icosphere(nsub: int = 4, radius: float = 0.15, centre=(0.5, 0.5, 0.5)):
    g = _native.geometry()
    nv_cap = 10 * 4 ** nsub + 2
    nt_cap = 20 * 4 ** nsub
    verts = np.zeros(3 * nv_cap)
    tris = np.zeros(3 * nt_cap, dtype=np.int32)
    nv, nt = ctypes.c_int(), ctypes.c_int()
    rc = g.fsi_geom_icosphere(nsub, radius, centre[0], centre[1], centre[2],
                              _native.ptr(verts, ctypes.c_double), nv_cap,
                              _native.ptr(tris, ctypes.c_int32), nt_cap, ctypes.byref(nv), ctypes.byref(nt))
    if rc != 0:
        raise RuntimeError("icosphere capacity" if rc == -1 else "icosphere: out of host memory")
    return verts[: 3 * nv.value].copy(), tris[: 3 * nt.value].copy()


def body_geometry(p: SolverParams, x, y, z, verts, tris, probe_length_normalized: float = 2.0) -> Geometry:
    """set_boundary for one solid unstructured body: iblank, ghost marks and list,
    image-point coefficients (IBM/BOUNDARY_SET.F90:8-51, IBM/GCM_SET_BOUNDARY.F90:2-304)."""
    g = _native.geometry()
    sh = full_shape(p)
    nv, nt = verts.size // 3, tris.size // 3
    iblank = np.zeros(sh, np.int8, order="F")
    ns = g.fsi_geom_iblank(p.nx, p.ny, p.nz, _native.ptr(x, ctypes.c_double), _native.ptr(y, ctypes.c_double),
                           _native.ptr(z, ctypes.c_double), nv, _native.ptr(verts, ctypes.c_double), nt,
                           _native.ptr(tris, ctypes.c_int32), iblank.ctypes.data_as(_native.c_i8_p))
    if ns < 0:
        raise RuntimeError("iblank: no reference marker for a band cell (the reference stops there)"
                           if ns == -1 else "iblank: out of host memory")
    ghost = np.zeros(sh, np.int8, order="F")
    cap = int(iblank.sum()) + 1
    iG = np.zeros(cap, np.int32); jG = np.zeros(cap, np.int32); kG = np.zeros(cap, np.int32)
    n = g.fsi_geom_ghost_list(p.nx, p.ny, p.nz, iblank.ctypes.data_as(_native.c_i8_p),
                              ghost.ctypes.data_as(_native.c_i8_p), cap,
                              _native.ptr(iG, ctypes.c_int32), _native.ptr(jG, ctypes.c_int32),
                              _native.ptr(kG, ctypes.c_int32))
    if n < 0:
        raise RuntimeError("ghost list capacity")
    iG, jG, kG = iG[:n].copy(), jG[:n].copy(), kG[:n].copy()
    iCI = np.zeros(n, np.int32); jCI = np.zeros(n, np.int32); kCI = np.zeros(n, np.int32)
    coeff = np.zeros((8, n), order="F")
    coeffD = np.zeros((8, n), order="F")
    xBI = np.zeros((3, n), order="F")
    xIP = np.zeros((3, n), order="F")
    probe = np.zeros(n)
    rc = g.fsi_geom_gcm_coeffs(p.nx, p.ny, p.nz, _native.ptr(x, ctypes.c_double), _native.ptr(y, ctypes.c_double),
                               _native.ptr(z, ctypes.c_double), nv, _native.ptr(verts, ctypes.c_double), nt,
                               _native.ptr(tris, ctypes.c_int32), probe_length_normalized, n,
                               _native.ptr(iG, ctypes.c_int32), _native.ptr(jG, ctypes.c_int32),
                               _native.ptr(kG, ctypes.c_int32), _native.ptr(iCI, ctypes.c_int32),
                               _native.ptr(jCI, ctypes.c_int32), _native.ptr(kCI, ctypes.c_int32),
                               coeff.ctypes.data_as(_native.c_double_p), _native.ptr(probe, ctypes.c_double),
                               xBI.ctypes.data_as(_native.c_double_p), xIP.ctypes.data_as(_native.c_double_p),
                               coeffD.ctypes.data_as(_native.c_double_p))
    if rc == -(n + 2):
        raise RuntimeError("image-point coefficients: out of host memory")
    if rc != 0:
        raise RuntimeError(f"image-point stencil search failed for ghost {-rc - 1}")
    return Geometry(iblank=iblank, ghost=ghost, flags=outer_flags(p), nGhost=n, iG=iG, jG=jG, kG=kG,
                    iCI=iCI, jCI=jCI, kCI=kCI, coeff=coeff, probe=probe, pgrad=np.zeros(pgrad_size(p)),
                    coeffD=coeffD, xBI=xBI, xIP=xIP)


# ---------------------------------------------------------------- RHS ----

def face_divergence(p: SolverParams, x, y, z, u, v, w, iblank, flags, dt: float = 1.0):
    """nlu0 = dtinv * div(face velocity) * (1 - iblank) with face velocities from
    the face_vel interpolation and masks (IBM/CORE_FRAC_STEP_ROUTINES.F90:80-109,
    178-195: zero boundary velocity on a face flagged from either side) and
    rhs_poisson (IBM/CORE_POISSON.F90:155-163).  u, v, w are cell-centred
    (0:nx+1,...) arrays."""
    mx, my, mz = Metrics(x), Metrics(y), Metrics(z)
    nxc, nyc, nzc = p.nx - 1, p.ny - 1, p.nz - 1
    I = slice(1, nxc + 1); J = slice(1, nyc + 1); K = slice(1, nzc + 1)
    ium, iup, jum, jup, kum, kup = [f[I, J, K].astype(np.float64) for f in flags]
    fx, fy, fz = mx.fx, my.fx, mz.fx

    def shifted(m, ax, step):
        # m of the neighbouring cell along ax (step -1: previous, +1: next); 0 past the interior
        out = np.zeros_like(m)
        src = [slice(None)] * 3
        dst = [slice(None)] * 3
        if step < 0:
            src[ax], dst[ax] = slice(0, -1), slice(1, None)
        else:
            src[ax], dst[ax] = slice(1, None), slice(0, -1)
        out[tuple(dst)] = m[tuple(src)]
        return out

    # face values on the + and - faces of each interior cell: a face is zero
    # (wall) when flagged from either side, the reference's final masks
    fu_p = (fx[2:nxc + 2, None, None] * u[2:nxc + 2, J, K] + (1 - fx[2:nxc + 2, None, None]) * u[I, J, K]) \
        * (1 - iup) * (1 - shifted(ium, 0, +1))
    fu_m = (fx[1:nxc + 1, None, None] * u[I, J, K] + (1 - fx[1:nxc + 1, None, None]) * u[0:nxc, J, K]) \
        * (1 - ium) * (1 - shifted(iup, 0, -1))
    fv_p = (fy[None, 2:nyc + 2, None] * v[I, 2:nyc + 2, K] + (1 - fy[None, 2:nyc + 2, None]) * v[I, J, K]) \
        * (1 - jup) * (1 - shifted(jum, 1, +1))
    fv_m = (fy[None, 1:nyc + 1, None] * v[I, J, K] + (1 - fy[None, 1:nyc + 1, None]) * v[I, 0:nyc, K]) \
        * (1 - jum) * (1 - shifted(jup, 1, -1))
    if p.ndim == DIM_3D:
        fw_p = (fz[None, None, 2:nzc + 2] * w[I, J, 2:nzc + 2] + (1 - fz[None, None, 2:nzc + 2]) * w[I, J, K]) \
            * (1 - kup) * (1 - shifted(kum, 2, +1))
        fw_m = (fz[None, None, 1:nzc + 1] * w[I, J, K] + (1 - fz[None, None, 1:nzc + 1]) * w[I, J, 0:nzc]) \
            * (1 - kum) * (1 - shifted(kup, 2, -1))
    else:
        fw_p = fw_m = 0.0
    div = ((fu_p - fu_m) * mx.dxinv[1:nxc + 1, None, None] + (fv_p - fv_m) * my.dxinv[None, 1:nyc + 1, None]
           + (fw_p - fw_m) * mz.dxinv[None, None, 1:nzc + 1]) / dt
    nlu0 = np.zeros(full_shape(p), order="F")
    nlu0[I, J, K] = div * (1 - iblank[I, J, K])
    return nlu0


def remove_fluid_mean(p: SolverParams, x, y, z, f, iblank):
    """Subtract the volume-weighted mean over fluid cells (interior only)."""
    mx, my, mz = Metrics(x), Metrics(y), Metrics(z)
    nxc, nyc, nzc = p.nx - 1, p.ny - 1, p.nz - 1
    vol = (mx.dx[1:nxc + 1, None, None] * my.dx[None, 1:nyc + 1, None] * mz.dx[None, None, 1:nzc + 1])
    fl = 1.0 - iblank[1:nxc + 1, 1:nyc + 1, 1:nzc + 1]
    sub = f[1:nxc + 1, 1:nyc + 1, 1:nzc + 1]
    mean = float((sub * vol * fl).sum() / (vol * fl).sum())
    f[1:nxc + 1, 1:nyc + 1, 1:nzc + 1] = (sub - mean) * fl
    return f


def gaussian_field(p: SolverParams, x, y, z, rng, kmax: int = 8, lengths=(1.0, 1.0, 1.0)):
    """Real Gaussian random field: finite Fourier sum over integer wavevectors
    with |k| <= kmax and i.i.d. normal coefficients, evaluated at cell centres
    (0:n+1).  Evaluated separably (one contraction per axis)."""
    mx, my, mz = Metrics(x), Metrics(y), Metrics(z)
    ks = np.arange(-kmax, kmax + 1)
    KX, KY, KZ = np.meshgrid(ks, ks, ks, indexing="ij")
    mask = (KX ** 2 + KY ** 2 + KZ ** 2) <= kmax * kmax
    if p.ndim == DIM_2D:
        mask &= (KZ == 0)
    coef = (rng.standard_normal(mask.shape) + 1j * rng.standard_normal(mask.shape)) * mask
    ex = np.exp(2j * np.pi * np.outer(mx.xc, ks) / lengths[0])
    ey = np.exp(2j * np.pi * np.outer(my.xc, ks) / lengths[1])
    ez = np.exp(2j * np.pi * np.outer(mz.xc, ks) / lengths[2])
    t1 = np.einsum("abc,ia->ibc", coef, ex)
    t2 = np.einsum("ibc,jb->ijc", t1, ey)
    out = np.empty((ex.shape[0], ey.shape[0], ez.shape[0]), order="F")
    out[...] = np.einsum("ijc,kc->ijk", t2, ez).real
    return out / np.sqrt(max(mask.sum(), 1))


def outflow_area(p: SolverParams, x, y, z, iblank) -> float:
    """set_outflow_area (IBM/BOUNDARY_SET.F90:134-221): the fluid area of the
    zero-gradient sides (the first / last cell layer of each side, cells with
    iblank = 0), the value fsi_mg_params.outflow_area carries."""
    mx, my, mz = Metrics(x), Metrics(y), Metrics(z)
    nxc, nyc, nzc = p.nx - 1, p.ny - 1, p.nz - 1
    dx, dy, dz = mx.dx[1:nxc + 1], my.dx[1:nyc + 1], mz.dx[1:nzc + 1]
    fl = 1.0 - iblank[1:nxc + 1, 1:nyc + 1, 1:nzc + 1]
    areas = [(dy[:, None] * dz[None, :] * fl[0]).sum(), (dy[:, None] * dz[None, :] * fl[-1]).sum(),
             (dx[:, None] * dz[None, :] * fl[:, 0, :]).sum(), (dx[:, None] * dz[None, :] * fl[:, -1, :]).sum(),
             (dx[:, None] * dy[None, :] * fl[:, :, 0]).sum(), (dx[:, None] * dy[None, :] * fl[:, :, -1]).sum()]
    return float(sum(a for a, t in zip(areas, p.bc) if t == BC_TYPE_ZERO_GRADIENT))


def default_params(ndim: int, nxc: int, nyc: int, nzc: int, body: bool, **kw) -> SolverParams:
    p = SolverParams(ndim=ndim, nx=nxc + 1, ny=nyc + 1, nz=(nzc + 1) if ndim == DIM_3D else 2)
    p.bc = (BC_TYPE_DIRICHLET,) * 6
    if body:
        p.internal_boundary_present = 1
        p.boundary_formulation = GCM_METHOD
    else:
        p.internal_boundary_present = 0
        p.boundary_formulation = NO_INTERNAL_BOUNDARY
    for k, v in kw.items():
        setattr(p, k, v)
    return p


def box2d(n: int = 128, seed: int = 1, **kw) -> Problem:
    """2D n x n uniform box on [0,1]^2, all-Neumann pressure, no body."""
    p = default_params(DIM_2D, n, n, 1, body=False, **kw)
    x, y, z = make_grid(p.nx, p.ny, p.nz, "uniform")
    geom = empty_geometry(p)
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = full_shape(p)
    u = np.asfortranarray(rng.standard_normal(sh))
    v = np.asfortranarray(rng.standard_normal(sh))
    w = np.zeros(sh, order="F")
    nlu0 = face_divergence(p, x, y, z, u, v, w, geom.iblank, geom.flags)
    remove_fluid_mean(p, x, y, z, nlu0, geom.iblank)
    return Problem(p, x, y, z, geom, nlu0, name=f"box2d_{n}")


def box3d(n=128, seed: int = 1, stretch: Optional[float] = 1.5, **kw) -> Problem:
    """3D box [0,1]^3 without a body, all-Neumann pressure; nlu0 from a seeded
    N(0,1) cell velocity field (face_vel interpolation), which is compatible
    (the zero boundary flux telescopes).  ``n`` is an int or (nxc, nyc, nzc)."""
    nxc, nyc, nzc = (n, n, n) if isinstance(n, int) else n
    p = default_params(DIM_3D, nxc, nyc, nzc, body=False, **kw)
    kind = "uniform" if stretch is None else "tanh"
    x, y, z = make_grid(p.nx, p.ny, p.nz, kind, beta=stretch or 1.5)
    geom = empty_geometry(p)
    rng = np.random.Generator(np.random.PCG64(seed))
    sh = full_shape(p)
    u, v, w = (np.asfortranarray(rng.standard_normal(sh)) for _ in range(3))
    nlu0 = face_divergence(p, x, y, z, u, v, w, geom.iblank, geom.flags)
    remove_fluid_mean(p, x, y, z, nlu0, geom.iblank)
    tag = "uniform" if stretch is None else f"tanh{stretch}"
    return Problem(p, x, y, z, geom, nlu0, name=f"box3d_{nxc}x{nyc}x{nzc}_{tag}")


def sphere(n=128, seed: int = 2, stretch: Optional[float] = 1.5, radius: float = 0.15, nsub: int = 4,
           kmax: int = 8, **kw) -> Problem:
    """3D box [0,1]^3 with a stationary ghost-cell sphere at the centre.
    ``n`` is an int or an (nxc, nyc, nzc) tuple; ``stretch`` None means uniform."""
    nxc, nyc, nzc = (n, n, n) if isinstance(n, int) else n
    p = default_params(DIM_3D, nxc, nyc, nzc, body=True, **kw)
    kind = "uniform" if stretch is None else "tanh"
    x, y, z = make_grid(p.nx, p.ny, p.nz, kind, beta=stretch or 1.5)
    verts, tris = icosphere(nsub, radius, (0.5, 0.5, 0.5))
    geom = body_geometry(p, x, y, z, verts, tris)
    rng = np.random.Generator(np.random.PCG64(seed))
    u = gaussian_field(p, x, y, z, rng, kmax)
    v = gaussian_field(p, x, y, z, rng, kmax)
    w = gaussian_field(p, x, y, z, rng, kmax)
    nlu0 = face_divergence(p, x, y, z, u, v, w, geom.iblank, geom.flags)
    remove_fluid_mean(p, x, y, z, nlu0, geom.iblank)
    tag = "uniform" if stretch is None else f"tanh{stretch}"
    return Problem(p, x, y, z, geom, nlu0, name=f"sphere_{nxc}x{nyc}x{nzc}_{tag}")


CHANNEL_BC = (1, 2, 4, 4, 4, 4)   # Dirichlet inflow, zero-gradient outflow, symmetry sides


def channel(cells=(192, 128, 128), lengths=(6.0, 4.0, 4.0), centre=(1.5, 2.0, 2.0), diameter: float = 1.0,
            nsub: int = 4, **kw) -> Problem:
    """Channel with a stationary ghost-cell sphere: uniform grid on
    [0,Lx] x [0,Ly] x [0,Lz], velocity BC types CHANNEL_BC (x1 inflow, x2
    zero-gradient outflow, symmetry sides), Neumann pressure, outflow_area
    from set_outflow_area.  nlu0 is zero: a time loop forms it every step.
    The default is the 192 x 128 x 128 channel of the sphere-wake rollout."""
    p = default_params(DIM_3D, *cells, body=True, **kw)
    p.bc = CHANNEL_BC
    x, y, z = make_grid(p.nx, p.ny, p.nz, "uniform", lengths=lengths)
    verts, tris = icosphere(nsub, 0.5 * diameter, centre)
    geom = body_geometry(p, x, y, z, verts, tris)
    p.outflow_area = outflow_area(p, x, y, z, geom.iblank)
    name = f"channel_{cells[0]}x{cells[1]}x{cells[2]}_sphere_d{diameter:g}"
    return Problem(p, x, y, z, geom, np.zeros(full_shape(p), order="F"), name=name)


def kat2d(n: int = 64, **kw) -> Problem:
    """Poisson_Tester known-answer case (IBM/CORE_POISSON.F90:1386-1444):
    domain [0,pi]^2, all-Neumann, nlu0 = -2 cos(xc) cos(yc); the exact answer is
    cos(x) cos(y) up to the Neumann constant."""
    p = default_params(DIM_2D, n, n, 1, body=False, **kw)
    x, y, z = make_grid(p.nx, p.ny, p.nz, "uniform", lengths=(np.pi, np.pi, 1.0))
    geom = empty_geometry(p)
    mx, my = Metrics(x), Metrics(y)
    nlu0 = np.zeros(full_shape(p), order="F")
    nlu0[1:n + 1, 1:n + 1, 1] = -2.0 * np.cos(mx.xc[1:n + 1, None]) * np.cos(my.xc[None, 1:n + 1])
    return Problem(p, x, y, z, geom, nlu0, name=f"kat2d_{n}")


# ------------------------------------------------------- compatibility ----

def fluid_indicator(problem: Problem) -> np.ndarray:
    p = problem.params
    one = np.zeros(problem.shape, order="F")
    n0, n1, n2 = p.nx - 1, p.ny - 1, p.nz - 1
    one[1:n0 + 1, 1:n1 + 1, 1:n2 + 1] = 1.0 - problem.geom.iblank[1:n0 + 1, 1:n1 + 1, 1:n2 + 1]
    return one


def residual_field(problem: Problem, pr: np.ndarray, f: np.ndarray) -> np.ndarray:
    """r - A p on fluid cells (the operator of calc_residual, IBM/CORE_POISSON.F90:
    1111-1222, with nlw0 = 0), vectorised.  Harness helper for input preparation."""
    p = problem.params
    mx, my, mz = Metrics(problem.x), Metrics(problem.y), Metrics(problem.z)
    n0, n1, n2 = p.nx - 1, p.ny - 1, p.nz - 1
    I, J, K = slice(1, n0 + 1), slice(1, n1 + 1), slice(1, n2 + 1)
    fl = [a[I, J, K].astype(np.float64) for a in problem.geom.flags]
    d2 = float(p.ndim - DIM_2D)
    bmx = (mx.dxcinv[1:n0 + 1] * mx.dxinv[1:n0 + 1])[:, None, None] * (1 - fl[0])
    bpx = (mx.dxcinv[2:n0 + 2] * mx.dxinv[1:n0 + 1])[:, None, None] * (1 - fl[1])
    bmy = (my.dxcinv[1:n1 + 1] * my.dxinv[1:n1 + 1])[None, :, None] * (1 - fl[2])
    bpy = (my.dxcinv[2:n1 + 2] * my.dxinv[1:n1 + 1])[None, :, None] * (1 - fl[3])
    bmz = (mz.dxcinv[1:n2 + 1] * mz.dxinv[1:n2 + 1])[None, None, :] * (1 - fl[4]) * d2
    bpz = (mz.dxcinv[2:n2 + 2] * mz.dxinv[1:n2 + 1])[None, None, :] * (1 - fl[5]) * d2
    bc = -(bmx + bpx) - (bmy + bpy) - (bmz + bpz)
    res = (f[I, J, K] - pr[I, J, K] * bc - pr[0:n0, J, K] * bmx - pr[2:n0 + 2, J, K] * bpx
           - pr[I, 0:n1, K] * bmy - pr[I, 2:n1 + 2, K] * bpy - pr[I, J, 0:n2] * bmz - pr[I, J, 2:n2 + 2] * bpz)
    out = np.zeros(problem.shape, order="F")
    out[I, J, K] = res * (1 - problem.geom.iblank[I, J, K])
    return out


def compatibility_shift(problem: Problem, stagnated_pressure) -> float:
    """Discrete compatibility constant of a ghost-cell Neumann problem.

    With ghost-cell rows the pure-Neumann operator is singular but not
    symmetric, so its left null vector is not the cell-volume vector and a
    volume-mean-free right-hand side can still be inconsistent: every iteration
    then stalls at a residual floor.  The stalled residual is a rank-one linear
    function of the right-hand side (its component outside the operator's
    range), so the uniform shift c that makes f + c*1_fluid consistent follows
    from two stalled solves: c = -<r(f), r(1)> / <r(1), r(1)>.
    ``stagnated_pressure(f)`` must return the pressure after the residual has
    stopped changing (e.g. 30 MG iterations with restol 0)."""
    one = fluid_indicator(problem)
    r0 = residual_field(problem, stagnated_pressure(problem.nlu0), problem.nlu0)
    r1 = residual_field(problem, stagnated_pressure(one), one)
    den = float((r1 * r1).sum())
    return 0.0 if den == 0.0 else -float((r0 * r1).sum()) / den


def stall_until_plateau(solve_from_zero, f, iters: int = 100, max_iters: int = 6400, rtol: float = 1e-10):
    """Pressure at the residual plateau of an inconsistent solve.

    ``solve_from_zero(f, iters) -> (p, history)`` runs ``iters`` outer
    iterations from pPrime = 0 in ONE solve.  A solve cannot be continued by
    restarting it from its own result: subtracting_average_pressure
    (IBM/CORE_POISSON.F90:419-490) zeroes every iblank = 1 cell, ghost cells
    included, so each restart re-injects an O(p/h^2) residual next to the body
    that a slowly contracting cycle does not remove within one chunk.  MG
    contracts everything but the inconsistent component geometrically, so the
    history approaches its plateau; the count doubles until the last quarter of
    the history moves by at most ``rtol`` relative (FP64: ~1e-10; the mixed
    form's plateau carries FP32 noise of a few 1e-6)."""
    while True:
        p, hist = solve_from_zero(f, iters)
        h = np.asarray(hist, dtype=float)
        a, b = float(h[(3 * len(h)) // 4]), float(h[-1])
        if abs(a - b) <= rtol * max(b, 1e-300) or iters >= max_iters:
            return p
        iters *= 2


def make_compatible(problem: Problem, stagnated_pressure) -> float:
    c = compatibility_shift(problem, stagnated_pressure)
    problem.nlu0 += c * fluid_indicator(problem)
    return c
