"""Grid nodes and metrics.

``make_grid`` restates IBM/CORE_GRID.F90:29-139: nodes x(1:nx) (uniform, or
read from xgrid.dat -- here a generated stretched distribution), ghost nodes
x(0) = -x(2) and x(nx+1) = 2 x(nx) - x(nx-1), cell centres, widths and their
inverses.  All arrays carry the reference's lower bound 0.
"""
from __future__ import annotations

import numpy as np


def uniform_nodes(n: int, length: float = 1.0) -> np.ndarray:
    """x(1:n) = (i-1) * length/(n-1) (IBM/CORE_GRID.F90:40-44)."""
    return np.arange(n, dtype=np.float64) * (length / (n - 1))


def tanh_stretched_nodes(n: int, beta: float = 1.5, length: float = 1.0) -> np.ndarray:
    """Nodes clustered toward the centre of [0, length]:
    x(s) = length * (0.5 + artanh((2s-1) tanh(beta)) / (2 beta)), s = (i-1)/(n-1).
    Spacing ratio edge/centre is cosh(beta)^2 (about 5.5 at beta = 1.5).  The
    reference reads such a distribution from xgrid.dat (IBM/CORE_GRID.F90:46-50)."""
    s = np.arange(n, dtype=np.float64) / (n - 1)
    x = 0.5 + np.arctanh((2.0 * s - 1.0) * np.tanh(beta)) / (2.0 * beta)
    x[0], x[-1] = 0.0, 1.0
    return x * length


def with_ghosts(nodes: np.ndarray) -> np.ndarray:
    """x(0:n+1) from x(1:n) (IBM/CORE_GRID.F90:52-53)."""
    n = nodes.size
    x = np.zeros(n + 2, dtype=np.float64)
    x[1:n + 1] = nodes
    x[0] = -x[2]
    x[n + 1] = x[n] + x[n] - x[n - 1]
    return x


class Metrics:
    """Cell metrics of one direction (IBM/CORE_GRID.F90:96-139)."""

    def __init__(self, x: np.ndarray):
        n = x.size - 2
        self.x = x
        self.xc = np.zeros(n + 2)
        self.dx = np.zeros(n + 2)
        self.dxinv = np.zeros(n + 2)
        self.dxc = np.zeros(n + 2)
        self.dxcinv = np.zeros(n + 2)
        self.xc[: n + 1] = 0.5 * (x[1:n + 2] + x[: n + 1])
        self.dx[: n + 1] = x[1:n + 2] - x[: n + 1]
        self.dxinv[: n + 1] = 1.0 / self.dx[: n + 1]
        self.xc[n + 1] = x[n + 1]
        self.dxc[1:n + 1] = self.xc[1:n + 1] - self.xc[0:n]
        self.dxcinv[1:n + 1] = 1.0 / self.dxc[1:n + 1]
        # interpolation weights fx(1:n) (IBM/CORE_GRID.F90:163-175)
        self.fx = np.zeros(n + 2)
        self.fx[1:n + 1] = (x[1:n + 1] - self.xc[0:n]) / (self.xc[1:n + 1] - self.xc[0:n])


def make_grid(nx: int, ny: int, nz: int, kind: str = "uniform", beta: float = 1.5,
              lengths=(1.0, 1.0, 1.0)):
    """Return (x, y, z) node arrays with ghosts for node counts (nx, ny, nz).
    ``kind`` is "uniform" or "tanh" (stretched toward the centre).  A 2D grid
    has nz = 2 with a unit-thickness z cell."""
    out = []
    for n, L in zip((nx, ny, nz), lengths):
        if kind == "tanh" and n > 2:
            nodes = tanh_stretched_nodes(n, beta, L)
        else:
            nodes = uniform_nodes(n, L)
        out.append(with_ghosts(nodes))
    return tuple(out)
