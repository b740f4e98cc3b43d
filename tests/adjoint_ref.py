"""Sparse-direct reference of the projection step and its gradient (test
infrastructure).  A_eff is assembled explicitly over the fluid cells (the
7-point operator of calc_residual with the ghost values eliminated through
the ghost rows) and every solve is a sparse LU of a bordered system:

    left null vector   [A^T 1; 1^T 0] [w; mu] = [0; vol]
    forward pressure   [A   1; 1^T 0] [p; mu] = [P f; 0]
    transposed solve   [A^T 1; 1^T 0] [z; mu] = [s; 0]   (1^T z = 0)

The divergence, gradient and ghost-row extension and their transposes are the
harness operators of flow_structure_interaction_fem_ibm_gb300.adjoint
(checked separately by dot-product tests).
"""
import numpy as np
import scipy.sparse as sp
import scipy.sparse.linalg as spla
import torch

from flow_structure_interaction_fem_ibm_gb300.adjoint import ProjectionOperators, fortran_zeros


def _flat(t):
    return t.permute(2, 1, 0).reshape(-1).cpu().numpy()


class SparseProjection:
    def __init__(self, problem):
        self.ops = o = ProjectionOperators(problem, "cpu")
        shape = problem.shape
        sx, sy = shape[0], shape[1]
        ntot = int(np.prod(shape))
        fluid = _flat(o.fluid) > 0.5
        self.fidx = np.nonzero(fluid)[0]
        nF = self.fidx.size
        col_of = -np.ones(ntot, dtype=np.int64)
        col_of[self.fidx] = np.arange(nF)
        # A_full restricted to fluid rows, columns over the full array
        rows, cols, vals = [], [], []
        n0, n1, n2 = o.n
        ii, jj, kk = np.meshgrid(np.arange(1, n0 + 1), np.arange(1, n1 + 1), np.arange(1, n2 + 1), indexing="ij")
        lin = (ii + sx * (jj + sy * kk)).reshape(-1, order="F")
        mask = o.mask.numpy().reshape(-1, order="F") > 0.5
        for coef, off in ((o.bc, 0), (o.bmx, -1), (o.bpx, 1), (o.bmy, -sx), (o.bpy, sx), (o.bmz, -sx * sy),
                          (o.bpz, sx * sy)):
            c = torch.broadcast_to(coef, o.mask.shape).numpy().reshape(-1, order="F")
            keep = mask & (c != 0.0)
            rows.append(col_of[lin[keep]]); cols.append(lin[keep] + off); vals.append(c[keep])
        Afull = sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                              shape=(nF, ntot))
        # E: fluid -> full (identity on fluid, ghost rows on ghosts)
        E = sp.csr_matrix((np.ones(nF), (self.fidx, np.arange(nF))), shape=(ntot, nF))
        if o.nG > 0:
            CGF = o.C_GF[:, self.fidx]                     # non-ghost stencil cells that are fluid
            X = spla.spsolve((sp.identity(o.nG) - o.C_GG).tocsc(), CGF.tocsc())
            X = sp.csr_matrix(X)
            Eg = sp.csr_matrix((np.ones(o.nG), (o.gidx_np, np.arange(o.nG))), shape=(ntot, o.nG))
            E = E + Eg @ X
        self.A = (Afull @ E).tocsc()
        one = np.ones((nF, 1))
        self.vol = _flat(o.vol)[self.fidx]
        BT = sp.bmat([[self.A.T, one], [one.T, None]]).tocsc()
        B = sp.bmat([[self.A, one], [one.T, None]]).tocsc()
        self.luT = spla.splu(BT)
        self.lu = spla.splu(B)
        sol = self.luT.solve(np.concatenate([np.zeros(nF), [self.vol.sum()]]))
        self.w = sol[:nF]

    def _full(self, xF):
        out = np.zeros(int(np.prod(self.ops.shape)))
        out[self.fidx] = xF
        return torch.as_tensor(out).reshape(tuple(reversed(self.ops.shape))).permute(2, 1, 0)

    def forward(self, u, v, w):
        o = self.ops
        f = _flat(o.div(u, v, w))[self.fidx]
        pf = f - self.w.dot(f) / self.w.sum()
        p = self.lu.solve(np.concatenate([pf, [0.0]]))[:-1]
        pfull = o.extend(self._full(p))
        gx, gy, gz = o.grad(pfull)
        return u - gx, v - gy, w - gz

    def gradient(self, lu, lv, lw):
        o = self.ops
        s = _flat(o.extend_T(o.grad_T(lu, lv, lw)))[self.fidx]
        z = self.luT.solve(np.concatenate([s, [0.0]]))[:-1]
        du, dv, dw = o.div_T(self._full(z))
        return lu - du, lv - dv, lw - dw
