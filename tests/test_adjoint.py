"""Adjoint of the projection step (flow_structure_interaction_fem_ibm_gb300.adjoint).

CPU: every hand-written transpose passes a dot-product test, and the
sparse-direct reference gradient (tests/adjoint_ref.py) matches FP64 central
differences.  GPU: the multigrid-based adjoint (transposed FGMRES with the
forward MG as preconditioner) matches the sparse-direct reference and FP64
central differences (h = 1e-6, relative 1e-6), and step checkpointing with
recomputation gives the same rollout gradient.
"""
import numpy as np
import pytest
import torch

from flow_structure_interaction_fem_ibm_gb300 import problem as P
from flow_structure_interaction_fem_ibm_gb300.adjoint import ProjectionOperators, box_kinetic_energy
from tests.adjoint_ref import SparseProjection


def _rand(shape, gen, device="cpu"):
    return torch.randn(tuple(reversed(shape)), dtype=torch.float64, generator=gen).permute(2, 1, 0).to(device)


def _velocity(pr, seed, device="cpu"):
    """Seeded Gaussian random velocity field with |k| <= 8 (cell-centred)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    comps = [P.gaussian_field(pr.params, pr.x, pr.y, pr.z, rng, 8) for _ in range(3)]
    return [torch.as_tensor(np.asfortranarray(c), device=device) for c in comps]


@pytest.mark.parametrize("case", ["sphere16_tanh", "box2d_16"])
def test_transposes_pass_dot_product_tests(case):
    pr = P.sphere(16, seed=2, stretch=1.5) if case == "sphere16_tanh" else P.box2d(16, seed=3)
    o = ProjectionOperators(pr, "cpu")
    g = torch.Generator().manual_seed(0)
    u, v, w, z, p, lx, ly, lz, y = (_rand(pr.shape, g) for _ in range(9))
    zf = z * o.fluid
    pf = p * o.fluid
    uT, vT, wT = o.div_T(z)
    pairs = [
        (o.dot(o.div(u, v, w), z), o.dot(u, uT) + o.dot(v, vT) + o.dot(w, wT)),
        (sum(o.dot(a, b) for a, b in zip(o.grad(p), (lx, ly, lz))), o.dot(p, o.grad_T(lx, ly, lz))),
        (o.dot(o.apply_full(p), z), o.dot(p, o.apply_full_T(z))),
        (o.dot(o.extend(pf), y), o.dot(pf, o.extend_T(y))),
        (o.dot(o.apply_eff(pf), zf), o.dot(pf, o.apply_eff_T(zf))),
    ]
    for a, b in pairs:
        assert abs(a - b) <= 1e-12 * max(abs(a), 1.0), (a, b)
    # constants: A_eff 1 = 0 and the gradient of the extended constant is 0
    one = o.fluid.clone()
    scale = float(o.bc.abs().max())
    assert float(o.apply_eff(one).abs().max()) <= 1e-13 * scale
    assert max(float(t.abs().max()) for t in o.grad(o.extend(one))) <= 1e-12


def _loss_grad(pr, fwd, grad, u, v, w):
    un, vn, wn = (t.detach().clone().requires_grad_() for t in fwd(u, v, w))
    L = box_kinetic_energy(pr, un, vn, wn)
    lu, lv, lw = torch.autograd.grad(L, [un, vn, wn])
    return float(L), grad(lu, lv, lw)


def _fd_check(pr, fwd, gradient, u, v, w, ndir, seed, h=1e-6, device="cpu"):
    g = torch.Generator().manual_seed(seed)
    L0, (gu, gv, gw) = _loss_grad(pr, fwd, gradient, u, v, w)
    loss = lambda a, b, c: float(box_kinetic_energy(pr, *fwd(a, b, c)))
    worst = 0.0
    for _ in range(ndir):
        du, dv, dw = (_rand(pr.shape, g, device) for _ in range(3))
        fd = (loss(u + h * du, v + h * dv, w + h * dw) - loss(u - h * du, v - h * dv, w - h * dw)) / (2 * h)
        an = float((gu * du).sum() + (gv * dv).sum() + (gw * dw).sum())
        worst = max(worst, abs(fd - an) / abs(an))
    return worst


def test_sparse_reference_gradient_matches_central_differences():
    pr = P.sphere(12, seed=2, stretch=None)
    S = SparseProjection(pr)
    u, v, w = _velocity(pr, 4)
    assert _fd_check(pr, S.forward, S.gradient, u, v, w, ndir=4, seed=5) < 1e-6


# ----------------------------------------------------------------- GPU --
@pytest.mark.gpu
def test_gpu_adjoint_matches_sparse_reference(gpu_built):
    from flow_structure_interaction_fem_ibm_gb300.adjoint import Projection
    pr = P.sphere(24, seed=4, stretch=None)
    S = SparseProjection(pr)
    proj = Projection(pr, "cuda")
    try:
        u, v, w = _velocity(pr, 4)
        ref = S.forward(u, v, w)
        got = proj.forward(*(t.cuda() for t in (u, v, w)))[:3]
        for a, b in zip(got, ref):
            assert float((a.cpu() - b).norm() / b.norm()) < 1e-9
        g = torch.Generator().manual_seed(7)
        lam = [_rand(pr.shape, g) for _ in range(3)]
        gref = S.gradient(*lam)
        ggpu = proj.backward(*(t.cuda() for t in lam))
        for a, b in zip(ggpu, gref):
            assert float((a.cpu() - b).norm() / b.norm()) < 1e-8
    finally:
        proj.close()


@pytest.mark.gpu
def test_gpu_adjoint_matches_central_differences(gpu_built):
    from flow_structure_interaction_fem_ibm_gb300.adjoint import Projection
    pr = P.sphere(32, seed=4, stretch=1.5)
    proj = Projection(pr, "cuda")
    try:
        u, v, w = _velocity(pr, 4, "cuda")
        fwd = lambda a, b, c: proj.forward(a, b, c)[:3]
        assert _fd_check(pr, fwd, proj.backward, u, v, w, ndir=3, seed=9, device="cuda") < 1e-6
    finally:
        proj.close()


@pytest.mark.gpu
def test_gpu_rollout_checkpointing_recomputes_the_same_gradient(gpu_built):
    from flow_structure_interaction_fem_ibm_gb300.adjoint import Projection, rollout
    pr = P.sphere(16, seed=4, stretch=1.5)
    proj = Projection(pr, "cuda")
    try:
        u0, v0, w0 = _velocity(pr, 6, "cuda")
        g = torch.Generator().manual_seed(3)
        forcing = [0.1 * _rand(pr.shape, g, "cuda") for _ in range(3)]
        grads = []
        for every in (0, 2):
            u, v, w = (t.clone().requires_grad_() for t in (u0, v0, w0))
            un, vn, wn = rollout(u, v, w, proj, steps=4, forcing=forcing, checkpoint_every=every)
            L = box_kinetic_energy(pr, un, vn, wn)
            grads.append(torch.autograd.grad(L, [u, v, w]))
        for a, b in zip(*grads):
            assert float((a - b).norm() / b.norm()) < 1e-10
    finally:
        proj.close()
