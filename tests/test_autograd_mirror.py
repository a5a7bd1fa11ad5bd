"""The forward/backward pair of the C ABI as a torch.autograd.Function (test harness only):
rdxg_metric is the forward, rdxg_gradient with the exact adjoint the backward.  Checked on
the adjoint-check workload (88x88, 3 channels x 8 frames, 36 KL modes) against directional
central differences of the FP64 oracle, through the constraint map into the free
parameters (Constraints::apply, constraints.hpp:128-133, against the oracle's), and by a
few descent steps of torch's own optimiser (marked gpu)."""
import numpy as np
import pytest

import oracle
from redux_gb300 import solver as S
from tests.conftest import workload

torch = pytest.importorskip("torch")

pytestmark = pytest.mark.gpu


class MomfbdMetric(torch.autograd.Function):
    """L(alpha) per patch through rdxg_metric; dL/dalpha through rdxg_gradient (exact)."""

    @staticmethod
    def forward(ctx, alpha, solver):
        ctx.solver = solver
        ctx.save_for_backward(alpha)
        L = solver.metric(alpha.detach().cpu().numpy().astype(np.float64))
        return torch.from_numpy(L).to(alpha.dtype)

    @staticmethod
    def backward(ctx, grad_L):
        (alpha,) = ctx.saved_tensors
        g, _ = ctx.solver.gradient(alpha.detach().cpu().numpy().astype(np.float64), "exact")
        return torch.from_numpy(g).to(alpha.dtype) * grad_L.view(-1, 1, 1), None


@pytest.fixture(scope="module")
def setup():
    w = workload("adjoint88", n_patches=1)
    s = S.Solver(w.job, max_patches=1)
    s.set_patches(w.patches.cutouts, None, w.patches.fixed_gamma)
    op = oracle.OraclePatch(w.job)
    op.set_images(w.patches.cutouts[0], None, None)
    yield w, s, op
    s.close()


def test_backward_is_the_directional_derivative(setup):
    w, s, op = setup
    rng = np.random.default_rng(7)
    a0 = w.patches.alpha_true * 0.5
    alpha = torch.tensor(a0, dtype=torch.float64, requires_grad=True)
    MomfbdMetric.apply(alpha, s).sum().backward()
    g = alpha.grad.numpy()[0]
    h = 1e-4 * w.job.wavelength
    for _ in range(3):
        v = rng.standard_normal(a0.shape[1:])
        v /= np.linalg.norm(v)
        fd = (op.metric(a0[0] + h * v) - op.metric(a0[0] - h * v)) / (2 * h)
        assert abs(np.sum(g * v) - fd) <= 1e-4 * abs(fd), (np.sum(g * v), fd)


def test_chain_through_the_constraint_map(setup):
    """alpha = N beta as a sparse product in torch: autograd's dL/dbeta equals the oracle's
    Constraints::apply of dL/dalpha."""
    w, s, op = setup
    ns = w.job.nullspace
    I, M = w.job.n_images, w.job.n_modes
    Nmat = torch.sparse_coo_tensor(np.stack([ns.rows, ns.cols]), ns.vals, (I * M, ns.n_free), dtype=torch.float64)
    rng = np.random.default_rng(8)
    beta = torch.tensor(1e-3 * w.job.wavelength * rng.standard_normal(ns.n_free), requires_grad=True)
    alpha = torch.sparse.mm(Nmat, beta[:, None])[:, 0].view(1, I, M)
    alpha.retain_grad()
    MomfbdMetric.apply(alpha, s).sum().backward()
    ref = op.cons_apply(alpha.grad.numpy()[0].ravel())
    np.testing.assert_allclose(beta.grad.numpy(), ref, rtol=1e-10, atol=1e-12 * np.abs(ref).max())


def test_torch_optimiser_descends(setup):
    """A step along the negative gradient lowers the metric by the first-order amount, and
    torch's SGD with that step keeps lowering it."""
    w, s, op = setup
    alpha = torch.zeros((1, w.job.n_images, w.job.n_modes), dtype=torch.float64, requires_grad=True)
    L = MomfbdMetric.apply(alpha, s).sum()
    L.backward()
    L0, g2 = float(L.detach()), float((alpha.grad ** 2).sum())
    t = 1e-5 * L0 / g2                        # a predicted decrease of 1e-5 of the metric
    with torch.no_grad():
        L1 = float(MomfbdMetric.apply(alpha - t * alpha.grad, s).sum())
    ratio = (L0 - L1) / (t * g2)
    assert 0.8 < ratio < 1.2, ratio
    opt = torch.optim.SGD([alpha], lr=t)
    losses = [L0]
    for _ in range(3):
        opt.zero_grad()
        L = MomfbdMetric.apply(alpha, s).sum()
        L.backward()
        opt.step()
        with torch.no_grad():
            losses.append(float(MomfbdMetric.apply(alpha, s).sum()))
    assert all(b < a for a, b in zip(losses, losses[1:])), losses
    # the device metric at the optimiser's point agrees with the FP64 oracle
    Lo = op.metric(alpha.detach().numpy()[0])
    assert abs(losses[-1] - Lo) <= 1e-5 * abs(Lo)
