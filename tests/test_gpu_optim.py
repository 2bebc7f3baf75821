"""GPU: multi-plane phase-hologram optimisation (hand-written adjoint, per-plane
recomputation).  Loss and gradient against the FP64 oracle, central finite
differences on a 256 x 256 crop, a torch.autograd.Function built on the
forward / adjoint C-ABI (test harness only), Adam against a numpy Adam on
oracle gradients, and checkpoint / resume."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2

pytestmark = pytest.mark.gpu
P, LAM = 6.4e-6, 532e-9


def problem(n=256, planes=3, seed=11):
    rng = np.random.default_rng(seed)
    phi = (2 * np.pi * rng.random((n, n))).astype(np.float32)
    t = og.make_targets(n, n, planes, seed=seed + 1)
    zs = [0.08 + 0.01 * k for k in range(planes)]
    return phi, t, zs


def test_loss_and_gradient_vs_fp64_oracle():
    phi, t, zs = problem()
    loss, grad = og.phase_loss_grad(torch.from_numpy(phi).cuda(), torch.from_numpy(t).cuda(), zs, dy=P, dx=P, lam=LAM)
    L, G = O.phase_loss_grad(phi, t, zs, P, LAM)
    assert abs(loss.item() - L) / L < 1e-5
    assert rel_l2(grad.cpu().numpy(), G) < 1e-4


def test_gradient_vs_central_finite_differences():
    """256 x 256 crop, central differences of the FP64 loss, h = 1e-3 rad."""
    phi, t, zs = problem(planes=2, seed=3)
    _, grad = og.phase_loss_grad(torch.from_numpy(phi).cuda(), torch.from_numpy(t).cuda(), zs, dy=P, dx=P, lam=LAM)
    g = grad.cpu().numpy()
    rng = np.random.default_rng(0)
    idx = [tuple(x) for x in rng.integers(0, 256, (8, 2))] + [(128, 128), (0, 0)]
    h = 1e-3
    for (i, j) in idx:
        a = phi.astype(np.float64)
        ap, am = a.copy(), a.copy()
        ap[i, j] += h
        am[i, j] -= h
        fd = (O.phase_loss(ap, t, zs, P, LAM) - O.phase_loss(am, t, zs, P, LAM)) / (2 * h)
        assert abs(fd - g[i, j]) <= 2e-3 * max(abs(fd), 1e-3 * np.abs(g).max()), (i, j, fd, g[i, j])


class AsmFn(torch.autograd.Function):
    """Test-harness autograd wrapper: forward = ASM, backward = its adjoint (C-ABI)."""

    @staticmethod
    def forward(ctx, u, z):
        ctx.z = z
        return og.asm_prop(u.contiguous(), torch.empty_like(u), dy=P, dx=P, lam=LAM, z=z)

    @staticmethod
    def backward(ctx, gout):
        # torch's convention for complex tensors: grad = dL/dconj(u), so the adjoint applies
        return og.asm_prop(gout.contiguous(), torch.empty_like(gout), dy=P, dx=P, lam=LAM, z=ctx.z, adjoint=True), None


def test_autograd_function_matches_fused_gradient():
    phi, t, zs = problem(planes=2, seed=5)
    ph = torch.from_numpy(phi).cuda().requires_grad_(True)
    tt = torch.from_numpy(t).cuda()
    u = torch.polar(torch.ones_like(ph), ph)
    loss = 0
    for k, z in enumerate(zs):
        v = AsmFn.apply(u, z)
        loss = loss + torch.mean((v.real ** 2 + v.imag ** 2 - tt[k]) ** 2)
    loss.backward()
    l2, g2 = og.phase_loss_grad(ph.detach(), tt, zs, dy=P, dx=P, lam=LAM)
    assert abs(loss.item() - l2.item()) / l2.item() < 1e-5
    assert rel_l2(ph.grad.cpu().numpy(), g2.cpu().numpy()) < 1e-4


def test_adam_matches_numpy_adam_on_oracle_gradients_and_resumes(tmp_path):
    phi, t, zs = problem(planes=2, seed=9)
    opt = og.PhaseOptimizer(torch.from_numpy(phi.copy()).cuda(), torch.from_numpy(t).cuda(), zs, dy=P, dx=P, lam=LAM,
                            lr=0.05)
    a = phi.astype(np.float64)
    m = np.zeros_like(a)
    v = np.zeros_like(a)
    b1, b2, eps = 0.9, 0.999, 1e-8
    losses = []
    for step in range(1, 4):
        L, G = O.phase_loss_grad(a, t, zs, P, LAM)
        m = b1 * m + (1 - b1) * G
        v = b2 * v + (1 - b2) * G * G
        a = a - 0.05 * (m / (1 - b1 ** step)) / (np.sqrt(v / (1 - b2 ** step)) + eps)
        losses.append(opt.step().item())
        assert abs(losses[-1] - L) / L < 1e-4
    assert np.abs(opt.phi.cpu().numpy() - a).max() < 2e-3
    # checkpoint after 3 steps, continue 2 more; a resumed optimiser must land on the same phase
    opt.save(tmp_path / "ckpt.npz")
    for _ in range(2):
        opt.step()
    fresh = og.PhaseOptimizer(torch.zeros_like(opt.phi), torch.from_numpy(t).cuda(), zs, dy=P, dx=P, lam=LAM, lr=0.05)
    fresh.load(tmp_path / "ckpt.npz")
    assert fresh.t == 3
    for _ in range(2):
        fresh.step()
    torch.cuda.synchronize()
    assert torch.equal(fresh.phi, opt.phi)


def test_adam_decreases_loss():
    phi, t, zs = problem(n=512, planes=4, seed=21)
    opt = og.PhaseOptimizer(torch.from_numpy(phi).cuda(), torch.from_numpy(t).cuda(), zs, dy=P, dx=P, lam=LAM, lr=0.1)
    first = opt.step().item()
    for _ in range(30):
        last = opt.step().item()
    assert last < 0.8 * first
