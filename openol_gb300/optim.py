"""Multi-plane phase-only hologram optimisation with the hand-written adjoint.

phi (ny x nx, float32 radians) is propagated by ASM to P depth planes; the
loss is sum_p mean((|A_p e^{i phi}|^2 - t_p)^2).  Gradients come from
olg_phase_loss_grad / olg_phase_adam_step, with no stored per-plane fields:
the planes share one forward spectrum of e^{i phi}; per plane an inverse
column transform, one row pass that forms the loss, the seed and the seed's
row transform, and a forward column transform summed into the adjoint
spectrum; one inverse transform of that sum gives dL/du*.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import call, lib
from .prop import _stream


def make_targets(ny, nx, n_planes, seed=20261207, density=0.05):
    """Seeded sparse intensity targets: `density` of the pixels U[0, 1], the rest 0."""
    rng = np.random.default_rng(seed)
    t = np.zeros((n_planes, ny, nx), np.float32)
    mask = rng.random((n_planes, ny, nx)) < density
    t[mask] = rng.random(int(mask.sum())).astype(np.float32)
    return t


def _zarr(z):
    z = np.ascontiguousarray(np.asarray(z, np.float64).reshape(-1))
    return z, z.ctypes.data_as(C.POINTER(C.c_double))


def workspace(ny, nx, device="cuda"):
    return torch.empty(int(lib().olg_phase_opt_workspace_bytes(ny, nx)), dtype=torch.uint8, device=device)


def _check(phi, targets):
    if not (phi.is_cuda and phi.dtype == torch.float32 and phi.is_contiguous() and phi.dim() == 2):
        raise TypeError("phi must be a contiguous CUDA float32 (ny, nx) tensor")
    ny, nx = phi.shape
    if not (targets.is_cuda and targets.dtype == torch.float32 and targets.is_contiguous()
            and tuple(targets.shape[1:]) == (ny, nx)):
        raise TypeError("targets must be a contiguous CUDA float32 (planes, ny, nx) tensor")
    return ny, nx


def phase_loss_grad(phi, targets, z, *, dy, dx, lam, grad=None, loss=None, work=None, stream=None):
    """Loss (device float64 scalar tensor) and dL/dphi (float32, ny x nx)."""
    ny, nx = _check(phi, targets)
    zz, zp = _zarr(z)
    if len(zz) != targets.shape[0]:
        raise ValueError("one z per target plane")
    grad = torch.empty_like(phi) if grad is None else grad
    loss = torch.zeros((), dtype=torch.float64, device=phi.device) if loss is None else loss
    wp, wb = (work.data_ptr(), work.numel()) if work is not None else (None, 0)
    call("olg_phase_loss_grad", phi.data_ptr(), targets.data_ptr(), zp, len(zz), ny, nx, float(dy), float(dx),
         float(lam), grad.data_ptr(), loss.data_ptr(), wp, wb, _stream(stream))
    return loss, grad


class PhaseOptimizer:
    """Adam on a phase-only hologram over several depth planes (one call per step)."""

    def __init__(self, phi, targets, z, *, dy, dx, lam, lr=0.05, betas=(0.9, 0.999), eps=1e-8):
        self.ny, self.nx = _check(phi, targets)
        self.phi, self.targets = phi, targets
        self.z, self._zp = _zarr(z)
        self.dy, self.dx, self.lam = float(dy), float(dx), float(lam)
        self.lr, self.betas, self.eps = float(lr), tuple(map(float, betas)), float(eps)
        self.m = torch.zeros_like(phi)
        self.v = torch.zeros_like(phi)
        self.t = 0
        self.loss = torch.zeros((), dtype=torch.float64, device=phi.device)
        self.work = workspace(self.ny, self.nx, phi.device)

    def step(self, stream=None):
        self.t += 1
        call("olg_phase_adam_step", self.phi.data_ptr(), self.m.data_ptr(), self.v.data_ptr(),
             self.targets.data_ptr(), self._zp, len(self.z), self.ny, self.nx, self.dy, self.dx, self.lam, self.lr,
             self.betas[0], self.betas[1], self.eps, self.t, self.loss.data_ptr(), self.work.data_ptr(),
             self.work.numel(), _stream(stream))
        return self.loss

    # checkpoint / resume: phi, Adam moments and the step counter
    def state_dict(self):
        return {"phi": self.phi.detach().cpu().numpy(), "m": self.m.cpu().numpy(), "v": self.v.cpu().numpy(),
                "t": np.int64(self.t)}

    def load_state_dict(self, sd):
        for k in ("phi", "m", "v"):
            getattr(self, k).copy_(torch.from_numpy(np.asarray(sd[k], np.float32)))
        self.t = int(sd["t"])

    def save(self, path):
        save_state(path, self.state_dict())

    def load(self, path):
        self.load_state_dict(load_state(path))


def save_state(path, sd):
    np.savez(path, **sd)


def load_state(path):
    with np.load(path) as f:
        return {k: f[k] for k in f.files}
