"""GPU parity at the production shapes of the phase-optimisation and batch
configurations, where the smaller tests do not reach:

* phase optimisation: a 2048 x 2048 phase, 8 planes at z = 80..150 mm,
  p = 6.4 um, 532 nm, 5 % sparse targets -- the shared forward spectrum and
  summed adjoint spectrum of the 4096 x 4096 padded grid.  Loss and gradient
  of one step against the FP64 oracle on the whole field.
* batch: the 96-field draw of the benchmark (sizes 512^2..4096^2, ASM /
  Fresnel / ARSS, z in [10, 300] mm, RGB wavelengths, p = 8 um) in one plan
  as the benchmark runs it -- the persistent kernel for the fields below
  2048^2 and the single-field passes for the 2048^2 and 4096^2 fields -- with
  one field of every (size, method) pair checked against the FP64 oracle.

Gates: relative L2 1e-5 for propagated fields (FP32 path vs FP64).  The
gradient is held to 1e-4: it is -2 Im(u conj(g)) with g the adjoint of the
seed (2/n)(|v|^2 - t) v, and the residual |v|^2 - t carries the FP32
rounding of |v|^2 (relative 1e-7..1e-6 of the intensity) wherever it is
small against |v|^2, so the gradient's relative error is the field's
multiplied by |v|^2 / |r|; the loss itself holds 1e-5."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_phase_step_at_config_size():
    n, planes, p, lam = 2048, 8, 6.4e-6, 532e-9
    rng = np.random.default_rng(20261203 + 4)
    phi = (2 * np.pi * rng.random((n, n))).astype(np.float32)
    t = og.make_targets(n, n, planes, seed=20261203 + 5)
    zs = [0.08 + 0.01 * k for k in range(planes)]
    loss, grad = og.phase_loss_grad(torch.from_numpy(phi).cuda(), torch.from_numpy(t).cuda(), zs, dy=p, dx=p, lam=lam)
    torch.cuda.synchronize()
    L, G = O.phase_loss_grad(phi, t, zs, p, lam)
    assert abs(loss.item() - L) / L < 1e-5
    assert rel_l2(grad.cpu().numpy(), G) < 1e-4


def _oracle(f, u):
    if f["method"] == "asm":
        return O.asm_prop(u, f["dy"], f["dx"], f["lam"], f["z"])
    if f["method"] == "fresnel":
        return O.fresnel_prop(u, f["dy"], f["dx"], f["lam"], f["z"])
    return O.arss_prop(u, f["dy"], f["dx"], f["lam"], f["z"], f["s"])


def test_batch_at_config_size():
    fields = og.config5_fields()
    assert len(fields) == 96
    plan = og.BatchPlan(fields)
    assert plan.n_direct > 0 and plan.n_items > 0   # both paths run
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            plan.execute(stream=s)
    g.replay()
    torch.cuda.synchronize()
    plan.check()
    checked = {}
    for k, f in enumerate(fields):
        key = (f["u_in"].shape[0], f["method"])
        if key in checked:
            continue
        u = f["u_in"].cpu().numpy().astype(np.complex128)
        checked[key] = rel_l2(f["u_out"].cpu().numpy(), _oracle(f, u))
    plan.close()
    assert len(checked) == 12, sorted(checked)   # 4 sizes x 3 methods
    bad = {k: v for k, v in checked.items() if not v < 1e-5}
    assert not bad, bad
