"""GPU: every launch variant of the three propagation passes (the shapes the
autotuner chooses among) gives the FP64 oracle's result, and the autotuner
runs and keeps a valid choice."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("shape", [(128, 256), (512, 512), (1024, 512), (2048, 1024), (64, 4096), (4096, 64)])
def test_every_launch_variant_matches_oracle(shape):
    ny, nx = shape
    rng = np.random.default_rng(ny + nx)
    u0 = ((rng.random(shape) < 0.5) * np.exp(2j * np.pi * rng.random(shape))).astype(np.complex64)
    uc = u0.astype(np.complex128)
    ref_asm = O.asm_prop(uc, 6e-6, 8e-6, 532e-9, 0.04)
    ref_arss = O.arss_prop(uc, 6e-6, 8e-6, 532e-9, 0.04, 0.5, 1e-4, -2e-4)
    # lengths below 256 have one fixed launch shape (no variants)
    lens = {k: n for k, n in {0: 2 * nx, 1: 2 * ny, 2: 2 * nx}.items() if n >= 256}
    tried = 0
    try:
        for kind, n in lens.items():
            for i in range(og.variant_count()):
                try:
                    og.set_variant(kind, n, i)
                except og.OlgError:
                    continue
                tried += 1
                src = torch.from_numpy(u0).cuda()
                a = og.asm_prop(src, torch.empty_like(src), dy=6e-6, dx=8e-6, lam=532e-9, z=0.04)
                b = og.arss_prop(src, torch.empty_like(src), dy=6e-6, dx=8e-6, lam=532e-9, z=0.04, s=0.5, oy=1e-4,
                                 ox=-2e-4)
                torch.cuda.synchronize()
                assert rel_l2(a.cpu().numpy(), ref_asm) < 1e-5, (kind, n, i)
                assert rel_l2(b.cpu().numpy(), ref_arss) < 1e-5, (kind, n, i)
            og.set_variant(kind, n, 0)
    finally:
        for kind, n in lens.items():
            og.set_variant(kind, n, 0)
    assert tried >= 2 * len(lens)


def test_autotune_keeps_a_valid_variant():
    chosen = og.autotune(1024, 1024, reps=2)
    for (kind, n), i in chosen.items():
        assert 0 <= i < og.variant_count()
    u = torch.ones((1024, 1024), dtype=torch.complex64, device="cuda")
    og.asm_prop(u, dy=8e-6, dx=8e-6, lam=532e-9, z=0.05)
    torch.cuda.synchronize()
    for kind, n in ((0, 2048), (1, 2048), (2, 2048)):
        og.set_variant(kind, n, 0)
