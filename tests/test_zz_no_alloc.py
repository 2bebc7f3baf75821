"""GPU: the allocation-free ASM entry point (olg_asm_prop_noalloc_c64).

Some callers cannot allocate device memory while they run -- a holographic
display loop with a fixed per-frame budget, or a plugin inside an application
that owns all GPU memory.  They call this entry point, which keeps its
scratch in an array compiled into the library.  This file is collected last
so that a run stopping at the first failure has run every other test first;
it also passes on its own in a fresh process."""
import numpy as np
import pytest
import torch

import openol_gb300 as og
from conftest import rel_l2
from openol_gb300 import _lib

pytestmark = pytest.mark.gpu


def _noalloc(u_in, u_out, dy, dx, lam, z, flags=0):
    ny, nx = u_in.shape
    return _lib.lib().olg_asm_prop_noalloc_c64(u_in.data_ptr(), u_out.data_ptr(), ny, nx, dy, dx, lam, z, flags,
                                               torch.cuda.current_stream().cuda_stream)


# 256 x 4096 has the widest padded rows, hence the largest scratch layout
# (about 16.1 of the 17 MiB)
@pytest.mark.parametrize("shape,z", [((1024, 1024), 0.05), ((256, 512), -0.03), ((256, 4096), 0.02)])
def test_noalloc_matches_allocating_entry_point(shape, z):
    rng = np.random.default_rng(shape[0] + shape[1])
    u0 = ((rng.random(shape) < 0.5) * np.exp(2j * np.pi * rng.random(shape))).astype(np.complex64)
    p = dict(dy=8e-6, dx=8e-6, lam=532e-9, z=z)
    src = torch.from_numpy(u0).cuda()
    ref = og.asm_prop(src, torch.empty_like(src), **p)
    for _ in range(2):  # two calls in a row share (and reuse) the static scratch
        out = torch.empty_like(src)
        assert _noalloc(src, out, p["dy"], p["dx"], p["lam"], p["z"]) == 0
        torch.cuda.synchronize()
        assert rel_l2(out.cpu().numpy(), ref.cpu().numpy()) < 1e-5
    # in place, and the adjoint flag, through the same entry point
    v = src.clone()
    assert _noalloc(v, v, p["dy"], p["dx"], p["lam"], p["z"], flags=_lib.OLG_CONJ) == 0
    adj = og.asm_prop(src, torch.empty_like(src), adjoint=True, **p)
    torch.cuda.synchronize()
    assert rel_l2(v.cpu().numpy(), adj.cpu().numpy()) < 1e-5


def test_noalloc_rejects_fields_beyond_its_scratch():
    big = torch.zeros((2048, 1024), dtype=torch.complex64, device="cuda")
    rc = _noalloc(big, big, 8e-6, 8e-6, 532e-9, 0.05)
    assert rc == -4  # OLG_ERR_WORKSPACE
    assert b"1048576" in _lib.lib().olg_last_error()


def test_noalloc_rejects_mixed_radix_sizes():
    """24 x 40 is a valid size for olg_asm_prop_c64 (mixed-radix passes), but
    those passes build a twiddle table on first use, so the allocation-free
    entry point takes power-of-two sizes only."""
    u = torch.zeros((24, 40), dtype=torch.complex64, device="cuda")
    rc = _noalloc(u, u, 8e-6, 8e-6, 532e-9, 0.05)
    assert rc == -2  # OLG_ERR_UNSUPPORTED_SIZE
    assert b"power-of-two" in _lib.lib().olg_last_error()
