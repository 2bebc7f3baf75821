"""GPU: ASM propagation of fields held in pinned (page-locked) host memory.

olg_host_device_pointer maps a pinned host field into the device address
space; pass 1 then reads the input and pass 3 writes the output over the host
link (NVLink-C2C on GB300) with no staging copies.  These are the same
kernels as for device fields, so the results must be the same values, and
within the 1e-5 relative-L2 gate of the FP64 oracle."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def test_asm_on_pinned_host_fields():
    ny, nx, kw = 512, 384, dict(dy=8e-6, dx=8e-6, lam=532e-9, z=0.03)
    rng = np.random.default_rng(21)
    u0 = ((rng.random((ny, nx)) < 0.5) * np.exp(2j * np.pi * rng.random((ny, nx)))).astype(np.complex64)
    ref_dev = og.asm_prop(torch.from_numpy(u0).cuda(), torch.empty((ny, nx), dtype=torch.complex64, device="cuda"),
                          **kw)
    hin = torch.from_numpy(u0).pin_memory()
    hout = torch.empty_like(hin).pin_memory()
    og.asm_prop(hin, hout, **kw)
    torch.cuda.synchronize()
    assert torch.equal(hout, ref_dev.cpu())
    ref = O.asm_prop(u0.astype(np.complex128), kw["dy"], kw["dx"], kw["lam"], kw["z"])
    assert rel_l2(hout.numpy().astype(np.complex128), ref) < 1e-5
    h2 = torch.from_numpy(u0.copy()).pin_memory()  # in place
    og.asm_prop(h2, **kw)
    torch.cuda.synchronize()
    assert torch.equal(h2, ref_dev.cpu())
    with pytest.raises(TypeError):  # pageable host memory is not taken
        og.asm_prop(torch.from_numpy(u0.copy()), **kw)
