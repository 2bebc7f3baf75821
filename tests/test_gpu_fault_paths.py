"""GPU: failure paths, exercised without faulting the GPU.

* A bounded device-side wait that runs out.  The persistent batch kernel
  waits, per item, for the earlier pass of its field (a counter read with
  ld.acquire).  Raising a field's completion target on the host makes those
  waits unsatisfiable; with a short budget (olg_wait_budget_cycles) each wait
  gives up, the kernel records the error, skips the item and returns.  The
  host reads the status (olg_batch_check), and the context stays usable.
* An allocation that fails, injected on the host (olg_inject_alloc_failures):
  the entry point returns OLG_ERR_NOMEM, leaks nothing, and the next call
  succeeds."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2
from openol_gb300 import _lib

pytestmark = pytest.mark.gpu
OLG_ERR_CUDA, OLG_ERR_NOMEM = -3, -5


def small_fields(seed):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(2):
        u = ((rng.random((256, 256)) < 0.5) * np.exp(2j * np.pi * rng.random((256, 256)))).astype(np.complex64)
        t = torch.from_numpy(u).cuda()
        out.append(dict(u_in=t, u_out=torch.empty_like(t), method="asm", dy=8e-6, dx=8e-6, lam=532e-9,
                        z=0.02 + 0.01 * k, host=u))
    return out


def test_batch_wait_runs_out_and_kernel_returns():
    L = _lib.lib()
    fields = small_fields(1)
    plan = og.BatchPlan(fields)
    assert plan.n_items > 0 and plan.n_direct == 0
    # field 0's pass-1 items now wait for one more set-up job than exists
    assert L.olg_batch_plan_raise_target(plan._plan, 0, 0, 1) == 0
    # ~2 ms per wait: every item is taken at once (more CTAs than items), so
    # field 1's last pass legitimately waits through its first two (~0.1 ms);
    # field 0's waits can never be met and each runs the budget out
    prev = L.olg_wait_budget_cycles(4000000)
    try:
        plan.execute()
        torch.cuda.synchronize()                  # the kernel returned
    finally:
        L.olg_wait_budget_cycles(prev)
    assert L.olg_batch_check(plan._plan) == OLG_ERR_CUDA
    assert b"bounded wait" in L.olg_last_error()
    # field 1's waits were all met: it is still right
    ref = O.asm_prop(fields[1]["host"].astype(np.complex128), 8e-6, 8e-6, 532e-9, fields[1]["z"])
    assert rel_l2(fields[1]["u_out"].cpu().numpy(), ref) < 1e-5
    plan.close()
    # the context is still usable: a fresh plan runs clean
    fields = small_fields(2)
    plan = og.BatchPlan(fields)
    plan.execute()
    torch.cuda.synchronize()
    plan.check()
    for f in fields:
        ref = O.asm_prop(f["host"].astype(np.complex128), 8e-6, 8e-6, 532e-9, f["z"])
        assert rel_l2(f["u_out"].cpu().numpy(), ref) < 1e-5
    plan.close()


def test_injected_allocation_failure():
    L = _lib.lib()
    rng = np.random.default_rng(4)
    u0 = ((rng.random((512, 512)) < 0.5) * np.exp(2j * np.pi * rng.random((512, 512)))).astype(np.complex64)
    u = torch.from_numpy(u0).cuda()
    out = torch.empty_like(u)
    stream = torch.cuda.current_stream().cuda_stream
    assert L.olg_inject_alloc_failures(1) == 0
    rc = L.olg_asm_prop_c64(u.data_ptr(), out.data_ptr(), 512, 512, 8e-6, 8e-6, 532e-9, 0.05, 0, None, 0, stream)
    assert rc == OLG_ERR_NOMEM
    assert b"injected" in L.olg_last_error()
    # one failure was injected: the next call allocates and succeeds
    og.asm_prop(u, out, dy=8e-6, dx=8e-6, lam=532e-9, z=0.05)
    torch.cuda.synchronize()
    ref = O.asm_prop(u0.astype(np.complex128), 8e-6, 8e-6, 532e-9, 0.05)
    assert rel_l2(out.cpu().numpy(), ref) < 1e-5
    assert L.olg_inject_alloc_failures(0) == 0
