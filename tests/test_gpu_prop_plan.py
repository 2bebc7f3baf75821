"""GPU: single-field propagation plans (olg_prop_plan_*) give the results of
the matching single calls bit for bit -- ASM, Fresnel, band-limited Fresnel
and ARSS, power-of-two and mixed-radix sizes -- over several executions on
different fields, in place and out of place, and against the FP64 oracle."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def field(seed, ny, nx):
    rng = np.random.default_rng(seed)
    return ((rng.random((ny, nx)) < 0.5) * np.exp(2j * np.pi * rng.random((ny, nx)))).astype(np.complex64)


CASES = [
    # method, ny, nx, dy, dx, lam, z, s
    ("asm", 256, 256, 8e-6, 8e-6, 532e-9, 0.05, None),
    ("fresnel", 128, 256, 8e-6, 6e-6, 633e-9, 0.08, None),
    ("fresnel_bandlimit", 256, 128, 8e-6, 8e-6, 450e-9, 0.12, None),
    ("arss", 128, 128, 8e-6, 8e-6, 532e-9, 0.02, 0.5),
    ("asm", 120, 200, 8e-6, 8e-6, 532e-9, 0.03, None),      # mixed radix (240 = 16 * 15, 400 = 16 * 25)
]


def single_call(method, u, out, dy, dx, lam, z, s):
    if method == "asm":
        return og.asm_prop(u, out, dy=dy, dx=dx, lam=lam, z=z)
    if method == "fresnel":
        return og.fresnel_prop(u, out, dy=dy, dx=dx, lam=lam, z=z)
    if method == "fresnel_bandlimit":
        return og.fresnel_prop(u, out, dy=dy, dx=dx, lam=lam, z=z, bandlimit=1)
    return og.arss_prop(u, out, dy=dy, dx=dx, lam=lam, z=z, s=s)


def oracle_of(method, u, dy, dx, lam, z, s):
    u = u.astype(np.complex128)
    if method == "asm":
        return O.asm_prop(u, dy, dx, lam, z)
    if method == "fresnel":
        return O.fresnel_prop(u, dy, dx, lam, z)
    if method == "fresnel_bandlimit":
        return O.fresnel_prop(u, dy, dx, lam, z, bandlimit=1)
    return O.arss_prop(u, dy, dx, lam, z, s)


@pytest.mark.parametrize("case", CASES, ids=[f"{c[0]}-{c[1]}x{c[2]}" for c in CASES])
def test_plan_equals_single_call(case):
    method, ny, nx, dy, dx, lam, z, s = case
    kw = dict(dy=dy, dx=dx, lam=lam, z=z)
    plan = og.PropPlan(method, ny, nx, s=s if s is not None else 0.5, **kw)
    for rep in range(3):
        h = field(100 * rep + ny, ny, nx)
        u = torch.from_numpy(h).cuda()
        want = torch.empty_like(u)
        single_call(method, u, want, dy, dx, lam, z, s)
        got = plan.execute(u, torch.empty_like(u))
        inplace = plan.execute(u.clone())
        torch.cuda.synchronize()
        assert torch.equal(got, want), rep
        assert torch.equal(inplace, want), rep
    assert rel_l2(got.cpu().numpy(), oracle_of(method, h, dy, dx, lam, z, s)) < 1e-5
    with pytest.raises(TypeError):
        plan.execute(torch.zeros((ny, nx + 2), dtype=torch.complex64, device="cuda"))
    plan.close()


@pytest.mark.parametrize("pinned", [True, False], ids=["pinned", "pageable"])
@pytest.mark.parametrize("case", [CASES[0], CASES[3], CASES[4]], ids=["asm", "arss", "asm-mixed-radix"])
def test_plan_host_sequence_equals_device_executions(case, pinned):
    """olg_prop_plan_execute_host: seven host fields (more than the three
    device slots, so slots are reused) give the device executions' results bit
    for bit, and the caller's stream is ordered after the last copy out.
    Pageable host memory gives the same results (its copies do not overlap)."""
    method, ny, nx, dy, dx, lam, z, s = case
    plan = og.PropPlan(method, ny, nx, dy=dy, dx=dx, lam=lam, z=z, s=s if s is not None else 0.5)
    hs = [field(7 * k + ny, ny, nx) for k in range(7)]
    pin = (lambda t: t.pin_memory()) if pinned else (lambda t: t)
    hin = [pin(torch.from_numpy(h)) for h in hs]
    hout = [pin(torch.full((ny, nx), complex(np.nan, np.nan), dtype=torch.complex64)) for _ in hs]
    stream = torch.cuda.Stream()
    with torch.cuda.stream(stream):
        plan.execute_host(hin, hout, stream=stream)
    stream.synchronize()
    for h, got in zip(hs, hout):
        u = torch.from_numpy(h).cuda()
        want = plan.execute(u, torch.empty_like(u))
        torch.cuda.synchronize()
        assert torch.equal(got, want.cpu())
    plan.execute_host([], [])  # an empty sequence is a no-op
