"""GPU parity: fused ASM / Fresnel / ARSS propagation through the C-ABI against
the reference's golden vectors and the FP64 oracle.  Gate: relative L2 <= 1e-5
(FP32 path vs FP64)."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def dev(u):
    return torch.from_numpy(np.ascontiguousarray(u, np.complex64)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().astype(np.complex128)


def c64(u):
    """the complex64 values the GPU sees, as complex128 for the oracle"""
    return np.asarray(u, np.complex64).astype(np.complex128)


def field(rng, shape):
    return (rng.random(shape) < 0.5) * np.exp(2j * np.pi * rng.random(shape))


POW2 = [0, 1, 2, 3, 4]  # golden cases with power-of-two sizes


@pytest.mark.parametrize("i", POW2)
def test_asm_golden(golden, i):
    ny, nx, dy, dx, lam, z = golden[f"prop{i}_params"]
    u = dev(golden[f"prop{i}_in"])
    og.gAsmProp(u, int(ny), int(nx), dy, dx, lam, z)
    assert rel_l2(host(u), golden[f"prop{i}_asm"]) < TOL


@pytest.mark.parametrize("i", POW2)
def test_fresnel_golden(golden, i):
    ny, nx, dy, dx, lam, z = golden[f"prop{i}_params"]
    u = dev(golden[f"prop{i}_in"])
    og.gFresnelProp(u, int(ny), int(nx), dy, dx, lam, z)
    assert rel_l2(host(u), golden[f"prop{i}_fresnel"]) < TOL
    # the CPU band limit (separate x / y limits, olprop.h:26-50)
    u = dev(golden[f"prop{i}_in"])
    og.fresnel_prop(u, dy=dy, dx=dx, lam=lam, z=z, bandlimit=2)
    assert rel_l2(host(u), golden[f"prop{i}_fresnel_bl"]) < TOL


@pytest.mark.parametrize("i", [0, 1, 2])
def test_auto_golden(golden, i):
    ny, nx, dy, dx, lam, z = golden[f"auto{i}_params"]
    u = dev(golden[f"auto{i}_in"])
    og.Prop(u, int(ny), int(nx), dy, dx, lam, z, single_precision=False, verbose=False)
    a, f = golden[f"auto{i}_branch"]
    assert og.Prop.last_choice == (0 if a else (1 if f else 2))
    if og.Prop.last_choice == 2:
        # the CPU dispatcher's band limit uses x and y limits (equal here: dy == dx)
        assert dy == dx
    assert rel_l2(host(u), golden[f"auto{i}_out"]) < TOL


def test_asm_workload_1024():
    """ASM at the benchmark size: 1024^2 -> 2048^2, p = 8 um, lambda = 532 nm, z = 50 mm."""
    rng = np.random.default_rng(20261204)
    u0 = field(rng, (1024, 1024)).astype(np.complex64)
    u = dev(u0)
    og.asm_prop(u, dy=8e-6, dx=8e-6, lam=532e-9, z=0.05)
    ref = O.asm_prop(c64(u0), 8e-6, 8e-6, 532e-9, 0.05)
    g = host(u)
    assert rel_l2(g, ref) < TOL
    assert rel_l2(np.abs(g) ** 2, np.abs(ref) ** 2) < TOL


# t = lambda^2 (u^2 + v^2) at the grid's corner: 0.0147 (just under the 1/64
# above which the phase remainder is evaluated in closed form instead of by
# its series; z / lambda = 3.8e5) and 0.089 (the closed form)
@pytest.mark.parametrize("p,lam,z", [(3.1e-6, 532e-9, 0.2), (1.5e-6, 633e-9, 0.01)])
@pytest.mark.parametrize("shape", [(256, 256), (128, 512)])
def test_asm_phase_remainder_forms_vs_oracle(p, lam, z, shape):
    rng = np.random.default_rng(int(p * 1e9) + shape[1])
    u0 = field(rng, shape).astype(np.complex64)
    u = dev(u0)
    og.asm_prop(u, dy=p, dx=p, lam=lam, z=z)
    assert rel_l2(host(u), O.asm_prop(c64(u0), p, p, lam, z)) < TOL


@pytest.mark.parametrize("shape", [(32, 32), (64, 256), (512, 128), (256, 256)])
@pytest.mark.parametrize("z", [0.02, -0.035])
def test_all_methods_vs_oracle(shape, z):
    rng = np.random.default_rng(abs(hash((shape, z))) % 2**32)
    u0 = field(rng, shape).astype(np.complex64)
    dy, dx, lam = 6e-6, 8e-6, 633e-9
    for kind in ("asm", "fresnel", "fresnel_bl1", "arss", "arss2"):
        u = dev(u0)
        if kind == "asm":
            og.asm_prop(u, dy=dy, dx=dx, lam=lam, z=z)
            ref = O.asm_prop(c64(u0), dy, dx, lam, z)
        elif kind == "fresnel":
            og.fresnel_prop(u, dy=dy, dx=dx, lam=lam, z=z)
            ref = O.fresnel_prop(c64(u0), dy, dx, lam, z)
        elif kind == "fresnel_bl1":
            og.fresnel_prop(u, dy=dy, dx=dx, lam=lam, z=z / 10, bandlimit=1)
            ref = O.fresnel_prop(c64(u0), dy, dx, lam, z / 10, bandlimit=1)
        elif kind == "arss":
            og.arss_prop(u, dy=dy, dx=dx, lam=lam, z=z, s=0.5)
            ref = O.arss_prop(c64(u0), dy, dx, lam, z, 0.5)
        else:
            og.arss_prop(u, dy=dy, dx=dx, lam=lam, z=z, s=2.0, oy=3e-4, ox=-5e-4)
            ref = O.arss_prop(c64(u0), dy, dx, lam, z, 2.0, 3e-4, -5e-4)
        assert rel_l2(host(u), ref) < TOL, kind


@pytest.mark.parametrize("kind", ["asm", "fresnel", "arss"])
def test_adjoints_vs_oracle(kind):
    rng = np.random.default_rng(5)
    u0 = (rng.standard_normal((128, 256)) + 1j * rng.standard_normal((128, 256))).astype(np.complex64)
    u = dev(u0)
    if kind == "asm":
        og.asm_prop(u, dy=8e-6, dx=8e-6, lam=532e-9, z=0.04, adjoint=True)
        ref = O.asm_prop(c64(u0), 8e-6, 8e-6, 532e-9, 0.04, flags=1)
    elif kind == "fresnel":
        og.fresnel_prop(u, dy=8e-6, dx=8e-6, lam=532e-9, z=0.04, adjoint=True)
        ref = O.fresnel_prop(c64(u0), 8e-6, 8e-6, 532e-9, 0.04, flags=1)
    else:
        og.arss_prop(u, dy=8e-6, dx=8e-6, lam=532e-9, z=0.06, s=0.25, oy=1e-4, ox=2e-4, adjoint=True)
        ref = O.arss_prop(c64(u0), 8e-6, 8e-6, 532e-9, 0.06, 0.25, 1e-4, 2e-4, flags=1)
    assert rel_l2(host(u), ref) < TOL


def test_host_overload_conventions():
    """Host-pointer overloads omit 1/Np (golprop.h:458-504, 70-124)."""
    rng = np.random.default_rng(9)
    u0 = field(rng, (64, 64)).astype(np.complex64)
    a = u0.copy()
    og.gAsmProp(a, 64, 64, 8e-6, 8e-6, 532e-9, 0.03)
    assert rel_l2(a, O.asm_prop(c64(u0), 8e-6, 8e-6, 532e-9, 0.03, flags=2)) < TOL
    f = u0.copy()
    og.gFresnelProp(f, 64, 64, 8e-6, 8e-6, 532e-9, 0.03)
    assert rel_l2(f, O.fresnel_prop(c64(u0), 8e-6, 8e-6, 532e-9, 0.03, flags=2)) < TOL


def test_out_of_place_and_workspace_reuse():
    rng = np.random.default_rng(2)
    u0 = field(rng, (256, 512)).astype(np.complex64)
    src = dev(u0)
    dst = torch.empty_like(src)
    ws = og.workspace(256, 512)
    for _ in range(2):
        og.asm_prop(src, dst, dy=8e-6, dx=8e-6, lam=532e-9, z=0.05, work=ws)
    assert np.array_equal(host(src), c64(u0))
    assert rel_l2(host(dst), O.asm_prop(c64(u0), 8e-6, 8e-6, 532e-9, 0.05)) < TOL


def test_linearity_and_adjoint_identity_full_size():
    """Size-independent properties at the WRP step-2 size (4096^2 -> 8192^2):
    linearity and <A x, y> = <x, A^H y>."""
    g = torch.Generator(device="cuda").manual_seed(1)
    n = 4096
    x = torch.randn((n, n), dtype=torch.complex64, device="cuda", generator=g)
    y = torch.randn((n, n), dtype=torch.complex64, device="cuda", generator=g)
    p = dict(dy=4e-6, dx=4e-6, lam=532e-9, z=0.15)
    Ax = og.asm_prop(x, torch.empty_like(x), **p)
    Ahy = og.asm_prop(y, torch.empty_like(y), adjoint=True, **p)
    lhs = torch.vdot(y.flatten(), Ax.flatten()).item()
    rhs = torch.vdot(Ahy.flatten(), x.flatten()).item()
    assert abs(lhs - rhs) / abs(lhs) < 1e-4
    A2x = og.asm_prop(2 * x - 3j * y, torch.empty_like(x), **p)
    Ay = og.asm_prop(y, torch.empty_like(y), **p)
    err = torch.linalg.vector_norm(A2x - (2 * Ax - 3j * Ay)) / torch.linalg.vector_norm(A2x)
    assert err.item() < 1e-5


def test_errors_raise():
    u = torch.zeros((14, 64), dtype=torch.complex64, device="cuda")  # 2 * 14 = 4 * 7: no plan
    with pytest.raises(og.OlgError):
        og.asm_prop(u, dy=8e-6, dx=8e-6, lam=532e-9, z=0.05)
    v = torch.zeros((64, 64), dtype=torch.complex64, device="cuda")
    with pytest.raises(og.OlgError):
        og.arss_prop(v, dy=8e-6, dx=8e-6, lam=532e-9, z=0.05, s=1.0)

