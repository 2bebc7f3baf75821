"""GPU: propagation at sizes whose padded lengths are not powers of two
(2n = 2^a 3^b 5^c), through the mixed-radix passes, against the reference's
golden vectors and the FP64 oracle."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def field(rng, shape):
    return ((rng.random(shape) < 0.5) * np.exp(2j * np.pi * rng.random(shape))).astype(np.complex64)


def dev(u):
    return torch.from_numpy(np.ascontiguousarray(u, np.complex64)).cuda()


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().astype(np.complex128)


def test_reference_golden_24x40(golden):
    """The reference's own outputs on a 24 x 40 field (padded 48 x 80)."""
    i = 5
    ny, nx, dy, dx, lam, z = golden[f"prop{i}_params"]
    assert (int(ny), int(nx)) == (24, 40)
    u = golden[f"prop{i}_in"]
    a = og.asm_prop(dev(u), dy=dy, dx=dx, lam=lam, z=z)
    assert rel_l2(host(a), golden[f"prop{i}_asm"]) < TOL
    f = og.fresnel_prop(dev(u), dy=dy, dx=dx, lam=lam, z=z)
    assert rel_l2(host(f), golden[f"prop{i}_fresnel"]) < TOL
    b = og.fresnel_prop(dev(u), dy=dy, dx=dx, lam=lam, z=z, bandlimit=2)
    assert rel_l2(host(b), golden[f"prop{i}_fresnel_bl"]) < TOL


@pytest.mark.parametrize("shape", [(1080, 1920), (600, 800), (512, 720), (360, 256), (96, 160)])
def test_asm_mixed_sizes(shape):
    ny, nx = shape
    u = field(np.random.default_rng(ny + nx), shape)
    ref = O.asm_prop(u.astype(np.complex128), 8e-6, 8e-6, 532e-9, 0.05)
    out = og.asm_prop(dev(u), torch.empty(shape, dtype=torch.complex64, device="cuda"), dy=8e-6, dx=8e-6,
                      lam=532e-9, z=0.05)
    assert rel_l2(host(out), ref) < TOL


def test_asm_reference_default_field():
    """The reference's default test field (tests/para.h: 3840 x 2160, p = 3.74 um,
    532 nm, d = -0.1 m): padded 7680 x 4320, the compile-time mixed-radix plans."""
    shape = (2160, 3840)
    u = field(np.random.default_rng(7), shape)
    ref = O.asm_prop(u.astype(np.complex128), 3.74e-6, 3.74e-6, 532e-9, -0.1)
    out = og.asm_prop(dev(u), torch.empty(shape, dtype=torch.complex64, device="cuda"), dy=3.74e-6, dx=3.74e-6,
                      lam=532e-9, z=-0.1)
    assert rel_l2(host(out), ref) < TOL


@pytest.mark.parametrize("shape", [(720, 1280), (1440, 2560)])
def test_asm_hd_and_qhd_fields(shape):
    """1280 x 720 and 2560 x 1440 fields (padded lengths 2560, 1440 and 5120,
    2880: compile-time plans)."""
    u = field(np.random.default_rng(shape[1]), shape)
    ref = O.asm_prop(u.astype(np.complex128), 5e-6, 5e-6, 532e-9, 0.08)
    out = og.asm_prop(dev(u), torch.empty(shape, dtype=torch.complex64, device="cuda"), dy=5e-6, dx=5e-6,
                      lam=532e-9, z=0.08)
    assert rel_l2(host(out), ref) < TOL
    f = og.fresnel_prop(dev(u), dy=5e-6, dx=5e-6, lam=532e-9, z=0.3)
    assert rel_l2(host(f), O.fresnel_prop(u.astype(np.complex128), 5e-6, 5e-6, 532e-9, 0.3)) < TOL


@pytest.mark.parametrize("kind", ["fresnel", "arss"])
def test_chirp_methods_at_1920x1080(kind):
    """Fresnel and ARSS (chirp spectra in the column pass) at 1920 x 1080."""
    shape = (1080, 1920)
    u = field(np.random.default_rng(11), shape)
    uc = u.astype(np.complex128)
    if kind == "fresnel":
        ref = O.fresnel_prop(uc, 8e-6, 8e-6, 532e-9, 0.2)
        out = og.fresnel_prop(dev(u), dy=8e-6, dx=8e-6, lam=532e-9, z=0.2)
    else:
        ref = O.arss_prop(uc, 8e-6, 8e-6, 532e-9, 0.2, 0.5, 1e-4, -2e-4)
        out = og.arss_prop(dev(u), dy=8e-6, dx=8e-6, lam=532e-9, z=0.2, s=0.5, oy=1e-4, ox=-2e-4)
    assert rel_l2(host(out), ref) < TOL


@pytest.mark.parametrize("shape", [(240, 320), (200, 256)])
def test_fresnel_and_arss_mixed_sizes(shape):
    u = field(np.random.default_rng(3), shape)
    uc = u.astype(np.complex128)
    for bl in (0, 1, 2):
        ref = O.fresnel_prop(uc, 6e-6, 8e-6, 633e-9, 0.03, bandlimit=bl)
        out = og.fresnel_prop(dev(u), dy=6e-6, dx=8e-6, lam=633e-9, z=0.03, bandlimit=bl)
        assert rel_l2(host(out), ref) < TOL, bl
    ref = O.arss_prop(uc, 6e-6, 8e-6, 633e-9, 0.03, 0.5, 1e-4, -2e-4)
    out = og.arss_prop(dev(u), torch.empty(shape, dtype=torch.complex64, device="cuda"), dy=6e-6, dx=8e-6,
                       lam=633e-9, z=0.03, s=0.5, oy=1e-4, ox=-2e-4)
    assert rel_l2(host(out), ref) < TOL


def test_shifted_and_adjoint_mixed_size():
    ny, nx = 150, 240
    rng = np.random.default_rng(9)
    u = field(rng, (ny, nx))
    ref = O.shifted_asm_prop(u.astype(np.complex128), 8e-6, 8e-6, 532e-9, 0.02, 2e-4, -1e-4)
    out = og.shifted_asm_prop(dev(u), torch.empty((ny, nx), dtype=torch.complex64, device="cuda"), dy=8e-6, dx=8e-6,
                              lam=532e-9, z=0.02, oy=2e-4, ox=-1e-4)
    assert rel_l2(host(out), ref) < TOL
    x = field(rng, (ny, nx)).astype(np.complex128)
    y = field(rng, (ny, nx)).astype(np.complex128)
    ax = host(og.asm_prop(dev(x), dy=8e-6, dx=8e-6, lam=532e-9, z=0.02))
    ay = host(og.asm_prop(dev(y), dy=8e-6, dx=8e-6, lam=532e-9, z=0.02, adjoint=True))
    assert abs(np.vdot(y, ax) - np.vdot(ay, x)) <= 1e-5 * abs(np.vdot(y, ax))


def test_unsupported_lengths_are_rejected():
    # 28 = 4 * 7 and 42 = 2 * 3 * 7 have a factor 7; 7776 does not fit one CTA
    for shape in [(14, 64), (64, 21), (3888, 16)]:
        u = torch.zeros(shape, dtype=torch.complex64, device="cuda")
        with pytest.raises(og.OlgError):
            og.asm_prop(u, dy=8e-6, dx=8e-6, lam=532e-9, z=0.05)
