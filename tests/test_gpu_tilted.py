"""GPU: tilted-plane propagation (source and reference forms, bilinear and
bicubic, ASM and Fresnel) against the reference's own outputs (golden
fixtures, PREC_T = double) and the FP64 oracle.  Gate: relative L2 <= 1e-5;
the FP32 spectrum and FP32 interpolation weights are the error budget, the
sampling positions are formed in FP64 as the reference forms them."""
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


def test_tilted_golden(golden):
    for i in range(int(golden["n_tilt"])):
        ny, nx, dy, dx, lam, z, ang, ip, mode, refm = golden[f"tilt{i}_params"]
        ny, nx = int(ny), int(nx)
        u = dev(golden[f"tilt{i}_in"])
        out = og.tilted_prop(u, torch.empty_like(u), dy=dy, dx=dx, lam=lam, z=z, angle=ang, interp=int(ip),
                             propmode=int(mode), reference=bool(refm))
        assert rel_l2(host(out), golden[f"tilt{i}_out"]) < TOL, i


CASES = [
    # ny, nx, dy, dx, lam, z, angle (source form), angle (reference form)
    (256, 256, 8e-6, 8e-6, 532e-9, 0.05, 0.12, 2e-3),
    (200, 240, 6e-6, 8e-6, 633e-9, 0.03, -0.25, -3e-3),
    (128, 512, 8e-6, 8e-6, 532e-9, -0.02, 0.05, 1e-3),
]


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("interp", [0, 1])
@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("refm", [False, True])
def test_tilted_matches_oracle(case, interp, mode, refm):
    ny, nx, dy, dx, lam, z, a_src, a_ref = case
    ang = a_ref if refm else a_src
    u = field(np.random.default_rng(ny + nx + interp + 2 * mode), (ny, nx))
    ref = O.tilted_prop(u.astype(np.complex128), dy, dx, lam, z, ang, interp, mode, refm)
    out = og.tilted_prop(dev(u), torch.empty((ny, nx), dtype=torch.complex64, device="cuda"), dy=dy, dx=dx, lam=lam,
                         z=z, angle=ang, interp=interp, propmode=mode, reference=refm)
    assert rel_l2(host(out), ref) < TOL


def test_tilted_in_place_and_mirrors():
    ny, nx, dy, dx, lam, z, ang = 64, 96, 8e-6, 8e-6, 532e-9, 0.02, 0.1
    u = field(np.random.default_rng(5), (ny, nx))
    ref = O.tilted_prop(u.astype(np.complex128), dy, dx, lam, z, ang, 1, 0, False)
    d = dev(u)
    og.TiltedSourceProp(d, ny, nx, dy, dx, lam, z, ang, og.BICUBIC, og.ASM)
    assert rel_l2(host(d), ref) < TOL
    h = u.copy()
    og.TiltedSourceProp(h, ny, nx, dy, dx, lam, z, ang, og.BICUBIC, og.ASM)
    assert rel_l2(h.astype(np.complex128), ref) < TOL
    ref = O.tilted_prop(u.astype(np.complex128), dy, dx, lam, z, 2e-3, 0, 1, True)
    h = u.copy()
    og.TiltedReferenceProp(h, ny, nx, dy, dx, lam, z, 2e-3, og.BILINEAR, og.FRESNEL)
    assert rel_l2(h.astype(np.complex128), ref) < TOL


def test_tilted_workspace_reuse():
    ny, nx = 128, 128
    w = og.tilted_workspace(ny, nx)
    rng = np.random.default_rng(8)
    for ang in (0.05, -0.1):
        u = field(rng, (ny, nx))
        ref = O.tilted_prop(u.astype(np.complex128), 8e-6, 8e-6, 532e-9, 0.03, ang, 0, 0, False)
        out = og.tilted_prop(dev(u), torch.empty((ny, nx), dtype=torch.complex64, device="cuda"), dy=8e-6, dx=8e-6,
                             lam=532e-9, z=0.03, angle=ang, work=w)
        assert rel_l2(host(out), ref) < TOL


def test_tilted_errors():
    u = torch.zeros((64, 64), dtype=torch.complex64, device="cuda")
    kw = dict(dy=8e-6, dx=8e-6, lam=532e-9, z=0.02, angle=0.1)
    with pytest.raises(og.OlgError):  # interpolation outside {BILINEAR, BICUBIC}
        og.tilted_prop(u, interp=2, **kw)
    with pytest.raises(ValueError):
        og.tilted_prop(u, propmode=og.AUTO, **kw)
    with pytest.raises(og.OlgError):  # a sub-wavelength pitch reaches evanescent frequencies
        og.tilted_prop(u, dy=2e-7, dx=2e-7, lam=532e-9, z=0.02, angle=0.1)
    with pytest.raises(og.OlgError):  # Fresnel at z = 0
        og.tilted_prop(u, dy=8e-6, dx=8e-6, lam=532e-9, z=0.0, angle=0.1, propmode=og.FRESNEL)
    with pytest.raises(og.OlgError):  # unsupported length (factor 7)
        og.tilted_prop(torch.zeros((14, 64), dtype=torch.complex64, device="cuda"), **kw)
