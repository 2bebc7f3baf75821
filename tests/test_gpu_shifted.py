"""GPU: shifted ASM / shifted Fresnel / split propagation against the FP64
oracle and against the reference's own CPU outputs (golden fixtures)."""
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


SHIFTED = [
    # ny, nx, dy, dx, lam, z, oy, ox
    (64, 64, 8e-6, 8e-6, 532e-9, 0.02, 1e-4, -2e-4),
    (128, 256, 6e-6, 8e-6, 633e-9, 0.05, 3e-4, 5e-4),
    (256, 128, 4e-6, 4e-6, 532e-9, -0.01, -1e-4, 2e-4),
    (512, 512, 8e-6, 8e-6, 532e-9, 0.1, 4.096e-3, -2.048e-3),
]


@pytest.mark.parametrize("case", SHIFTED)
@pytest.mark.parametrize("band", [0, 1, 2])
def test_shifted_asm_matches_oracle(case, band):
    ny, nx, dy, dx, lam, z, oy, ox = case
    rng = np.random.default_rng(ny + nx + band)
    u = field(rng, (ny, nx))
    flags = {0: 0, 1: O.OLC_BANDLIMIT, 2: O.OLC_BANDLIMIT | 0x10}[band]
    ref = O.shifted_asm_prop(u.astype(np.complex128), dy, dx, lam, z, oy, ox, flags=flags)
    out = og.shifted_asm_prop(dev(u), torch.empty((ny, nx), dtype=torch.complex64, device="cuda"), dy=dy, dx=dx,
                              lam=lam, z=z, oy=oy, ox=ox, bandlimit=band > 0, window_f32=band == 2)
    g = host(out)
    if np.linalg.norm(ref) == 0:
        assert np.abs(g).max() == 0
    else:
        assert rel_l2(g, ref) < TOL


def test_shifted_asm_host_mirror_matches_reference(golden):
    """ol::shiftedAsmProp<double> outputs, made by the reference's own CPU build."""
    for i in range(int(golden["n_shasm"])):
        ny, nx, dy, dx, lam, z, oy, ox = golden[f"shasm{i}_params"]
        ny, nx = int(ny), int(nx)
        u = golden[f"shasm{i}_in"].astype(np.complex64)
        out = np.zeros((ny, nx), np.complex64)
        og.shiftedAsmProp(u, out, ny, nx, dy, dx, lam, z, oy, ox)
        ref = golden[f"shasm{i}_out"]
        if np.linalg.norm(ref) == 0:
            assert np.abs(out).max() == 0
        else:
            assert rel_l2(out.astype(np.complex128), ref) < TOL, i


@pytest.mark.parametrize("s", [1.0, 0.7, 1.3])
def test_shifted_fresnel_matches_oracle(s):
    ny, nx, dy, dx, lam, z, oy, ox = 128, 256, 6e-6, 8e-6, 633e-9, 0.05, 2e-4, -3e-4
    u = field(np.random.default_rng(7), (ny, nx))
    ref = O.shifted_fresnel_prop(u.astype(np.complex128), dy, dx, lam, z, s, oy, ox)
    out = og.shifted_fresnel_prop(dev(u), torch.empty((ny, nx), dtype=torch.complex64, device="cuda"), dy=dy, dx=dx,
                                  lam=lam, z=z, s=s, oy=oy, ox=ox)
    assert rel_l2(host(out), ref) < TOL


def test_shifted_fresnel_host_mirror_matches_reference(golden):
    """ol::shiftedFresnelProp<double> outputs, made by the reference's own CPU build."""
    for i in range(int(golden["n_shfr"])):
        ny, nx, dy, dx, lam, z, s, oy, ox = golden[f"shfr{i}_params"]
        ny, nx = int(ny), int(nx)
        u = golden[f"shfr{i}_in"].astype(np.complex64).copy()
        og.shiftedFresnelProp(u, ny, nx, dy, dx, lam, z, s, oy, ox)
        assert rel_l2(u.astype(np.complex128), golden[f"shfr{i}_out"]) < TOL, i


@pytest.mark.parametrize("kind", ["asm", "asm_band", "fresnel"])
def test_shifted_adjoint_identity(kind):
    ny, nx = 256, 128
    rng = np.random.default_rng(11)
    x = (rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))).astype(np.complex64)
    y = (rng.standard_normal((ny, nx)) + 1j * rng.standard_normal((ny, nx))).astype(np.complex64)
    kw = dict(dy=6e-6, dx=8e-6, lam=633e-9, z=0.03, oy=2e-4, ox=-1e-4)

    def A(v, adj):
        o = torch.empty_like(v)
        if kind == "fresnel":
            return og.shifted_fresnel_prop(v, o, s=0.8, adjoint=adj, **kw)
        return og.shifted_asm_prop(v, o, bandlimit=kind == "asm_band", adjoint=adj, **kw)

    lhs = np.vdot(y.astype(np.complex128), host(A(dev(x), False)))
    rhs = np.vdot(host(A(dev(y), True)), x.astype(np.complex128))
    assert abs(lhs - rhs) <= 1e-5 * abs(lhs)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("blocks", [(2, 2), (2, 4), (1, 2)])
def test_split_matches_oracle(mode, blocks):
    by, bx = blocks
    ny, nx, dy, dx, lam, z = 128, 256, 8e-6, 8e-6, 532e-9, 0.02
    u = field(np.random.default_rng(by * 10 + bx + mode), (ny, nx))
    ref = O.split_prop(u.astype(np.complex128), dy, dx, lam, z, mode, by, bx)
    out = og.split_prop(dev(u), torch.empty((ny, nx), dtype=torch.complex64, device="cuda"), dy=dy, dx=dx, lam=lam,
                        z=z, propmode=mode, blocks_y=by, blocks_x=bx)
    assert rel_l2(host(out), ref) < TOL


def test_split_band_f32_window_matches_oracle():
    ny, nx, dy, dx, lam, z, by, bx = 128, 128, 8e-6, 8e-6, 532e-9, 0.01, 2, 2
    u = field(np.random.default_rng(21), (ny, nx))
    ref = O.split_prop(u.astype(np.complex128), dy, dx, lam, z, 0, by, bx, flags=O.OLC_BANDLIMIT | 0x10)
    out = og.split_prop(dev(u), torch.empty((ny, nx), dtype=torch.complex64, device="cuda"), dy=dy, dx=dx, lam=lam,
                        z=z, blocks_y=by, blocks_x=bx, bandlimit=True, window_f32=True)
    assert rel_l2(host(out), ref) < TOL


def test_split_host_mirror_follows_reference(golden):
    """ol::splitAsmProp's reference outputs are single precision (its only
    instantiation is PREC_T = float): about 1e-2 of relative L2 from FP64."""
    for i in range(int(golden["n_split"])):
        ny, nx, dy, dx, lam, z, by, bx = golden[f"split{i}_params"]
        ny, nx, by, bx = int(ny), int(nx), int(by), int(bx)
        u = golden[f"split{i}_in"].astype(np.complex64).copy()
        og.splitAsmProp(u, ny, nx, dy, dx, lam, z, by, bx)
        assert rel_l2(u.astype(np.complex128), golden[f"split{i}_out"]) < 2e-2, i


def test_shifted_prop_dispatch_and_errors():
    ny, nx = 64, 64
    u = dev(field(np.random.default_rng(5), (ny, nx)))
    o = torch.empty_like(u)
    og.shiftedProp(u, o, ny, nx, 8e-6, 8e-6, 532e-9, 0.02, 1e-4, 1e-4, og.ASM)
    ref = O.shifted_asm_prop(u.cpu().numpy().astype(np.complex128), 8e-6, 8e-6, 532e-9, 0.02, 1e-4, 1e-4)
    assert rel_l2(host(o), ref) < TOL
    og.shiftedProp(u, o, ny, nx, 8e-6, 8e-6, 532e-9, 0.02, 1e-4, 1e-4, og.FRESNEL)
    ref = O.shifted_fresnel_prop(u.cpu().numpy().astype(np.complex128), 8e-6, 8e-6, 532e-9, 0.02, 1.0, 1e-4, 1e-4)
    assert rel_l2(host(o), ref) < TOL
    with pytest.raises(ValueError):
        og.shiftedProp(u, o, ny, nx, 8e-6, 8e-6, 532e-9, 0.02, 1e-4, 1e-4, og.AUTO)
    with pytest.raises(og.OlgError):  # output overlapping the input
        og.split_prop(u, u, dy=8e-6, dx=8e-6, lam=532e-9, z=0.02)
    with pytest.raises(og.OlgError):  # blocks that do not divide the field
        og.split_prop(u, o, dy=8e-6, dx=8e-6, lam=532e-9, z=0.02, blocks_y=3)
