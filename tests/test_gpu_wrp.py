"""GPU parity: WRP step 1 (binned windowed spherical waves), the whole WRP
method and the 8-bit quantisers, against the FP64 oracle."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def host(t):
    torch.cuda.synchronize()
    return t.cpu().numpy().astype(np.complex128)


def wrp_points(n, N, p, zw, seed, extent=None):
    rng = np.random.default_rng(seed)
    ext = extent if extent is not None else N * p
    c = N * p / 2
    x = c + (rng.random(n) - 0.5) * ext
    y = c + (rng.random(n) - 0.5) * ext
    z = zw + 1e-3 + rng.random(n) * 4e-3
    return np.stack([x, y, z], 1).astype(np.float32)


@pytest.mark.parametrize("window", [0, 1])
@pytest.mark.parametrize("N,n", [(256, 300), (512, 2000)])
def test_wrp_step1_vs_oracle(window, N, n):
    p, lam, zw = np.float32(4e-6), np.float32(532e-9), np.float32(0.15)
    pts = wrp_points(n, N, float(p), float(zw), seed=N + n + window)
    U = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
    fn = og.WRPStep1 if window == 0 else og.WRPStep1_D
    fn(og.gObject(pts), U, N, N, p, lam, zw)
    ref = O.wrp_step1(pts, N, N, p, lam, zw, window=window)
    assert np.count_nonzero(ref) > N * N // 4
    assert rel_l2(host(U), ref) < TOL


def test_wrp_step1_workload_subset():
    """The WRP workload geometry (4096^2 WRP, p = 4 um, points 1-5 mm behind it,
    10 x 10 mm) with a 20,000-point seeded subset of the 200,000."""
    N, p, lam, zw = 4096, np.float32(4e-6), np.float32(532e-9), np.float32(0.15)
    pts = wrp_points(20000, N, float(p), float(zw), seed=20261206, extent=10e-3)
    U = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
    og.WRPStep1(og.gObject(pts), U, N, N, p, lam, zw)
    ref = O.wrp_step1(pts, N, N, p, lam, zw, window=0)
    assert rel_l2(host(U), ref) < TOL


def test_wrp_method_end_to_end():
    N, p, lam = 512, np.float32(4e-6), np.float32(532e-9)
    zmin = np.float32(0.02)
    pts = wrp_points(500, N, float(p), float(zmin), seed=3)
    pts[:, 2] = zmin + 1e-3 + (pts[:, 2] - pts[:, 2].min())
    U = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
    U, pz = og.WRPMethod(og.gObject(pts), U, N, N, p, lam, float(pts[:, 2].min()), s=0.9, verbose=False)
    pz = np.float32(pz)
    assert pz == np.float32(np.float32(pts[:, 2].min()) * np.float32(0.9))
    ref = O.wrp_step1(pts, N, N, p, lam, pz, window=0)
    ref = O.prop(ref, float(p), float(p), float(lam), float(pz))
    assert rel_l2(host(U), ref) < TOL


def test_quantisers_vs_oracle(golden):
    u64 = golden["q_in"]
    u = torch.from_numpy(u64.astype(np.complex64)).cuda()
    uc = u64.astype(np.complex64).astype(np.complex128)
    for mode in range(4):
        img = og.complex2img(u, 16, 24, mode).cpu().numpy()
        ref = O.complex2img(uc, mode)
        diff = img.astype(int) - ref.astype(int)
        assert np.abs(diff).max() <= 1
        assert np.count_nonzero(diff) <= 2, mode
    b = og.binarize(u, 16, 24).cpu().numpy()
    assert np.array_equal(b, O.binarize(uc))


def test_quantisers_large_threshold_pixels():
    """At 1024^2 every mismatch must sit within FP32 rounding of a .5 level."""
    rng = np.random.default_rng(8)
    u0 = (rng.standard_normal((1024, 1024)) + 1j * rng.standard_normal((1024, 1024))).astype(np.complex64)
    u = torch.from_numpy(u0).cuda()
    uc = u0.astype(np.complex128)
    for mode in range(4):
        img = og.complex2img(u, 1024, 1024, mode).cpu().numpy().astype(int)
        ref = O.complex2img(uc, mode).astype(int)
        bad = np.nonzero(img != ref)
        assert np.abs(img - ref).max() <= 1
        # value before rounding in FP64
        v = [np.angle(uc), uc.real, uc.imag, np.abs(uc)][mode]
        lo, hi = (-np.pi, np.pi) if mode == 0 else (v.min(), v.max())
        x = 255 * (v - lo) / (hi - lo)
        frac = np.abs(x[bad] - np.floor(x[bad]) - 0.5)
        assert (frac < 1e-4).all(), (mode, len(bad[0]))
