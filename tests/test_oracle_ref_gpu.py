"""The oracle pinned to the reference's OWN GPU code for the rows the
reference implements only in CUDA: ARSS propagation (golprop.h:816-995) and
the windowed WRP step 1 (golcgh.h:291-491, circle and square windows).

tests/golden/ref_gpu_golden.npz holds outputs of the unmodified reference
templates, built with nvcc for sm_103a and run on a GB300 by
tests/golden/make_gpu_golden.py (inputs seeded there).  The reference computes
in FP32 (PREC_T = float), so values agree to FP32 rounding (relative L2
1e-5), while the window supports -- which pixels a window includes -- are
compared exactly:

  * ARSS: the pre-chirp stage (zero outside its window), the impulse-response
    chirp on the padded grid (zero outside its window, whose limit comes from
    x on both axes, golprop.h:892-893) and the post-chirp applied to a field
    of ones (exactly 1 outside its window, golprop.h:910), plus the whole
    propagation; one case has s < 0, where the pre-chirp window is empty.
  * WRP: single points and sparse clouds whose windows do not overlap, so the
    output's nonzero set is exactly the union of the windows; dense clouds for
    the values.
"""
import numpy as np
import pytest

import oracle as O
from conftest import rel_l2

ARSS = ["arss_a", "arss_b", "arss_c", "arss_d", "arss_e", "arss_f"]
WRP = ["wrp_single_w0", "wrp_single_w1", "wrp_sparse_w0", "wrp_sparse_w1", "wrp_plimit_w0", "wrp_plimit_w1",
       "wrp_dense_w0", "wrp_dense_w1"]
F32_TOL = 1e-5   # reference values are FP32


@pytest.fixture(scope="module")
def gold(golden_dir):
    return np.load(golden_dir / "ref_gpu_golden.npz")


def f32(v):
    return float(np.float32(v))


def arss_params(g, name):
    ny, nx, dy, dx, lam, z, s, oy, ox = g[name + "_par"]
    return int(ny), int(nx), *map(f32, (dy, dx, lam, z, s, oy, ox))


def arss_masks(ny, nx, dy, dx, lam, z, s):
    """Window masks from the oracle's limits (olc_arss_windows)."""
    L = np.zeros(6, np.int64)
    assert O.cpu().olc_arss_windows(ny, nx, dy, dx, lam, z, s, L.ctypes.data) == 0
    H, W = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    pre = (np.abs(W - nx // 2) < L[1]) & (np.abs(H - ny // 2) < L[0])
    post = (np.abs(W - nx // 2) < L[4]) & (np.abs(H - ny // 2) < L[3])
    H2, W2 = np.meshgrid(np.arange(2 * ny), np.arange(2 * nx), indexing="ij")
    resp = (np.abs(W2 - nx) < L[2]) & (np.abs(H2 - ny) < L[2])
    return pre, post, resp


@pytest.mark.parametrize("name", ARSS)
def test_arss_windows_match_reference_gpu(gold, name):
    ny, nx, dy, dx, lam, z, s, oy, ox = arss_params(gold, name)
    u = gold[name + "_in"]
    pre, post, resp = arss_masks(ny, nx, dy, dx, lam, z, s)
    # pre-chirp: zero outside the window; inside, zero only where the input is
    stage_u = gold[name + "_u"]
    assert np.array_equal(stage_u != 0, pre & (u != 0))
    # response chirp on the padded grid: nonzero exactly inside its window
    assert np.array_equal(gold[name + "_h"] != 0, resp)
    # post-chirp on ones: untouched (exactly 1) outside its window; inside it
    # is exp(i phi_c), which the oracle's window must agree is a chirp sample
    cz = gold[name + "_cz"]
    assert np.all(cz[~post] == np.complex64(1.0))
    H, W = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    x2, y2 = (W - nx // 2) * dx, (H - ny // 2) * dy
    phc = ((1 - s) * x2 * x2 + 2 * ox * x2 + ox * ox + (1 - s) * y2 * y2 + 2 * oy * y2 + oy * oy) * np.pi / (lam * z)
    assert np.abs(cz[post] - np.exp(1j * phc[post])).max() < 1e-4


@pytest.mark.parametrize("name", ARSS)
def test_arss_output_matches_reference_gpu(gold, name):
    ny, nx, dy, dx, lam, z, s, oy, ox = arss_params(gold, name)
    ref = gold[name + "_out"].astype(np.complex128)
    got = O.arss_prop(gold[name + "_in"].astype(np.complex128), dy, dx, lam, z, s, oy, ox)
    if s < 0:
        # the reference's pre-chirp window is empty for s < 0 (its limit is negative)
        assert not np.any(ref) and not np.any(got)
        return
    assert rel_l2(got, ref) < F32_TOL


def wrp_case(g, name):
    ny, nx, p, lam, pz, window, plimit = g[name + "_par"]
    pts = g[name + "_pts"]
    return pts, int(ny), int(nx), np.float32(p), np.float32(lam), np.float32(pz), int(window), \
        (np.float32(plimit) if plimit > 0 else None)


@pytest.mark.parametrize("name", WRP)
def test_wrp_step1_matches_reference_gpu(gold, name):
    pts, ny, nx, p, lam, pz, window, plimit = wrp_case(gold, name)
    ref = gold[name + "_out"]
    U = O.wrp_step1(pts, ny, nx, p, lam, pz, plimit, window)
    # window membership is decided in float32 as the reference's kernel decides it
    assert np.array_equal(U != 0, ref != 0)
    assert rel_l2(U, ref.astype(np.complex128)) < F32_TOL
    if "sparse" in name or "single" in name or "plimit" in name:
        assert 0 < np.count_nonzero(ref) < ref.size
