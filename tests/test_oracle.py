"""CPU: the oracle restatement against the reference's golden vectors and its
own mathematical properties.  No GPU."""
import numpy as np
import pytest

import oracle as O
from conftest import rel_l2


@pytest.mark.parametrize("shape", [(16, 16), (24, 40), (30, 7), (64, 128), (1, 32)])
def test_fft_matches_numpy(shape):
    rng = np.random.default_rng(1)
    u = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    assert rel_l2(O.fft2(u, -1), np.fft.fft2(u)) < 1e-14
    assert rel_l2(O.fft2(u, +1), np.fft.ifft2(u) * u.size) < 1e-14


def test_golden_propagation(golden):
    for i in range(int(golden["n_prop"])):
        ny, nx, dy, dx, lam, z = golden[f"prop{i}_params"]
        u = golden[f"prop{i}_in"]
        assert rel_l2(O.asm_prop(u, dy, dx, lam, z), golden[f"prop{i}_asm"]) < 1e-13
        assert rel_l2(O.fresnel_prop(u, dy, dx, lam, z), golden[f"prop{i}_fresnel"]) < 1e-13
        assert rel_l2(O.fresnel_prop(u, dy, dx, lam, z, bandlimit=2), golden[f"prop{i}_fresnel_bl"]) < 1e-13


def test_golden_auto_dispatch(golden):
    for i in range(int(golden["n_auto"])):
        ny, nx, dy, dx, lam, z = golden[f"auto{i}_params"]
        a, f = golden[f"auto{i}_branch"]
        assert O.asm_prop_check(int(ny), int(nx), dy, dx, lam, z) == bool(a)
        assert O.fresnel_prop_check(int(ny), int(nx), dy, dx, lam, z) == bool(f)
        assert rel_l2(O.prop(golden[f"auto{i}_in"], dy, dx, lam, z), golden[f"auto{i}_out"]) < 1e-13


def test_golden_checks_double(golden):
    for ny, nx, p, lam, z, a64, a32, f64, f32 in golden["checks"]:
        assert O.asm_prop_check(int(ny), int(nx), p, p, lam, z) == bool(a64)
        assert O.fresnel_prop_check(int(ny), int(nx), p, p, lam, z) == bool(f64)


def test_golden_cgh(golden):
    for i in range(int(golden["n_cgh"])):
        ny, nx, py, px, lam = golden[f"cgh{i}_params"]
        pts = golden[f"cgh{i}_pts"]
        U, ph = O.cgh_fresnel(pts, int(ny), int(nx), py, px, lam, want_phase=True)
        assert rel_l2(U, golden[f"cgh{i}_U"]) < 1e-13
        if f"cgh{i}_phase" in golden:
            assert np.allclose(ph, golden[f"cgh{i}_phase"], atol=1e-12)


def test_golden_quantisers(golden):
    u = golden["q_in"]
    for mode in range(4):
        assert np.array_equal(O.complex2img(u, mode), golden[f"q_mode{mode}"])
    assert np.array_equal(O.quant8bit(u.real), golden["q_quant8bit"])


def _rand_field(rng, shape):
    return (rng.random(shape) < 0.5) * np.exp(2j * np.pi * rng.random(shape))


def _dot(a, b):
    return np.vdot(b, a)  # <a, b> = sum a conj(b)


@pytest.mark.parametrize("kind", ["asm", "fresnel", "fresnel_bl", "arss", "arss_off"])
def test_adjoint_dot_product(kind):
    rng = np.random.default_rng(7)
    x = rng.standard_normal((32, 48)) + 1j * rng.standard_normal((32, 48))
    y = rng.standard_normal((32, 48)) + 1j * rng.standard_normal((32, 48))
    p = dict(dy=8e-6, dx=8e-6, lam=532e-9, z=0.03)
    if kind == "asm":
        A = lambda v, f: O.asm_prop(v, p["dy"], p["dx"], p["lam"], p["z"], flags=f)
    elif kind == "fresnel":
        A = lambda v, f: O.fresnel_prop(v, p["dy"], p["dx"], p["lam"], p["z"], flags=f)
    elif kind == "fresnel_bl":
        A = lambda v, f: O.fresnel_prop(v, 20e-6, 20e-6, p["lam"], 0.005, bandlimit=1, flags=f)
    elif kind == "arss":
        A = lambda v, f: O.arss_prop(v, 8e-6, 8e-6, p["lam"], 0.05, 0.5, flags=f)
    else:
        A = lambda v, f: O.arss_prop(v, 6e-6, 8e-6, p["lam"], -0.04, 2.0, oy=1e-4, ox=-2e-4, flags=f)
    lhs = _dot(A(x, 0), y)
    rhs = _dot(x, A(y, O_CONJ))
    assert abs(lhs - rhs) <= 1e-10 * abs(lhs)


O_CONJ = 1


def test_cgh_adjoint_dot_product():
    rng = np.random.default_rng(3)
    pts = np.stack([rng.random(9) * 20 * 8e-6, rng.random(9) * 12 * 8e-6, 0.01 + rng.random(9) * 0.01], 1)
    c = rng.standard_normal(9) + 1j * rng.standard_normal(9)
    G = rng.standard_normal((12, 20)) + 1j * rng.standard_normal((12, 20))
    for fwd, adj in [(O.cgh_fresnel, O.cgh_fresnel_adjoint), (O.cgh_exact, O.cgh_exact_adjoint)]:
        # forward with complex weights c_j = a_j exp(i phi_j)
        U = fwd(pts, 12, 20, 8e-6, 8e-6, 532e-9, amp=np.abs(c), phase0=np.angle(c))
        g = adj(pts, G, 8e-6, 8e-6, 532e-9)
        assert abs(_dot(U, G) - _dot(c, g)) <= 1e-10 * abs(_dot(U, G))


def test_cgh_fresnel_unit_weights_equal_reference_form(golden):
    ny, nx, py, px, lam = golden["cgh0_params"]
    pts = golden["cgh0_pts"]
    n = len(pts)
    U1 = O.cgh_fresnel(pts, int(ny), int(nx), py, px, lam, amp=np.ones(n), phase0=np.zeros(n))
    assert rel_l2(U1, golden["cgh0_U"]) < 1e-14


def _wrp_literal(pts, ny, nx, p, lam, plane_z, plimit, window):
    """Per-pixel loop over ALL points, as golcgh.h:303-328 / 403-441 writes it,
    with float32 window tests (numpy float32 arithmetic rounds every operation)."""
    f = np.float32
    pts = np.asarray(pts, np.float32)
    R = O.wrp_radius(pts, plimit, lam, plane_z, window)
    U = np.zeros((ny, nx), np.complex128)
    for h in range(ny):
        for w in range(nx):
            dxf = f(f(p) * f(w)) - pts[:, 0]
            dyf = f(f(p) * f(h)) - pts[:, 1]
            if window == 0:
                inside = (dxf * dxf + dyf * dyf) < R * R
            else:
                inside = (np.abs(dxf) * f(2) <= R) & (np.abs(dyf) * f(2) <= R)
            dz = pts[:, 2].astype(np.float64) - np.float64(plane_z)
            ddx = np.float64(p) * w - pts[:, 0].astype(np.float64)
            ddy = np.float64(p) * h - pts[:, 1].astype(np.float64)
            th = np.pi * (ddx * ddx + ddy * ddy) / (np.float64(lam) * dz)
            U[h, w] = np.sum(np.where(inside, np.exp(1j * th) / np.abs(dz), 0))
    return U


@pytest.mark.parametrize("window", [0, 1])
def test_wrp_scatter_equals_literal_gather(window):
    rng = np.random.default_rng(11)
    ny, nx, p, lam = 24, 32, np.float32(4e-6), np.float32(532e-9)
    plane_z = np.float32(0.1)
    n = 15
    pts = np.stack([rng.random(n) * nx * 4e-6, rng.random(n) * ny * 4e-6, 0.1 + 1e-4 + rng.random(n) * 3e-4],
                   1).astype(np.float32)
    U = O.wrp_step1(pts, ny, nx, p, lam, plane_z, window=window)
    L = _wrp_literal(pts, ny, nx, p, lam, plane_z, p, window)
    assert np.count_nonzero(L) > 20
    assert rel_l2(U, L) < 1e-12


def test_arss_windows_and_rejects_s1():
    w = O.arss_windows(64, 64, 8e-6, 8e-6, 532e-9, 0.05, 0.5)
    assert (w[:5] > 0).all()
    with pytest.raises(ValueError):
        O.arss_windows(64, 64, 8e-6, 8e-6, 532e-9, 0.05, 1.0)


def _rel_or_zero(a, b):
    nb = np.linalg.norm(b)
    return rel_l2(a, b) if nb > 0 else np.abs(a).max()


def test_golden_shifted_asm(golden):
    """ol::shiftedAsmProp<double> (olprop.h:307-327): band window, 1/Np twice."""
    for i in range(int(golden["n_shasm"])):
        ny, nx, dy, dx, lam, z, oy, ox = golden[f"shasm{i}_params"]
        out = O.shifted_asm_prop(golden[f"shasm{i}_in"], dy, dx, lam, z, oy, ox, flags=O.OLC_BANDLIMIT)
        assert _rel_or_zero(out / (4 * ny * nx), golden[f"shasm{i}_out"]) < 1e-13, i


def test_golden_shifted_fresnel(golden):
    """ol::shiftedFresnelProp<double> (olprop.h:338-406): one more 1/Np than
    gshiftedFresnelProp, which the oracle follows."""
    for i in range(int(golden["n_shfr"])):
        ny, nx, dy, dx, lam, z, s, oy, ox = golden[f"shfr{i}_params"]
        out = O.shifted_fresnel_prop(golden[f"shfr{i}_in"], dy, dx, lam, z, s, oy, ox)
        assert rel_l2(out / (4 * ny * nx), golden[f"shfr{i}_out"]) < 1e-13, i


def test_golden_split_asm(golden):
    """ol::splitAsmProp (olprop.h:618-654) only instantiates with PREC_T = float:
    its phases are single precision (about 1e-2 of relative L2 against FP64;
    a single-block split shows the same).  The oracle takes the float-rounded
    parameters and decides the band windows in float like it; adjacent blocks
    sit exactly on the window's branch boundary, where a double decision would
    give a different window (about 0.8 relative L2)."""
    f32 = lambda v: float(np.float32(v))
    for i in range(int(golden["n_split"])):
        ny, nx, dy, dx, lam, z, by, bx = golden[f"split{i}_params"]
        ny, nx, by, bx = int(ny), int(nx), int(by), int(bx)
        out = O.split_prop(golden[f"split{i}_in"], f32(dy), f32(dx), f32(lam), f32(z), 0, by, bx,
                           flags=O.OLC_BANDLIMIT | 0x10)
        out /= 4 * (ny // by) * (nx // bx)
        assert rel_l2(out, golden[f"split{i}_out"]) < 2e-2, i
        wrong = O.split_prop(golden[f"split{i}_in"], dy, dx, lam, z, 0, by, bx, flags=O.OLC_BANDLIMIT)
        assert rel_l2(wrong / (4 * (ny // by) * (nx // bx)), golden[f"split{i}_out"]) > 0.3


@pytest.mark.parametrize("kind", ["shifted_asm", "shifted_asm_band", "shifted_fresnel"])
def test_shifted_adjoint_dot_product(kind):
    rng = np.random.default_rng(3)
    x = rng.standard_normal((32, 64)) + 1j * rng.standard_normal((32, 64))
    y = rng.standard_normal((32, 64)) + 1j * rng.standard_normal((32, 64))
    args = (6e-6, 8e-6, 633e-9, 0.03)
    if kind == "shifted_fresnel":
        A = lambda v, f: O.shifted_fresnel_prop(v, *args, 0.8, 2e-4, -1e-4, flags=f)
    else:
        band = O.OLC_BANDLIMIT if kind.endswith("band") else 0
        A = lambda v, f: O.shifted_asm_prop(v, *args, 2e-4, -1e-4, flags=f | band)
    lhs = np.vdot(y, A(x, 0))
    rhs = np.vdot(A(y, 0x1), x)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)


def test_split_sums_shifted_blocks():
    """Split propagation == sum of shifted propagations of the blocks."""
    rng = np.random.default_rng(4)
    u = rng.standard_normal((32, 64)) + 1j * rng.standard_normal((32, 64))
    args = (8e-6, 8e-6, 532e-9, 0.01)
    out = O.split_prop(u, *args, 0, 2, 2)
    ref = np.zeros_like(u)
    for gn in range(2):
        for gm in range(2):
            blk = np.zeros_like(u)
            blk[gn * 16:(gn + 1) * 16, gm * 32:(gm + 1) * 32] = u[gn * 16:(gn + 1) * 16, gm * 32:(gm + 1) * 32]
            for dn in range(2):
                for dm in range(2):
                    oy = float(np.float32((gn - dn) * 16) * np.float32(8e-6))
                    ox = float(np.float32((gm - dm) * 32) * np.float32(8e-6))
                    s = O.shifted_asm_prop(u[gn * 16:(gn + 1) * 16, gm * 32:(gm + 1) * 32], *args, oy, ox)
                    ref[dn * 16:(dn + 1) * 16, dm * 32:(dm + 1) * 32] += s
    assert rel_l2(out, ref) < 1e-14


def test_golden_tilted(golden):
    """ol::TiltedSourceProp / ol::TiltedReferenceProp (PREC_T = double) outputs."""
    for i in range(int(golden["n_tilt"])):
        ny, nx, dy, dx, lam, z, ang, ip, mode, refm = golden[f"tilt{i}_params"]
        out = O.tilted_prop(golden[f"tilt{i}_in"], dy, dx, lam, z, ang, int(ip), int(mode), bool(refm))
        assert rel_l2(out, golden[f"tilt{i}_out"]) < 1e-13, i


def test_tilted_zero_angle_is_plain_propagation():
    """At angle 0 both tilted forms resample on the unrotated grid (J = 1); the
    source form with ASM is then the ASM propagation with one more 1/N."""
    rng = np.random.default_rng(3)
    u = (rng.random((32, 48)) < 0.5) * np.exp(2j * np.pi * rng.random((32, 48)))
    n = 4 * u.size
    ref = O.asm_prop(u, 8e-6, 8e-6, 532e-9, 0.02) / n
    for refm in (False, True):
        out = O.tilted_prop(u, 8e-6, 8e-6, 532e-9, 0.02, 0.0, 0, 0, refm)
        assert rel_l2(out, ref) < 1e-12
