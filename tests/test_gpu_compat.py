"""GPU: a C++ caller written against the reference's GPU API (gAsmProp,
gFresnelProp, ARSSFresnelProp, Prop, gCgh -- the shape of the reference's own
demos) compiles unchanged against include/openol_gb300/*.h, links
libolgb300.so, and its results match the FP64 oracle."""
import os
import subprocess

import numpy as np
import pytest

import oracle as O
import openol_gb300 as og
from conftest import ROOT, rel_l2
from openol_gb300 import build as B

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def demo_out(tmp_path_factory):
    out = tmp_path_factory.mktemp("compat")
    exe = str(out / "compat_demo")
    subprocess.run([B._nvcc(), *B.ARCH, "-std=c++17", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "compat_demo.cu"), "-L", os.path.dirname(B.LIB), "-lolgb300",
                    "-Xlinker", "-rpath=" + os.path.dirname(B.LIB), "-o", exe], check=True)
    r = subprocess.run([exe, str(out)], capture_output=True, text=True, check=True)
    assert "compat_demo ok" in r.stdout
    return out, r.stdout


def load(out, name, dtype=np.complex64, shape=(128, 256)):
    return np.fromfile(out / f"{name}.bin", dtype=dtype).reshape(shape)


def test_compat_propagation(demo_out):
    out, stdout = demo_out
    u = load(out, "input").astype(np.complex128)
    p, lam, d = float(np.float32(8e-6)), float(np.float32(532e-9)), float(np.float32(0.05))
    assert rel_l2(load(out, "asm"), O.asm_prop(u, p, p, lam, d)) < 1e-5
    assert rel_l2(load(out, "fresnel"), O.fresnel_prop(u, p, p, lam, d)) < 1e-5
    q = float(np.float32(np.float32(8e-6) / np.float32(0.5)))
    assert rel_l2(load(out, "arss"), O.arss_prop(u, q, q, lam, d, 0.5)) < 1e-5
    assert rel_l2(load(out, "prop_auto"), O.prop(u, p, p, lam, d)) < 1e-5
    assert "AsmProp" in stdout
    assert rel_l2(load(out, "asm_host"), O.asm_prop(u, p, p, lam, d, flags=2)) < 1e-5
    f = lambda v: float(np.float32(v))
    assert rel_l2(load(out, "shifted_asm"), O.shifted_asm_prop(u, p, p, lam, d, f(2e-4), f(-1e-4))) < 1e-5
    assert rel_l2(load(out, "split_asm"), O.split_prop(u, p, p, lam, d, 0, 2, 2)) < 1e-5
    assert rel_l2(load(out, "tilted_source"), O.tilted_prop(u, p, p, lam, d, f(0.1), 1, 0, False)) < 1e-5
    assert rel_l2(load(out, "tilted_reference"), O.tilted_prop(u, p, p, lam, d, f(2e-3), 0, 1, True)) < 1e-5


def test_compat_cgh(demo_out):
    out, _ = demo_out
    pts = np.fromfile(out / "points.bin", dtype=np.float32).reshape(-1, 3).astype(np.float64)
    p, lam = float(np.float32(8e-6)), float(np.float32(532e-9))
    U, ph = O.cgh_fresnel(pts, 128, 256, p, p, lam, want_phase=True)
    assert rel_l2(load(out, "cgh"), U) < 1e-3          # tensor-core path (>= 1024 points)
    g = load(out, "cgh_phase", np.float32)
    assert np.abs(np.angle(np.exp(1j * (g - ph)))).max() < 1e-3


def test_compat_objects(demo_out):
    """ol::objread / objset / objsort / bmpwrite through the drop-in headers."""
    out, _ = demo_out
    cloud = og.objread(out / "cloud.3d")
    g = og.gObject(cloud)
    p = float(np.float32(8e-6))
    og.objset(g, np.float32(2e-3), (np.float32(256 / 2 * p), np.float32(128 / 2 * p), np.float32(0.03)), og.ZMIN)
    og.objsort(g)
    got = np.fromfile(out / "cloud_set_sorted.bin", dtype=np.float32).reshape(-1, 3)
    assert np.array_equal(got, g.points.cpu().numpy())
    img = (np.arange(128 * 256) * 7 % 256).astype(np.uint8).reshape(128, 256)
    assert np.array_equal(og.bmpread(out / "img.bmp", 128, 256), img)


def test_compat_host_field_templates(demo_out):
    """olprop.h / olcgh.h: the reference's CPU templates for host fields
    (AsmProp, FresnelProp, FresnelPropBandLimit, Prop, shiftedAsmProp,
    shiftedFresnelProp, splitAsmProp, Cgh, the CPU WRPStep1) and WRPStep2,
    called from C++ with float and double fields.  Every field propagates in
    FP32 on the GPU, so results are held to the FP32 gate against the FP64
    oracle whatever COMPLEX_T the caller used."""
    out, stdout = demo_out
    u = load(out, "input").astype(np.complex128)
    f = lambda v: float(np.float32(v))
    p, lam = f(8e-6), f(532e-9)
    c128 = lambda name: load(out, name, np.complex128)
    assert rel_l2(c128("host_asm_f64"), O.asm_prop(u, p, p, lam, 0.02)) < 1e-5
    assert rel_l2(load(out, "host_asm_f32"), O.asm_prop(u, p, p, lam, f(0.02))) < 1e-5
    assert rel_l2(c128("host_fresnel"), O.fresnel_prop(u, p, p, lam, 0.1)) < 1e-5
    assert rel_l2(c128("host_fresnel_bl"), O.fresnel_prop(u, p, p, lam, 0.05, bandlimit=2)) < 1e-5
    for k, z in enumerate((0.02, 0.05, 0.1)):
        assert rel_l2(c128(f"host_prop_auto{k}"), O.prop(u, p, p, lam, z)) < 1e-5, z
    # the three AUTO branches were taken (ASM, band-limited warning, Fresnel)
    assert "warning!!" in stdout and "FresnelProp" in stdout
    ref = O.shifted_asm_prop(u, p, p, lam, 0.02, 2e-4, -1e-4, flags=O.OLC_BANDLIMIT) / (4.0 * 128 * 256)
    assert rel_l2(c128("host_shifted_asm"), ref) < 1e-5
    ref = O.shifted_fresnel_prop(u, p, p, lam, f(0.05), f(0.7), f(1e-4), 0.0) / (4.0 * 128 * 256)
    assert rel_l2(load(out, "host_shifted_fresnel"), ref) < 1e-5
    ref = O.split_prop(u, p, p, lam, f(0.02), 0, 2, 2, flags=O.OLC_BANDLIMIT | 0x10) / (4.0 * 64 * 128)
    assert rel_l2(load(out, "host_split_asm"), ref) < 1e-5


def test_compat_host_cgh_and_wrp_step2(demo_out):
    out, stdout = demo_out
    pts = np.fromfile(out / "points.bin", dtype=np.float32).reshape(-1, 3).astype(np.float64)
    f = lambda v: float(np.float32(v))
    p, lam = f(8e-6), f(532e-9)
    U, ph = O.cgh_fresnel(pts, 128, 256, p, p, lam, want_phase=True)
    # 1500 points take the split-FP16 tensor-core form (gate 1e-3)
    assert rel_l2(load(out, "host_cgh", np.complex128), U) < 1e-3
    assert rel_l2(load(out, "host_cgh_pypx"), U) < 1e-3
    assert rel_l2(load(out, "host_wrp_step1"), U) < 1e-3
    for name, dt in (("host_cgh_phase", np.float32), ("host_cgh_phase_f64", np.float64)):
        g = load(out, name, dt)
        assert np.abs(np.angle(np.exp(1j * (g - ph)))).max() < 1e-3, name
    u = load(out, "input").astype(np.complex128)
    assert rel_l2(load(out, "wrp_step2_0"), O.asm_prop(u, p, p, lam, f(0.02))) < 1e-5
    assert rel_l2(load(out, "wrp_step2_1"), O.fresnel_prop(u, p, p, lam, f(0.1))) < 1e-5
    assert "WRP Step2 is AsmProp" in stdout and "WRP Step2 is FresnelProp" in stdout


def test_python_host_field_mirrors():
    """The Python mirrors of the same olprop.h / olcgh.h host templates, on
    numpy arrays (complex128 in, complex128 out, FP32 inside)."""
    rng = np.random.default_rng(12)
    u = (rng.random((128, 256)) < 0.5) * np.exp(2j * np.pi * rng.random((128, 256)))
    u = u.astype(np.complex64).astype(np.complex128)
    p, lam = 8e-6, 532e-9
    a = og.AsmProp(u.copy(), 128, 256, p, p, lam, 0.02)
    assert rel_l2(a, O.asm_prop(u, p, p, lam, 0.02)) < 1e-5
    b = og.FresnelPropBandLimit(u.copy(), 128, 256, p, p, lam, 0.05)
    assert rel_l2(b, O.fresnel_prop(u, p, p, lam, 0.05, bandlimit=2)) < 1e-5
    for z in (0.02, 0.05, 0.1):
        c = og.PropHost(u.copy(), 128, 256, p, p, lam, z, verbose=False)
        assert rel_l2(c, O.prop(u, p, p, lam, z)) < 1e-5, z
    pts = np.stack([rng.random(300) * 256 * p, rng.random(300) * 128 * p, 0.02 + 0.01 * rng.random(300)], 1)
    pts32 = pts.astype(np.float32).astype(np.float64)
    U = og.Cgh(pts, np.zeros((128, 256), np.complex128), 128, 256, p, lam)
    Ur, ph = O.cgh_fresnel(pts32, 128, 256, p, p, lam, want_phase=True)
    assert rel_l2(U, Ur) < 1e-5
    g = og.Cgh(pts, np.zeros((128, 256), np.float64), 128, 256, p, p, lam)
    assert np.abs(np.angle(np.exp(1j * (g - ph)))).max() < 1e-3
