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
