"""Generate tests/golden/ref_golden.npz from the reference's OWN CPU code.

The reference (somamake/openol) ships no golden vectors and no assertions, so
the fixtures are made by running its CPU templates -- ``ol::AsmProp``,
``ol::FresnelProp``, ``ol::FresnelPropBandLimit``, ``ol::Prop``,
``ol::AsmPropCheck`` / ``ol::FresnelPropCheck``, ``ol::Cgh`` (complex and phase
outputs), ``ol::complex2img``, ``ol::quant8bit``, ``ol::shiftedAsmProp``,
``ol::shiftedFresnelProp``, ``ol::splitAsmProp``, ``ol::objread``,
``ol::objset``, ``ol::objsort``, ``ol::bmpwrite``, ``ol::TiltedSourceProp`` and
``ol::TiltedReferenceProp`` -- compiled unmodified by
``oracle/Makefile`` (``make -C oracle ref``; needs the reference sources) on
seeded inputs.  Run from the repository root:

    make -C oracle ref && python tests/golden/make_golden.py
"""
from __future__ import annotations

import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle as O  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "ref_golden.npz")


def field(rng, shape):
    """Binary amplitude (p = 0.5) x uniform phase, the propagation workload's distribution."""
    amp = (rng.random(shape) < 0.5).astype(np.float64)
    return amp * np.exp(2j * np.pi * rng.random(shape))


def refcall(fn, u, *args):
    u = np.ascontiguousarray(u, np.complex128).copy()
    fn(O._ptr(u), u.shape[0], u.shape[1], *args)
    return u


def main():
    R = O.ref()
    rng = np.random.default_rng(20261203)
    g = {}
    prop_cases = [
        # (ny, nx, dy, dx, lambda, z)
        (16, 16, 8e-6, 8e-6, 532e-9, 0.05),
        (32, 64, 8e-6, 8e-6, 532e-9, 0.05),
        (64, 32, 4e-6, 6e-6, 633e-9, -0.02),
        (64, 64, 20e-6, 20e-6, 532e-9, 0.01),   # band limit active
        (128, 128, 3.74e-6, 3.74e-6, 532e-9, 0.1),
        (24, 40, 8e-6, 8e-6, 450e-9, 0.03),     # not a power of two: oracle-only case
    ]
    for i, (ny, nx, dy, dx, lam, z) in enumerate(prop_cases):
        u = field(rng, (ny, nx))
        g[f"prop{i}_params"] = np.array([ny, nx, dy, dx, lam, z])
        g[f"prop{i}_in"] = u
        g[f"prop{i}_asm"] = refcall(R.ref_asm_prop, u, dy, dx, lam, z)
        g[f"prop{i}_fresnel"] = refcall(R.ref_fresnel_prop, u, dy, dx, lam, z)
        g[f"prop{i}_fresnel_bl"] = refcall(R.ref_fresnel_prop_bandlimit, u, dy, dx, lam, z)
    g["n_prop"] = np.array(len(prop_cases))

    # AUTO dispatcher: one case per branch (ASM / Fresnel / band-limited Fresnel)
    n2, p2, l2 = 64, 2e-6, 633e-9
    u2 = 1.0 / (2 * p2)
    zmax = np.sqrt(1 / l2**2 - 2 * u2**2) / (2 * u2 * (1 / (p2 * n2)))
    zmin = n2 * p2 * p2 / l2
    auto_cases = [(32, 32, 8e-6, 8e-6, 532e-9, 0.005), (32, 32, 8e-6, 8e-6, 532e-9, 2.0),
                  (32, 32, p2, p2, l2, 0.5 * (zmax + zmin))]
    for i, (ny, nx, dy, dx, lam, z) in enumerate(auto_cases):
        u = field(rng, (ny, nx))
        g[f"auto{i}_params"] = np.array([ny, nx, dy, dx, lam, z])
        g[f"auto{i}_in"] = u
        g[f"auto{i}_out"] = refcall(R.ref_prop, u, dy, dx, lam, z, 2)
        g[f"auto{i}_branch"] = np.array([R.ref_asm_prop_check(ny, nx, dy, dx, lam, z),
                                         R.ref_fresnel_prop_check(ny, nx, dy, dx, lam, z)])
    g["n_auto"] = np.array(len(auto_cases))

    # AUTO checks in float and double over a sweep of distances
    chk = []
    for (ny, nx, p, lam) in [(1024, 1024, 8e-6, 532e-9), (4096, 4096, 4e-6, 532e-9), (2160, 3840, 3.74e-6, 532e-9)]:
        for z in np.geomspace(1e-3, 3.0, 25):
            chk.append([ny, nx, p, lam, z,
                        R.ref_asm_prop_check(ny, nx, p, p, lam, z), R.ref_asm_prop_check_f(ny, nx, p, p, lam, z),
                        R.ref_fresnel_prop_check(ny, nx, p, p, lam, z), R.ref_fresnel_prop_check_f(ny, nx, p, p, lam, z)])
    g["checks"] = np.array(chk)

    # Fresnel-form point-cloud CGH
    for i, (ny, nx, py, px, lam, n) in enumerate([(24, 40, 8e-6, 8e-6, 532e-9, 7), (32, 48, 6e-6, 8e-6, 633e-9, 13)]):
        pts = np.stack([rng.random(n) * nx * px, rng.random(n) * ny * py, 0.02 + rng.random(n) * 0.02], 1)
        pts = pts.astype(np.float32).astype(np.float64)  # representable as the float32 points the GPU takes
        U = np.zeros((ny, nx), np.complex128)
        R.ref_cgh(O._ptr(np.ascontiguousarray(pts)), n, O._ptr(U), ny, nx, py, px, lam)
        g[f"cgh{i}_params"] = np.array([ny, nx, py, px, lam])
        g[f"cgh{i}_pts"] = pts
        g[f"cgh{i}_U"] = U
        if py == px:
            ph = np.zeros((ny, nx), np.float64)
            R.ref_cgh_phase(O._ptr(np.ascontiguousarray(pts)), n, O._ptr(ph), ny, nx, py, lam)
            g[f"cgh{i}_phase"] = ph
    g["n_cgh"] = np.array(2)

    # 8-bit quantisers
    u = field(rng, (16, 24)) * (0.2 + rng.random((16, 24)))
    g["q_in"] = u
    for mode in range(4):
        img = np.zeros((16, 24), np.uint8)
        R.ref_complex2img(O._ptr(np.ascontiguousarray(u)), O._ptr(img), 16, 24, mode)
        g[f"q_mode{mode}"] = img
    real = np.ascontiguousarray(u.real)
    img = np.zeros((16, 24), np.uint8)
    R.ref_quant8bit(O._ptr(real.copy()), O._ptr(img), 16, 24)
    g["q_quant8bit"] = img

    # shifted / split propagation (a separate generator: the cases above stay as they were)
    rs = np.random.default_rng(20261204)
    shifted = [(32, 32, 8e-6, 8e-6, 532e-9, 0.02, 1e-4, -2e-4), (32, 64, 6e-6, 8e-6, 633e-9, 0.05, 3e-4, 5e-4),
               (64, 32, 4e-6, 4e-6, 532e-9, -0.01, -1e-4, 2e-4), (32, 32, 8e-6, 8e-6, 532e-9, 0.02, 2.56e-4, 0.0)]
    for i, (ny, nx, dy, dx, lam, z, oy, ox) in enumerate(shifted):
        u = field(rs, (ny, nx))
        d = np.zeros_like(u)
        R.ref_shifted_asm_prop(O._ptr(np.ascontiguousarray(u)), O._ptr(d), ny, nx, dy, dx, lam, z, oy, ox)
        g[f"shasm{i}_params"] = np.array([ny, nx, dy, dx, lam, z, oy, ox])
        g[f"shasm{i}_in"] = u
        g[f"shasm{i}_out"] = d
    g["n_shasm"] = np.array(len(shifted))
    shfr = [(32, 32, 8e-6, 8e-6, 532e-9, 0.02, 1.0, 1e-4, -2e-4), (32, 64, 6e-6, 8e-6, 633e-9, 0.05, 0.7, 3e-4, 5e-4),
            (64, 32, 4e-6, 4e-6, 450e-9, -0.03, 1.3, 0.0, 1e-4)]
    for i, (ny, nx, dy, dx, lam, z, sc, oy, ox) in enumerate(shfr):
        u = field(rs, (ny, nx))
        g[f"shfr{i}_params"] = np.array([ny, nx, dy, dx, lam, z, sc, oy, ox])
        g[f"shfr{i}_in"] = u
        g[f"shfr{i}_out"] = refcall(R.ref_shifted_fresnel_prop, u, dy, dx, lam, z, sc, oy, ox)
    g["n_shfr"] = np.array(len(shfr))
    split = [(64, 64, 8e-6, 8e-6, 532e-9, 0.01, 2, 2), (64, 128, 8e-6, 8e-6, 532e-9, 0.02, 2, 4)]
    for i, (ny, nx, dy, dx, lam, z, by, bx) in enumerate(split):
        u = field(rs, (ny, nx))
        g[f"split{i}_params"] = np.array([ny, nx, dy, dx, lam, z, by, bx])
        g[f"split{i}_in"] = u
        g[f"split{i}_out"] = refcall(R.ref_split_asm_prop, u, dy, dx, lam, z, by, bx)
    g["n_split"] = np.array(len(split))

    # tilted-plane propagation (its own generator): ol::TiltedSourceProp /
    # ol::TiltedReferenceProp in PREC_T = double
    rt = np.random.default_rng(20261206)
    tilt = [
        # ny, nx, dy, dx, lam, z, angle, interp, mode, reference
        (32, 32, 8e-6, 8e-6, 532e-9, 0.02, 0.1, 0, 0, 0),
        (32, 48, 8e-6, 6e-6, 633e-9, 0.01, -0.2, 1, 0, 0),
        (32, 32, 8e-6, 8e-6, 532e-9, 0.02, 0.15, 0, 1, 0),
        (24, 40, 8e-6, 8e-6, 532e-9, 0.03, 0.05, 1, 1, 0),
        (32, 32, 8e-6, 8e-6, 532e-9, 0.02, 2e-3, 0, 0, 1),
        (32, 32, 8e-6, 8e-6, 532e-9, -0.02, -4e-3, 1, 0, 1),
        (32, 64, 8e-6, 8e-6, 532e-9, 0.02, 3e-3, 0, 1, 1),
        (40, 24, 6e-6, 8e-6, 633e-9, 0.03, -2e-3, 1, 1, 1),
    ]
    for i, (ny, nx, dy, dx, lam, z, ang, ip, mode, refm) in enumerate(tilt):
        u = field(rt, (ny, nx))
        g[f"tilt{i}_params"] = np.array([ny, nx, dy, dx, lam, z, ang, ip, mode, refm], np.float64)
        g[f"tilt{i}_in"] = u
        g[f"tilt{i}_out"] = refcall(R.ref_tilted_prop, u, dy, dx, lam, z, ang, ip, mode, refm)
    g["n_tilt"] = np.array(len(tilt))

    # point files, objset / objsort and BMP files (their own generator)
    import tempfile
    ro = np.random.default_rng(20261205)
    pts = np.stack([ro.integers(-200, 201, 500), ro.integers(-150, 151, 500), ro.integers(0, 40, 500)], 1)
    with tempfile.TemporaryDirectory() as td:
        f3d = os.path.join(td, "obj.3d")
        with open(f3d, "wb") as f:
            f.write(np.int32(len(pts)).tobytes() + pts.astype(np.int32).tobytes())
        g["obj_3d_bytes"] = np.frombuffer(open(f3d, "rb").read(), np.uint8)
        out = np.zeros((len(pts), 3), np.float32)
        assert R.ref_objread(f3d.encode(), O._ptr(out), len(pts)) == len(pts)
        g["obj_read"] = out.copy()
        sc = np.zeros_like(out)
        R.ref_objread_scaled(f3d.encode(), 1e-3, -2e-3, 0.1, 1.7e-5, O._ptr(sc), len(pts))
        g["obj_read_scaled"] = sc
        f3df = os.path.join(td, "obj.3df")
        fl = (ro.random((64, 3)) * 0.01 - 0.005).astype(np.float32)
        with open(f3df, "wb") as f:
            f.write(np.int32(len(fl)).tobytes() + fl.tobytes())
        g["obj_3df_bytes"] = np.frombuffer(open(f3df, "rb").read(), np.uint8)
        o2 = np.zeros((64, 3), np.float32)
        R.ref_objread(f3df.encode(), O._ptr(o2), 64)
        g["obj_read_3df"] = o2
        cases = [(5e-3, -1.0, 0), (5e-3, -1.0, 1), (6e-3, 4e-3, 0), (3e-3, 7e-3, 1)]
        for i, (xr, yr, mode) in enumerate(cases):
            q = out.copy()
            R.ref_objset(O._ptr(q), len(q), xr, yr, 7.68e-3, 4.32e-3, 0.1, mode)
            g[f"objset{i}_params"] = np.array([xr, yr, 7.68e-3, 4.32e-3, 0.1, mode], np.float64)
            g[f"objset{i}_out"] = q
        g["n_objset"] = np.array(len(cases))
        q = out.copy()
        R.ref_objsort(O._ptr(q), len(q))
        g["objsort_out"] = q
        for i, (ny, nx) in enumerate([(5, 8), (4, 9), (3, 10), (6, 11)]):
            img = ro.integers(0, 256, (ny, nx)).astype(np.uint8)
            fb = os.path.join(td, f"img{i}.bmp")
            R.ref_bmpwrite(fb.encode(), O._ptr(img), ny, nx)
            g[f"bmp{i}_img"] = img
            g[f"bmp{i}_bytes"] = np.frombuffer(open(fb, "rb").read(), np.uint8)
        g["n_bmp"] = np.array(4)

    np.savez_compressed(OUT, **g)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
