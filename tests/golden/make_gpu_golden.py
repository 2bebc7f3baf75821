"""Generate tests/golden/ref_gpu_golden.npz from the reference's OWN GPU code.

The reference implements ARSS propagation (golprop.h:816-995) and the
windowed WRP step 1 (golcgh.h:291-491) only as CUDA kernels; it has no CPU
version to build.  This script builds oracle/ref_gpu_harness.cu (a
project-written driver) against an unmodified copy of the reference headers
in oracle/_ref/include (`make -C oracle ref-gpu-src` copies them where the
reference tree exists; they are never committed), runs the harness on
seeded inputs on a GPU, and stores inputs and outputs.

Run on a machine with a GPU:
    python tests/golden/make_gpu_golden.py [OUT.npz]

Cases:
  arss_*  ARSSFresnelProp<float> (golprop.h:941-990) and its three stages:
          gARSSFresnelProp_u (windowed pre-chirp), gARSSFresnelProp_Cz on a
          field of ones (post-chirp, 1 outside its window), gARSSFresnelProp_h
          (impulse-response chirp with its window, padded grid).  The window
          limits cut into the field in all but one case; one case has s < 0,
          where the reference's pre-chirp window is empty.
  wrp_*   WRPStep1 (circle, golcgh.h:369-389) and WRPStep1_D (square,
          golcgh.h:470-491), with and without p_limit: single points and
          sparse grids whose windows do not overlap (so the output support IS
          the window set), and dense random clouds for the values.
"""
from __future__ import annotations

import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
ORACLE = os.path.join(ROOT, "oracle")
HARNESS = os.path.join(ORACLE, "_ref", "ref_gpu_harness")
SEED = 20261204

ARSS_CASES = [
    # name, ny, nx, dy, dx, lambda, z, s, oy, ox
    ("arss_a", 64, 64, 8e-6, 8e-6, 532e-9, 1.0e-3, 0.5, 0.0, 0.0),
    ("arss_b", 32, 64, 16e-6, 8e-6, 633e-9, 2.0e-3, 2.0, 1.0e-4, -5.0e-5),
    ("arss_c", 64, 64, 8e-6, 8e-6, 532e-9, -1.5e-3, 0.7, 0.0, 3.0e-5),
    ("arss_d", 64, 64, 8e-6, 8e-6, 532e-9, 5.0e-2, 0.5, 0.0, 0.0),
    ("arss_e", 64, 32, 8e-6, 8e-6, 450e-9, 1.2e-3, 1.6, -4.0e-5, 0.0),
    ("arss_f", 32, 32, 8e-6, 8e-6, 532e-9, 1.0e-3, -0.5, 0.0, 0.0),
]


def _field(rng, ny, nx):
    amp = (rng.random((ny, nx)) < 0.5).astype(np.float64)
    return (amp * np.exp(2j * np.pi * rng.random((ny, nx)))).astype(np.complex64)


def _sparse_points(rng, ny, nx, p, plane_z, step, dz_lo, dz_hi):
    """One point per step x step cell, near the cell centre, so windows of
    radius < step / 2 pixels never overlap."""
    pts = []
    for cy in range(step // 2, ny, step):
        for cx in range(step // 2, nx, step):
            x = (cx + rng.uniform(-0.5, 0.5)) * p
            y = (cy + rng.uniform(-0.5, 0.5)) * p
            pts.append((x, y, plane_z + rng.uniform(dz_lo, dz_hi)))
    return np.asarray(pts, np.float32)


def wrp_cases(rng):
    p, lam, pz = 4e-6, 532e-9, 0.01
    cases = []
    one = np.asarray([[(31.3) * p, (30.7) * p, pz + 1.0e-3]], np.float32)
    for window in (0, 1):
        cases.append((f"wrp_single_w{window}", one, 64, 64, p, lam, pz, window, 0.0))
    sp = _sparse_points(rng, 128, 128, p, pz, 32, 0.3e-3, 0.9e-3)
    for window in (0, 1):
        cases.append((f"wrp_sparse_w{window}", sp, 128, 128, p, lam, pz, window, 0.0))
    # p_limit = 8 um doubles the divisor of W_j (about 30): radii 5-14.5 px
    sp2 = _sparse_points(rng, 128, 128, p, pz, 32, 0.6e-3, 1.75e-3)
    for window in (0, 1):
        cases.append((f"wrp_plimit_w{window}", sp2, 128, 128, p, lam, pz, window, 8e-6))
    # dense: points beyond the edges, 20 % in front of the plane (dz < 0)
    n = 600
    dz = rng.uniform(0.3e-3, 2.0e-3, n) * np.where(rng.random(n) < 0.2, -1.0, 1.0)
    dense = np.stack([rng.uniform(-8, 136, n) * p, rng.uniform(-8, 136, n) * p, pz + dz], 1).astype(np.float32)
    for window in (0, 1):
        cases.append((f"wrp_dense_w{window}", dense, 128, 128, p, lam, pz, window, 0.0))
    return cases


def run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(cmd) + "\n" + r.stdout + r.stderr)


def main(out_path: str) -> None:
    run(["make", "-s", "-C", ORACLE, "ref-gpu"])
    rng = np.random.default_rng(SEED)
    out = {}
    with tempfile.TemporaryDirectory() as tmp:
        for name, ny, nx, dy, dx, lam, z, s, oy, ox in ARSS_CASES:
            u = _field(rng, ny, nx)
            fin = os.path.join(tmp, "in.bin")
            u.tofile(fin)
            run([HARNESS, "arss", fin, tmp, str(ny), str(nx), repr(dy), repr(dx), repr(lam), repr(z), repr(s),
                 repr(oy), repr(ox)])
            out[name + "_in"] = u
            out[name + "_par"] = np.asarray([ny, nx, dy, dx, lam, z, s, oy, ox], np.float64)
            for stage, shape in (("u", (ny, nx)), ("cz", (ny, nx)), ("h", (2 * ny, 2 * nx)), ("out", (ny, nx))):
                out[f"{name}_{stage}"] = np.fromfile(os.path.join(tmp, f"arss_{stage}.bin"),
                                                     np.complex64).reshape(shape)
        for name, pts, ny, nx, p, lam, pz, window, plimit in wrp_cases(rng):
            fp = os.path.join(tmp, "pts.bin")
            fo = os.path.join(tmp, "wrp.bin")
            pts.tofile(fp)
            run([HARNESS, "wrp", fp, fo, str(len(pts)), str(ny), str(nx), repr(p), repr(lam), repr(pz),
                 str(window), repr(plimit)])
            out[name + "_pts"] = pts
            out[name + "_par"] = np.asarray([ny, nx, p, lam, pz, window, plimit], np.float64)
            out[name + "_out"] = np.fromfile(fo, np.complex64).reshape(ny, nx)
    np.savez_compressed(out_path, **out)
    print(f"wrote {out_path}: {len(ARSS_CASES)} ARSS cases, {len(wrp_cases(np.random.default_rng(0)))} WRP cases")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "ref_gpu_golden.npz"))
