"""Time the reference's OWN GPU implementation of the hot path on this GPU.

TEST INFRASTRUCTURE ONLY: a measurement of the reference for comparison, not
part of the product.  Builds oracle/ref_gpu_harness.cu against the staged
copy of the reference headers (oracle/_ref/include; `make -C oracle
ref-gpu-src` where the reference tree exists) and runs its timing modes on
the workloads of the benchmark:

  asm      gAsmProp (golprop.h:507-534), 1024^2 field, p = 8 um, 532 nm, 50 mm
  fresnel  gFresnelProp (golprop.h:167-198), the same field
  arss     ARSSFresnelProp (golprop.h:941-990), the same field, s = 0.5
  cgh      gCgh -> gCghShared (golcgh.h:47-88, 137-145), 10,000 points in a
           5 mm box at 100 mm, p = 8 um, 532 nm, on 1920 x 1088: gCghShared
           calls __syncthreads() inside its bounds check, so a hologram whose
           height is not a multiple of its 16-row blocks (1080) would run a
           barrier that only part of a block reaches; 1088 rows avoid that,
           and the rate is reported per point.pixel
  wrp      WRPMethod (golcgh.h:561-581), 200,000 points 1-5 mm behind a 4096^2
           WRP, p = 4 um, 532 nm (its step 1 tests every point at every pixel)

Each call is the reference's whole wrapper (its own allocations, cuFFT plan
creation and synchronisation), timed with CUDA events.  Prints one JSON line.

    python oracle/time_reference_gpu.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
HARNESS = os.path.join(HERE, "_ref", "ref_gpu_harness")


def run(args):
    r = subprocess.run([HARNESS, *map(str, args)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(map(str, args)) + "\n" + r.stdout + r.stderr)
    mode, ms, reps = r.stdout.strip().splitlines()[-1].split()
    return float(ms)


def main():
    subprocess.run(["make", "-s", "-C", HERE, "ref-gpu"], check=True)
    out = {}
    for mode in ("asm", "fresnel", "arss"):
        ms = run([f"time-{mode}", 1024, 1024, 8e-6, 532e-9, 0.05, 20])
        out[mode] = {"ms": ms, "props/s": 1e3 / ms, "workload": "1024^2 padded 2048^2, p=8um, 532nm, z=50mm"}
    ms = run(["time-cgh", 1088, 1920, 10000, 8e-6, 532e-9, 5])
    out["cgh"] = {"ms": ms, "point.pixel/s": 1088 * 1920 * 10000 / (ms * 1e-3),
                  "workload": "gCghShared, 1920x1088 (see docstring), 10000 points, p=8um, 532nm, 5mm box at 100mm"}
    ms = run(["time-wrp", 4096, 200000, 4e-6, 532e-9, 1])
    out["wrp"] = {"ms": ms, "holograms/s": 1e3 / ms,
                  "workload": "WRPMethod, 200000 points 1-5mm behind a 4096^2 WRP, p=4um, 532nm"}
    print(json.dumps({"reference_gpu": out}))
    return 0


if __name__ == "__main__":
    sys.exit(main())
