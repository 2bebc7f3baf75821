#!/usr/bin/env python
"""Benchmark of the OpenOL hot path on GB300.

Default workload (N = 1): point-cloud CGH on a 1920 x 1080 hologram, pitch
8 um, lambda = 532 nm, 10,000 points uniform in a 5 x 5 x 5 mm box centred at
(W/2 p, H/2 p, 100 mm), amplitudes U[0.5, 1], phases U[0, 2 pi) -- metric
point.pixel/s (one step = one hologram = 2.07e10 point.pixels).  Other
workloads: ``--workload asm`` (1024^2 field padded to 2048^2, p = 8 um,
532 nm, z = 50 mm; props/s), ``--workload wrp`` (200,000 points 1-5 mm behind
a 4096^2 WRP, p = 4 um, then ASM by 150 mm and the binarised 8-bit hologram;
holograms/s), ``--workload adam`` (2048^2 phase, 8 planes at 80..150 mm,
p = 6.4 um; one Adam step with the adjoint gradient; grad-steps/s),
``--workload batch`` (96 fields of 512^2..4096^2, ASM / Fresnel / ARSS, RGB,
one CUDA graph; props/s), ``--workload tilt`` (tilted planes beside the path).

Our arm prints one JSON line with value (device-resident inputs, CUDA events
on the launching stream, L2 flushed between steps), e2e (host buffers, copies
inside the timed region, through the public API), roofline of the dominant
kernel, accuracy (relative L2 and maximum phase error against the FP64
oracle; for the binarised WRP hologram, the pixels that differ and how many
of them lie within one float32 ulp of the threshold), a CPU baseline (the
FP64 oracle port on the host cores, bounded sample) and the clocks sampled
during the timed region.  The default line also carries ``configs``: the
ASM, WRP, Adam and batch configurations, each run briefly (at most 5 timed
steps) with its value, e2e, roofline fraction and accuracy
(``--no-configs`` skips them).

``--impl reference`` times the reference's CPU implementation of the same
workload (the FP64 restatement in oracle/, OpenMP over all host threads) on a
bounded sample per step; under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WRP_DESC = "wrp 200000 points 1-5mm behind a 4096x4096 WRP, p=4um, lambda=532nm, ASM 150mm, binarised 8-bit"
ADAM_DESC = "adam 2048x2048 phase, 8 planes z=80..150mm, p=6.4um, lambda=532nm, 5% sparse targets"
CGH = dict(ny=1080, nx=1920, p=8e-6, lam=532e-9, n=10000, zc=0.1, box=5e-3, seed=20261203 + 2)
ASM = dict(n=1024, p=8e-6, lam=532e-9, z=0.05, seed=20261203 + 1)
# the reference's default test field (tests/para.h: 1920*2 x 1080*2, p = 3.74 um,
# 532 nm, d = -0.1 m), padded to 7680 x 4320: mixed-radix passes
UHD = dict(ny=2160, nx=3840, p=3.74e-6, lam=532e-9, z=-0.1, seed=20261203 + 7)
UHD_DESC = "asm 3840x2160 padded 7680x4320 (mixed radix), p=3.74um, lambda=532nm, z=-100mm"
WRP = dict(N=4096, p=4e-6, lam=532e-9, n=200000, zw=0.15, ext=10e-3, seed=20261203 + 3)
# tilted planes (the row beside the path): the ASM workload's field, rotated 0.1 rad (source form)
# or 2 mrad (reference form: its frequency shift a13 / (lambda du) is ~30 samples per mrad here)
BATCH_DESC = ("batch 96 fields, sizes U{512,1024,2048,4096}^2, ASM/Fresnel/ARSS (s=0.5), z U[10,300]mm, "
              "lambda U{640,532,450}nm, p=8um; one CUDA graph: one persistent launch for the fields below 2048^2, "
              "then the autotuned single-field passes for the 2048^2 and 4096^2 fields")
TILT = dict(n=1024, p=8e-6, lam=532e-9, z=0.05, angle=0.1, angle_ref=2e-3, seed=20261203 + 1)
TILT_DESC = ("tilt 1024x1024 padded 2048x2048, p=8um, lambda=532nm, z=50mm, TiltedSourceProp ASM bilinear, "
             "0.1 rad")
ADAM = dict(n=2048, p=6.4e-6, lam=532e-9, planes=8, z0=0.08, dz=0.01, lr=0.05, seed=20261203 + 4)


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of the
# kernels each roofline covers, from ncu captures of this bench's own timed
# region (--ncu-range); the profile file named beside each holds the command.
TRAFFIC = {
    "cgh": (360.2e6 + 14.6e6, "k_cgh_gemm2 (two-SM tiles), profiles/cgh_gemm_1920x1080_10k.md"),
    "asm": ((8.5 + 16.9 + 16.8) * 1e6, "the three passes, profiles/asm_1024_kernels.md (S stays in L2)"),
    "wrp": ((134.4 + 205.0 + 268.5 + 211.6 + 268.5 + 99.1) * 1e6,
            "the three 8192-point passes of step 2, profiles/asm_4096_to_8192_wrp_step2.md"),
    "uhd": ((66.5 + 70.8 + 132.8 + 76.0 + 132.8 + 33.3) * 1e6,
            "the three mixed-radix passes, profiles/asm_3840x2160_mixed_radix.md"),
    "adam": (4656.1e6, "every kernel of one step, the bench's L2 flush excluded (S and the spectra partly stay in "
                       "L2), profiles/phase_grad_2048_8planes.md"),
}


def traffic(name):
    t = TRAFFIC.get(name)
    return (t[0], t[1]) if t else (None, None)


def pinned_variants(og, tuned, spec):
    """--variants "kind:n=i,...": set these launch shapes after the autotuner
    (so that a profiler run launches the kernels a plain run chose, whatever
    the autotuner's timings under the profiler say) and report them."""
    if not spec:
        return tuned
    for item in spec.split(","):
        key, idx = item.split("=")
        kind, n = (int(v) for v in key.split(":"))
        og.set_variant(kind, n, int(idx))
        tuned[(kind, n)] = int(idx)
    return tuned


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f), "measured"
    except OSError:
        return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0, "sm_max_mhz": 2070.0}, \
            "fallback"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.idx = gpu_index
        self.proc = None
        self.f = None

    def __enter__(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:  # nvidia-smi missing: the line then says so
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if self.proc is None or self.f is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        mx = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in rows for k in range(4) if r[5 + k].lower().startswith("active")})
        busy = [s for s in sm if s > 0.5 * max(sm)] or sm
        return {"sm_mhz": statistics.median(busy) if busy else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(rows)}


# ------------------------------------------------------------------ helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def cgh_inputs():
    c = CGH
    rng = np.random.default_rng(c["seed"])
    ctr = np.array([c["nx"] / 2 * c["p"], c["ny"] / 2 * c["p"], c["zc"]])
    pts = (ctr + (rng.random((c["n"], 3)) - 0.5) * c["box"]).astype(np.float32)
    amp = (0.5 + 0.5 * rng.random(c["n"])).astype(np.float32)
    ph = (2 * np.pi * rng.random(c["n"])).astype(np.float32)
    return pts, amp, ph


def asm_input():
    rng = np.random.default_rng(ASM["seed"])
    n = ASM["n"]
    return ((rng.random((n, n)) < 0.5) * np.exp(2j * np.pi * rng.random((n, n)))).astype(np.complex64)


def cpu_cgh_sample(rows):
    """FP64 oracle (OpenMP, all host threads) on `rows` hologram rows: point.pixels/s."""
    import oracle as O
    pts, amp, ph = cgh_inputs()
    c = CGH
    sp = pts.astype(np.float64)
    t0 = time.perf_counter()
    U = O.cgh_fresnel(sp, rows, c["nx"], c["p"], c["p"], c["lam"], amp=amp.astype(np.float64),
                      phase0=ph.astype(np.float64))
    dt = time.perf_counter() - t0
    return rows * c["nx"] * c["n"] / dt, dt, U


def cpu_asm_sample():
    import oracle as O
    u = asm_input().astype(np.complex128)
    t0 = time.perf_counter()
    r = O.asm_prop(u, ASM["p"], ASM["p"], ASM["lam"], ASM["z"])
    return 1.0 / (time.perf_counter() - t0), r


def uhd_input():
    rng = np.random.default_rng(UHD["seed"])
    shape = (UHD["ny"], UHD["nx"])
    return ((rng.random(shape) < 0.5) * np.exp(2j * np.pi * rng.random(shape))).astype(np.complex64)


def cpu_uhd_sample():
    import oracle as O
    u = uhd_input().astype(np.complex128)
    t0 = time.perf_counter()
    r = O.asm_prop(u, UHD["p"], UHD["p"], UHD["lam"], UHD["z"])
    return 1.0 / (time.perf_counter() - t0), r


def cpu_tilt_sample():
    import oracle as O
    u = asm_input().astype(np.complex128)
    t0 = time.perf_counter()
    r = O.tilted_prop(u, TILT["p"], TILT["p"], TILT["lam"], TILT["z"], TILT["angle"], 0, 0, False)
    return 1.0 / (time.perf_counter() - t0), r


def batch_draw():
    """Sizes, methods, distances and wavelengths of the 96 batch fields, drawn
    as openol_gb300.config5_fields draws them."""
    rng = np.random.default_rng(20261203 + 5)
    sizes = rng.choice([512, 1024, 2048, 4096], 96)
    methods = rng.choice(["asm", "fresnel", "arss"], 96)
    zs = 0.01 + 0.29 * rng.random(96)
    lams = rng.choice([640e-9, 532e-9, 450e-9], 96)
    return sizes, methods, zs, lams


def cpu_batch_sample(inputs=None):
    """One field of each size class propagated by the FP64 oracle (its own
    method, z, lambda), every field of that class costed as it.  inputs:
    {size: (field index, complex64 field)} -- the GPU batch's own inputs --
    or None for seeded fields.  Returns props/s, the per-class seconds and
    {size: (field index, FP64 result)}."""
    import oracle as O
    sizes, methods, zs, lams = batch_draw()
    t_cls, refs = {}, {}
    fr = np.random.default_rng(5)
    for m in (512, 1024, 2048, 4096):
        k = int(np.nonzero(sizes == m)[0][0])
        if inputs is not None:
            k, u = inputs[m]
        else:
            u = (fr.random((m, m)) < 0.5) * np.exp(2j * np.pi * fr.random((m, m)))
        u = np.asarray(u, np.complex128)
        t0 = time.perf_counter()
        if methods[k] == "asm":
            r = O.asm_prop(u, 8e-6, 8e-6, float(lams[k]), float(zs[k]))
        elif methods[k] == "fresnel":
            r = O.fresnel_prop(u, 8e-6, 8e-6, float(lams[k]), float(zs[k]))
        else:
            r = O.arss_prop(u, 8e-6, 8e-6, float(lams[k]), float(zs[k]), 0.5)
        t_cls[m] = time.perf_counter() - t0
        refs[m] = (k, r)
    total = sum(t_cls[int(m)] for m in sizes)
    return 96 / total, t_cls, refs


def wrp_points():
    c = WRP
    rng = np.random.default_rng(c["seed"])
    ctr = c["N"] * c["p"] / 2
    x = ctr + (rng.random(c["n"]) - 0.5) * c["ext"]
    y = ctr + (rng.random(c["n"]) - 0.5) * c["ext"]
    z = c["zw"] + 1e-3 + rng.random(c["n"]) * 4e-3
    return np.stack([x, y, z], 1).astype(np.float32)


def adam_problem():
    from openol_gb300.optim import make_targets
    c = ADAM
    rng = np.random.default_rng(c["seed"])
    phi = (2 * np.pi * rng.random((c["n"], c["n"]))).astype(np.float32)
    t = make_targets(c["n"], c["n"], c["planes"], seed=c["seed"] + 1)
    zs = [c["z0"] + c["dz"] * k for k in range(c["planes"])]
    return phi, t, zs


def cpu_wrp_sample(frac=0.01):
    """FP64 oracle WRP step 1 on a seeded 1% subset of the points + the 4096^2 ASM (FP64), scaled."""
    import oracle as O
    c = WRP
    pts = wrp_points()
    sub = pts[: int(len(pts) * frac)]
    p, lam, zw = np.float32(c["p"]), np.float32(c["lam"]), np.float32(c["zw"])
    t0 = time.perf_counter()
    U = O.wrp_step1(sub, c["N"], c["N"], p, lam, zw)
    t1 = time.perf_counter()
    U = O.asm_prop(U, float(p), float(p), float(lam), float(zw))
    t2 = time.perf_counter()
    return 1.0 / ((t1 - t0) / frac + (t2 - t1)), (t1 - t0, t2 - t1), sub, U


def cpu_adam_sample():
    """FP64 oracle loss+gradient for one of the 8 planes at 2048^2 (2 propagations), scaled x8."""
    import oracle as O
    phi, t, zs = adam_problem()
    t0 = time.perf_counter()
    r = O.phase_loss_grad(phi, t[:1], zs[:1], ADAM["p"], ADAM["lam"])
    dt = time.perf_counter() - t0
    return 1.0 / (dt * ADAM["planes"]), dt, r


def accuracy(got, ref, floor=1e-3):
    """Relative L2 and maximum phase error (rad) of a GPU result against its
    FP64 oracle; the phase is compared where |ref| > floor x rms(ref)."""
    got = np.asarray(got, np.complex128)
    ref = np.asarray(ref, np.complex128)
    rel = float(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300))
    rms = float(np.sqrt(np.mean(np.abs(ref) ** 2)))
    m = np.abs(ref) > floor * rms
    ph = float(np.abs(np.angle(got[m] * np.conj(ref[m]))).max()) if m.any() else 0.0
    return {"rel_l2": rel, "max_phase_err_rad": ph, "phase_where": f"|ref| > {floor:g} rms"}


def binarized_accuracy(img, got, ref):
    """The binarised 8-bit hologram (255 where Re U >= 0) against the one the
    FP64 field gives: mismatched pixels, and how many of them lie within one
    float32 ulp of |U| of the threshold, or within the GPU result's own error."""
    img = np.asarray(img)
    ref = np.asarray(ref, np.complex128)
    want = np.where(ref.real >= 0, 255, 0).astype(np.uint8)
    mism = img != want
    ulp = np.spacing(np.abs(ref).astype(np.float32)).astype(np.float64)
    err = float(np.abs(np.asarray(got, np.complex128) - ref).max())
    return {"pixels": int(img.size), "mismatch": int(mism.sum()),
            "mismatch_within_1ulp": int((mism & (np.abs(ref.real) <= ulp)).sum()),
            "mismatch_within_error": int((mism & (np.abs(ref.real) <= err)).sum()),
            "pixels_within_1ulp": int((np.abs(ref.real) <= ulp).sum())}


def cpu_threads():
    return len(os.sched_getaffinity(0)) if hasattr(os, "sched_getaffinity") else os.cpu_count()


# ------------------------------------------------------------- reference arm
def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    wl = args.workload
    vals = []
    if wl == "cgh":
        rows = args.ref_rows
        for k in range(args.warmup + args.steps):
            v, _, _ = cpu_cgh_sample(rows)
            if k >= args.warmup:
                vals.append(v)
        metric, unit = "CGH point.pixel/s", "point.pixel/s"
        sample = f"{rows} of {CGH['ny']} rows x {CGH['nx']} px x {CGH['n']} points per step (FP64 Fresnel-form sum)"
        config = {"workload": "cgh 1920x1080, 10000 points, p=8um, lambda=532nm, 5mm box at z=100mm"}
    elif wl == "asm":
        for k in range(args.warmup + args.steps):
            v, _ = cpu_asm_sample()
            if k >= args.warmup:
                vals.append(v)
        metric, unit = "ASM props/s", "props/s"
        sample = "one full 1024^2 -> 2048^2 FP64 ASM propagation per step"
        config = {"workload": "asm 1024x1024 padded 2048x2048, p=8um, lambda=532nm, z=50mm"}
    elif wl == "wrp":
        for k in range(1 + min(args.steps, 2)):
            v, _, _, _ = cpu_wrp_sample()
            if k >= 1:
                vals.append(v)
        metric, unit = "WRP holograms/s", "holograms/s"
        sample = "WRP step 1 on a seeded 1% point subset (scaled x100) + full 4096^2 FP64 ASM, per step"
        config = {"workload": WRP_DESC}
    elif wl == "batch":
        for k in range(1 + min(args.steps, 2)):
            v, _, _ = cpu_batch_sample()
            if k >= 1:
                vals.append(v)
        metric, unit = "batched props/s", "props/s"
        sample = ("one field per size class (512^2 .. 4096^2) of the 96-field batch, FP64, each class costed "
                  "for all its fields, per step")
        config = {"workload": BATCH_DESC}
    elif wl == "uhd":
        for k in range(1 + min(args.steps, 2)):
            v, _ = cpu_uhd_sample()
            if k >= 1:
                vals.append(v)
        metric, unit = "mixed-radix ASM props/s", "props/s"
        sample = "one full 3840x2160 -> 7680x4320 FP64 ASM propagation per step"
        config = {"workload": UHD_DESC}
    elif wl == "tilt":
        for k in range(1 + min(args.steps, 3)):
            v, _ = cpu_tilt_sample()
            if k >= 1:
                vals.append(v)
        metric, unit = "tilted props/s", "props/s"
        sample = "one full 1024^2 -> 2048^2 FP64 TiltedSourceProp (ASM, bilinear) per step"
        config = {"workload": TILT_DESC}
    else:
        for k in range(1 + min(args.steps, 3)):
            v, _, _ = cpu_adam_sample()
            if k >= 1:
                vals.append(v)
        metric, unit = "grad-steps/s", "grad-steps/s"
        sample = "loss + adjoint gradient for 1 of 8 planes at 2048^2 per step (scaled x8), FP64"
        config = {"workload": ADAM_DESC}
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": config,
            "cpu_baseline": {"value": v, "unit": unit, "cores": cpu_threads(), "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------- our arm
# --ncu-range: the first timed region of the run (the headline form) is
# bracketed by cudaProfilerStart / Stop, so that `ncu --profile-from-start off`
# captures the tuned launches of the measured step, not autotuner trials.
NCU_RANGE = {"on": False, "done": False}


def timed(torch, fn, K, W, flush, stream, barrier):
    for _ in range(W):
        fn()
    torch.cuda.synchronize()
    barrier()
    rng = NCU_RANGE["on"] and not NCU_RANGE["done"]
    if rng:
        torch.cuda.profiler.start()
    evs = []
    for _ in range(K):
        if flush is not None:
            flush.zero_()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        fn()
        e1.record(stream)
        evs.append((e0, e1))
    torch.cuda.synchronize()
    if rng:
        torch.cuda.profiler.stop()
        NCU_RANGE["done"] = True
    barrier()
    return [a.elapsed_time(b) for a, b in evs]


def timed_sequence(torch, fn, K, W, flush, stream, barrier):
    """One timed region around fn(K): a call that runs K steps as one pipelined
    sequence (each step's host copies in and out overlapping its neighbours'
    computation).  Warm-up: one sequence of max(W, 3) steps.  L2 is flushed
    once, before the region; each step's inputs are copied in from host memory
    inside it.  Returns the region's time per step (ms)."""
    fn(max(W, 3))
    torch.cuda.synchronize()
    barrier()
    if flush is not None:
        flush.zero_()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    fn(K)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    return e0.elapsed_time(e1) / K


class _Ctx:
    pass


def wl_cgh(x, K, W, cpu):
    torch, og, pk, pk_kind = x.torch, x.og, x.pk, x.pk_kind
    stream, flush, barrier, max_over_ranks = x.stream, x.flush, x.barrier, x.max_over_ranks
    ws, rank, local, args = x.ws, x.rank, x.local, x.args
    c = CGH
    pts, amp, ph = cgh_inputs()
    obj = og.gObject(pts)
    a = torch.from_numpy(amp).cuda()
    f = torch.from_numpy(ph).cuda()
    U = torch.zeros((c["ny"], c["nx"]), dtype=torch.complex64, device="cuda")
    units = c["ny"] * c["nx"] * c["n"]

    def step_fresnel():
        og.cgh_fresnel(obj, U, ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"], amp=a, phase0=f)

    def step_exact():
        og.cgh_exact(obj, U, ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"], amp=a, phase0=f)

    gemm_pairs, tail_w = og.autotune_cgh_gemm(c["n"], c["ny"], c["nx"])
    gws = og.cgh_gemm_workspace(c["n"], c["ny"], c["nx"])

    def step_gemm():
        og.cgh_fresnel_gemm(obj, U, ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"], amp=a,
                            phase0=f, work=gws)

    def step_gemm_only():
        og.cgh_fresnel_gemm(obj, U, ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"], amp=a,
                            phase0=f, work=gws, reuse_operands=True)

    from openol_gb300.plain import plain_cgh_fresnel

    def step_plain():
        plain_cgh_fresnel(obj, U, ny=c["ny"], nx=c["nx"], p=c["p"], lam=c["lam"])

    # the adjoints (transposed sums) of the two forms, onto the point amplitudes
    Gadj = torch.complex(torch.randn((c["ny"], c["nx"]), device="cuda"), torch.randn((c["ny"], c["nx"]), device="cuda"))
    gadj = torch.zeros(c["n"], dtype=torch.complex64, device="cuda")
    aws = torch.empty(int(og.lib().olg_cgh_adjoint_workspace_bytes(c["n"], c["ny"], c["nx"], 1)), dtype=torch.uint8,
                      device="cuda")

    def step_adj_fresnel():
        og.cgh_fresnel_adjoint(obj, Gadj, gadj, ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"], work=aws)

    def step_adj_exact():
        og.cgh_exact_adjoint(obj, Gadj, gadj, ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"], work=aws)

    agws = og.cgh_adjoint_gemm_workspace(c["n"], c["ny"], c["nx"])

    def step_adj_gemm():
        og.cgh_fresnel_adjoint_gemm(obj, Gadj, gadj, ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"],
                                    work=agws)

    forms = {"fresnel_gemm": step_gemm, "fresnel_gemm_kernel_only": step_gemm_only,
             "fresnel_direct": step_fresnel, "exact": step_exact, "plain_simt": step_plain,
             "fresnel_adjoint": step_adj_fresnel, "fresnel_adjoint_gemm": step_adj_gemm,
             "exact_adjoint": step_adj_exact}
    chosen = "fresnel_gemm"
    res = {}
    with ClockSampler(local) as clk:
        for name, fn in forms.items():
            l0 = og.launch_count()
            ms = timed(torch, fn, K, W, flush, stream, barrier)
            launches = (og.launch_count() - l0) // (K + W) * K
            res[name] = (ms, launches)
    clocks = clk.summary()
    og.device_fault_check()
    ms_c, launches = res[chosen]
    t_step = max_over_ranks(statistics.mean(ms_c))
    value = ws * units / (t_step * 1e-3)
    # e2e: pinned host inputs in, hologram out, through the public API
    hp = torch.from_numpy(pts).pin_memory()
    ha = torch.from_numpy(amp).pin_memory()
    hf = torch.from_numpy(ph).pin_memory()
    hU = torch.empty((c["ny"], c["nx"]), dtype=torch.complex64).pin_memory()

    def step_e2e():
        obj.points.copy_(hp, non_blocking=True)
        a.copy_(ha, non_blocking=True)
        f.copy_(hf, non_blocking=True)
        step_gemm()
        hU.copy_(U, non_blocking=True)

    ms_e = timed(torch, step_e2e, K, W, flush, stream, barrier)
    # e2e, pipelined: the K steps as one sequence through the host-cloud call
    # (olg_cgh_fresnel_gemm_host_c64): every step's cloud goes up and its
    # hologram comes down inside the region, hologram i-1's copy out and cloud
    # i+1's copy in overlapping hologram i's GEMM
    hseq = [torch.empty((c["ny"], c["nx"]), dtype=torch.complex64).pin_memory() for _ in range(max(K, W, 3))]
    hp3 = hp.reshape(-1, 3)

    def seq_e2e(k):
        og.cgh_fresnel_gemm_host([hp3] * k, hseq[:k], ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"],
                                 amp=[ha] * k, phase0=[hf] * k, stream=stream)

    ms_seq = timed_sequence(torch, seq_e2e, K, W, flush, stream, barrier)
    step_gemm()
    torch.cuda.synchronize()
    seq_err = float(np.linalg.norm(hseq[K - 1].numpy() - U.cpu().numpy()) / np.linalg.norm(U.cpu().numpy()))
    seq_ok = seq_err < 1e-6
    e2e_form = "pipelined_sequence" if seq_ok and ms_seq < statistics.mean(ms_e) else "per_step_copies"
    t_e2e = max_over_ranks(ms_seq if e2e_form == "pipelined_sequence" else statistics.mean(ms_e))
    # tensor roofline of the dominant kernel (k_cgh_gemm, timed alone with the
    # operands already built): issued f16 MMA work 24 M N K flop per hologram
    ms_g = statistics.mean(res["fresnel_gemm_kernel_only"][0])
    kpad = ((2 * c["n"] + 63) // 64) * 64 // 2
    issued = 24.0 * c["ny"] * c["nx"] * kpad
    ach_tf = issued / (ms_g * 1e-3) / 1e12
    nsm = torch.cuda.get_device_properties(0).multi_processor_count
    mhz = clocks.get("sm_mhz") or pk.get("sm_max_mhz", 2070.0)
    peak_gops = nsm * 16 * mhz * 1e6 / 1e9
    sfu_gops = 2 * units / (statistics.mean(res["exact"][0]) * 1e-3) / 1e9
    out = {
        "metric": "CGH point.pixel/s", "value": value, "unit": "point.pixel/s",
        "ms_per_step": t_step,
        "dtype": "f16x3 split products, f32 accumulate",
        "config": {"workload": "cgh 1920x1080, 10000 points, p=8um, lambda=532nm, 5mm box at z=100mm",
                   "form": chosen, "l2": "flushed between steps (256 MiB write)",
                   "gemm_tail_weight": tail_w, "gemm_tiles": "two-SM 256xBN" if gemm_pairs else "single-SM 128xBN"},
        "e2e": {"value": ws * units / (t_e2e * 1e-3), "unit": "point.pixel/s",
                "h2d_bytes_per_step": pts.nbytes + amp.nbytes + ph.nbytes,
                "d2h_bytes_per_step": c["ny"] * c["nx"] * 8, "form": e2e_form,
                "per_step_copies": {"point.pixel/s": ws * units / (statistics.mean(ms_e) * 1e-3),
                                    "ms": statistics.mean(ms_e)},
                "pipelined_sequence": {"point.pixel/s": ws * units / (ms_seq * 1e-3), "ms": ms_seq,
                                       "steps": K, "rel_l2_vs_device_call": seq_err,
                                       "note": "K steps in one olg_cgh_fresnel_gemm_host_c64 call; L2 flushed "
                                               "once before the region"}},
        "gpu_launches": int(launches),
        "roofline": {"bound": "tensor", "achieved": ach_tf, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                     "frac": ach_tf / pk["bf16_tflops"], "traffic": traffic("cgh")[0],
                     "traffic_source": traffic("cgh")[1],
                     "note": f"the GEMM kernel alone ({ms_g:.3f} ms): 24 M N K f16 flop (3 split products x "
                             f"4 real GEMMs; tile padding not counted), useful 8 M N K; "
                             f"peak = {pk_kind} dense bf16 (f16 same rate)"},
        "exact_kernel_sfu": {"achieved": sfu_gops, "peak": peak_gops, "unit": "Gop/s (MUFU)",
                             "frac": sfu_gops / peak_gops,
                             "note": f"exact kernel: 2 MUFU (sin, cos) per term; peak {nsm} SM x 16 MUFU/clk x "
                                     f"{mhz} MHz (a loop of independent __sinf measures 14.9 per SM per clk)"},
        "forms": {k: {"point.pixel/s": units / (statistics.mean(v[0]) * 1e-3), "ms": statistics.mean(v[0])}
                  for k, v in res.items()},
        "clocks": clocks,
    }
    # accuracy against the FP64 oracle on the first rows: the chosen (GEMM)
    # form, the direct FP32 form, the exact kernel
    rows = args.cpu_rows if (rank == 0 and ws == 1 and cpu) else 8
    got = {}
    for name, fn in (("fresnel_gemm", step_gemm), ("fresnel_direct", step_fresnel), ("exact", step_exact)):
        fn()
        torch.cuda.synchronize()
        got[name] = U[:rows].cpu().numpy()
    v, dt, Uref = cpu_cgh_sample(rows)
    import oracle as O
    Uex = O.cgh_exact(pts.astype(np.float64), min(rows, 16), c["nx"], c["p"], c["p"], c["lam"],
                      amp=amp.astype(np.float64), phase0=ph.astype(np.float64))
    out["accuracy"] = {"fresnel_gemm": accuracy(got["fresnel_gemm"], Uref),
                       "fresnel_direct": accuracy(got["fresnel_direct"], Uref),
                       "exact": accuracy(got["exact"][:min(rows, 16)], Uex),
                       "against": f"FP64 oracle, rows 0..{rows - 1} (exact: 0..{min(rows, 16) - 1}) of 1080"}
    if rank == 0 and ws == 1 and cpu:
        out["cpu_baseline"] = {"value": v, "unit": "point.pixel/s", "cores": cpu_threads(), "kind": "port",
                               "sample": f"{args.cpu_rows} of 1080 rows x 1920 px x 10000 points, FP64 oracle, "
                                         f"{dt:.1f} s"}
    return out


def wl_asm(x, K, W, cpu):
    torch, og, pk, pk_kind = x.torch, x.og, x.pk, x.pk_kind
    stream, flush, barrier, max_over_ranks = x.stream, x.flush, x.barrier, x.max_over_ranks
    ws, rank, local, args = x.ws, x.rank, x.local, x.args
    n = ASM["n"]
    tuned = pinned_variants(og, og.autotune(n, n), args.variants)
    u0 = asm_input()
    src = torch.from_numpy(u0).cuda()
    dst = torch.empty_like(src)
    ws_buf = og.workspace(n, n)

    def step():
        og.asm_prop(src, dst, dy=ASM["p"], dx=ASM["p"], lam=ASM["lam"], z=ASM["z"], work=ws_buf)

    from openol_gb300.plain import plain_asm_prop

    def step_plain():
        plain_asm_prop(src, dst, dy=ASM["p"], dx=ASM["p"], lam=ASM["lam"], z=ASM["z"])

    with ClockSampler(local) as clk:
        l0 = og.launch_count()
        ms = timed(torch, step, K, W, flush, stream, barrier)
        launches = (og.launch_count() - l0) // (K + W) * K
        ms_plain = timed(torch, step_plain, K, W, flush, stream, barrier)
    clocks = clk.summary()
    t_step = max_over_ranks(statistics.mean(ms))
    hsrc = torch.from_numpy(u0).pin_memory()
    hdst = torch.empty_like(hsrc).pin_memory()

    def step_e2e():
        src.copy_(hsrc, non_blocking=True)
        step()
        hdst.copy_(dst, non_blocking=True)

    ms_e = timed(torch, step_e2e, K, W, flush, stream, barrier)

    def step_e2e_zero_copy():
        # the public call on the pinned host fields: pass 1 reads the input and
        # pass 3 writes the result over the host link, no staging copies
        og.asm_prop(hsrc, hdst, dy=ASM["p"], dx=ASM["p"], lam=ASM["lam"], z=ASM["z"], work=ws_buf)

    ms_z = timed(torch, step_e2e_zero_copy, K, W, flush, stream, barrier)
    torch.cuda.synchronize()
    zc_equal = bool(torch.equal(hdst, dst.cpu()))  # the same kernels: the same values as the device run
    # pipelined: the K steps as one sequence of host fields through a plan
    # (olg_prop_plan_execute_host), field i+1's copy in and field i-1's copy
    # out overlapping field i's passes
    plan = og.PropPlan("asm", n, n, dy=ASM["p"], dx=ASM["p"], lam=ASM["lam"], z=ASM["z"])
    houts = [torch.empty_like(hsrc).pin_memory() for _ in range(max(K, W, 3))]

    def seq_e2e(k):
        plan.execute_host([hsrc] * k, houts[:k], stream=stream)

    ms_seq = timed_sequence(torch, seq_e2e, K, W, flush, stream, barrier)
    step()
    torch.cuda.synchronize()
    seq_equal = bool(torch.equal(houts[K - 1], dst.cpu()))
    plan.close()
    forms_e2e = {"staged_copies": statistics.mean(ms_e)}
    if zc_equal:
        forms_e2e["zero_copy"] = statistics.mean(ms_z)
    if seq_equal:
        forms_e2e["pipelined_sequence"] = ms_seq
    e2e_form = min(forms_e2e, key=forms_e2e.get)
    t_e2e = max_over_ranks(forms_e2e[e2e_form])
    b_alg = 80 * n * n
    ach = b_alg / (statistics.mean(ms) * 1e-3) / 1e9
    out = {
        "metric": "ASM props/s", "value": ws / (t_step * 1e-3), "unit": "props/s", "ms_per_step": t_step,
        "dtype": "f32",
        "config": {"workload": "asm 1024x1024 padded 2048x2048, p=8um, lambda=532nm, z=50mm",
                   "l2": "flushed between steps (256 MiB write)",
                   "launch_variants": {f"{k}:{m}": v for (k, m), v in tuned.items()}},
        "e2e": {"value": ws / (t_e2e * 1e-3), "unit": "props/s", "h2d_bytes_per_step": u0.nbytes,
                "d2h_bytes_per_step": u0.nbytes, "form": e2e_form},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": traffic("asm")[0],
                     "traffic_source": traffic("asm")[1],
                     "note": f"80 n bytes per propagation (n = 1024^2) over the 3-pass propagation time; "
                             f"peak {pk_kind}"},
        "forms": {"fused": {"props/s": 1e3 / statistics.mean(ms), "ms": statistics.mean(ms)},
                  "plain_cufft": {"props/s": 1e3 / statistics.mean(ms_plain), "ms": statistics.mean(ms_plain)},
                  "e2e_staged_copies": {"props/s": 1e3 / statistics.mean(ms_e), "ms": statistics.mean(ms_e)},
                  "e2e_zero_copy": {"props/s": 1e3 / statistics.mean(ms_z), "ms": statistics.mean(ms_z),
                                    "equal_to_device_run": zc_equal},
                  "e2e_pipelined_sequence": {"props/s": 1e3 / ms_seq, "ms": ms_seq, "steps": K,
                                             "equal_to_device_run": seq_equal,
                                             "note": "K steps in one olg_prop_plan_execute_host call; L2 "
                                                     "flushed once before the region"}},
        "clocks": clocks,
    }
    step()
    torch.cuda.synchronize()
    v, ref = cpu_asm_sample()
    out["accuracy"] = dict(accuracy(dst.cpu().numpy(), ref), against="FP64 oracle, the whole 1024^2 field")
    if rank == 0 and ws == 1 and cpu:
        out["cpu_baseline"] = {"value": v, "unit": "props/s", "cores": cpu_threads(),
                               "kind": "port", "sample": "one full 1024^2 FP64 ASM propagation"}
    return out


def wl_wrp(x, K, W, cpu):
    torch, og, pk, pk_kind = x.torch, x.og, x.pk, x.pk_kind
    stream, flush, barrier, max_over_ranks = x.stream, x.flush, x.barrier, x.max_over_ranks
    ws, rank, local, args = x.ws, x.rank, x.local, x.args
    c = WRP
    N = c["N"]
    tuned = pinned_variants(og, og.autotune(N, N), args.variants)
    pts = wrp_points()
    obj = og.gObject(pts)
    U = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
    img = torch.empty((N, N), dtype=torch.uint8, device="cuda")
    pws = og.workspace(N, N)
    p, lam, zw = np.float32(c["p"]), np.float32(c["lam"]), np.float32(c["zw"])

    def step1():
        og.WRPStep1(obj, U, N, N, p, lam, zw)

    def step2():
        og.asm_prop(U, dy=float(p), dx=float(p), lam=float(lam), z=float(zw), work=pws)

    def step():
        step1()
        step2()
        og.binarize(U, N, N, img)

    with ClockSampler(local) as clk:
        l0 = og.launch_count()
        ms = timed(torch, step, K, W, flush, stream, barrier)
        launches = (og.launch_count() - l0) // (K + W) * K
        ms1 = timed(torch, step1, K, W, flush, stream, barrier)
        ms2 = timed(torch, step2, K, W, flush, stream, barrier)
    clocks = clk.summary()
    t_step = max_over_ranks(statistics.mean(ms))
    hp = torch.from_numpy(pts).pin_memory()
    himg = torch.empty((N, N), dtype=torch.uint8).pin_memory()

    def step_e2e():
        obj.points.copy_(hp, non_blocking=True)
        step()
        himg.copy_(img, non_blocking=True)

    ms_e = timed(torch, step_e2e, K, W, flush, stream, barrier)
    t_e2e = max_over_ranks(statistics.mean(ms_e))
    # useful window terms sum_j pi W_j^2 / p^2 (W_j as the reference computes it)
    dz = pts[:, 2].astype(np.float64) - float(zw)
    Wj = np.abs(dz) / np.sqrt(4 * (float(p) / float(lam)) ** 2 - 1)
    terms = float(np.sum(np.pi * Wj ** 2) / float(p) ** 2)
    b_alg = 80 * N * N
    ach = b_alg / (statistics.mean(ms2) * 1e-3) / 1e9
    out = {
        "metric": "WRP holograms/s", "value": ws / (t_step * 1e-3), "unit": "holograms/s", "ms_per_step": t_step,
        "dtype": "f32 (double-float phase anchor)",
        "config": {"workload": WRP_DESC, "l2": "flushed between steps (256 MiB write)",
                   "launch_variants": {f"{k}:{m}": v for (k, m), v in tuned.items()}},
        "e2e": {"value": ws / (t_e2e * 1e-3), "unit": "holograms/s", "h2d_bytes_per_step": pts.nbytes,
                "d2h_bytes_per_step": N * N},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": traffic("wrp")[0],
                     "traffic_source": traffic("wrp")[1],
                     "note": f"step 2 (4096^2 -> 8192^2 ASM, {statistics.mean(ms2):.3f} ms): 80 n bytes; "
                             f"peak {pk_kind}"},
        "forms": {"step1_ms": statistics.mean(ms1), "step2_ms": statistics.mean(ms2),
                  "step1_window_terms": terms,
                  "step1_terms_per_s": terms / (statistics.mean(ms1) * 1e-3),
                  "window_radius_px": [float(Wj.min() / float(p)), float(Wj.max() / float(p))]},
        "clocks": clocks,
    }
    # accuracy: the same pipeline (step 1, step 2, binarisation) on the seeded
    # 1% point subset that the CPU sample uses, against the FP64 oracle
    v, (t1, t2), sub, Uref = cpu_wrp_sample()
    Us = torch.zeros((N, N), dtype=torch.complex64, device="cuda")
    og.WRPStep1(og.gObject(sub), Us, N, N, p, lam, zw)
    og.asm_prop(Us, dy=float(p), dx=float(p), lam=float(lam), z=float(zw), work=pws)
    imgs = torch.empty((N, N), dtype=torch.uint8, device="cuda")
    og.binarize(Us, N, N, imgs)
    torch.cuda.synchronize()
    got = Us.cpu().numpy()
    out["accuracy"] = dict(accuracy(got, Uref), binarized=binarized_accuracy(imgs.cpu().numpy(), got, Uref),
                           against=f"FP64 oracle, whole 4096^2 hologram of a seeded {len(sub)}-point subset")
    del Us, imgs
    if rank == 0 and ws == 1 and cpu:
        out["cpu_baseline"] = {"value": v, "unit": "holograms/s", "cores": cpu_threads(), "kind": "port",
                               "sample": f"FP64 WRP step 1 on 1% of the points ({t1:.1f} s, scaled x100) + "
                                         f"full FP64 4096^2 ASM ({t2:.1f} s)"}
    return out


def wl_adam(x, K, W, cpu):
    torch, og, pk, pk_kind = x.torch, x.og, x.pk, x.pk_kind
    stream, flush, barrier, max_over_ranks = x.stream, x.flush, x.barrier, x.max_over_ranks
    ws, rank, local, args = x.ws, x.rank, x.local, x.args
    c = ADAM
    n = c["n"]
    tuned = pinned_variants(og, og.autotune(n, n), args.variants)
    phi0, t, zs = adam_problem()
    phi = torch.from_numpy(phi0.copy()).cuda()
    tt = torch.from_numpy(t).cuda()
    opt = og.PhaseOptimizer(phi, tt, zs, dy=c["p"], dx=c["p"], lam=c["lam"], lr=c["lr"])

    def step():
        opt.step()

    # plain form: autograd through torch.fft (cuFFT) + torch.optim.Adam
    import math
    pphi = torch.from_numpy(phi0.copy()).cuda().requires_grad_(True)
    popt = torch.optim.Adam([pphi], lr=c["lr"])
    N2 = 2 * n
    fx = torch.fft.fftfreq(N2, d=c["p"], device="cuda", dtype=torch.float64)
    FY, FX = torch.meshgrid(fx, fx, indexing="ij")
    Hs = [torch.exp(1j * (2 * math.pi * z * torch.sqrt(1 / c["lam"] ** 2 - FX ** 2 - FY ** 2)))
          .to(torch.complex64) / (N2 * N2) for z in zs]

    def step_plain():
        popt.zero_grad(set_to_none=True)
        u = torch.polar(torch.ones_like(pphi), pphi)
        up = torch.nn.functional.pad(u, (n // 2, n // 2, n // 2, n // 2))
        F = torch.fft.fft2(up)
        loss = 0
        for k, H in enumerate(Hs):
            v = torch.fft.ifft2(F * H, norm="forward")[n // 2: n // 2 + n, n // 2: n // 2 + n]
            loss = loss + torch.mean((v.real ** 2 + v.imag ** 2 - tt[k]) ** 2)
        loss.backward()
        popt.step()

    with ClockSampler(local) as clk:
        l0 = og.launch_count()
        ms = timed(torch, step, K, W, flush, stream, barrier)
        launches = (og.launch_count() - l0) // (K + W) * K
        ms_plain = timed(torch, step_plain, K, W, flush, stream, barrier)
    clocks = clk.summary()
    t_step = max_over_ranks(statistics.mean(ms))
    hphi = torch.from_numpy(phi0.copy()).pin_memory()
    hout = torch.empty_like(hphi).pin_memory()

    def step_e2e():
        opt.phi.copy_(hphi, non_blocking=True)
        opt.step()
        hout.copy_(opt.phi, non_blocking=True)

    ms_e = timed(torch, step_e2e, K, W, flush, stream, barrier)
    t_e2e = max_over_ranks(statistics.mean(ms_e))
    # bytes of the shared-spectrum gradient (n = 2048^2 elements, P planes):
    # e^{i phi} row pass 20 n + forward column pass to the full spectrum 48 n;
    # per plane: inverse column pass 48 n, the fused seed row pass (row
    # spectrum in and out, targets) 36 n, forward column pass into the summed
    # spectrum 80 n (48 n for the first); the final inverse column + row
    # passes 72 n; Adam 32 n
    P = len(zs)
    b_alg = (68 + 84 * P + 80 * P - 32 + 72 + 32) * n * n
    ach = b_alg / (statistics.mean(ms) * 1e-3) / 1e9
    out = {
        "metric": "grad-steps/s", "value": ws / (t_step * 1e-3), "unit": "grad-steps/s", "ms_per_step": t_step,
        "dtype": "f32",
        "config": {"workload": ADAM_DESC, "lr": c["lr"], "l2": "flushed between steps (256 MiB write)",
                   "launch_variants": {f"{k}:{m}": v for (k, m), v in tuned.items()}},
        "e2e": {"value": ws / (t_e2e * 1e-3), "unit": "grad-steps/s", "h2d_bytes_per_step": phi0.nbytes,
                "d2h_bytes_per_step": phi0.nbytes},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": traffic("adam")[0],
                     "traffic_source": traffic("adam")[1],
                     "note": f"{b_alg // (n * n)} n bytes per step (one shared forward spectrum, per plane an "
                             f"inverse column pass, the fused seed row pass and a forward column pass into the "
                             f"summed adjoint spectrum; Adam), n = 2048^2; peak {pk_kind}"},
        "forms": {"fused_adjoint": {"grad-steps/s": 1e3 / statistics.mean(ms), "ms": statistics.mean(ms)},
                  "plain_torch_autograd_cufft": {"grad-steps/s": 1e3 / statistics.mean(ms_plain),
                                                  "ms": statistics.mean(ms_plain)},
                  "loss_after_steps": float(opt.loss.item())},
        "clocks": clocks,
    }
    # accuracy: loss and gradient of the first plane against the FP64 oracle
    phi_t = torch.from_numpy(phi0.copy()).cuda()
    l1, g1 = og.phase_loss_grad(phi_t, tt[:1].contiguous(), zs[:1], dy=c["p"], dx=c["p"], lam=c["lam"])
    torch.cuda.synchronize()
    v, dt, (lref, gref) = cpu_adam_sample()
    out["accuracy"] = {"grad_rel_l2": float(np.linalg.norm(g1.cpu().numpy() - gref) / np.linalg.norm(gref)),
                       "loss_rel_err": abs(float(l1) - float(lref)) / abs(float(lref)),
                       "against": "FP64 oracle loss and gradient, plane 1 of 8, whole 2048^2 phase"}
    if rank == 0 and ws == 1 and cpu:
        out["cpu_baseline"] = {"value": v, "unit": "grad-steps/s", "cores": cpu_threads(), "kind": "port",
                               "sample": f"FP64 loss + adjoint gradient of 1 of 8 planes ({dt:.1f} s), scaled x8"}
    return out


def wl_batch(x, K, W, cpu):
    torch, og, pk, pk_kind = x.torch, x.og, x.pk, x.pk_kind
    stream, flush, barrier, max_over_ranks = x.stream, x.flush, x.barrier, x.max_over_ranks
    ws, rank, local, args = x.ws, x.rank, x.local, x.args
    # launch shapes of the 4096- and 8192-point passes that the large fields run
    tuned = {}
    for n in (2048, 4096):
        tuned.update(pinned_variants(og, og.autotune(n, n), args.variants))
    fields = og.config5_fields()
    plan = og.BatchPlan(fields)
    nprop = len(fields)
    b_alg = sum(80 * f["u_in"].numel() for f in fields)
    gs = torch.cuda.Stream()
    graph = torch.cuda.CUDAGraph()
    plan.execute()
    torch.cuda.synchronize()
    with torch.cuda.stream(gs):
        with torch.cuda.graph(graph, stream=gs):
            plan.execute(stream=gs)
    torch.cuda.synchronize()

    def step():
        graph.replay()

    def step_serial():
        plan.execute_serial()

    from openol_gb300.plain import plain_prop

    def step_plain():
        for f in fields:
            plain_prop(f)

    with ClockSampler(local) as clk:
        l0 = og.launch_count()
        ms_direct = timed(torch, plan.execute, K, W, flush, stream, barrier)
        launches = (og.launch_count() - l0) // (K + W) * K
        ms = timed(torch, step, K, W, flush, stream, barrier)
        ms_serial = timed(torch, step_serial, K, W, flush, stream, barrier)
        ms_plain = timed(torch, step_plain, K, W, flush, stream, barrier)
    clocks = clk.summary()
    plan.check()
    t_step = max_over_ranks(statistics.mean(ms))
    # launch-bound regime: 96 small (256^2) fields, persistent vs one by one
    small = og.config5_fields(n=96, seed=77)
    for f in small:
        f["u_in"] = f["u_in"][:256, :256].contiguous()
        f["u_out"] = torch.empty_like(f["u_in"])
    splan = og.BatchPlan(small)
    ms_small = timed(torch, splan.execute, K, W, None, stream, barrier)
    ms_small_serial = timed(torch, splan.execute_serial, K, W, None, stream, barrier)
    ms_small_plain = timed(torch, lambda: [plain_prop(f) for f in small], K, W, None, stream, barrier)
    splan.check()
    splan.close()
    hin = [f["u_in"].cpu().pin_memory() for f in fields]
    hout = [torch.empty_like(h).pin_memory() for h in hin]

    def step_e2e():
        # the public host-field call: copies in, propagations and copies out
        # pipelined over the plan's copy streams and this stream
        plan.execute_host(hin, hout, stream=torch.cuda.current_stream())

    def step_e2e_serial_copies():
        for f, h in zip(fields, hin):
            f["u_in"].copy_(h, non_blocking=True)
        graph.replay()
        for f, h in zip(fields, hout):
            h.copy_(f["u_out"], non_blocking=True)

    ms_e = timed(torch, step_e2e, K, W, flush, stream, barrier)
    plan.check()
    ms_es = timed(torch, step_e2e_serial_copies, K, W, flush, stream, barrier)
    t_e2e = max_over_ranks(statistics.mean(ms_e))
    nbytes = sum(f["u_in"].numel() * 8 for f in fields)
    ach = b_alg / (statistics.mean(ms) * 1e-3) / 1e9
    out = {
        "metric": "batched props/s", "value": ws * nprop / (t_step * 1e-3), "unit": "props/s",
        "ms_per_step": t_step, "dtype": "f32",
        "config": {"workload": BATCH_DESC, "items": plan.n_items, "direct_fields": plan.n_direct,
                   "launch_variants": {f"{k}:{m}": v for (k, m), v in tuned.items()},
                   "l2": "inputs larger than L2 (%.1f GB)" % (nbytes / 1e9)},
        "e2e": {"value": ws * nprop / (t_e2e * 1e-3), "unit": "props/s", "h2d_bytes_per_step": nbytes,
                "d2h_bytes_per_step": nbytes, "form": "olg_batch_execute_host: copies pipelined with the passes"},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": None,
                     "note": f"sum of 80 n bytes over the 96 propagations per step; peak {pk_kind}"},
        "forms": {"persistent_graph": {"props/s": nprop * 1e3 / statistics.mean(ms), "ms": statistics.mean(ms)},
                  "persistent_direct": {"ms": statistics.mean(ms_direct)},
                  "e2e_serial_copies": {"props/s": nprop * 1e3 / statistics.mean(ms_es), "ms": statistics.mean(ms_es),
                                        "note": "all copies in, the graph, all copies out, one after another"},
                  "serial_per_field": {"props/s": nprop * 1e3 / statistics.mean(ms_serial),
                                       "ms": statistics.mean(ms_serial)},
                  "serial_plain_cufft": {"props/s": nprop * 1e3 / statistics.mean(ms_plain),
                                         "ms": statistics.mean(ms_plain),
                                         "note": "each field through the reference-structured cuFFT chain"},
                  "small_256sq_persistent": {"props/s": 96e3 / statistics.mean(ms_small),
                                             "ms": statistics.mean(ms_small)},
                  "small_256sq_serial": {"props/s": 96e3 / statistics.mean(ms_small_serial),
                                         "ms": statistics.mean(ms_small_serial)},
                  "small_256sq_plain_cufft": {"props/s": 96e3 / statistics.mean(ms_small_plain),
                                              "ms": statistics.mean(ms_small_plain)}},
        "clocks": clocks,
    }
    # accuracy: one field per size class, from the last graph replay, against
    # the FP64 oracle on the same input
    graph.replay()
    torch.cuda.synchronize()
    sizes = batch_draw()[0]
    inputs = {}
    for m in (512, 1024, 2048, 4096):
        k = int(np.nonzero(sizes == m)[0][0])
        inputs[m] = (k, fields[k]["u_in"].cpu().numpy())
    v, t_cls, refs = cpu_batch_sample(inputs)
    acc = {f"{m}^2 {fields[k]['method']}": accuracy(fields[k]["u_out"].cpu().numpy(), r) for m, (k, r) in refs.items()}
    out["accuracy"] = dict(acc, max_rel_l2=max(a["rel_l2"] for a in acc.values()),
                           against="FP64 oracle, one whole field per size class")
    plan.close()
    if rank == 0 and ws == 1 and cpu:
        out["cpu_baseline"] = {"value": v, "unit": "props/s", "cores": cpu_threads(), "kind": "port",
                               "sample": "one FP64 field per size class (%s s), each class costed for all its "
                                         "fields" % ", ".join("%d^2 %.2f" % (m, t) for m, t in t_cls.items())}
    return out


def wl_tilt(x, K, W, cpu):
    torch, og, pk, pk_kind = x.torch, x.og, x.pk, x.pk_kind
    stream, flush, barrier, max_over_ranks = x.stream, x.flush, x.barrier, x.max_over_ranks
    ws, rank, local, args = x.ws, x.rank, x.local, x.args
    c = TILT
    n = c["n"]
    tuned = pinned_variants(og, og.autotune(n, n), args.variants)
    u0 = asm_input()
    src = torch.from_numpy(u0).cuda()
    dst = torch.empty_like(src)
    tws = og.tilted_workspace(n, n)
    kw = dict(dy=c["p"], dx=c["p"], lam=c["lam"], z=c["z"], work=tws)

    def run(interp, mode, refm):
        ang = c["angle_ref"] if refm else c["angle"]
        return lambda: og.tilted_prop(src, dst, angle=ang, interp=interp, propmode=mode, reference=refm, **kw)

    step = run(0, 0, False)
    with ClockSampler(local) as clk:
        l0 = og.launch_count()
        ms = timed(torch, step, K, W, flush, stream, barrier)
        launches = (og.launch_count() - l0) // (K + W) * K
        forms = {}
        for refm in (False, True):
            for mode in (0, 1):
                for interp in (0, 1):
                    name = "%s_%s_%s" % ("reference" if refm else "source", "fresnel" if mode else "asm",
                                         "bicubic" if interp else "bilinear")
                    mf = timed(torch, run(interp, mode, refm), K, W, flush, stream, barrier)
                    forms[name] = {"props/s": 1e3 / statistics.mean(mf), "ms": statistics.mean(mf)}
        ms_asm = timed(torch, lambda: og.asm_prop(src, dst, dy=c["p"], dx=c["p"], lam=c["lam"], z=c["z"]),
                       K, W, flush, stream, barrier)
    clocks = clk.summary()
    t_step = max_over_ranks(statistics.mean(ms))
    hsrc = torch.from_numpy(u0).pin_memory()
    hdst = torch.empty_like(hsrc).pin_memory()

    def step_e2e():
        src.copy_(hsrc, non_blocking=True)
        step()
        hdst.copy_(dst, non_blocking=True)

    ms_e = timed(torch, step_e2e, K, W, flush, stream, barrier)
    t_e2e = max_over_ranks(statistics.mean(ms_e))
    # row pass 8n in + 16n out, column FFTs 16n + 32n, resample 32n + 32n,
    # inverse columns 32n + 16n, inverse rows 16n + 8n
    b_alg = 208 * n * n
    ach = b_alg / (statistics.mean(ms) * 1e-3) / 1e9
    forms["plain_asm_same_field"] = {"props/s": 1e3 / statistics.mean(ms_asm), "ms": statistics.mean(ms_asm)}
    out = {
        "metric": "tilted props/s", "value": ws / (t_step * 1e-3), "unit": "props/s", "ms_per_step": t_step,
        "dtype": "f32 (FP64 sampling positions at the grid edges)",
        "config": {"workload": TILT_DESC, "l2": "flushed between steps (256 MiB write)",
                   "launch_variants": {f"{k}:{m}": v for (k, m), v in tuned.items()}},
        "e2e": {"value": ws / (t_e2e * 1e-3), "unit": "props/s", "h2d_bytes_per_step": u0.nbytes,
                "d2h_bytes_per_step": u0.nbytes},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": None,
                     "note": f"208 n bytes per tilted propagation (n = 1024^2); peak {pk_kind}"},
        "forms": forms,
        "clocks": clocks,
    }
    step()
    torch.cuda.synchronize()
    v, ref = cpu_tilt_sample()
    out["accuracy"] = dict(accuracy(dst.cpu().numpy(), ref), against="FP64 oracle, the whole 1024^2 field")
    if rank == 0 and ws == 1 and cpu:
        out["cpu_baseline"] = {"value": v, "unit": "props/s", "cores": cpu_threads(),
                               "kind": "port", "sample": "one full 1024^2 FP64 TiltedSourceProp (ASM, bilinear)"}
    return out


def wl_uhd(x, K, W, cpu):
    """ASM of the reference's default 3840 x 2160 test field: padded lengths
    7680 = 2^9 3 5 and 4320 = 2^5 3^3 5 through the mixed-radix passes."""
    torch, og, pk, pk_kind = x.torch, x.og, x.pk, x.pk_kind
    stream, flush, barrier, max_over_ranks = x.stream, x.flush, x.barrier, x.max_over_ranks
    ws, rank, local, args = x.ws, x.rank, x.local, x.args
    c = UHD
    ny, nx = c["ny"], c["nx"]
    u0 = uhd_input()
    src = torch.from_numpy(u0).cuda()
    dst = torch.empty_like(src)
    ws_buf = og.workspace(ny, nx)
    kw = dict(dy=c["p"], dx=c["p"], lam=c["lam"], z=c["z"])

    def step():
        og.asm_prop(src, dst, work=ws_buf, **kw)

    from openol_gb300.plain import plain_asm_prop

    with ClockSampler(local) as clk:
        l0 = og.launch_count()
        ms = timed(torch, step, K, W, flush, stream, barrier)
        launches = (og.launch_count() - l0) // (K + W) * K
        ms_plain = timed(torch, lambda: plain_asm_prop(src, dst, **kw), K, W, flush, stream, barrier)
    clocks = clk.summary()
    t_step = max_over_ranks(statistics.mean(ms))
    hsrc = torch.from_numpy(u0).pin_memory()
    hdst = torch.empty_like(hsrc).pin_memory()

    def step_e2e():
        src.copy_(hsrc, non_blocking=True)
        step()
        hdst.copy_(dst, non_blocking=True)

    ms_e = timed(torch, step_e2e, K, W, flush, stream, barrier)
    plan = og.PropPlan("asm", ny, nx, **kw)
    houts = [torch.empty_like(hsrc).pin_memory() for _ in range(max(K, W, 3))]
    ms_seq = timed_sequence(torch, lambda k: plan.execute_host([hsrc] * k, houts[:k], stream=stream), K, W, flush,
                            stream, barrier)
    step()
    torch.cuda.synchronize()
    seq_equal = bool(torch.equal(houts[K - 1], dst.cpu()))
    plan.close()
    forms_e2e = {"per_step_copies": statistics.mean(ms_e)}
    if seq_equal:
        forms_e2e["pipelined_sequence"] = ms_seq
    e2e_form = min(forms_e2e, key=forms_e2e.get)
    t_e2e = max_over_ranks(forms_e2e[e2e_form])
    n = ny * nx
    b_alg = 80 * n
    ach = b_alg / (statistics.mean(ms) * 1e-3) / 1e9
    out = {
        "metric": "mixed-radix ASM props/s", "value": ws / (t_step * 1e-3), "unit": "props/s", "ms_per_step": t_step,
        "dtype": "f32",
        "config": {"workload": UHD_DESC, "l2": "inputs larger than L2 (S: %.0f MB), flushed between steps"
                   % (ny * 2 * nx * 8 / 1e6)},
        "e2e": {"value": ws / (t_e2e * 1e-3), "unit": "props/s", "h2d_bytes_per_step": u0.nbytes,
                "d2h_bytes_per_step": u0.nbytes, "form": e2e_form},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                     "frac": ach / pk["hbm_gbs"], "traffic": traffic("uhd")[0], "traffic_source": traffic("uhd")[1],
                     "note": f"80 n bytes per propagation (n = 3840 x 2160) over the 3-pass propagation time; "
                             f"peak {pk_kind}"},
        "forms": {"fused_mixed_radix": {"props/s": 1e3 / statistics.mean(ms), "ms": statistics.mean(ms)},
                  "plain_cufft": {"props/s": 1e3 / statistics.mean(ms_plain), "ms": statistics.mean(ms_plain)},
                  "e2e_per_step_copies": {"props/s": 1e3 / statistics.mean(ms_e), "ms": statistics.mean(ms_e)},
                  "e2e_pipelined_sequence": {"props/s": 1e3 / ms_seq, "ms": ms_seq, "steps": K,
                                             "equal_to_device_run": seq_equal}},
        "clocks": clocks,
    }
    v, ref = cpu_uhd_sample()
    out["accuracy"] = dict(accuracy(dst.cpu().numpy(), ref), against="FP64 oracle, the whole 3840 x 2160 field")
    if rank == 0 and ws == 1 and cpu:
        out["cpu_baseline"] = {"value": v, "unit": "props/s", "cores": cpu_threads(), "kind": "port",
                               "sample": "one full 3840x2160 -> 7680x4320 FP64 ASM propagation"}
    return out


def run_ours(args):
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")

    def barrier():
        if dist is not None:
            dist.barrier()

    def max_over_ranks(x):
        if dist is None:
            return x
        t = torch.tensor([x], dtype=torch.float64, device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        return float(t.item())

    import openol_gb300 as og
    pk, pk_kind = peaks()
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    K, W = args.steps, args.warmup

    x = _Ctx()
    x.torch, x.og, x.pk, x.pk_kind = torch, og, pk, pk_kind
    x.stream, x.flush, x.barrier, x.max_over_ranks = stream, flush, barrier, max_over_ranks
    x.ws, x.rank, x.local, x.args = ws, rank, local, args
    out = WORKLOADS[args.workload](x, K, W, not args.no_cpu)
    # The default (CGH) line also carries the other benchmark configurations
    # and the reference's default 3840 x 2160 field, each run briefly (at most
    # 5 timed steps) with its accuracy against the FP64 oracle; their CPU
    # baselines are left to their own --workload runs.
    configs = {}
    if args.workload == "cgh" and not args.no_configs:
        for name in ("asm", "wrp", "adam", "batch", "uhd"):
            o = WORKLOADS[name](x, min(K, 5), 3, False)
            configs[name] = {"metric": o["metric"], "value": o["value"], "unit": o["unit"],
                             "ms_per_step": o["ms_per_step"], "workload": o["config"]["workload"],
                             "e2e": o["e2e"]["value"], "gpu_launches": o["gpu_launches"],
                             "roofline": {k: o["roofline"][k] for k in ("bound", "achieved", "peak", "unit", "frac",
                                                                        "traffic")},
                             "accuracy": o.get("accuracy"), "clocks": o["clocks"]}
            del o
            torch.cuda.empty_cache()
    if rank == 0:
        line = {"metric": out["metric"], "value": out["value"], "unit": out["unit"], "n_gpus": ws, "steps": K,
                "warmup": W, "ms_per_step": out["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": out["dtype"], "data": "synthetic (seeded)", "config": out["config"]}
        for k in ("e2e", "gpu_launches", "roofline", "accuracy", "cpu_baseline", "clocks", "forms",
                  "exact_kernel_sfu"):
            if k in out:
                line[k] = out[k]
        if configs:
            line["configs"] = configs
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


WORKLOADS = {"cgh": wl_cgh, "asm": wl_asm, "wrp": wl_wrp, "adam": wl_adam, "batch": wl_batch, "tilt": wl_tilt,
             "uhd": wl_uhd}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cgh", choices=["cgh", "asm", "wrp", "adam", "batch", "tilt", "uhd"])
    ap.add_argument("--cpu-rows", type=int, default=48)
    ap.add_argument("--ref-rows", type=int, default=24)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--ncu-range", action="store_true",
                    help="bracket the first timed region with cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--variants", default="",
                    help='launch shapes to set after the autotuner, "kind:n=i,..." (kind 0/1/2: pass 1/2/3)')
    ap.add_argument("--no-configs", action="store_true",
                    help="default workload only: skip the brief runs of the other configurations")
    args = ap.parse_args()
    NCU_RANGE["on"] = args.ncu_range
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
