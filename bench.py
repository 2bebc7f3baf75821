#!/usr/bin/env python
"""Benchmark of the OpenOL hot path on GB300.

Default workload (N = 1): point-cloud CGH on a 1920 x 1080 hologram, pitch
8 um, lambda = 532 nm, 10,000 points uniform in a 5 x 5 x 5 mm box centred at
(W/2 p, H/2 p, 100 mm), amplitudes U[0.5, 1], phases U[0, 2 pi) -- metric
point.pixel/s (one step = one hologram = 2.07e10 point.pixels).  Other
workloads: ``--workload asm`` (1024^2 field padded to 2048^2, p = 8 um,
532 nm, z = 50 mm; props/s).

Our arm prints one JSON line with value (device-resident inputs, CUDA events
on the launching stream, L2 flushed between steps), e2e (host buffers, copies
inside the timed region, through the public API), roofline of the dominant
kernel, a CPU baseline (the FP64 oracle port on the host cores, bounded
sample) and the clocks sampled during the timed region.

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

CGH = dict(ny=1080, nx=1920, p=8e-6, lam=532e-9, n=10000, zc=0.1, box=5e-3, seed=20261203 + 2)
ASM = dict(n=1024, p=8e-6, lam=532e-9, z=0.05, seed=20261203 + 1)


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
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
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
    O.cgh_fresnel(sp, rows, c["nx"], c["p"], c["p"], c["lam"], amp=amp.astype(np.float64),
                  phase0=ph.astype(np.float64))
    dt = time.perf_counter() - t0
    return rows * c["nx"] * c["n"] / dt, dt


def cpu_asm_sample():
    import oracle as O
    u = asm_input().astype(np.complex128)
    t0 = time.perf_counter()
    O.asm_prop(u, ASM["p"], ASM["p"], ASM["lam"], ASM["z"])
    return 1.0 / (time.perf_counter() - t0)


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
            v, _ = cpu_cgh_sample(rows)
            if k >= args.warmup:
                vals.append(v)
        metric, unit = "CGH point.pixel/s", "point.pixel/s"
        sample = f"{rows} of {CGH['ny']} rows x {CGH['nx']} px x {CGH['n']} points per step (FP64 Fresnel-form sum)"
        config = {"workload": "cgh 1920x1080, 10000 points, p=8um, lambda=532nm, 5mm box at z=100mm"}
    else:
        for k in range(args.warmup + args.steps):
            v = cpu_asm_sample()
            if k >= args.warmup:
                vals.append(v)
        metric, unit = "ASM props/s", "props/s"
        sample = "one full 1024^2 -> 2048^2 FP64 ASM propagation per step"
        config = {"workload": "asm 1024x1024 padded 2048x2048, p=8um, lambda=532nm, z=50mm"}
    v = statistics.median(vals)
    line = {"impl": "reference", "metric": metric, "value": v, "unit": unit, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded)", "config": config,
            "cpu_baseline": {"value": v, "unit": unit, "cores": cpu_threads(), "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------- our arm
def timed(torch, fn, K, W, flush, stream, barrier):
    for _ in range(W):
        fn()
    torch.cuda.synchronize()
    barrier()
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
    barrier()
    return [a.elapsed_time(b) for a, b in evs]


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
    out = {}

    if args.workload == "cgh":
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

        gws = og.cgh_gemm_workspace(c["n"], c["ny"], c["nx"])

        def step_gemm():
            og.cgh_fresnel_gemm(obj, U, ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"], amp=a,
                                phase0=f, work=gws)

        def step_gemm_only():
            og.cgh_fresnel_gemm(obj, U, ny=c["ny"], nx=c["nx"], py=c["p"], px=c["p"], lam=c["lam"], amp=a,
                                phase0=f, work=gws, reuse_operands=True)

        forms = {"fresnel_gemm": step_gemm, "fresnel_gemm_kernel_only": step_gemm_only,
                 "fresnel_direct": step_fresnel, "exact": step_exact}
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
        t_e2e = max_over_ranks(statistics.mean(ms_e))
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
                       "form": chosen, "l2": "flushed between steps (256 MiB write)"},
            "e2e": {"value": ws * units / (t_e2e * 1e-3), "unit": "point.pixel/s",
                    "h2d_bytes_per_step": pts.nbytes + amp.nbytes + ph.nbytes,
                    "d2h_bytes_per_step": c["ny"] * c["nx"] * 8},
            "gpu_launches": int(launches),
            "roofline": {"bound": "tensor", "achieved": ach_tf, "peak": pk["bf16_tflops"], "unit": "TFLOP/s",
                         "frac": ach_tf / pk["bf16_tflops"], "traffic": None,
                         "note": f"k_cgh_gemm alone ({ms_g:.3f} ms): 24 M N K issued f16 flop (3 split products x "
                                 f"4 real GEMMs), useful 8 M N K; peak = {pk_kind} dense bf16 (f16 same rate)"},
            "exact_kernel_sfu": {"achieved": sfu_gops, "peak": peak_gops, "unit": "Gop/s (MUFU)",
                                 "frac": sfu_gops / peak_gops,
                                 "note": f"2 MUFU per term; peak {nsm} SM x 16 MUFU/clk x {mhz} MHz"},
            "forms": {k: {"point.pixel/s": units / (statistics.mean(v[0]) * 1e-3), "ms": statistics.mean(v[0])}
                      for k, v in res.items()},
            "clocks": clocks,
        }
        if rank == 0 and ws == 1 and not args.no_cpu:
            v, dt = cpu_cgh_sample(args.cpu_rows)
            out["cpu_baseline"] = {"value": v, "unit": "point.pixel/s", "cores": cpu_threads(), "kind": "port",
                                   "sample": f"{args.cpu_rows} of 1080 rows x 1920 px x 10000 points, FP64 oracle, "
                                             f"{dt:.1f} s"}
    else:
        n = ASM["n"]
        u0 = asm_input()
        src = torch.from_numpy(u0).cuda()
        dst = torch.empty_like(src)
        ws_buf = og.workspace(n, n)

        def step():
            og.asm_prop(src, dst, dy=ASM["p"], dx=ASM["p"], lam=ASM["lam"], z=ASM["z"], work=ws_buf)

        with ClockSampler(local) as clk:
            l0 = og.launch_count()
            ms = timed(torch, step, K, W, flush, stream, barrier)
            launches = (og.launch_count() - l0) // (K + W) * K
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
        b_alg = 80 * n * n
        ach = b_alg / (statistics.mean(ms) * 1e-3) / 1e9
        out = {
            "metric": "ASM props/s", "value": ws / (t_step * 1e-3), "unit": "props/s", "ms_per_step": t_step,
            "dtype": "f32",
            "config": {"workload": "asm 1024x1024 padded 2048x2048, p=8um, lambda=532nm, z=50mm",
                       "l2": "flushed between steps (256 MiB write)"},
            "e2e": {"value": ws / (t_e2e * 1e-3), "unit": "props/s", "h2d_bytes_per_step": u0.nbytes,
                    "d2h_bytes_per_step": u0.nbytes},
            "gpu_launches": int(launches),
            "roofline": {"bound": "hbm", "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                         "frac": ach / pk["hbm_gbs"], "traffic": None,
                         "note": f"80 n bytes per propagation (n = 1024^2) over the 3-pass propagation time; "
                                 f"peak {pk_kind}"},
            "clocks": clocks,
        }
        if rank == 0 and ws == 1 and not args.no_cpu:
            out["cpu_baseline"] = {"value": cpu_asm_sample(), "unit": "props/s", "cores": cpu_threads(),
                                   "kind": "port", "sample": "one full 1024^2 FP64 ASM propagation"}

    if rank == 0:
        line = {"metric": out["metric"], "value": out["value"], "unit": out["unit"], "n_gpus": ws, "steps": K,
                "warmup": W, "ms_per_step": out["ms_per_step"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": out["dtype"], "data": "synthetic (seeded)", "config": out["config"]}
        for k in ("e2e", "gpu_launches", "roofline", "cpu_baseline", "clocks", "forms"):
            if k in out:
                line[k] = out[k]
        print(json.dumps(line))
    if dist is not None:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cgh", choices=["cgh", "asm"])
    ap.add_argument("--cpu-rows", type=int, default=48)
    ap.add_argument("--ref-rows", type=int, default=24)
    ap.add_argument("--no-cpu", action="store_true")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
