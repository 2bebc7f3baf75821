"""CPU: the C-ABI library loads, exports every declared entry point, and its
host-side logic (AUTO checks, WRP plane, argument validation) matches the
reference.  No kernel is launched here."""
import ctypes as C
import os
import re
import subprocess

import numpy as np

from conftest import ROOT
from openol_gb300 import _lib
from openol_gb300 import build as B

HEADERS = [os.path.join(ROOT, "include", h) for h in ("olgb300.h", "olgb300_plain.h")]


def declared_symbols():
    txt = "".join(open(h).read() for h in HEADERS)
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(olg_\w+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    syms = declared_symbols()
    assert len(syms) >= 18
    out = subprocess.run(["nm", "-D", "--defined-only", B.LIB], capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (olg_\w+)", out))
    missing = [s for s in syms if s not in exported]
    assert not missing, missing
    L = C.CDLL(B.LIB)
    for s in syms:
        assert hasattr(L, s)


def test_python_binding_covers_header():
    assert set(declared_symbols()) <= set(_lib.SIGNATURES)


def test_status_strings():
    L = _lib.lib()
    assert L.olg_version() >= 100
    assert L.olg_status_string(0) == b"ok"
    assert b"argument" in L.olg_status_string(-1)


def test_batch_direct_threshold_without_gpu():
    L = _lib.lib()
    cur = L.olg_batch_direct_pixels(0)
    assert cur == 2048 * 2048
    assert L.olg_batch_direct_pixels(1000) == cur
    assert L.olg_batch_direct_pixels(-5) == 1000  # <= 0 only reads
    assert L.olg_batch_direct_pixels(cur) == 1000
    assert L.olg_batch_plan_direct_fields(None) == 0
    import openol_gb300 as og
    assert og.batch_direct_pixels() == cur
    assert og.batch_direct_pixels(4096) == cur and og.batch_direct_pixels(cur) == 4096


def test_tuning_knobs_without_gpu():
    L = _lib.lib()
    # launch-shape table of the three passes (host state only)
    n_var = L.olg_prop_variant_count()
    assert n_var >= 10
    old = L.olg_prop_get_variant(1, 2048)
    assert 0 <= old < n_var
    assert L.olg_prop_set_variant(1, 2048, 8) == 0 and L.olg_prop_get_variant(1, 2048) == 8
    assert L.olg_prop_set_variant(1, 2048, n_var) == -1  # no such shape
    assert L.olg_prop_set_variant(3, 2048, 0) == -1      # no such pass
    assert L.olg_prop_set_variant(0, 3000, 0) == -1      # not a tuned length
    assert L.olg_prop_get_variant(0, 100) == -1
    assert L.olg_prop_set_variant(1, 2048, old) == 0
    # GEMM K-tail weight: out-of-range values leave it unchanged
    w = L.olg_cgh_gemm_tail_weight(-1.0)
    assert w == 1.2
    assert L.olg_cgh_gemm_tail_weight(2.0) == w
    assert L.olg_cgh_gemm_tail_weight(99.0) == 2.0
    assert L.olg_cgh_gemm_tail_weight(w) == 2.0
    # GEMM tile form: 0 / 1 set it, anything else only reads it
    f = L.olg_cgh_gemm_pairs(-1)
    assert f == 1
    assert L.olg_cgh_gemm_pairs(0) == 1
    assert L.olg_cgh_gemm_pairs(7) == 0
    assert L.olg_cgh_gemm_pairs(f) == 0
    # GEMM accumulation chunk: 1..64 K blocks
    ch = L.olg_cgh_gemm_chunk(-1)
    assert ch == 8
    assert L.olg_cgh_gemm_chunk(16) == 8
    assert L.olg_cgh_gemm_chunk(0) == 16 and L.olg_cgh_gemm_chunk(65) == 16
    assert L.olg_cgh_gemm_chunk(ch) == 16


def test_auto_checks_match_reference_float_and_double(golden):
    L = _lib.lib()
    for ny, nx, p, lam, z, a64, a32, f64, f32 in golden["checks"]:
        ny, nx = int(ny), int(nx)
        assert L.olg_asm_prop_check(ny, nx, p, p, lam, z, 0) == int(a64)
        assert L.olg_asm_prop_check(ny, nx, p, p, lam, z, 1) == int(a32)
        assert L.olg_fresnel_prop_check(ny, nx, p, p, lam, z, 0) == int(f64)
        assert L.olg_fresnel_prop_check(ny, nx, p, p, lam, z, 1) == int(f32)


def _plane_z_ref(window, ny, nx, p, plimit, lam, zmin, s):
    """golcgh.h:561-581 / 519-559 evaluated with the reference's float/double mix."""
    f = np.float32
    p, plimit, lam, zmin, s = f(p), f(plimit), f(lam), f(zmin), f(s)
    if s >= 0:
        return f(zmin * s)
    if window == 0:
        Wpow2 = f(np.float64(f(f(f(nx * ny) * p) * p)) / np.pi * 1 / 1024.0)
        q = np.float64(f(p / lam))
        d = f(np.sqrt((4 * q ** 2 - 1) * np.float64(Wpow2)))
        return f(zmin - d)
    D = f(np.float64(f(f(nx) * p)) * 0.05)
    q = np.float64(f(plimit / lam))
    d = f(np.sqrt(4 * q ** 2 - 1) / np.sqrt(2.0) * np.float64(D))
    return f(zmin - d)


def test_wrp_plane_z():
    L = _lib.lib()
    for window in (0, 1):
        for (ny, nx, p, lam, zmin, s) in [(4096, 4096, 4e-6, 532e-9, 0.151, -1.0), (2160, 3840, 3.74e-6, 532e-9, -0.1, -1.0),
                                          (1080, 1920, 8e-6, 633e-9, 0.2, 0.9)]:
            got = L.olg_wrp_plane_z(window, ny, nx, p, 0.0, lam, zmin, s)
            assert np.float32(got) == _plane_z_ref(window, ny, nx, p, p, lam, zmin, s)


def test_fault_knobs_without_gpu():
    """The wait budget and the injected allocation failures are host state."""
    L = _lib.lib()
    b = L.olg_wait_budget_cycles(0)
    assert b == 4000000000
    assert L.olg_wait_budget_cycles(12345) == b and L.olg_wait_budget_cycles(0) == 12345
    assert L.olg_wait_budget_cycles(b) == 12345
    assert L.olg_inject_alloc_failures(2) == 0
    assert L.olg_inject_alloc_failures(-3) == 2   # negative counts clear
    assert L.olg_inject_alloc_failures(0) == 0
    assert L.olg_batch_plan_raise_target(None, 0, 0, 1) == -1


def test_cgh_adjoint_validation_without_gpu():
    L = _lib.lib()
    buf = (C.c_char * 64)()
    base = (C.addressof(buf) + 15) // 16 * 16
    adj = L.olg_cgh_fresnel_adjoint_c64
    assert adj(base, -1, base, base, 8, 8, 8e-6, 8e-6, 532e-9, 0, None, 0, None) == -1   # bad point count
    assert adj(None, 5, base, base, 8, 8, 8e-6, 8e-6, 532e-9, 0, None, 0, None) == -1    # null points
    assert adj(base, 5, base + 4, base, 8, 8, 8e-6, 8e-6, 532e-9, 0, None, 0, None) == -1  # misaligned G
    assert L.olg_cgh_exact_adjoint_c64(base, 5, base, base, 8, 8, 8e-6, 0.0, 532e-9, 0, None, 0, None) == -1
    assert adj(base, 0, base, base, 8, 8, 8e-6, 8e-6, 532e-9, 0, None, 0, None) == 0     # nothing to do
    assert L.olg_cgh_adjoint_workspace_bytes(0, 8, 8, 0) == 0


def test_argument_validation_without_gpu():
    L = _lib.lib()
    # rejected before any device work
    assert L.olg_asm_prop_c64(None, None, 64, 64, 8e-6, 8e-6, 532e-9, 0.05, 0, None, 0, None) == -1
    buf = (C.c_char * 64)()
    base = (C.addressof(buf) + 15) // 16 * 16
    assert L.olg_asm_prop_c64(base, base, 14, 64, 8e-6, 8e-6, 532e-9, 0.05, 0, None, 0, None) == -2  # 28 = 4 * 7
    assert L.olg_asm_prop_c64(base, base, 64, 8192, 8e-6, 8e-6, 532e-9, 0.05, 0, None, 0, None) == -2
    assert L.olg_asm_prop_c64(base + 8, base, 64, 64, 8e-6, 8e-6, 532e-9, 0.05, 0, None, 0, None) == -1
    assert L.olg_arss_prop_c64(base, base, 64, 64, 8e-6, 8e-6, 532e-9, 0.05, 1.0, 0, 0, 0, None, 0, None) == -1
    assert b"s = 1" in L.olg_last_error() or b"s|s-1|" in L.olg_last_error()
    assert L.olg_cgh_fresnel_c64(None, None, None, 5, None, None, 8, 8, 8e-6, 8e-6, 532e-9, 0, None) == -1
    assert L.olg_prop_c64(base, 64, 64, 8e-6, 8e-6, 532e-9, 0.05, 7, 0, None, None, 0, None) == -1
    # shifted / split: bad mode, blocks that do not divide the field, overlapping output
    assert L.olg_shifted_prop_c64(base, base, 64, 64, 8e-6, 8e-6, 532e-9, 0.05, 0, 0, 2, 0, None, 0, None) == -1
    assert L.olg_split_prop_c64(base, base + 16, 64, 64, 8e-6, 8e-6, 532e-9, 0.05, 0, 3, 2, 0, None, 0, None) == -1
    assert L.olg_split_prop_c64(base, base, 64, 64, 8e-6, 8e-6, 532e-9, 0.05, 0, 2, 2, 0, None, 0, None) == -1
    assert b"overlap" in L.olg_last_error()
    assert L.olg_split_prop_c64(base, base + 16, 64, 64, 8e-6, 8e-6, 532e-9, 0.05, 2, 2, 2, 0, None, 0, None) == -1
    out = C.c_void_p()
    assert L.olg_host_device_pointer(None, C.byref(out)) == -1 and out.value is None
    # tilted planes: interpolation, mode, evanescent grid, Fresnel at z = 0, unsupported length
    tp = L.olg_tilted_prop_c64
    assert tp(base, base, 64, 64, 8e-6, 8e-6, 532e-9, 0.02, 0.1, 2, 0, 0, None, 0, None) == -1
    assert tp(base, base, 64, 64, 8e-6, 8e-6, 532e-9, 0.02, 0.1, 0, 2, 0, None, 0, None) == -1
    assert tp(base, base, 64, 64, 2e-7, 2e-7, 532e-9, 0.02, 0.1, 0, 0, 0, None, 0, None) == -1
    assert b"evanescent" in L.olg_last_error()
    assert tp(base, base, 64, 64, 8e-6, 8e-6, 532e-9, 0.0, 0.1, 0, 1, 0, None, 0, None) == -1
    assert tp(base, base, 14, 64, 8e-6, 8e-6, 532e-9, 0.02, 0.1, 0, 0, 0, None, 0, None) == -2
    assert tp(base, base, 64, 64, 8e-6, 8e-6, 532e-9, 0.02, float("nan"), 0, 0, 0, None, 0, None) == -1
    assert L.olg_tilted_workspace_bytes(64, 64) >= 2 * 128 * 128 * 8


def test_plan_validation_without_gpu():
    """Propagation and batch plans check the field description (size, method,
    physical parameters, ARSS s) before any device work."""
    L = _lib.lib()
    buf = (C.c_char * 64)()
    base = (C.addressof(buf) + 15) // 16 * 16
    F = _lib.OlgField

    def desc(**kw):
        d = dict(in_=base, out=base, ny=64, nx=64, method=0, flags=0, dy=8e-6, dx=8e-6, lam=532e-9, z=0.05, s=0.5,
                 oy=0.0, ox=0.0)
        d.update(kw)
        return F(**d)

    plan = C.c_void_p()
    assert L.olg_prop_plan_create(None, C.byref(plan)) == -1
    assert L.olg_prop_plan_create(C.byref(desc(ny=14)), C.byref(plan)) == -2       # 28 = 4 * 7
    assert L.olg_prop_plan_create(C.byref(desc(method=9)), C.byref(plan)) == -1
    assert L.olg_prop_plan_create(C.byref(desc(lam=float("nan"))), C.byref(plan)) == -1
    assert L.olg_prop_plan_create(C.byref(desc(method=1, z=0.0)), C.byref(plan)) == -1   # Fresnel at z = 0
    assert L.olg_prop_plan_create(C.byref(desc(method=2, s=1.0)), C.byref(plan)) == -1   # ARSS, s = 1
    assert L.olg_prop_plan_create(C.byref(desc(method=2, ox=float("inf"))), C.byref(plan)) == -1
    assert plan.value is None
    assert L.olg_prop_plan_execute(None, base, base, None) == -1
    ptrs = (C.c_void_p * 1)(base)
    assert L.olg_prop_plan_execute_host(None, ptrs, ptrs, 1, None) == -1
    assert L.olg_prop_plan_destroy(None) == 0
    # the batch plan runs the same checks on every field
    arr = (F * 2)(desc(ny=256, nx=256), desc(ny=256, nx=256, method=2, s=0.0))
    bplan = C.c_void_p()
    assert L.olg_batch_plan_create(arr, 2, C.byref(bplan)) == -1
    assert b"s = 0" in L.olg_last_error() or b"s|s-1|" in L.olg_last_error()


def test_cgh_host_sequence_validation_without_gpu():
    """The host-cloud CGH sequence checks its arguments before any device work."""
    L = _lib.lib()
    buf = (C.c_float * 16)()
    p = (C.c_void_p * 1)(C.addressof(buf))
    n = (C.c_int * 1)(1)
    args = (6, 8, 8e-6, 8e-6, 532e-9)
    assert L.olg_cgh_fresnel_gemm_host_c64(p, None, None, n, p, 0, *args, 0, None) == 0      # nothing to do
    assert L.olg_cgh_fresnel_gemm_host_c64(p, None, None, n, p, -1, *args, 0, None) == -1
    assert L.olg_cgh_fresnel_gemm_host_c64(None, None, None, n, p, 1, *args, 0, None) == -1
    assert L.olg_cgh_fresnel_gemm_host_c64(p, None, None, n, p, 1, *args, _lib.OLG_ACCUMULATE, None) == -1
    assert L.olg_cgh_fresnel_gemm_host_c64(p, None, None, n, p, 1, 6, 5000, 8e-6, 8e-6, 532e-9, 0, None) == -2
    assert L.olg_cgh_fresnel_gemm_host_c64(p, None, None, n, p, 1, 6, 8, 8e-6, 8e-6, -1.0, 0, None) == -1
    bad = (C.c_int * 1)(-3)
    assert L.olg_cgh_fresnel_gemm_host_c64(p, None, None, bad, p, 1, *args, 0, None) == -1
    nullh = (C.c_void_p * 1)(None)
    assert L.olg_cgh_fresnel_gemm_host_c64(p, None, None, n, nullh, 1, *args, 0, None) == -1


def test_workspace_size():
    L = _lib.lib()
    ws = L.olg_prop_workspace_bytes(1024, 1024)
    assert ws >= 1024 * 2048 * 8
    assert ws < 1024 * 2048 * 8 * 1.1


def test_cgh_host_sequence_python_checks_without_gpu():
    """openol_gb300.cgh_fresnel_gemm_host checks its host tensors before any
    device work: one hologram per cloud, n x 3 float32 clouds, ny x nx
    complex64 holograms, per-point amplitudes of the cloud's length."""
    import pytest
    import torch

    import openol_gb300 as og

    pts = [torch.zeros((4, 3), dtype=torch.float32)]
    holo = [torch.zeros((6, 8), dtype=torch.complex64)]
    kw = dict(ny=6, nx=8, py=8e-6, px=8e-6, lam=532e-9)
    with pytest.raises(ValueError):
        og.cgh_fresnel_gemm_host(pts, holo * 2, **kw)
    with pytest.raises(TypeError):
        og.cgh_fresnel_gemm_host([torch.zeros((4, 3), dtype=torch.float64)], holo, **kw)
    with pytest.raises(ValueError):
        og.cgh_fresnel_gemm_host([torch.zeros((4, 2), dtype=torch.float32)], holo, **kw)
    with pytest.raises(ValueError):
        og.cgh_fresnel_gemm_host(pts, [torch.zeros((5, 8), dtype=torch.complex64)], **kw)
    with pytest.raises(ValueError):
        og.cgh_fresnel_gemm_host(pts, holo, amp=[torch.zeros(3, dtype=torch.float32)], **kw)
    with pytest.raises(TypeError):
        og.cgh_fresnel_gemm_host(pts, [torch.zeros((6, 8), dtype=torch.complex128)], **kw)
