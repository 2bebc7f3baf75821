"""Batched propagation: many fields of different sizes, methods, distances and
wavelengths in one persistent launch (olg_batch_*), replayable from a CUDA graph.
Fields of at least ``direct_pixels()`` pixels (default 2048 x 2048) each fill the
GPU alone and run after it through the single-field passes."""
from __future__ import annotations

import ctypes as C

import torch

from ._lib import OlgField, call, lib
from .prop import _stream

METHODS = {"asm": 0, "fresnel": 1, "arss": 2, "fresnel_bandlimit": 3}


class BatchPlan:
    """fields: dicts with keys u_in, u_out (CUDA complex64 (ny, nx), may be the same
    tensor), method ('asm' | 'fresnel' | 'arss' | 'fresnel_bandlimit'), dy, dx, lam, z
    and, for ARSS, s (oy, ox optional)."""

    def __init__(self, fields):
        self._keep = []
        arr = (OlgField * len(fields))()
        for i, f in enumerate(fields):
            u_in, u_out = f["u_in"], f.get("u_out", f["u_in"])
            for t in (u_in, u_out):
                if not (t.is_cuda and t.dtype == torch.complex64 and t.is_contiguous()):
                    raise TypeError("fields must be contiguous CUDA complex64 tensors")
            self._keep += [u_in, u_out]
            ny, nx = u_in.shape
            arr[i] = OlgField(u_in.data_ptr(), u_out.data_ptr(), ny, nx, METHODS[f["method"]], int(f.get("flags", 0)),
                              float(f["dy"]), float(f["dx"]), float(f["lam"]), float(f["z"]), float(f.get("s", 0.5)),
                              float(f.get("oy", 0.0)), float(f.get("ox", 0.0)))
        self._plan = C.c_void_p()
        call("olg_batch_plan_create", arr, len(fields), C.byref(self._plan))
        self.n_fields = len(fields)
        self.n_items = int(lib().olg_batch_plan_items(self._plan))
        self.n_direct = int(lib().olg_batch_plan_direct_fields(self._plan))

    def execute(self, stream=None):
        """One persistent launch for the small fields, then the single-field passes
        for the large ones (capturable in a CUDA graph)."""
        call("olg_batch_execute", self._plan, _stream(stream))

    def execute_host(self, host_in, host_out, stream=None):
        """The plan's fields from host tensors and back (olg_batch_execute_host):
        ``host_in[i]`` is copied into field i's input, the plan runs, and field i's
        output is copied into ``host_out[i]``, with the copies in, the propagations
        and the copies out pipelined over three streams.  Host tensors: CPU
        complex64 of each field's shape, contiguous; pinned memory
        (``pin_memory()``) for the copies to run asynchronously.  Ordered on
        ``stream``: synchronize it before reading ``host_out``."""
        if len(host_in) != self.n_fields or len(host_out) != self.n_fields:
            raise ValueError("one host tensor per field, in and out")
        for t in list(host_in) + list(host_out):
            if t.is_cuda or t.dtype != torch.complex64 or not t.is_contiguous():
                raise TypeError("host fields must be contiguous CPU complex64 tensors")
        for t, d in zip(host_in, self._keep[0::2]):
            if tuple(t.shape) != tuple(d.shape):
                raise ValueError("host field shape differs from the plan's")
        hin = (C.c_void_p * self.n_fields)(*[t.data_ptr() for t in host_in])
        hout = (C.c_void_p * self.n_fields)(*[t.data_ptr() for t in host_out])
        call("olg_batch_execute_host", self._plan, hin, hout, _stream(stream))

    def execute_serial(self, stream=None):
        """The same fields one after another through the single-field entry points."""
        call("olg_batch_execute_serial", self._plan, _stream(stream))

    def check(self):
        """Raises OlgError if an item of the last persistent launch gave up on its bounded wait."""
        call("olg_batch_check", self._plan)

    def close(self):
        if self._plan:
            lib().olg_batch_plan_destroy(self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class PropPlan:
    """One propagation set up once (olg_prop_plan_*): method ('asm' | 'fresnel' |
    'arss' | 'fresnel_bandlimit'), field shape (ny, nx), dy, dx, lam, z and, for
    ARSS, s (oy, ox optional); flags as the single calls take.  Creation checks
    the parameters, allocates the scratch and computes the Fresnel / ARSS chirp
    spectra; ``execute`` binds device fields and runs the three passes.
    Executions share the plan's scratch: keep them on one stream."""

    def __init__(self, method, ny, nx, *, dy, dx, lam, z, s=0.5, oy=0.0, ox=0.0, flags=0):
        self.shape = (int(ny), int(nx))
        desc = OlgField(None, None, int(ny), int(nx), METHODS[method], int(flags), float(dy), float(dx), float(lam),
                        float(z), float(s), float(oy), float(ox))
        self._plan = C.c_void_p()
        call("olg_prop_plan_create", C.byref(desc), C.byref(self._plan))

    def execute(self, u_in, u_out=None, stream=None):
        """Propagate ``u_in`` into ``u_out`` (in place when omitted): contiguous
        CUDA complex64 tensors of the plan's shape."""
        u_out = u_in if u_out is None else u_out
        for t in (u_in, u_out):
            if not (t.is_cuda and t.dtype == torch.complex64 and t.is_contiguous()) or tuple(t.shape) != self.shape:
                raise TypeError("fields must be contiguous CUDA complex64 tensors of the plan's shape")
        call("olg_prop_plan_execute", self._plan, u_in.data_ptr(), u_out.data_ptr(), _stream(stream))
        return u_out

    def execute_host(self, host_in, host_out, stream=None):
        """A sequence of host fields through the plan (olg_prop_plan_execute_host):
        ``host_out[i]`` = the propagation of ``host_in[i]``, with field i+1's copy
        in and field i-1's copy out overlapping field i's passes.  Host tensors:
        contiguous CPU complex64 of the plan's shape, pinned (``pin_memory()``)
        for the copies to run asynchronously.  Ordered on ``stream``: synchronize
        it before reading ``host_out``."""
        if len(host_in) != len(host_out):
            raise ValueError("one host output per host input")
        for t in list(host_in) + list(host_out):
            if t.is_cuda or t.dtype != torch.complex64 or not t.is_contiguous() or tuple(t.shape) != self.shape:
                raise TypeError("host fields must be contiguous CPU complex64 tensors of the plan's shape")
        n = len(host_in)
        hin = (C.c_void_p * max(n, 1))(*[t.data_ptr() for t in host_in])
        hout = (C.c_void_p * max(n, 1))(*[t.data_ptr() for t in host_out])
        call("olg_prop_plan_execute_host", self._plan, hin, hout, n, _stream(stream))
        return host_out

    def close(self):
        if self._plan:
            lib().olg_prop_plan_destroy(self._plan)
            self._plan = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def direct_pixels(pixels=None):
    """The size (ny * nx) from which plans created afterwards run a field through
    the single-field passes instead of the persistent kernel; with ``pixels``,
    sets it and returns the previous value."""
    return int(lib().olg_batch_direct_pixels(int(pixels) if pixels else 0))


def config5_fields(n=96, seed=20261203 + 5, p=8e-6, s=0.5, device="cuda"):
    """The mixed batch workload: sizes U{512^2, 1024^2, 2048^2, 4096^2}, methods
    U{ASM, Fresnel, ARSS}, z ~ U[10, 300] mm, lambda U{640, 532, 450} nm, binary
    amplitude x uniform phase fields (seeded)."""
    import numpy as np
    rng = np.random.default_rng(seed)
    sizes = rng.choice([512, 1024, 2048, 4096], n)
    methods = rng.choice(["asm", "fresnel", "arss"], n)
    zs = 0.01 + 0.29 * rng.random(n)
    lams = rng.choice([640e-9, 532e-9, 450e-9], n)
    fields = []
    g = torch.Generator(device=device).manual_seed(seed)
    for k in range(n):
        m = int(sizes[k])
        amp = (torch.rand((m, m), generator=g, device=device) < 0.5).float()
        ph = 2 * np.pi * torch.rand((m, m), generator=g, device=device)
        u = torch.polar(amp, ph).to(torch.complex64)
        fields.append(dict(u_in=u, u_out=torch.empty_like(u), method=str(methods[k]), dy=p, dx=p,
                           lam=float(lams[k]), z=float(zs[k]), s=s))
    return fields
