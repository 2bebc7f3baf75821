"""Point-cloud CGH and the WRP method: the Python mirror of golcgh.h.

Point clouds are ``gObject`` instances holding a CUDA float32 tensor of shape
(N, 3) -- the reference's ``ol::gObject<float>`` (golclass.h:58-71), an AoS of
``Vect3<float>``.  Holograms are CUDA complex64 tensors (ny, nx), or float32
tensors for the phase-output kernels.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from ._lib import OLG_ACCUMULATE, OLG_REUSE_OPERANDS, OLG_VERBOSE, call, lib
from .prop import PROPMODE, _dev_field, _stream


class gObject:
    """Device point cloud, ol::gObject<float> (golclass.h:58-71)."""

    def __init__(self, points, device="cuda"):
        if isinstance(points, int):
            self.points = torch.zeros((points, 3), dtype=torch.float32, device=device)
        else:
            t = torch.as_tensor(np.asarray(points, dtype=np.float32) if not isinstance(points, torch.Tensor)
                                else points)
            self.points = t.to(device=device, dtype=torch.float32).reshape(-1, 3).contiguous()

    @property
    def size(self) -> int:
        return int(self.points.shape[0])

    def __len__(self):
        return self.size


def Object2cuda(obj) -> gObject:
    """ol::Object2cuda (golclass.h:73-78): host (N, 3) points -> gObject."""
    if isinstance(obj, gObject):
        return obj
    return gObject(obj)


def _opt(t):
    if t is None:
        return None
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32 and t.is_contiguous()):
        raise TypeError("per-point arrays must be contiguous CUDA float32 tensors")
    return t.data_ptr()


def cgh_fresnel(gobj, U=None, *, ny, nx, py, px, lam, amp=None, phase0=None, phase_out=None, accumulate=False,
                stream=None):
    """Fresnel-form CGH (olg_cgh_fresnel_c64): U[h,w] = sum_j a_j exp(i(pi rho^2/(lambda z_j) + phi_j))."""
    if U is not None:
        _dev_field(U, ny, nx, "U")
    if phase_out is not None and (phase_out.dtype != torch.float32 or not phase_out.is_cuda):
        raise TypeError("phase_out must be a CUDA float32 tensor")
    call("olg_cgh_fresnel_c64", gobj.points.data_ptr(), _opt(amp), _opt(phase0), gobj.size,
         U.data_ptr() if U is not None else None, phase_out.data_ptr() if phase_out is not None else None,
         ny, nx, float(py), float(px), float(lam), OLG_ACCUMULATE if accumulate else 0, _stream(stream))
    return U if U is not None else phase_out


def cgh_exact(gobj, U, *, ny, nx, py, px, lam, amp=None, phase0=None, accumulate=False, stream=None):
    """Exact spherical CGH (olg_cgh_exact_c64): U = sum_j a_j exp(i(k r_j + phi_j)) / r_j."""
    _dev_field(U, ny, nx, "U")
    call("olg_cgh_exact_c64", gobj.points.data_ptr(), _opt(amp), _opt(phase0), gobj.size, U.data_ptr(), ny, nx,
         float(py), float(px), float(lam), OLG_ACCUMULATE if accumulate else 0, _stream(stream))
    return U


def _cgh_adjoint(fn, gobj, G, g, ny, nx, py, px, lam, accumulate, stream, work):
    _dev_field(G, ny, nx, "G")
    n = gobj.size
    if g is None:
        g = torch.zeros(n, dtype=torch.complex64, device=G.device)
    if not (g.is_cuda and g.dtype == torch.complex64 and g.is_contiguous() and g.numel() == n):
        raise TypeError("g must be a contiguous CUDA complex64 tensor with one entry per point")
    wp, wb = (work.data_ptr(), work.numel() * work.element_size()) if work is not None else (None, 0)
    call(fn, gobj.points.data_ptr(), n, G.data_ptr(), g.data_ptr(), ny, nx, float(py), float(px), float(lam),
         OLG_ACCUMULATE if accumulate else 0, wp, wb, _stream(stream))
    return g


def cgh_fresnel_adjoint(gobj, G, g=None, *, ny, nx, py, px, lam, accumulate=False, stream=None, work=None):
    """Adjoint of the Fresnel-form CGH (olg_cgh_fresnel_adjoint_c64):
    g_j = sum_{h,w} conj(exp(i pi rho^2 / (lambda z_j))) G[h,w]."""
    return _cgh_adjoint("olg_cgh_fresnel_adjoint_c64", gobj, G, g, ny, nx, py, px, lam, accumulate, stream, work)


def cgh_fresnel_adjoint_gemm(gobj, G, g=None, *, ny, nx, py, px, lam, accumulate=False, stream=None, work=None):
    """The Fresnel adjoint on the tensor cores (olg_cgh_fresnel_adjoint_gemm_c64):
    the same g_j as cgh_fresnel_adjoint, through T = G conj(X) as a split-FP16
    tcgen05 GEMM and a per-point reduction over rows."""
    return _cgh_adjoint("olg_cgh_fresnel_adjoint_gemm_c64", gobj, G, g, ny, nx, py, px, lam, accumulate, stream, work)


def cgh_adjoint_gemm_workspace(n_points, ny, nx, device="cuda"):
    return torch.empty(int(lib().olg_cgh_adjoint_gemm_workspace_bytes(n_points, ny, nx)), dtype=torch.uint8,
                       device=device)


def cgh_exact_adjoint(gobj, G, g=None, *, ny, nx, py, px, lam, accumulate=False, stream=None, work=None):
    """Adjoint of the exact spherical CGH (olg_cgh_exact_adjoint_c64):
    g_j = sum_{h,w} conj(exp(i k r_j) / r_j) G[h,w]."""
    return _cgh_adjoint("olg_cgh_exact_adjoint_c64", gobj, G, g, ny, nx, py, px, lam, accumulate, stream, work)


def cgh_fresnel_gemm(gobj, U, *, ny, nx, py, px, lam, amp=None, phase0=None, accumulate=False, stream=None,
                     work=None, reuse_operands=False):
    """Fresnel-form CGH as a split-FP16 tensor-core GEMM (olg_cgh_fresnel_gemm_c64).
    ``reuse_operands``: the f16 operands are already in ``work`` from a previous
    call with the same points, pitch and wavelength; only the GEMM runs."""
    _dev_field(U, ny, nx, "U")
    wp, wb = (work.data_ptr(), work.numel() * work.element_size()) if work is not None else (None, 0)
    flags = (OLG_ACCUMULATE if accumulate else 0) | (OLG_REUSE_OPERANDS if reuse_operands else 0)
    call("olg_cgh_fresnel_gemm_c64", gobj.points.data_ptr(), _opt(amp), _opt(phase0), gobj.size, U.data_ptr(),
         ny, nx, float(py), float(px), float(lam), flags, wp, wb, _stream(stream))
    return U


def cgh_fresnel_gemm_host(points, holograms, *, ny, nx, py, px, lam, amp=None, phase0=None, stream=None):
    """A sequence of holograms from host point clouds (olg_cgh_fresnel_gemm_host_c64):
    ``holograms[i]`` (CPU complex64, ny x nx) = the Fresnel-form hologram of
    ``points[i]`` (CPU float32, n_i x 3), with ``amp[i]`` / ``phase0[i]`` (CPU
    float32, n_i; lists or entries may be None).  Cloud i+1's copy in and
    hologram i-1's copy out overlap hologram i's GEMM; pinned tensors
    (``pin_memory()``) for the copies to run asynchronously.  Ordered on
    ``stream``: synchronize it before reading the holograms."""
    n = len(points)
    if len(holograms) != n:
        raise ValueError("one hologram per point cloud")

    def host(t, dtype, what):
        if t is None:
            return None
        if not (isinstance(t, torch.Tensor) and not t.is_cuda and t.dtype == dtype and t.is_contiguous()):
            raise TypeError(f"{what} must be contiguous CPU {dtype} tensors")
        return t

    amp = list(amp) if amp is not None else [None] * n
    phase0 = list(phase0) if phase0 is not None else [None] * n
    if len(amp) != n or len(phase0) != n:
        raise ValueError("one amplitude / phase entry per point cloud")
    counts = []
    for i in range(n):
        p = host(points[i], torch.float32, "points")
        if p.dim() != 2 or p.shape[1] != 3:
            raise ValueError("points must be n x 3")
        counts.append(int(p.shape[0]))
        for t, what in ((amp[i], "amp"), (phase0[i], "phase0")):
            if host(t, torch.float32, what) is not None and t.numel() != counts[-1]:
                raise ValueError(f"{what}[{i}] must have one entry per point")
        h = host(holograms[i], torch.complex64, "holograms")
        if tuple(h.shape) != (ny, nx):
            raise ValueError("holograms must be ny x nx")
    arr = lambda ts: (C.c_void_p * max(n, 1))(*[t.data_ptr() if t is not None else None for t in ts])
    call("olg_cgh_fresnel_gemm_host_c64", arr(points), arr(amp), arr(phase0), (C.c_int * max(n, 1))(*counts),
         arr(holograms), n, int(ny), int(nx), float(py), float(px), float(lam), 0, _stream(stream))
    return holograms


def autotune_cgh_gemm(n_points, ny, nx, reps=5, stream=None):
    """Time the GEMM's tile form and K-tail split for this hologram shape
    (olg_autotune_cgh_gemm) and keep the fastest; returns (pairs, tail weight)."""
    call("olg_autotune_cgh_gemm", int(n_points), int(ny), int(nx), int(reps), _stream(stream))
    return int(lib().olg_cgh_gemm_pairs(-1)), float(lib().olg_cgh_gemm_tail_weight(-1.0))


def cgh_gemm_pairs(on=None):
    """Tile form of the GEMM (olg_cgh_gemm_pairs): True = two-SM pairs,
    False = single-SM tiles; None only reads it.  Returns the previous form."""
    return bool(lib().olg_cgh_gemm_pairs(-1 if on is None else int(bool(on))))


def cgh_gemm_workspace(n_points, ny, nx, device="cuda"):
    return torch.empty(int(lib().olg_cgh_gemm_workspace_bytes(n_points, ny, nx)), dtype=torch.uint8, device=device)


def device_fault_check(clear=True):
    """Raise OlgError if a tensor-core kernel gave up on a bounded wait (synchronises)."""
    call("olg_device_fault_check", int(clear))


def gCgh(gobj, U, ny, nx, *params):
    """ol::gCgh.  gCgh(gobj, U, ny, nx, p, lambda) -> complex hologram (gCghShared,
    golcgh.h:137-145); gCgh(gobj, U, ny, nx, py, px, lambda) -> complex hologram
    (golcgh.h:108-135) or, when U is a float32 tensor, its phase (golcgh.h:26-45)."""
    if len(params) == 2:
        p, lam = params
        py = px = p
    elif len(params) == 3:
        py, px, lam = params
    else:
        raise TypeError("gCgh(gobj, U, ny, nx, p, lambda) or gCgh(gobj, U, ny, nx, py, px, lambda)")
    if U.dtype == torch.float32:
        return cgh_fresnel(gobj, None, ny=ny, nx=nx, py=py, px=px, lam=lam, phase_out=U)
    return cgh_fresnel(gobj, U, ny=ny, nx=nx, py=py, px=px, lam=lam)


def gCghReduction(gobj, U, ny, nx, p, lam):
    """ol::gCghReduction (golcgh.h:147-195): U += the Fresnel-form hologram."""
    return cgh_fresnel(gobj, U, ny=ny, nx=nx, py=p, px=p, lam=lam, accumulate=True)


# ---------------------------------------------------------------------- WRP
def Cgh(obj, out, ny, nx, *params):
    """ol::Cgh for host point clouds and host holograms (olcgh.h:351-379):
    ``Cgh(obj, out, ny, nx, p, lam)`` or ``Cgh(obj, out, ny, nx, py, px, lam)``.
    ``obj``: (N, 3) host points (rounded to float32, the GPU path's point type);
    ``out``: a complex host array (the hologram) or a real one (its phase,
    atan2 as _CghFresnel olcgh.h:276-295 returns it), written in place."""
    if len(params) == 2:
        py = px = params[0]
        lam = params[1]
    elif len(params) == 3:
        py, px, lam = params
    else:
        raise TypeError("Cgh(obj, out, ny, nx, p, lam) or Cgh(obj, out, ny, nx, py, px, lam)")
    g = gObject(np.asarray(obj, np.float32).reshape(-1, 3))
    if np.iscomplexobj(out):
        U = torch.zeros((ny, nx), dtype=torch.complex64, device="cuda")
        gCgh(g, U, ny, nx, py, px, lam)
        res = U.cpu().numpy()
    else:
        ph = torch.zeros((ny, nx), dtype=torch.float32, device="cuda")
        cgh_fresnel(g, None, ny=ny, nx=nx, py=py, px=px, lam=lam, phase_out=ph)
        res = ph.cpu().numpy()
    out[...] = res.reshape(out.shape).astype(out.dtype, copy=False)
    return out


def wrp_plane_z(window, ny, nx, p, lam, zmin, s, p_limit=None) -> float:
    return float(lib().olg_wrp_plane_z(int(window), ny, nx, p, 0.0 if p_limit is None else p_limit, lam, zmin, s))


def _wrp_step1(obj, U, ny, nx, p, lam, d, plimit, window):
    _dev_field(U, ny, nx, "U")
    call("olg_wrp_step1_c64", obj.points.data_ptr(), obj.size, U.data_ptr(), ny, nx, float(p), float(lam),
         float(d), 0.0 if plimit is None else float(plimit), int(window), _stream())
    return U


def WRPStep1(obj, U, ny, nx, p, lam, d, plimit=None):
    """ol::WRPStep1 (golcgh.h:369-389): circular windows W_j = |z_j - d| / sqrt(4 (p/lambda)^2 - 1)."""
    return _wrp_step1(obj, U, ny, nx, p, lam, d, plimit, 0)


def WRPStep1_D(obj, U, ny, nx, p, lam, d, plimit=None):
    """ol::WRPStep1_D (golcgh.h:470-491): square windows of side D_j = sqrt(2) W_j."""
    return _wrp_step1(obj, U, ny, nx, p, lam, d, plimit, 1)


def WRPStep2(U, ny, nx, p, lam, d, propmode=PROPMODE.AUTO, verbose=True):
    """ol::WRPStep2 (golcgh.h:494-517)."""
    from .prop import AsmPropCheck, FresnelPropCheck, asm_prop, fresnel_prop
    _dev_field(U, ny, nx, "U")
    V = U.view(ny, nx)
    if propmode == PROPMODE.FRESNEL:
        return fresnel_prop(V, dy=p, dx=p, lam=lam, z=d)
    if propmode == PROPMODE.ASM:
        return asm_prop(V, dy=p, dx=p, lam=lam, z=d)
    if AsmPropCheck(ny, nx, p, p, lam, d):
        if verbose:
            print("WRP Step2 is AsmProp")
        return asm_prop(V, dy=p, dx=p, lam=lam, z=d)
    if not FresnelPropCheck(ny, nx, p, p, lam, d):
        if verbose:
            print("warning!!\neither AsmProp or FresnelProp does not meet the condition.")
        return asm_prop(V, dy=p, dx=p, lam=lam, z=d)
    if verbose:
        print("WRP Step2 is FresnelProp")
    return fresnel_prop(V, dy=p, dx=p, lam=lam, z=d)


def _wrp_method(obj, U, ny, nx, p, lam, zmin, s, propmode, p_limit, window, verbose):
    _dev_field(U, ny, nx, "U")
    pz = C.c_float(0.0)
    call("olg_wrp_method_c64", obj.points.data_ptr(), obj.size, U.data_ptr(), ny, nx, float(p), float(lam),
         float(zmin), float(s), 0.0 if p_limit is None else float(p_limit), int(window), int(propmode),
         OLG_VERBOSE if verbose else 0, C.byref(pz), _stream())
    return U, pz.value


def WRPMethod(obj, U, ny, nx, p, lam, zmin, s=0.9, propmode=PROPMODE.AUTO, verbose=True):
    """ol::WRPMethod (golcgh.h:561-581).  Returns (U, plane_z)."""
    return _wrp_method(obj, U, ny, nx, p, lam, zmin, s, propmode, None, 0, verbose)


def WRPMethod_D(obj, U, ny, nx, p, lam, zmin, s=0.9, propmode=PROPMODE.AUTO, p_limit=None, verbose=True):
    """ol::WRPMethod_D (golcgh.h:519-559, p_limit overload :540-559).  Returns (U, plane_z)."""
    return _wrp_method(obj, U, ny, nx, p, lam, zmin, s, propmode, p_limit, 1, verbose)
