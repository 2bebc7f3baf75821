"""Propagation: the Python mirror of the reference's golprop.h API.

Names, argument order and meaning follow the reference (``ol::gAsmProp``,
``ol::gFresnelProp``, ``ol::gFresnelPropBandLimit``, ``ol::ARSSFresnelProp``,
``ol::Prop``, ``ol::AsmPropCheck``, ``ol::FresnelPropCheck``).  A device field is
a CUDA ``torch.complex64`` tensor of shape (ny, nx) (the reference's
``cuda::unique_ptr<thrust::complex<float>[]>``); like the reference, the result
is written back into it.  A host field (numpy array or CPU tensor, the
reference's ``std::unique_ptr<std::complex<float>[]>`` overloads) is copied to
the GPU, propagated with the host overload's conventions, and copied back.

Everything runs through libolgb300.so; failures raise ``OlgError``.
"""
from __future__ import annotations

import ctypes as C
from enum import IntEnum

import numpy as np
import torch

from ._lib import (OLG_ACCUMULATE, OLG_BANDLIMIT, OLG_CHECK_F32, OLG_CONJ, OLG_NO_NORMALIZE, OLG_VERBOSE, call,
                   lib)


class PROPMODE(IntEnum):
    """ol::PROPMODE (oldefine.h:7-9)."""

    ASM = 0
    FRESNEL = 1
    AUTO = 2


ASM, FRESNEL, AUTO = PROPMODE.ASM, PROPMODE.FRESNEL, PROPMODE.AUTO


def _stream(stream=None) -> int:
    s = stream if stream is not None else torch.cuda.current_stream()
    return int(s.cuda_stream)


def _dev_field(u, ny, nx, name="u"):
    if not isinstance(u, torch.Tensor) or not u.is_cuda:
        raise TypeError(f"{name} must be a CUDA tensor")
    if u.dtype != torch.complex64 or not u.is_contiguous() or u.numel() != ny * nx:
        raise ValueError(f"{name} must be a contiguous complex64 tensor with ny*nx = {ny * nx} elements")
    return u


def _is_host(u) -> bool:
    return isinstance(u, np.ndarray) or (isinstance(u, torch.Tensor) and not u.is_cuda)


def _host_roundtrip(u, ny, nx, fn):
    """Copy a host field to the GPU, run fn(device_tensor), copy back in place."""
    if isinstance(u, np.ndarray):
        d = torch.from_numpy(np.ascontiguousarray(u, np.complex64).reshape(ny, nx)).cuda()
        fn(d)
        u[...] = d.cpu().numpy().reshape(u.shape).astype(u.dtype, copy=False)
        return u
    d = u.reshape(ny, nx).to(device="cuda", dtype=torch.complex64).contiguous()
    fn(d)
    u.copy_(d.cpu().reshape(u.shape).to(u.dtype))
    return u


# ------------------------------------------------------------------ general
def _pinned_ptr(u, ny, nx, name):
    """Device address of a page-locked host field (olg_host_device_pointer)."""
    if u.dtype != torch.complex64 or not u.is_contiguous() or u.numel() != ny * nx:
        raise ValueError(f"{name} must be a contiguous complex64 tensor with ny*nx = {ny * nx} elements")
    d = C.c_void_p()
    call("olg_host_device_pointer", u.data_ptr(), C.byref(d))
    return d.value


def _field_ptr(u, ny, nx, name):
    """CUDA tensors by address; pinned CPU tensors by their mapped device address."""
    if isinstance(u, torch.Tensor) and not u.is_cuda and u.is_pinned():
        return _pinned_ptr(u, ny, nx, name)
    return _dev_field(u, ny, nx, name).data_ptr()


def asm_prop(u_in, u_out=None, *, dy, dx, lam, z, adjoint=False, normalize=True, stream=None, work=None):
    """Angular spectrum method (olg_asm_prop_c64) on CUDA tensors or on pinned
    (page-locked) CPU tensors.  For pinned fields pass 1 reads the input and
    pass 3 writes the output over the host link directly, with no staging
    copies; as for device fields, the result is ready once ``stream`` is.

    ``adjoint`` applies the conjugate transfer function (the adjoint operator);
    ``normalize=False`` omits 1/Np like the host-pointer overload.
    """
    ny, nx = u_in.shape
    pin = _field_ptr(u_in, ny, nx, "u_in")
    u_out = u_in if u_out is None else u_out
    pout = _field_ptr(u_out, ny, nx, "u_out")
    flags = (OLG_CONJ if adjoint else 0) | (0 if normalize else OLG_NO_NORMALIZE)
    wp, wb = (work.data_ptr(), work.numel() * work.element_size()) if work is not None else (None, 0)
    call("olg_asm_prop_c64", pin, pout, ny, nx, float(dy), float(dx), float(lam), float(z), flags, wp, wb,
         _stream(stream))
    return u_out


def fresnel_prop(u_in, u_out=None, *, dy, dx, lam, z, bandlimit=0, adjoint=False, normalize=True, stream=None,
                 work=None):
    """Fresnel convolution propagation (olg_fresnel_prop_c64).  bandlimit: 0 none,
    1 the GPU band limit (golprop.h:225-233), 2 the CPU band limit (olprop.h:26-50)."""
    ny, nx = u_in.shape
    _dev_field(u_in, ny, nx, "u_in")
    u_out = u_in if u_out is None else _dev_field(u_out, ny, nx, "u_out")
    flags = (OLG_CONJ if adjoint else 0) | (0 if normalize else OLG_NO_NORMALIZE)
    wp, wb = (work.data_ptr(), work.numel() * work.element_size()) if work is not None else (None, 0)
    call("olg_fresnel_prop_c64", u_in.data_ptr(), u_out.data_ptr(), ny, nx, float(dy), float(dx), float(lam),
         float(z), int(bandlimit), flags, wp, wb, _stream(stream))
    return u_out


def arss_prop(u_src, u_dst=None, *, dy, dx, lam, z, s, oy=0.0, ox=0.0, adjoint=False, stream=None, work=None):
    """ARSS scaled Fresnel propagation (olg_arss_prop_c64)."""
    ny, nx = u_src.shape
    _dev_field(u_src, ny, nx, "u_src")
    u_dst = u_src if u_dst is None else _dev_field(u_dst, ny, nx, "u_dst")
    wp, wb = (work.data_ptr(), work.numel() * work.element_size()) if work is not None else (None, 0)
    call("olg_arss_prop_c64", u_src.data_ptr(), u_dst.data_ptr(), ny, nx, float(dy), float(dx), float(lam),
         float(z), float(s), float(oy), float(ox), OLG_CONJ if adjoint else 0, wp, wb, _stream(stream))
    return u_dst


def workspace_bytes(ny, nx) -> int:
    return int(lib().olg_prop_workspace_bytes(ny, nx))


def workspace(ny, nx, device="cuda"):
    """A reusable scratch buffer for one propagation of an ny x nx field."""
    return torch.empty(workspace_bytes(ny, nx), dtype=torch.uint8, device=device)


# ------------------------------------------------------- reference mirror
def gAsmProp(u, ny, nx, dy, dx, lam, d):
    """ol::gAsmProp: device overload golprop.h:507-534 (1/Np applied) or, for a
    host field, the host overload golprop.h:458-504 (no 1/Np)."""
    if _is_host(u):
        return _host_roundtrip(u, ny, nx, lambda t: asm_prop(t, dy=dy, dx=dx, lam=lam, z=d, normalize=False))
    return asm_prop(_dev_field(u, ny, nx).view(ny, nx), dy=dy, dx=dx, lam=lam, z=d)


def gFresnelProp(u, ny, nx, dy, dx, lam, d):
    """ol::gFresnelProp: device overload golprop.h:167-198, host overload golprop.h:70-124."""
    if _is_host(u):
        return _host_roundtrip(u, ny, nx, lambda t: fresnel_prop(t, dy=dy, dx=dx, lam=lam, z=d, normalize=False))
    return fresnel_prop(_dev_field(u, ny, nx).view(ny, nx), dy=dy, dx=dx, lam=lam, z=d)


def gFresnelPropBandLimit(u, ny, nx, dy, dx, lam, d):
    """ol::gFresnelPropBandLimit, golprop.h:278-302."""
    return fresnel_prop(_dev_field(u, ny, nx).view(ny, nx), dy=dy, dx=dx, lam=lam, z=d, bandlimit=1)


def ARSSFresnelProp(usrc, udst, ny, nx, dy, dx, lam, z, s, oy=0.0, ox=0.0):
    """ol::ARSSFresnelProp, golprop.h:941-995 (and the 9-argument form :990-995)."""
    return arss_prop(_dev_field(usrc, ny, nx, "usrc").view(ny, nx), _dev_field(udst, ny, nx, "udst").view(ny, nx),
                     dy=dy, dx=dx, lam=lam, z=z, s=s, oy=oy, ox=ox)


def AsmPropCheck(ny, nx, dy, dx, lam, z, single_precision=True) -> bool:
    """ol::AsmPropCheck, olprop.h:209-225 (float evaluation by default, as the GPU path uses it)."""
    return bool(lib().olg_asm_prop_check(ny, nx, float(dy), float(dx), float(lam), float(z), int(single_precision)))


def FresnelPropCheck(ny, nx, dy, dx, lam, z, single_precision=True) -> bool:
    """ol::FresnelPropCheck, olprop.h:109-123."""
    return bool(lib().olg_fresnel_prop_check(ny, nx, float(dy), float(dx), float(lam), float(z),
                                             int(single_precision)))


def Prop(u, ny, nx, dy, dx, lam, d, propmode=PROPMODE.AUTO, verbose=True, single_precision=True):
    """ol::Prop, golprop.h:578-604: ASM / FRESNEL / AUTO (ASM if its check passes,
    else Fresnel if its check passes, else band-limited Fresnel).  Prints the
    chosen method like the reference when ``verbose``.  Returns the field;
    the chosen branch (0 ASM, 1 Fresnel, 2 band-limited) is in ``Prop.last_choice``."""
    t = _dev_field(u, ny, nx)
    chosen = C.c_int(-1)
    flags = (OLG_VERBOSE if verbose else 0) | (OLG_CHECK_F32 if single_precision else 0)
    call("olg_prop_c64", t.data_ptr(), ny, nx, float(dy), float(dx), float(lam), float(d), int(propmode), flags,
         C.byref(chosen), None, 0, _stream())
    Prop.last_choice = chosen.value
    return u


Prop.last_choice = -1


# ------------------------------------------- host-field templates of olprop.h
# The reference's CPU templates take host fields of any std::complex<COMPLEX_T>;
# these mirrors take host arrays (numpy or CPU tensors) of any complex dtype,
# propagate them in complex64 on the GPU and write the result back in place.
def AsmProp(u, height, width, dy, dx, lam, z):
    """ol::AsmProp, olprop.h:227-248: crop(IFFT(H FFT(pad u)) / Np), in place."""
    return _host_roundtrip(u, height, width, lambda d: asm_prop(d, dy=dy, dx=dx, lam=lam, z=z))


def FresnelProp(u, height, width, dy, dx, lam, z):
    """ol::FresnelProp, olprop.h:125-148 (both spectra scaled by 1/Np), in place."""
    return _host_roundtrip(u, height, width, lambda d: fresnel_prop(d, dy=dy, dx=dx, lam=lam, z=z))


def FresnelPropBandLimit(u, height, width, dy, dx, lam, z):
    """ol::FresnelPropBandLimit, olprop.h:150-170: the response zeroed outside the
    x and y limits of FresnelResponseBandLimit (olprop.h:26-50), in place."""
    return _host_roundtrip(u, height, width, lambda d: fresnel_prop(d, dy=dy, dx=dx, lam=lam, z=z, bandlimit=2))


def PropHost(u, ny, nx, dy, dx, lam, d, propmode=PROPMODE.AUTO, verbose=True, single_precision=False):
    """ol::Prop for host fields, olprop.h:656-682: AUTO takes AsmProp when
    AsmPropCheck passes, else FresnelProp when FresnelPropCheck passes, else the
    CPU FresnelPropBandLimit.  The checks run in double unless
    ``single_precision`` (the reference's PREC_T)."""
    say = print if verbose else (lambda *a: None)
    pm = int(propmode)
    if pm == PROPMODE.FRESNEL:
        say("FresnelProp")
        return FresnelProp(u, ny, nx, dy, dx, lam, d)
    if pm == PROPMODE.ASM:
        say("AsmProp")
        return AsmProp(u, ny, nx, dy, dx, lam, d)
    if pm != PROPMODE.AUTO:
        raise ValueError("invalid PROPMODE")
    if AsmPropCheck(ny, nx, dy, dx, lam, d, single_precision):
        say("AsmProp")
        return AsmProp(u, ny, nx, dy, dx, lam, d)
    if not FresnelPropCheck(ny, nx, dy, dx, lam, d, single_precision):
        say("warning!!\neither AsmProp or FresnelProp does not meet the condition.")
        return FresnelPropBandLimit(u, ny, nx, dy, dx, lam, d)
    say("FresnelProp")
    return FresnelProp(u, ny, nx, dy, dx, lam, d)


# ------------------------------------------------------- shifted / split
def _work(work):
    return (work.data_ptr(), work.numel() * work.element_size()) if work is not None else (None, 0)


def shifted_asm_prop(u_in, u_out=None, *, dy, dx, lam, z, oy, ox, bandlimit=False, window_f32=False, adjoint=False,
                     normalize=True, stream=None, work=None):
    """Shifted angular spectrum method (olg_shifted_asm_prop_c64): the destination
    plane is offset by (oy, ox).  ``bandlimit`` adds the host overload's band
    window (decided in float with ``window_f32``)."""
    ny, nx = u_in.shape
    _dev_field(u_in, ny, nx, "u_in")
    u_out = u_in if u_out is None else _dev_field(u_out, ny, nx, "u_out")
    flags = ((OLG_CONJ if adjoint else 0) | (0 if normalize else OLG_NO_NORMALIZE) |
             (OLG_BANDLIMIT if bandlimit else 0) | (OLG_CHECK_F32 if window_f32 else 0))
    wp, wb = _work(work)
    call("olg_shifted_asm_prop_c64", u_in.data_ptr(), u_out.data_ptr(), ny, nx, float(dy), float(dx), float(lam),
         float(z), float(oy), float(ox), flags, wp, wb, _stream(stream))
    return u_out


def shifted_fresnel_prop(u_src, u_dst=None, *, dy, dx, lam, z, s=1.0, oy=0.0, ox=0.0, adjoint=False, stream=None,
                         work=None):
    """Shifted (scaled) Fresnel propagation (olg_shifted_fresnel_prop_c64)."""
    ny, nx = u_src.shape
    _dev_field(u_src, ny, nx, "u_src")
    u_dst = u_src if u_dst is None else _dev_field(u_dst, ny, nx, "u_dst")
    wp, wb = _work(work)
    call("olg_shifted_fresnel_prop_c64", u_src.data_ptr(), u_dst.data_ptr(), ny, nx, float(dy), float(dx), float(lam),
         float(z), float(s), float(oy), float(ox), OLG_CONJ if adjoint else 0, wp, wb, _stream(stream))
    return u_dst


def split_workspace(ny, nx, blocks_y=2, blocks_x=2, device="cuda"):
    n = int(lib().olg_split_prop_workspace_bytes(ny, nx, blocks_y, blocks_x))
    return torch.empty(n, dtype=torch.uint8, device=device)


def split_prop(u_in, u_out, *, dy, dx, lam, z, propmode=PROPMODE.ASM, blocks_y=2, blocks_x=2, bandlimit=False,
               window_f32=False, accumulate=False, stream=None, work=None):
    """Split propagation (olg_split_prop_c64): every (source, destination) block
    pair adds a shifted propagation; ``u_out`` must be a separate tensor."""
    ny, nx = u_in.shape
    _dev_field(u_in, ny, nx, "u_in")
    _dev_field(u_out, ny, nx, "u_out")
    flags = ((OLG_BANDLIMIT if bandlimit else 0) | (OLG_CHECK_F32 if window_f32 else 0) |
             (OLG_ACCUMULATE if accumulate else 0))
    wp, wb = _work(work)
    call("olg_split_prop_c64", u_in.data_ptr(), u_out.data_ptr(), ny, nx, float(dy), float(dx), float(lam), float(z),
         int(propmode), int(blocks_y), int(blocks_x), flags, wp, wb, _stream(stream))
    return u_out


def gshiftedAsmProp(usrc, udst, ny, nx, dy, dx, lam, d, oy, ox):
    """ol::gshiftedAsmProp, golprop.h:537-575 (device fields, no band window, 1/Np)."""
    return shifted_asm_prop(_dev_field(usrc, ny, nx, "usrc").view(ny, nx), _dev_field(udst, ny, nx, "udst").view(ny, nx),
                            dy=dy, dx=dx, lam=lam, z=d, oy=oy, ox=ox)


def gshiftedFresnelProp(usrc, udst, ny, nx, dy, dx, lam, z, s, oy, ox):
    """ol::gshiftedFresnelProp, golprop.h:706-752."""
    return shifted_fresnel_prop(_dev_field(usrc, ny, nx, "usrc").view(ny, nx),
                                _dev_field(udst, ny, nx, "udst").view(ny, nx), dy=dy, dx=dx, lam=lam, z=z, s=s, oy=oy,
                                ox=ox)


def shiftedProp(usrc, udst, ny, nx, dy, dx, lam, d, oy, ox, propmode):
    """ol::shiftedProp, golprop.h:755-768: ASM or Fresnel (s = 1) on device fields."""
    if int(propmode) == PROPMODE.ASM:
        return gshiftedAsmProp(usrc, udst, ny, nx, dy, dx, lam, d, oy, ox)
    if int(propmode) == PROPMODE.FRESNEL:
        return gshiftedFresnelProp(usrc, udst, ny, nx, dy, dx, lam, d, 1.0, oy, ox)
    raise ValueError("shiftedProp takes PROPMODE.ASM or PROPMODE.FRESNEL")


def _host_c64(u, ny, nx):
    return torch.from_numpy(np.ascontiguousarray(np.asarray(u).reshape(ny, nx), np.complex64)).cuda()


def _write_host(u, d):
    u[...] = d.cpu().numpy().reshape(u.shape).astype(u.dtype, copy=False)
    return u


def shiftedAsmProp(usrc, udst, height, width, dy, dx, lam, z, oy, ox):
    """ol::shiftedAsmProp, olprop.h:307-327, on host arrays: the band window of
    shiftedAsmTransferF (olprop.h:251-305) and 1/Np twice."""
    d = _host_c64(usrc, height, width)
    o = torch.empty_like(d)
    shifted_asm_prop(d, o, dy=dy, dx=dx, lam=lam, z=z, oy=oy, ox=ox, bandlimit=True)
    return _write_host(udst, o / (4.0 * height * width))


def shiftedFresnelProp(u, height, width, dy, dx, lam, z, s, oy, ox):
    """ol::shiftedFresnelProp, olprop.h:338-406, in place on a host array (its
    normalisation carries one more 1/Np than the device version)."""
    d = _host_c64(u, height, width)
    shifted_fresnel_prop(d, dy=dy, dx=dx, lam=lam, z=z, s=s, oy=oy, ox=ox)
    return _write_host(u, d / (4.0 * height * width))


def splitAsmProp(u, height, width, dy, dx, lam, z, blocknum_y=2, blocknum_x=2):
    """ol::splitAsmProp, olprop.h:618-654, in place on a host array: per-block
    shiftedAsmProp (band window decided in float -- the template's only
    instantiation is PREC_T = float -- and 1/Np_block twice)."""
    d = _host_c64(u, height, width)
    o = torch.empty_like(d)
    split_prop(d, o, dy=dy, dx=dx, lam=lam, z=z, propmode=PROPMODE.ASM, blocks_y=blocknum_y, blocks_x=blocknum_x,
               bandlimit=True, window_f32=True)
    nb = 4.0 * (height // blocknum_y) * (width // blocknum_x)
    return _write_host(u, o / nb)


def gsplitProp(u, height, width, dy, dx, lam, z, propmode, blocknum_y=2, blocknum_x=2):
    """ol::gsplitProp, golprop.h:772-813: a host field, each block pair through
    the device shiftedProp (no band window)."""
    d = _host_c64(u, height, width)
    o = torch.empty_like(d)
    split_prop(d, o, dy=dy, dx=dx, lam=lam, z=z, propmode=propmode, blocks_y=blocknum_y, blocks_x=blocknum_x)
    return _write_host(u, o)


# ------------------------------------------------------------------ tilted
class INTERPOLATION(IntEnum):
    """ol::INTERPOLATION (olprop.h:408-410)."""

    BILINEAR = 0
    BICUBIC = 1


BILINEAR, BICUBIC = INTERPOLATION.BILINEAR, INTERPOLATION.BICUBIC


def tilted_workspace(ny, nx, device="cuda"):
    n = int(lib().olg_tilted_workspace_bytes(ny, nx))
    return torch.empty(n, dtype=torch.uint8, device=device)


def tilted_prop(u_in, u_out=None, *, dy, dx, lam, z, angle, interp=INTERPOLATION.BILINEAR, propmode=PROPMODE.ASM,
                reference=False, stream=None, work=None):
    """Tilted-plane propagation (olg_tilted_prop_c64) on device fields.

    ``reference=False`` is TiltedSourceProp (the destination plane rotated by
    ``angle`` about y as seen from the source); ``reference=True`` is
    TiltedReferenceProp (propagate, then resample for a plane rotated by
    ``angle``).  ``interp`` BILINEAR / BICUBIC, ``propmode`` ASM / FRESNEL."""
    ny, nx = u_in.shape
    _dev_field(u_in, ny, nx, "u_in")
    u_out = u_in if u_out is None else _dev_field(u_out, ny, nx, "u_out")
    if int(propmode) not in (PROPMODE.ASM, PROPMODE.FRESNEL):
        raise ValueError("tilted propagation takes PROPMODE.ASM or PROPMODE.FRESNEL")
    wp, wb = _work(work)
    call("olg_tilted_prop_c64", u_in.data_ptr(), u_out.data_ptr(), ny, nx, float(dy), float(dx), float(lam),
         float(z), float(angle), int(interp), int(propmode), 1 if reference else 0, wp, wb, _stream(stream))
    return u_out


def _tilted_mirror(u, ny, nx, dy, dx, lam, z, angle, inp, propmode, reference):
    if _is_host(u):
        d = _host_c64(u, ny, nx)
        tilted_prop(d, dy=dy, dx=dx, lam=lam, z=z, angle=angle, interp=inp, propmode=propmode, reference=reference)
        return _write_host(u, d)
    d = _dev_field(u, ny, nx).view(ny, nx)
    tilted_prop(d, dy=dy, dx=dx, lam=lam, z=z, angle=angle, interp=inp, propmode=propmode, reference=reference)
    return u


def TiltedSourceProp(u, ny, nx, dy, dx, lam, z, angle_src2dst, inp=INTERPOLATION.BILINEAR, propmode=PROPMODE.ASM):
    """ol::TiltedSourceProp, olprop.h:414-521, in place (host array or device tensor)."""
    return _tilted_mirror(u, ny, nx, dy, dx, lam, z, angle_src2dst, inp, propmode, False)


def TiltedReferenceProp(u, ny, nx, dy, dx, lam, z, rotate, inp=INTERPOLATION.BILINEAR, propmode=PROPMODE.ASM):
    """ol::TiltedReferenceProp, olprop.h:523-600, in place (host array or device tensor)."""
    return _tilted_mirror(u, ny, nx, dy, dx, lam, z, rotate, inp, propmode, True)


# ------------------------------------------------------------------ autotuner
def autotune(ny, nx, reps=5, stream=None):
    """Time every launch variant of the three passes for an ny x nx field and keep
    the fastest (olg_autotune_prop).  Returns {(kind, n): variant}."""
    call("olg_autotune_prop", int(ny), int(nx), int(reps), _stream(stream))
    return {(k, n): int(lib().olg_prop_get_variant(k, n)) for k, n in ((0, 2 * nx), (1, 2 * ny), (2, 2 * nx))}


def set_variant(kind, n, idx):
    call("olg_prop_set_variant", int(kind), int(n), int(idx))


def get_variant(kind, n):
    return int(lib().olg_prop_get_variant(int(kind), int(n)))


def variant_count():
    return int(lib().olg_prop_variant_count())
