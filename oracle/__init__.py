"""CPU oracle for the OpenOL propagation / CGH / WRP path.

TEST INFRASTRUCTURE ONLY.  Only ``tests/``, ``__graft_entry__.smoke()`` and
``bench.py``'s CPU-baseline legs import this package, and only as the checker
or as the timed CPU baseline.  The GPU product (``openol_gb300``) never imports
it.

Two libraries are wrapped here:

* ``libolcpu.so`` -- the project's FP64 C restatement (``olcpu.c``) of the
  reference functions, each citing the reference file:line it follows.  It is
  built from this directory by ``make`` on any machine.
* ``_ref/libolref.so`` -- the reference's OWN CPU templates (``olprop.h``,
  ``olcgh.h``, ``olimg.h``) compiled unmodified with a project-written FFTW
  shim.  It exists only where the reference sources are present; it pins the
  restatement and generates ``tests/golden``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_CPU = None
_REF = None

_d = C.c_double
_f = C.c_float
_l = C.c_long
_i = C.c_int
_p = C.c_void_p


def build(ref: bool = False) -> None:
    """Compile libolcpu.so.  With ``ref``, also the reference's own CPU build
    and a staged copy of its headers for the GPU harness (both only where the
    reference tree is present; the recipe skips them elsewhere)."""
    subprocess.run(["make", "-s", "-C", HERE, "libolcpu.so"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)
        subprocess.run(["make", "-s", "-C", HERE, "ref-gpu-src"], check=False,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)


def _ptr(a):
    return a.ctypes.data_as(_p) if a is not None else None


def cpu():
    global _CPU
    if _CPU is None:
        path = os.path.join(HERE, "libolcpu.so")
        if not os.path.exists(path):
            build()
        lib = C.CDLL(path)
        lib.olc_asm_prop.argtypes = [_p, _l, _l, _d, _d, _d, _d, _i]
        lib.olc_fresnel_prop.argtypes = [_p, _l, _l, _d, _d, _d, _d, _i, _i]
        lib.olc_arss_prop.argtypes = [_p, _p, _l, _l, _d, _d, _d, _d, _d, _d, _d, _i]
        lib.olc_arss_prop.restype = _i
        lib.olc_arss_windows.argtypes = [_l, _l, _d, _d, _d, _d, _d, _p]
        lib.olc_arss_windows.restype = _i
        lib.olc_shifted_asm_prop.argtypes = [_p, _p, _l, _l, _d, _d, _d, _d, _d, _d, _i]
        lib.olc_split_prop.argtypes = [_p, _p, _l, _l, _d, _d, _d, _d, _i, _i, _i, _i]
        lib.olc_split_prop.restype = _i
        lib.olc_asm_prop_check.argtypes = [_l, _l, _d, _d, _d, _d]
        lib.olc_fresnel_prop_check.argtypes = [_l, _l, _d, _d, _d, _d]
        lib.olc_cgh_fresnel.argtypes = [_p, _p, _p, _l, _p, _p, _l, _l, _d, _d, _d, _i]
        lib.olc_cgh_exact.argtypes = [_p, _p, _p, _l, _p, _l, _l, _d, _d, _d, _i]
        lib.olc_cgh_fresnel_adjoint.argtypes = [_p, _l, _p, _p, _l, _l, _d, _d, _d]
        lib.olc_cgh_exact_adjoint.argtypes = [_p, _l, _p, _p, _l, _l, _d, _d, _d]
        lib.olc_wrp_step1.argtypes = [_p, _l, _p, _l, _l, _f, _f, _f, _f, _i]
        lib.olc_wrp_radius.argtypes = [_p, _l, _p, _f, _f, _f, _i]
        lib.olc_complex2img.argtypes = [_p, _p, _l, _l, _i]
        lib.olc_quant8bit.argtypes = [_p, _p, _l, _l]
        lib.olc_binarize.argtypes = [_p, _p, _l, _l]
        lib.olc_fft2d.argtypes = [_p, _l, _l, _i, _i]
        lib.olc_tilted_prop.argtypes = [_p, _l, _l, _d, _d, _d, _d, _d, _i, _i, _i]
        _CPU = lib
    return _CPU


def ref_available() -> bool:
    return os.path.exists(os.path.join(HERE, "_ref", "libolref.so"))


def ref():
    """The reference's own CPU code (only where it was built from its sources)."""
    global _REF
    if _REF is None:
        lib = C.CDLL(os.path.join(HERE, "_ref", "libolref.so"))
        for nm in ("ref_asm_prop", "ref_fresnel_prop", "ref_fresnel_prop_bandlimit"):
            getattr(lib, nm).argtypes = [_p, _i, _i, _d, _d, _d, _d]
        lib.ref_prop.argtypes = [_p, _i, _i, _d, _d, _d, _d, _i]
        lib.ref_asm_prop_check.argtypes = [_i, _i, _d, _d, _d, _d]
        lib.ref_asm_prop_check_f.argtypes = [_i, _i, _f, _f, _f, _f]
        lib.ref_fresnel_prop_check.argtypes = [_i, _i, _d, _d, _d, _d]
        lib.ref_fresnel_prop_check_f.argtypes = [_i, _i, _f, _f, _f, _f]
        lib.ref_cgh.argtypes = [_p, _i, _p, _i, _i, _d, _d, _d]
        lib.ref_cgh_phase.argtypes = [_p, _i, _p, _i, _i, _d, _d]
        lib.ref_complex2img.argtypes = [_p, _p, _i, _i, _i]
        lib.ref_quant8bit.argtypes = [_p, _p, _i, _i]
        lib.ref_shifted_asm_prop.argtypes = [_p, _p, _i, _i, _d, _d, _d, _d, _d, _d]
        lib.ref_shifted_fresnel_prop.argtypes = [_p, _i, _i, _d, _d, _d, _d, _d, _d, _d]
        lib.ref_split_asm_prop.argtypes = [_p, _i, _i, _d, _d, _d, _d, _i, _i]
        lib.ref_objread.argtypes = [C.c_char_p, _p, _i]
        lib.ref_objread.restype = _i
        lib.ref_objread_scaled.argtypes = [C.c_char_p, _f, _f, _f, _f, _p, _i]
        lib.ref_objread_scaled.restype = _i
        lib.ref_objset.argtypes = [_p, _i, _f, _f, _f, _f, _f, _i]
        lib.ref_objsort.argtypes = [_p, _i]
        lib.ref_bmpwrite.argtypes = [C.c_char_p, _p, _i, _i]
        lib.ref_tilted_prop.argtypes = [_p, _i, _i, _d, _d, _d, _d, _d, _i, _i, _i]
        _REF = lib
    return _REF


def _c128(u):
    return np.ascontiguousarray(u, dtype=np.complex128)


# --------------------------------------------------------------- propagation
def asm_prop(u, dy, dx, lam, z, flags=0):
    u = _c128(u).copy()
    cpu().olc_asm_prop(_ptr(u), u.shape[0], u.shape[1], dy, dx, lam, z, flags)
    return u


def fresnel_prop(u, dy, dx, lam, z, bandlimit=0, flags=0):
    u = _c128(u).copy()
    cpu().olc_fresnel_prop(_ptr(u), u.shape[0], u.shape[1], dy, dx, lam, z, bandlimit, flags)
    return u


def arss_prop(u, dy, dx, lam, z, s, oy=0.0, ox=0.0, flags=0):
    u = _c128(u)
    out = np.empty_like(u)
    rc = cpu().olc_arss_prop(_ptr(u), _ptr(out), u.shape[0], u.shape[1], dy, dx, lam, z, s, oy, ox, flags)
    if rc != 0:
        raise ValueError("ARSS undefined for s in {0, 1}")
    return out


OLC_BANDLIMIT = 0x40
OLC_NO_WINDOWS = 0x80


def shifted_asm_prop(u, dy, dx, lam, z, oy, ox, flags=0):
    """Shifted ASM (golprop.h:537-575); flags may add OLC_BANDLIMIT (olprop.h:251-305)."""
    u = _c128(u)
    out = np.empty_like(u)
    cpu().olc_shifted_asm_prop(_ptr(u), _ptr(out), u.shape[0], u.shape[1], dy, dx, lam, z, oy, ox, flags)
    return out


def shifted_fresnel_prop(u, dy, dx, lam, z, s, oy=0.0, ox=0.0, flags=0):
    """Shifted Fresnel (golprop.h:606-752): the ARSS chirps without windows."""
    return arss_prop(u, dy, dx, lam, z, s, oy, ox, flags | OLC_NO_WINDOWS)


def split_prop(u, dy, dx, lam, z, mode, blocks_y=2, blocks_x=2, flags=0):
    """Split propagation (golprop.h:772-813); mode 0 ASM, 1 Fresnel (s = 1)."""
    u = _c128(u)
    out = np.zeros_like(u)
    if cpu().olc_split_prop(_ptr(u), _ptr(out), u.shape[0], u.shape[1], dy, dx, lam, z, mode, blocks_y, blocks_x,
                            flags) != 0:
        raise ValueError("bad split arguments")
    return out


def tilted_prop(u, dy, dx, lam, z, angle, interp=0, mode=0, reference=False, use_ref=False):
    """Tilted-plane propagation: TiltedSourceProp (olprop.h:414-521) or, with
    ``reference``, TiltedReferenceProp (olprop.h:523-600); interp 0 bilinear /
    1 bicubic, mode 0 ASM / 1 Fresnel.  ``use_ref`` runs the reference's own
    build instead of the restatement."""
    u = _c128(u).copy()
    fn = ref().ref_tilted_prop if use_ref else cpu().olc_tilted_prop
    fn(_ptr(u), u.shape[0], u.shape[1], dy, dx, lam, z, angle, interp, mode, int(bool(reference)))
    return u


def arss_windows(ny, nx, dy, dx, lam, z, s):
    out = np.zeros(6, np.int64)
    if cpu().olc_arss_windows(ny, nx, dy, dx, lam, z, s, _ptr(out)) != 0:
        raise ValueError("ARSS undefined for s in {0, 1}")
    return out


def asm_prop_check(ny, nx, dy, dx, lam, z):
    return bool(cpu().olc_asm_prop_check(ny, nx, dy, dx, lam, z))


def fresnel_prop_check(ny, nx, dy, dx, lam, z):
    return bool(cpu().olc_fresnel_prop_check(ny, nx, dy, dx, lam, z))


def prop(u, dy, dx, lam, z, mode=2):
    """CPU dispatcher olprop.h:656-682 (mode: 0 ASM, 1 FRESNEL, 2 AUTO)."""
    ny, nx = u.shape
    if mode == 1:
        return fresnel_prop(u, dy, dx, lam, z)
    if mode == 0 or asm_prop_check(ny, nx, dy, dx, lam, z):
        return asm_prop(u, dy, dx, lam, z)
    if not fresnel_prop_check(ny, nx, dy, dx, lam, z):
        return fresnel_prop(u, dy, dx, lam, z, bandlimit=2)
    return fresnel_prop(u, dy, dx, lam, z)


def fft2(u, sign=-1):
    u = _c128(u).copy()
    cpu().olc_fft2d(_ptr(u), u.shape[0], u.shape[1], sign, 0)
    return u


# ----------------------------------------------------------------------- CGH
def _pts(p):
    return np.ascontiguousarray(p, dtype=np.float64).reshape(-1, 3)


def cgh_fresnel(pts, ny, nx, py, px, lam, amp=None, phase0=None, U=None, flags=0, want_phase=False):
    pts = _pts(pts)
    U = np.zeros((ny, nx), np.complex128) if U is None else _c128(U).copy()
    amp = None if amp is None else np.ascontiguousarray(amp, np.float64)
    phase0 = None if phase0 is None else np.ascontiguousarray(phase0, np.float64)
    ph = np.zeros((ny, nx), np.float64) if want_phase else None
    cpu().olc_cgh_fresnel(_ptr(pts), _ptr(amp), _ptr(phase0), pts.shape[0], _ptr(U), _ptr(ph),
                          ny, nx, py, px, lam, flags)
    return (U, ph) if want_phase else U


def cgh_exact(pts, ny, nx, py, px, lam, amp=None, phase0=None, U=None, flags=0):
    pts = _pts(pts)
    U = np.zeros((ny, nx), np.complex128) if U is None else _c128(U).copy()
    amp = None if amp is None else np.ascontiguousarray(amp, np.float64)
    phase0 = None if phase0 is None else np.ascontiguousarray(phase0, np.float64)
    cpu().olc_cgh_exact(_ptr(pts), _ptr(amp), _ptr(phase0), pts.shape[0], _ptr(U), ny, nx, py, px, lam, flags)
    return U


def cgh_fresnel_adjoint(pts, G, py, px, lam):
    pts = _pts(pts)
    G = _c128(G)
    g = np.zeros(pts.shape[0], np.complex128)
    cpu().olc_cgh_fresnel_adjoint(_ptr(pts), pts.shape[0], _ptr(G), _ptr(g), G.shape[0], G.shape[1], py, px, lam)
    return g


def cgh_exact_adjoint(pts, G, py, px, lam):
    pts = _pts(pts)
    G = _c128(G)
    g = np.zeros(pts.shape[0], np.complex128)
    cpu().olc_cgh_exact_adjoint(_ptr(pts), pts.shape[0], _ptr(G), _ptr(g), G.shape[0], G.shape[1], py, px, lam)
    return g


# ----------------------------------------------------------------------- WRP
def wrp_step1(pts, ny, nx, p, lam, plane_z, plimit=None, window=0):
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    U = np.zeros((ny, nx), np.complex128)
    cpu().olc_wrp_step1(_ptr(pts), pts.shape[0], _ptr(U), ny, nx, p, lam, plane_z,
                        p if plimit is None else plimit, window)
    return U


def wrp_radius(pts, plimit, lam, plane_z, window=0):
    pts = np.ascontiguousarray(pts, np.float32).reshape(-1, 3)
    W = np.zeros(pts.shape[0], np.float32)
    cpu().olc_wrp_radius(_ptr(pts), pts.shape[0], _ptr(W), plimit, lam, plane_z, window)
    return W


# ---------------------------------------------------------------- quantisers
def complex2img(u, mode):
    u = _c128(u)
    img = np.zeros(u.shape, np.uint8)
    cpu().olc_complex2img(_ptr(u), _ptr(img), u.shape[0], u.shape[1], mode)
    return img


def quant8bit(real):
    real = np.ascontiguousarray(real, np.float64)
    img = np.zeros(real.shape, np.uint8)
    cpu().olc_quant8bit(_ptr(real), _ptr(img), real.shape[0], real.shape[1])
    return img


def binarize(u):
    u = _c128(u)
    img = np.zeros(u.shape, np.uint8)
    cpu().olc_binarize(_ptr(u), _ptr(img), u.shape[0], u.shape[1])
    return img


# ------------------------------------------------------ phase optimisation
def phase_loss_grad(phi, targets, zs, p, lam):
    """FP64 loss sum_p mean((|ASM_z(e^{i phi})|^2 - t_p)^2) and dL/dphi, by the
    adjoint (conj transfer function) of the FP64 ASM restatement."""
    u = np.exp(1j * np.asarray(phi, np.float64))
    n = u.size
    L = 0.0
    g = np.zeros_like(u)
    for t, z in zip(targets, zs):
        v = asm_prop(u, p, p, lam, z)
        r = np.abs(v) ** 2 - np.asarray(t, np.float64)
        L += float(np.mean(r * r))
        g += asm_prop(2.0 * r * v / n, p, p, lam, z, flags=1)
    return L, -2.0 * np.imag(u * np.conj(g))


def phase_loss(phi, targets, zs, p, lam):
    u = np.exp(1j * np.asarray(phi, np.float64))
    L = 0.0
    for t, z in zip(targets, zs):
        v = asm_prop(u, p, p, lam, z)
        r = np.abs(v) ** 2 - np.asarray(t, np.float64)
        L += float(np.mean(r * r))
    return L
