"""Point clouds and image files around the hologram path: the Python mirror of
the reference's olobject.h (objread, objinfo, objset, objsort) and of its 8-bit
BMP reader and writer (olimg.h).  objinfo / objset / objsort run on the GPU on
a gObject's device points; the file formats are read and written on the host,
byte for byte as the reference does."""
from __future__ import annotations

import ctypes as C
from enum import IntEnum

import numpy as np
import torch

from ._lib import OLG_VERBOSE, call, lib
from .cgh import gObject
from .prop import _stream


class OBJSET_MODE(IntEnum):
    """ol::OBJSET_MODE (olobject.h:192-194)."""

    ZMIN = 0
    ZMIDDLE = 1


ZMIN, ZMIDDLE = OBJSET_MODE.ZMIN, OBJSET_MODE.ZMIDDLE


def _path(p) -> bytes:
    return str(p).encode()


def objread(path, offset=None, scale=None) -> np.ndarray:
    """ol::objread (olobject.h:79-161): the (N, 3) float32 points of a .3d
    (int32) or .3df (float) file.  With ``offset`` and ``scale`` (the scaled
    form, int32 records): p = xint * scale + offset in float."""
    n = C.c_int(0)
    if offset is None:
        call("olg_objread", _path(path), None, 0, C.byref(n))
        out = np.zeros((n.value, 3), np.float32)
        call("olg_objread", _path(path), out.ctypes.data, n.value, C.byref(n))
    else:
        off = np.ascontiguousarray(offset, np.float32).reshape(3)
        sc = 1.0 if scale is None else float(scale)
        call("olg_objread_scaled", _path(path), off.ctypes.data, sc, None, 0, C.byref(n))
        out = np.zeros((n.value, 3), np.float32)
        call("olg_objread_scaled", _path(path), off.ctypes.data, sc, out.ctypes.data, n.value, C.byref(n))
    return out


def objwrite_3d(path, points) -> None:
    """Write a .3d file (int32 count, then int32 x, y, z per point), the format objread takes."""
    p = np.asarray(points).reshape(-1, 3)
    with open(path, "wb") as f:
        f.write(np.int32(p.shape[0]).tobytes())
        f.write(np.ascontiguousarray(p, np.int32).tobytes())


def _gobj(obj) -> gObject:
    if not isinstance(obj, gObject):
        raise TypeError("objinfo / objset / objsort take a gObject (device points)")
    return obj


def objinfo(obj, verbose=True):
    """ol::objinfo (olobject.h:163-174): extents of x, y, z; prints them like the reference."""
    g = _gobj(obj)
    mm = np.zeros(6, np.float32)
    call("olg_obj_minmax_f32", g.points.data_ptr(), g.size, mm.ctypes.data, _stream())
    if verbose:
        for c, name in enumerate("xyz"):
            print(f"{name}max: {mm[3 + c]:g}  {name}min: {mm[c]:g}")
    return mm[:3].copy(), mm[3:].copy()


def objset(obj, xy_range, offset, mode=OBJSET_MODE.ZMIN, y_range=None, verbose=False):
    """ol::objset on the device, in place.  One range (olobject.h:196-230): the
    larger x/y extent is scaled to ``xy_range``; with ``y_range`` (the two-range
    form, olobject.h:232-264) the smaller of the two scales is taken.  Then the
    x/y centre and zmin (ZMIN) or the z centre (ZMIDDLE) move to ``offset``."""
    g = _gobj(obj)
    off = np.ascontiguousarray(offset, np.float32).reshape(3)
    call("olg_objset_f32", g.points.data_ptr(), g.size, float(xy_range), -1.0 if y_range is None else float(y_range),
         off.ctypes.data, int(mode), OLG_VERBOSE if verbose else 0, _stream())
    return obj


def objsort(obj, work=None):
    """ol::objsort (olobject.h:176-181) on the device: by z, largest first
    (stable: equal z keep their order)."""
    g = _gobj(obj)
    wp, wb = (work.data_ptr(), work.numel() * work.element_size()) if work is not None else (None, 0)
    call("olg_objsort_f32", g.points.data_ptr(), g.size, wp, wb, _stream())
    return obj


def objsort_workspace(n, device="cuda"):
    return torch.empty(int(lib().olg_objsort_workspace_bytes(n)), dtype=torch.uint8, device=device)


def bmpwrite(fname, img, ny, nx) -> None:
    """ol::bmpwrite (olimg.h:136-165): an 8-bit grey BMP of a host or device image."""
    a = img.cpu().numpy() if isinstance(img, torch.Tensor) else np.asarray(img)
    a = np.ascontiguousarray(a, np.uint8).reshape(ny, nx)
    call("olg_bmpwrite_u8", _path(fname), a.ctypes.data, ny, nx)


def bmpread(fname, ny, nx) -> np.ndarray:
    """ol::bmpread (olimg.h:55-99): the ny x nx bytes of an 8-bit BMP written as bmpwrite writes it."""
    out = np.zeros((ny, nx), np.uint8)
    call("olg_bmpread_u8", _path(fname), out.ctypes.data, ny, nx)
    return out
