"""8-bit quantisers: the Python mirror of olimg.h's complex2img (olimg.h:348-391)."""
from __future__ import annotations

from enum import IntEnum

import torch

from ._lib import call
from .prop import _dev_field, _stream


class MODE(IntEnum):
    """ol::MODE (olimg.h:268)."""

    PHASE = 0
    REAL = 1
    IMAG = 2
    AMP = 3


def complex2img(u, ny, nx, mode=MODE.PHASE, img=None):
    """ol::complex2img(u, img, ny, nx, MODE): uint8 CUDA tensor (ny, nx)."""
    _dev_field(u, ny, nx)
    img = torch.empty((ny, nx), dtype=torch.uint8, device=u.device) if img is None else img
    call("olg_complex2img_u8", u.data_ptr(), img.data_ptr(), ny, nx, int(mode), _stream())
    return img


def binarize(u, ny, nx, img=None):
    """Binarised 8-bit hologram (project rule): 255 where Re(U) >= 0, else 0."""
    _dev_field(u, ny, nx)
    img = torch.empty((ny, nx), dtype=torch.uint8, device=u.device) if img is None else img
    call("olg_binarize_u8", u.data_ptr(), img.data_ptr(), ny, nx, _stream())
    return img
