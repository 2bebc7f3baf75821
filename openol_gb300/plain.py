"""Plain-form GPU baselines (reference-structured kernels on this GPU), for measurement."""
from __future__ import annotations

from ._lib import call
from .prop import _dev_field, _stream


def plain_asm_prop(u_in, u_out, *, dy, dx, lam, z, stream=None):
    ny, nx = u_in.shape
    _dev_field(u_in, ny, nx, "u_in")
    _dev_field(u_out, ny, nx, "u_out")
    call("olg_plain_asm_prop_c64", u_in.data_ptr(), u_out.data_ptr(), ny, nx, float(dy), float(dx), float(lam),
         float(z), _stream(stream))
    return u_out


def plain_cgh_fresnel(gobj, U, *, ny, nx, p, lam, stream=None):
    _dev_field(U, ny, nx, "U")
    call("olg_plain_cgh_fresnel_c64", gobj.points.data_ptr(), gobj.size, U.data_ptr(), ny, nx, float(p), float(lam),
         _stream(stream))
    return U
