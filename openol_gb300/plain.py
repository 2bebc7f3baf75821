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


def plain_fresnel_prop(u_in, u_out, *, dy, dx, lam, z, stream=None):
    ny, nx = u_in.shape
    _dev_field(u_in, ny, nx, "u_in")
    _dev_field(u_out, ny, nx, "u_out")
    call("olg_plain_fresnel_prop_c64", u_in.data_ptr(), u_out.data_ptr(), ny, nx, float(dy), float(dx), float(lam),
         float(z), _stream(stream))
    return u_out


def plain_arss_prop(u_src, u_dst, *, dy, dx, lam, z, s, oy=0.0, ox=0.0, stream=None):
    ny, nx = u_src.shape
    _dev_field(u_src, ny, nx, "u_src")
    _dev_field(u_dst, ny, nx, "u_dst")
    call("olg_plain_arss_prop_c64", u_src.data_ptr(), u_dst.data_ptr(), ny, nx, float(dy), float(dx), float(lam),
         float(z), float(s), float(oy), float(ox), _stream(stream))
    return u_dst


def plain_prop(f, stream=None):
    """One batch field (config5_fields entry) through its plain form."""
    kw = dict(dy=f["dy"], dx=f["dx"], lam=f["lam"], z=f["z"], stream=stream)
    if f["method"] == "asm":
        return plain_asm_prop(f["u_in"], f["u_out"], **kw)
    if f["method"] == "fresnel":
        return plain_fresnel_prop(f["u_in"], f["u_out"], **kw)
    return plain_arss_prop(f["u_in"], f["u_out"], s=f["s"], **kw)


def plain_cgh_fresnel(gobj, U, *, ny, nx, p, lam, stream=None):
    _dev_field(U, ny, nx, "U")
    call("olg_plain_cgh_fresnel_c64", gobj.points.data_ptr(), gobj.size, U.data_ptr(), ny, nx, float(p), float(lam),
         _stream(stream))
    return U
