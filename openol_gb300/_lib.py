"""ctypes binding of libolgb300.so (the C-ABI declared in include/olgb300.h).

The library is the product: there is no CPU fallback.  Importing a routine
whose library is missing raises immediately, and every non-zero status of the
C-ABI is raised as ``OlgError`` (the analogue of the reference's
``CHECK_CUDA_ERROR`` throwing ``std::runtime_error``, golclass.h:9-21).
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libolgb300.so")

OLG_OK = 0
OLG_CONJ = 0x1
OLG_NO_NORMALIZE = 0x2
OLG_ACCUMULATE = 0x4
OLG_VERBOSE = 0x8
OLG_CHECK_F32 = 0x10
OLG_REUSE_OPERANDS = 0x20
OLG_BANDLIMIT = 0x40

_d, _f, _i, _p, _sz = C.c_double, C.c_float, C.c_int, C.c_void_p, C.c_size_t

class OlgField(C.Structure):
    """olg_field (include/olgb300.h)."""
    _fields_ = [("in_", C.c_void_p), ("out", C.c_void_p), ("ny", C.c_int), ("nx", C.c_int), ("method", C.c_int),
                ("flags", C.c_int), ("dy", C.c_double), ("dx", C.c_double), ("lam", C.c_double), ("z", C.c_double),
                ("s", C.c_double), ("oy", C.c_double), ("ox", C.c_double)]


# name -> (restype, argtypes)
SIGNATURES = {
    "olg_version": (_i, []),
    "olg_status_string": (C.c_char_p, [_i]),
    "olg_last_error": (C.c_char_p, []),
    "olg_launch_count": (C.c_ulonglong, []),
    "olg_host_device_pointer": (_i, [_p, C.POINTER(_p)]),
    "olg_prop_workspace_bytes": (_sz, [_i, _i]),
    "olg_asm_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _i, _p, _sz, _p]),
    "olg_shifted_asm_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _d, _d, _i, _p, _sz, _p]),
    "olg_shifted_fresnel_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _d, _d, _d, _i, _p, _sz, _p]),
    "olg_shifted_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _d, _d, _i, _i, _p, _sz, _p]),
    "olg_split_prop_workspace_bytes": (_sz, [_i, _i, _i, _i]),
    "olg_split_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _i, _i, _i, _i, _p, _sz, _p]),
    "olg_asm_prop_noalloc_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _i, _p]),
    "olg_tilted_workspace_bytes": (_sz, [_i, _i]),
    "olg_cgh_gemm_tail_weight": (_d, [_d]),
    "olg_cgh_gemm_pairs": (_i, [_i]),
    "olg_cgh_gemm_chunk": (_i, [_i]),
    "olg_tilted_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _d, _i, _i, _i, _p, _sz, _p]),
    "olg_fresnel_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _i, _i, _p, _sz, _p]),
    "olg_arss_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _d, _d, _d, _i, _p, _sz, _p]),
    "olg_autotune_prop": (_i, [_i, _i, _i, _p]),
    "olg_prop_variant_count": (_i, []),
    "olg_prop_get_variant": (_i, [_i, _i]),
    "olg_prop_set_variant": (_i, [_i, _i, _i]),
    "olg_asm_prop_check": (_i, [_i, _i, _d, _d, _d, _d, _i]),
    "olg_fresnel_prop_check": (_i, [_i, _i, _d, _d, _d, _d, _i]),
    "olg_prop_c64": (_i, [_p, _i, _i, _d, _d, _d, _d, _i, _i, C.POINTER(_i), _p, _sz, _p]),
    "olg_batch_plan_create": (_i, [C.POINTER(OlgField), _i, C.POINTER(_p)]),
    "olg_batch_direct_pixels": (C.c_longlong, [C.c_longlong]),
    "olg_batch_plan_direct_fields": (_i, [_p]),
    "olg_batch_execute": (_i, [_p, _p]),
    "olg_batch_execute_serial": (_i, [_p, _p]),
    "olg_batch_execute_host": (_i, [_p, _p, _p, _p]),
    "olg_prop_plan_create": (_i, [_p, _p]),
    "olg_prop_plan_execute": (_i, [_p, _p, _p, _p]),
    "olg_prop_plan_execute_host": (_i, [_p, _p, _p, _i, _p]),
    "olg_prop_plan_destroy": (_i, [_p]),
    "olg_batch_check": (_i, [_p]),
    "olg_batch_plan_items": (_i, [_p]),
    "olg_batch_plan_destroy": (_i, [_p]),
    "olg_phase_opt_workspace_bytes": (_sz, [_i, _i]),
    "olg_phase_loss_grad": (_i, [_p, _p, C.POINTER(_d), _i, _i, _i, _d, _d, _d, _p, _p, _p, _sz, _p]),
    "olg_phase_adam_step": (_i, [_p, _p, _p, _p, C.POINTER(_d), _i, _i, _i, _d, _d, _d, _d, _d, _d, _d, _i, _p, _p,
                                 _sz, _p]),
    "olg_cgh_fresnel_c64": (_i, [_p, _p, _p, _i, _p, _p, _i, _i, _d, _d, _d, _i, _p]),
    "olg_cgh_exact_c64": (_i, [_p, _p, _p, _i, _p, _i, _i, _d, _d, _d, _i, _p]),
    "olg_cgh_adjoint_workspace_bytes": (_sz, [_i, _i, _i, _i]),
    "olg_wait_budget_cycles": (C.c_longlong, [C.c_longlong]),
    "olg_autotune_cgh_gemm": (_i, [_i, _i, _i, _i, _p]),
    "olg_inject_alloc_failures": (_i, [_i]),
    "olg_batch_plan_raise_target": (_i, [_p, _i, _i, _i]),
    "olg_cgh_fresnel_adjoint_c64": (_i, [_p, _i, _p, _p, _i, _i, _d, _d, _d, _i, _p, _sz, _p]),
    "olg_cgh_fresnel_adjoint_gemm_c64": (_i, [_p, _i, _p, _p, _i, _i, _d, _d, _d, _i, _p, _sz, _p]),
    "olg_cgh_adjoint_gemm_workspace_bytes": (_sz, [_i, _i, _i]),
    "olg_cgh_exact_adjoint_c64": (_i, [_p, _i, _p, _p, _i, _i, _d, _d, _d, _i, _p, _sz, _p]),
    "olg_cgh_gemm_workspace_bytes": (_sz, [_i, _i, _i]),
    "olg_cgh_fresnel_gemm_c64": (_i, [_p, _p, _p, _i, _p, _i, _i, _d, _d, _d, _i, _p, _sz, _p]),
    "olg_cgh_fresnel_gemm_host_c64": (_i, [_p, _p, _p, _p, _p, _i, _i, _i, _d, _d, _d, _i, _p]),
    "olg_device_fault_check": (_i, [_i]),
    "olg_wrp_plane_z": (_f, [_i, _i, _i, _f, _f, _f, _f, _f]),
    "olg_wrp_step1_c64": (_i, [_p, _i, _p, _i, _i, _f, _f, _f, _f, _i, _p]),
    "olg_wrp_method_c64": (_i, [_p, _i, _p, _i, _i, _f, _f, _f, _f, _f, _i, _i, _i, C.POINTER(_f), _p]),
    "olg_obj_minmax_f32": (_i, [_p, _i, _p, _p]),
    "olg_objset_f32": (_i, [_p, _i, _f, _f, _p, _i, _i, _p]),
    "olg_objsort_workspace_bytes": (_sz, [_i]),
    "olg_objsort_f32": (_i, [_p, _i, _p, _sz, _p]),
    "olg_objread": (_i, [C.c_char_p, _p, _i, C.POINTER(_i)]),
    "olg_objread_scaled": (_i, [C.c_char_p, _p, _f, _p, _i, C.POINTER(_i)]),
    "olg_bmpwrite_u8": (_i, [C.c_char_p, _p, _i, _i]),
    "olg_bmpread_u8": (_i, [C.c_char_p, _p, _i, _i]),
    "olg_plain_asm_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _p]),
    "olg_plain_fresnel_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _p]),
    "olg_plain_arss_prop_c64": (_i, [_p, _p, _i, _i, _d, _d, _d, _d, _d, _d, _d, _p]),
    "olg_plain_cgh_fresnel_c64": (_i, [_p, _i, _p, _i, _i, _d, _d, _p]),
    "olg_complex2img_u8": (_i, [_p, _p, _i, _i, _i, _p]),
    "olg_binarize_u8": (_i, [_p, _p, _i, _i, _p]),
}


class OlgError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        super().__init__(f"{where}: status {status}: {msg}")
        self.status = status


_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is not built; run `python -c 'import __graft_entry__ as g; g.build()'`")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(status: int, where: str) -> None:
    if status != OLG_OK:
        L = lib()
        raise OlgError(status, where, (L.olg_last_error() or b"").decode() or L.olg_status_string(status).decode())


def call(name: str, *args):
    fn = getattr(lib(), name)
    rc = fn(*args)
    check(rc, name)
    return rc


def launch_count() -> int:
    return int(lib().olg_launch_count())
