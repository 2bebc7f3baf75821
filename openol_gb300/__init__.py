"""openol_gb300 -- GB300-native (sm_103a) engine for OpenOL's propagation and
hologram hot path, behind the reference's own API names.

The compute lives in libolgb300.so (C-ABI: include/olgb300.h).  This package is
the host-side mirror of the reference's golprop.h / golcgh.h / olimg.h calls,
with PyTorch CUDA tensors standing in for the reference's device buffers.
"""
from ._lib import OlgError, launch_count, lib  # noqa: F401
from .cgh import (Cgh, Object2cuda, autotune_cgh_gemm, WRPMethod, WRPMethod_D, WRPStep1, WRPStep1_D, WRPStep2,  # noqa: F401
                  cgh_adjoint_gemm_workspace, cgh_exact, cgh_exact_adjoint, cgh_fresnel, cgh_fresnel_adjoint, cgh_fresnel_adjoint_gemm, cgh_fresnel_gemm, cgh_fresnel_gemm_host, cgh_gemm_pairs, cgh_gemm_workspace, device_fault_check, gCgh, gCghReduction, gObject, wrp_plane_z)
from .img import MODE, binarize, complex2img  # noqa: F401
from .objects import (OBJSET_MODE, ZMIDDLE, ZMIN, bmpread, bmpwrite, objinfo, objread, objset, objsort,  # noqa: F401
                      objwrite_3d)
from .batch import BatchPlan, PropPlan, config5_fields, direct_pixels as batch_direct_pixels  # noqa: F401
from .optim import PhaseOptimizer, make_targets, phase_loss_grad  # noqa: F401
from .prop import (ASM, AUTO, FRESNEL, PROPMODE, ARSSFresnelProp, AsmProp, AsmPropCheck, FresnelProp,
                   FresnelPropBandLimit, FresnelPropCheck, PropHost,  # noqa: F401
                   Prop, arss_prop, asm_prop, fresnel_prop, gAsmProp, gFresnelProp, gFresnelPropBandLimit,
                   autotune, get_variant, set_variant, variant_count, workspace, workspace_bytes,
                   gshiftedAsmProp, gshiftedFresnelProp, gsplitProp, shiftedAsmProp, shiftedFresnelProp, shiftedProp,
                   shifted_asm_prop, shifted_fresnel_prop, split_prop, split_workspace, splitAsmProp,
                   BICUBIC, BILINEAR, INTERPOLATION, TiltedReferenceProp, TiltedSourceProp, tilted_prop,
                   tilted_workspace)

__version__ = "0.1.0"
