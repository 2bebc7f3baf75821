"""GPU parity against the reference's OWN GPU code: the CUDA ARSS propagation
(olg_arss_prop_c64) and WRP step 1 (olg_wrp_step1_c64) on the inputs of
tests/golden/ref_gpu_golden.npz, whose outputs the unmodified reference
templates ARSSFresnelProp (golprop.h:941-990), WRPStep1 (golcgh.h:369-389)
and WRPStep1_D (golcgh.h:470-491) produced on a GB300.

Both sides compute in FP32, so values agree to relative L2 1e-5; the WRP
window supports (which pixels each point's window reaches) must be equal
exactly.  The same fixtures pin the FP64 oracle (tests/test_oracle_ref_gpu.py)."""
import numpy as np
import pytest
import torch

import openol_gb300 as og
from conftest import rel_l2
from test_oracle_ref_gpu import ARSS, WRP, arss_params, wrp_case

pytestmark = pytest.mark.gpu
TOL = 1e-5


@pytest.fixture(scope="module")
def gold(golden_dir):
    return np.load(golden_dir / "ref_gpu_golden.npz")


@pytest.mark.parametrize("name", ARSS)
def test_arss_matches_reference_gpu(gold, name):
    ny, nx, dy, dx, lam, z, s, oy, ox = arss_params(gold, name)
    src = torch.from_numpy(gold[name + "_in"].copy()).cuda()
    dst = torch.empty_like(src)
    og.arss_prop(src, dst, dy=dy, dx=dx, lam=lam, z=z, s=s, oy=oy, ox=ox)
    torch.cuda.synchronize()
    got = dst.cpu().numpy().astype(np.complex128)
    ref = gold[name + "_out"].astype(np.complex128)
    if s < 0:
        assert not np.any(ref) and not np.any(got)   # empty pre-chirp window
        return
    assert rel_l2(got, ref) < TOL


@pytest.mark.parametrize("name", WRP)
def test_wrp_step1_matches_reference_gpu(gold, name):
    pts, ny, nx, p, lam, pz, window, plimit = wrp_case(gold, name)
    U = torch.full((ny, nx), 7 + 7j, dtype=torch.complex64, device="cuda")   # step 1 overwrites U
    fn = og.WRPStep1 if window == 0 else og.WRPStep1_D
    fn(og.gObject(pts), U, ny, nx, p, lam, pz, plimit)
    torch.cuda.synchronize()
    got = U.cpu().numpy()
    ref = gold[name + "_out"]
    assert np.array_equal(got != 0, ref != 0)
    assert rel_l2(got, ref) < TOL
