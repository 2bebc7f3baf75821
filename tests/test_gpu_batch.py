"""GPU: the batched persistent launch gives the same fields as the single-field
entry points and as the FP64 oracle, is replayable from a CUDA graph, and
matches its serial baseline."""
import numpy as np
import pytest
import torch

import oracle as O
import openol_gb300 as og
from conftest import rel_l2

pytestmark = pytest.mark.gpu


def mixed_fields(seed=3):
    rng = np.random.default_rng(seed)
    fields = []
    shapes = [(256, 256), (512, 256), (256, 1024), (1024, 1024), (512, 512), (256, 512), (2048, 256)]
    methods = ["asm", "fresnel", "arss", "asm", "arss", "fresnel_bandlimit", "fresnel"]
    for k, ((ny, nx), m) in enumerate(zip(shapes, methods)):
        u = ((rng.random((ny, nx)) < 0.5) * np.exp(2j * np.pi * rng.random((ny, nx)))).astype(np.complex64)
        t = torch.from_numpy(u).cuda()
        fields.append(dict(u_in=t, u_out=torch.empty_like(t), method=m, dy=8e-6, dx=6e-6,
                           lam=[640e-9, 532e-9, 450e-9][k % 3], z=0.01 + 0.04 * k, s=0.5 if k % 2 else 2.0,
                           host=u))
    return fields


def oracle_of(f):
    u = f["host"].astype(np.complex128)
    m = f["method"]
    if m == "asm":
        return O.asm_prop(u, f["dy"], f["dx"], f["lam"], f["z"])
    if m == "fresnel":
        return O.fresnel_prop(u, f["dy"], f["dx"], f["lam"], f["z"])
    if m == "fresnel_bandlimit":
        return O.fresnel_prop(u, f["dy"], f["dx"], f["lam"], f["z"], bandlimit=1)
    return O.arss_prop(u, f["dy"], f["dx"], f["lam"], f["z"], f["s"])


def test_batch_matches_oracle_and_serial():
    fields = mixed_fields()
    plan = og.BatchPlan(fields)
    plan.execute()
    torch.cuda.synchronize()
    plan.check()
    persistent = [f["u_out"].cpu().numpy() for f in fields]
    for f in fields:
        f["u_out"].zero_()
    plan.execute_serial()
    torch.cuda.synchronize()
    for f, got in zip(fields, persistent):
        ref = oracle_of(f)
        assert rel_l2(got, ref) < 1e-5, f["method"]
        assert rel_l2(got, f["u_out"].cpu().numpy()) < 1e-6
    plan.close()


def test_batch_cuda_graph_replay_and_in_place():
    fields = mixed_fields(seed=8)
    for f in fields:  # in place: u_out is u_in
        f["u_out"] = f["u_in"]
    plan = og.BatchPlan(fields)
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.stream(s):
        with torch.cuda.graph(g, stream=s):
            plan.execute(stream=s)
    for f in fields:  # capture does not run: restore inputs, then replay twice (propagate twice)
        f["u_in"].copy_(torch.from_numpy(f["host"]))
    g.replay()
    g.replay()
    torch.cuda.synchronize()
    plan.check()
    for f in fields:
        once = oracle_of(f)
        f2 = dict(f, host=once.astype(np.complex64))
        twice = oracle_of(f2)
        assert rel_l2(f["u_in"].cpu().numpy(), twice) < 2e-5, f["method"]
    plan.close()


def test_batch_large_fields_run_through_single_field_passes():
    # lower the threshold so that four of the seven mixed fields (ASM, Fresnel
    # and ARSS among them) leave the persistent kernel, then capture and replay
    old = og.batch_direct_pixels(512 * 512)
    try:
        fields = mixed_fields(seed=11)
        plan = og.BatchPlan(fields)
        assert plan.n_direct == 4
        s = torch.cuda.Stream()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.stream(s):
            with torch.cuda.graph(g, stream=s):
                plan.execute(stream=s)
        for f in fields:
            f["u_out"].zero_()
        g.replay()
        torch.cuda.synchronize()
        plan.check()
        for f in fields:
            assert rel_l2(f["u_out"].cpu().numpy(), oracle_of(f)) < 1e-5, (f["method"], tuple(f["u_in"].shape))
        plan.close()
    finally:
        og.batch_direct_pixels(old)
    assert og.batch_direct_pixels() == old


def test_batch_host_fields_pipelined():
    """olg_batch_execute_host: host fields copied in, the plan run and the
    results copied out over three streams give exactly what execute() gives on
    the same inputs, for persistent-kernel and single-field-pass fields alike,
    and twice in a row on the same buffers."""
    old = og.batch_direct_pixels(512 * 512)
    try:
        fields = mixed_fields(seed=13)
        plan = og.BatchPlan(fields)
        assert 0 < plan.n_direct < len(fields)
        plan.execute()
        torch.cuda.synchronize()
        want = [f["u_out"].cpu().numpy() for f in fields]
        hin = [torch.from_numpy(f["host"]).pin_memory() for f in fields]
        for f in fields:  # the device inputs are overwritten by the copies in
            f["u_in"].zero_()
            f["u_out"].zero_()
        s = torch.cuda.Stream()
        for rep in range(2):
            hout = [torch.full_like(h, complex(7.0, 7.0)).pin_memory() for h in hin]
            plan.execute_host(hin, hout, stream=s)
            s.synchronize()
            plan.check()
            for f, got, ref in zip(fields, hout, want):
                assert np.array_equal(got.numpy(), ref), (rep, f["method"], tuple(f["u_in"].shape))
        with pytest.raises(ValueError):
            plan.execute_host(hin[:-1], hout[:-1])
        plan.close()
    finally:
        og.batch_direct_pixels(old)
