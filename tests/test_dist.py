"""CPU, world_size 2 over gloo: the partitioner covers every work unit exactly
once, and row shards of a CGH computed on separate ranks reassemble into the
whole hologram (FP64 oracle as the per-rank worker)."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from openol_gb300.dist import hologram_rows, shard_by_cost, shard_items


def test_shard_items_cover_exactly_once():
    for n in (0, 1, 7, 96, 1000):
        for world in (1, 2, 3, 8):
            seen = []
            for r in range(world):
                a, b = shard_items(n, r, world)
                seen += list(range(a, b))
            assert seen == list(range(n))


def test_shard_by_cost_balances_uneven_batch():
    rng = np.random.default_rng(0)
    sizes = rng.choice([512, 1024, 2048, 4096], 96)
    costs = [float(s) ** 2 for s in sizes]
    parts = shard_by_cost(costs, 4)
    assert sorted(i for p in parts for i in p) == list(range(96))
    loads = [sum(costs[i] for i in p) for p in parts]
    assert max(loads) / min(loads) < 1.1


def _worker(rank, world, port, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import oracle as O
    ny, nx, p, lam = 24, 20, 8e-6, 532e-9
    rng = np.random.default_rng(5)
    pts = np.stack([rng.random(9) * nx * p, rng.random(9) * ny * p, 0.02 + rng.random(9) * 0.01], 1)
    h0, h1 = hologram_rows(ny, rank, world)
    sp = pts.copy()
    sp[:, 1] -= p * h0
    part = O.cgh_fresnel(sp, h1 - h0, nx, p, p, lam)
    t = torch.from_numpy(np.stack([part.real, part.imag], -1)).float().contiguous()
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([t.shape[0]]))
    m = int(max(s.item() for s in sizes))
    pad = torch.zeros((m, nx, 2))
    pad[: t.shape[0]] = t
    gathered = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(gathered, pad)
    if rank == 0:
        rows = [g[: int(s.item())] for g, s in zip(gathered, sizes)]
        full = torch.cat(rows).numpy()
        ref = O.cgh_fresnel(pts, ny, nx, p, p, lam)
        out.put(float(np.abs(full[..., 0] + 1j * full[..., 1] - ref).max()))
    dist.barrier()
    dist.destroy_process_group()


def test_row_shards_reassemble_over_gloo():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29600 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for pr in procs:
        pr.start()
    err = q.get(timeout=120)
    for pr in procs:
        pr.join(timeout=60)
        assert pr.exitcode == 0
    assert err < 1e-4  # float32 transport of values of magnitude ~10
