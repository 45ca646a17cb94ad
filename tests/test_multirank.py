"""Multi-rank host logic on CPU (gloo, world_size 2): pixel shards need no
data exchange and reproduce the single-process result; the diffusion-law
partial sums reduce to the single-process mean and variance."""
import os

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

import oracle
from imaging_fcs_1_52_gb300 import engine, shard
from tests.helpers import oracle_kwargs
from tests.synth import brownian_stack


def test_shard_rows_cover_exactly():
    for out_h in (1, 7, 128):
        for world in (1, 2, 3, 8):
            rows = [shard.shard_rows(out_h, world, r) for r in range(world)]
            assert sum(n for _, n in rows) == out_h
            assert [s for s, _ in rows] == list(np.cumsum([0] + [n for _, n in rows[:-1]]))


def test_diffusion_point_of_empty_binning_is_nan():
    mean, var = shard.diffusion_point(shard.diffusion_partials(np.zeros((4, 11)), np.zeros(4, np.int32)))
    assert np.isnan(mean) and np.isnan(var)


def _worker(rank, world, port, stack, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    cfg = engine.FCSConfig(width=6, height=6, frames=3000, background=100, binx=1, biny=1)
    part = shard.shard_config(cfg, world, rank)
    r = oracle.run(stack, **oracle_kwargs(part))
    acf = torch.from_numpy(r["acf"])
    sizes = [torch.zeros(1, dtype=torch.int64) for _ in range(world)]
    dist.all_gather(sizes, torch.tensor([acf.shape[0]]))
    maxn = int(max(s.item() for s in sizes))
    pad = torch.zeros((maxn, acf.shape[1]), dtype=acf.dtype)
    pad[: acf.shape[0]] = acf
    gathered = [torch.zeros_like(pad) for _ in range(world)]
    dist.all_gather(gathered, pad)
    partials = torch.from_numpy(shard.diffusion_partials(r["fitres"], r["fitted"]))
    dist.all_reduce(partials)
    if rank == 0:
        full = torch.cat([g[: int(s.item())] for g, s in zip(gathered, sizes)]).numpy()
        q.put((full, partials.numpy()))
    dist.destroy_process_group()


def test_two_rank_shards_match_single_process():
    stack = brownian_stack(6, 6, 3000, seed=12, density=2.0, cps=3e4)
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, stack, q)) for r in range(2)]
    for p in procs:
        p.start()
    full, partials = q.get(timeout=300)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    cfg = engine.FCSConfig(width=6, height=6, frames=3000, background=100)
    ref = oracle.run(stack, **oracle_kwargs(cfg))
    np.testing.assert_array_equal(full, ref["acf"])
    mean, var = shard.diffusion_point(partials)
    m_ref, v_ref = shard.diffusion_point(shard.diffusion_partials(ref["fitres"], ref["fitted"]))
    assert mean == pytest.approx(m_ref, rel=1e-12) and var == pytest.approx(v_ref, rel=1e-9, abs=1e-12)
