"""Log-weight summaries of sample shards merge to the summary of the whole set
(CPU; world_size 2 over gloo, and the merge rule itself against the oracle)."""
import math
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _oracle_summary(lw):
    lw = np.asarray(lw, dtype=np.float64)
    live = lw[lw > -np.inf]
    if live.size == 0:
        return (-math.inf, 0.0, 0.0)
    m = live.max()
    e = np.exp(live - m)
    return (m, e.sum(), (e * e).sum())


def test_merge_matches_whole_set(issm):
    merge_summaries = issm.shards.merge_summaries

    rng = np.random.default_rng(0)
    lw = rng.normal(size=10_000) * 6
    lw[rng.random(lw.size) < 0.05] = -np.inf
    parts = np.array_split(lw, 7)
    parts.append(np.full(5, -np.inf))  # an all -Inf shard contributes nothing
    merged = merge_summaries(_oracle_summary(p) for p in parts)
    whole = _oracle_summary(lw)
    assert merged[0] == whole[0]
    assert merged[1] == pytest.approx(whole[1], rel=1e-13)
    assert merged[2] == pytest.approx(whole[2], rel=1e-13)
    assert merge_summaries([(-math.inf, 0.0, 0.0)]) == (-math.inf, 0.0, 0.0)


def _worker(rank, world, port, lw, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import __graft_entry__

        shards = __graft_entry__.load_package().shards
        allreduce_summary, ess_and_logz = shards.allreduce_summary, shards.ess_and_logz

        shard = np.array_split(lw, world)[rank]
        merged = allreduce_summary(_oracle_summary(shard))
        out[rank] = (merged, ess_and_logz(merged, lw.size))
    finally:
        dist.destroy_process_group()


def test_two_rank_gloo_merge(issm):
    rng = np.random.default_rng(1)
    lw = rng.normal(size=4_001) * 3 + 2.0
    lw[:17] = -np.inf
    port = _free_port()
    # spawn, never fork: the test process may already hold a CUDA context
    with mp.get_context("spawn").Manager() as manager:
        out = manager.dict()
        mp.spawn(_worker, args=(2, port, lw, out), nprocs=2, join=True)
        results = dict(out)
    whole = _oracle_summary(lw)
    for rank in (0, 1):
        merged, (ess, logz) = results[rank]
        assert merged[0] == whole[0]
        assert merged[1] == pytest.approx(whole[1], rel=1e-13)
        ess_ref = whole[1] ** 2 / whole[2]
        logz_ref = whole[0] + math.log(whole[1]) - math.log(lw.size)
        assert ess == pytest.approx(ess_ref, rel=1e-12)
        assert logz == pytest.approx(logz_ref, rel=1e-12, abs=1e-12)


@pytest.mark.gpu
def test_gpu_shard_summaries_merge(issm, cuda):
    """Device summaries of four shards merge to the device summary of the whole."""
    g = torch.Generator(device=cuda).manual_seed(5)
    lw = torch.randn(3_000_017, device=cuda, generator=g, dtype=torch.float64) * 4
    whole = issm.ops.logweight_summary(lw).cpu().numpy()
    parts = [issm.ops.logweight_summary(c.contiguous()).cpu().numpy() for c in torch.chunk(lw, 4)]
    merged = issm.shards.merge_summaries(parts)
    assert merged[0] == whole[0]
    assert merged[1] == pytest.approx(whole[1], rel=1e-12)
    assert merged[2] == pytest.approx(whole[2], rel=1e-12)
