"""Merging log-weight summaries across sample shards.

A summary is the triple (m, S, S2) = (max l, sum exp(l - m), sum exp(2(l - m)))
that issm_logweight_summary writes (FP64). Shards of one set of log weights
merge exactly as the reference merges per-block moments
(_merge_logweight_moments, src/execution.jl:166-173): rescale each shard's
sums to the common maximum and add. An all -Inf shard (S = 0) contributes
nothing. With torch.distributed, every rank gets the merged summary of all
ranks' shards (one all-gather of three words per rank).
"""
import math

import numpy as np
import torch


def merge_summaries(summaries):
    """Merge (m, S, S2) triples (any iterable of 3-sequences) into one."""
    rows = [tuple(float(v) for v in s) for s in summaries]
    live = [r for r in rows if r[1] != 0.0]
    if not live:
        return (-math.inf, 0.0, 0.0)
    m = max(r[0] for r in live)
    s = s2 = 0.0
    for mk, sk, s2k in live:
        f = math.exp(mk - m) if mk != m else 1.0
        s += sk * f
        s2 += s2k * f * f
    return (m, s, s2)


def ess_and_logz(summary, n):
    """ESS = S^2 / S2 and log Z = m + log S - log n of a (merged) summary."""
    m, s, s2 = summary
    if s == 0.0:
        return 0.0, -math.inf
    return s * s / s2, m + math.log(s) - math.log(n)


def allreduce_summary(summary, group=None):
    """Merge this rank's summary with every other rank's (torch.distributed).

    `summary` is a 3-element tensor or sequence (device or host). Returns the
    merged triple on every rank."""
    local = torch.as_tensor(np.asarray([float(v) for v in (summary.tolist() if isinstance(summary, torch.Tensor)
                                                          else summary)], dtype=np.float64))
    world = torch.distributed.get_world_size(group)
    parts = [torch.zeros(3, dtype=torch.float64) for _ in range(world)]
    torch.distributed.all_gather(parts, local, group=group)
    return merge_summaries(p.tolist() for p in parts)
