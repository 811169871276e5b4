"""Permutation sharding across ranks (one GPU per rank).

Permutations are independent and keyed by their global index (the
generator is seeded with index + 42), so a run over P permutations splits into
contiguous ranges, one per rank, with no exchange until the statistics: each
rank computes the ES columns of its range (``Plan(perm_offset=...)``), the
columns are gathered in rank order into the [K][P] matrix a single run would
produce, and the statistics are computed on it once.  Only torch.distributed
is used for the exchange (gloo on CPU, NCCL on GPUs); the data path of every
rank is the library's.
"""
from __future__ import annotations

from typing import Optional, Tuple

import numpy as np


def shard_range(num_perms: int, rank: int, world: int) -> Tuple[int, int]:
    """(first global permutation, count) of `rank`; counts differ by at most one."""
    base, extra = divmod(num_perms, world)
    count = base + (1 if rank < extra else 0)
    first = rank * base + min(rank, extra)
    return first, count


def gather_es(es_local: np.ndarray, num_perms: int, group=None) -> Optional[np.ndarray]:
    """All-gather the ES columns of every rank into the full [K][P] matrix
    (every rank receives it).  es_local: [K][count] of this rank's range."""
    import torch
    import torch.distributed as dist
    world = dist.get_world_size(group)
    K = es_local.shape[0]
    width = -(-num_perms // world)  # padded column count
    buf = np.zeros((K, width), es_local.dtype)
    buf[:, :es_local.shape[1]] = es_local
    t = torch.from_numpy(buf)
    if dist.get_backend(group) == "nccl":
        t = t.cuda()
    parts = [torch.empty_like(t) for _ in range(world)]
    dist.all_gather(parts, t, group=group)
    cols = []
    for r, p in enumerate(parts):
        _, count = shard_range(num_perms, r, world)
        cols.append(p.cpu().numpy()[:, :count])
    return np.concatenate(cols, axis=1)


def run_sharded(d, num_perms: int, metric="twopass_signal2noise", precision: int = 32, form: int = 0,
                group=None):
    """Every rank runs its permutation range of data set `d` on its current
    GPU; returns (es [K][P], stats [5K]) on every rank."""
    import ctypes
    import torch
    import torch.distributed as dist
    from . import api
    from . import _native as N
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    first, count = shard_range(num_perms, rank, world)
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, max(count, 1), metric, precision=precision,
                    form=form, perm_offset=first)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es_local, _ = plan.read(stats=False)
    plan.close()
    es = gather_es(es_local[:, :count], num_perms, group)
    # statistics of the merged matrix, on this rank's GPU, without allocating in the library
    dt = torch.float64 if precision == 64 else torch.float32
    es_dev = torch.from_numpy(np.ascontiguousarray(es)).to(device="cuda", dtype=dt)
    st_dev = torch.empty(5 * d.num_sets, dtype=dt, device="cuda")
    N.check(N.lib().gsea_stats_device_noalloc(ctypes.c_void_p(es_dev.data_ptr()), d.num_sets, num_perms,
                                              precision, ctypes.c_void_p(st_dev.data_ptr()),
                                              ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return es, st_dev.cpu().numpy()
