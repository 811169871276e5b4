"""Permutation sharding across ranks (one GPU per rank).

Permutations are independent and keyed by their global index (the
generator is seeded with index + 42), so a run over P permutations splits into
contiguous ranges, one per rank, with no exchange until the statistics.  Two
ways to finish:

* ``run_sharded`` gathers the ES columns in rank order into the [K][P] matrix
  a single run would produce (needed when the caller wants the matrix, e.g.
  for the .es dump) and computes the statistics on it;
* ``run_sharded_stats`` merges O(K) partial results instead
  (``merge_stats``): the sequential sum of |ES| behind NES chained from rank
  to rank in permutation order, then NP / FWER counts and the FDR null
  histogram summed over the ranks -- bit-identical to a single run, with no
  K x P exchange.

Only torch.distributed carries the exchange (gloo on CPU, NCCL on GPUs); the
data path of every rank is the library's.
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
    # statistics of the merged matrix on this rank's GPU; the working memory
    # comes from torch's allocator (no size limit but the device's memory)
    dt = torch.float64 if precision == 64 else torch.float32
    es_dev = torch.from_numpy(np.ascontiguousarray(es)).to(device="cuda", dtype=dt)
    st_dev = torch.empty(5 * d.num_sets, dtype=dt, device="cuda")
    L = N.lib()
    need = ctypes.c_size_t(0)
    N.check(L.gsea_stats_scratch_bytes(d.num_sets, num_perms, precision, ctypes.byref(need)))
    scratch = torch.empty(need.value, dtype=torch.uint8, device="cuda")
    N.check(L.gsea_stats_device(ctypes.c_void_p(es_dev.data_ptr()), d.num_sets, num_perms, precision,
                                ctypes.c_void_p(st_dev.data_ptr()), ctypes.c_void_p(scratch.data_ptr()),
                                need.value, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return es, st_dev.cpu().numpy()


# ---------------------------------------------------------------------------
# O(K) merge of the statistics


class DeviceOps:
    """The partial-statistics steps as the library's kernels on torch CUDA
    tensors (gsea_shard_sum / _head / _partial / _finish)."""

    def __init__(self, precision: int = 32):
        import torch
        self.torch = torch
        self.precision = precision
        self.dtype = torch.float64 if precision == 64 else torch.float32

    def _p(self, t):
        import ctypes
        return None if t is None else ctypes.c_void_p(t.data_ptr())

    def _stream(self):
        import ctypes
        return ctypes.c_void_p(self.torch.cuda.current_stream().cuda_stream)

    def chain_sum(self, es, init):
        from . import _native as N
        K, count = es.shape
        out = self.torch.empty(K, dtype=self.dtype, device=es.device)
        N.check(N.lib().gsea_shard_sum(self._p(es), K, count, es.stride(0), self.precision, self._p(init),
                                       self._p(out), self._stream()))
        return out

    def observed(self, es):
        return es[:, 0].contiguous()

    def head(self, es_obs, total, num_perms):
        from . import _native as N
        K = es_obs.shape[0]
        out = self.torch.empty(3 * K, dtype=self.dtype, device=es_obs.device)
        N.check(N.lib().gsea_shard_head(self._p(es_obs), self._p(total), K, num_perms, self.precision,
                                        self._p(out), self._stream()))
        return out

    def partial(self, es, first, head):
        from . import _native as N
        K, count = es.shape
        counts = self.torch.empty(2 * K, dtype=self.torch.int64, device=es.device)
        hist = self.torch.empty(2 * (K + 2) + 2, dtype=self.torch.float64, device=es.device)
        N.check(N.lib().gsea_shard_partial(self._p(es), K, count, es.stride(0), self.precision, first,
                                           self._p(head), self._p(counts), self._p(hist), self._stream()))
        return counts, hist

    def finish(self, head, num_perms, counts, hist):
        from . import _native as N
        K = head.shape[0] // 3
        out = self.torch.empty(5 * K, dtype=self.dtype, device=head.device)
        N.check(N.lib().gsea_shard_finish(self._p(head), K, num_perms, self.precision, self._p(counts),
                                          self._p(hist), self._p(out), self._stream()))
        return out

    def empty_like_sum(self, K, like):
        return self.torch.empty(K, dtype=self.dtype, device=like.device)

    def to_comm(self, x, device):
        return x.to(device)

    def from_comm(self, t, like):
        return t.to(like.device)


def merge_stats(ops, es_local, first: int, num_perms: int, group=None):
    """Statistics of the whole run from this rank's ES columns [K][count]
    (global permutations first .. first + count - 1; the ranks' ranges
    contiguous and in rank order, rank 0 holding permutation 0).  `ops`
    computes the partial steps (DeviceOps for the library's kernels); every
    rank returns the same [5K] statistics."""
    import torch
    import torch.distributed as dist
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    comm_dev = torch.device("cuda", torch.cuda.current_device()) if dist.get_backend(group) == "nccl" \
        else torch.device("cpu")
    K = es_local.shape[0]
    # 1. sequential |ES| sum, chained in rank (= permutation) order
    init = None
    if rank > 0:
        buf = ops.to_comm(ops.empty_like_sum(K, es_local), comm_dev)
        dist.recv(buf, src=dist.get_global_rank(group, rank - 1) if group is not None else rank - 1, group=group)
        init = ops.from_comm(buf, es_local)
    total = ops.chain_sum(es_local, init)
    if rank < world - 1:
        dist.send(ops.to_comm(total, comm_dev),
                  dst=dist.get_global_rank(group, rank + 1) if group is not None else rank + 1, group=group)
    last = dist.get_global_rank(group, world - 1) if group is not None else world - 1
    t = ops.to_comm(total, comm_dev)
    dist.broadcast(t, src=last, group=group)
    total = ops.from_comm(t, es_local)
    # 2. observed scores from the rank holding permutation 0
    src0 = dist.get_global_rank(group, 0) if group is not None else 0
    obs = ops.to_comm(ops.observed(es_local) if rank == 0 else ops.empty_like_sum(K, es_local), comm_dev)
    dist.broadcast(obs, src=src0, group=group)
    head = ops.head(ops.from_comm(obs, es_local), total, num_perms)
    # 3. partial counts and histograms, summed over the ranks (exact)
    counts, hist = ops.partial(es_local, first, head)
    c, h = ops.to_comm(counts, comm_dev), ops.to_comm(hist, comm_dev)
    dist.all_reduce(c, group=group)
    dist.all_reduce(h, group=group)
    return ops.finish(head, num_perms, ops.from_comm(c, counts), ops.from_comm(h, hist))


def run_sharded_stats(d, num_perms: int, metric="twopass_signal2noise", precision: int = 32, form: int = 0,
                      group=None):
    """Every rank runs its permutation range of data set `d` on its current
    GPU and the statistics are merged from O(K) partial results; returns the
    [5K] statistics (numpy) on every rank."""
    import torch
    import torch.distributed as dist
    from . import api
    rank, world = dist.get_rank(group), dist.get_world_size(group)
    first, count = shard_range(num_perms, rank, world)
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, max(count, 1), metric, precision=precision,
                    form=form, perm_offset=first)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es_local, _ = plan.read(stats=False)
    plan.close()
    ops = DeviceOps(precision)
    es_dev = torch.from_numpy(np.ascontiguousarray(es_local[:, :count])).to(device="cuda", dtype=ops.dtype)
    return merge_stats(ops, es_dev, first, num_perms, group).cpu().numpy()
