"""Permutation shards on two gloo ranks (CPU): the gathered columns equal a
single run's ES matrix, so the statistics are identical.  Each rank computes
its columns with the oracle (no GPU here); the host logic under test is the
range split and the gather order of cudagsea_gb300.shard."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from cudagsea_gb300.shard import shard_range


def test_shard_ranges_cover_exactly():
    for P in (1, 7, 1000, 1024):
        for world in (1, 2, 3, 8):
            spans = [shard_range(P, r, world) for r in range(world)]
            assert spans[0][0] == 0
            for (a, n), (b, _) in zip(spans, spans[1:]):
                assert a + n == b
            assert sum(n for _, n in spans) == P
            assert max(n for _, n in spans) - min(n for _, n in spans) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, P, out_dir):
    import torch.distributed as dist
    import oracle
    from cudagsea_gb300 import synthetic
    from cudagsea_gb300.shard import gather_es, shard_range
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    d = synthetic.make(400, 16, 12, P, seed=9, n_class_b=8, set_min=5, set_max=40)
    first, count = shard_range(P, rank, world)
    keys = oracle.metric(8, d.exprs, d.labels, count, shift=first)
    sk, order = oracle.sort(keys)
    es_local = oracle.es(sk, order, d.set_offsets, d.set_genes)
    es = gather_es(es_local, P)
    if rank == 0:
        np.save(os.path.join(out_dir, "merged.npy"), es)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("P", [50, 64])
def test_two_rank_gather_equals_single_run(tmp_path, P):
    import oracle
    from cudagsea_gb300 import synthetic
    mp.start_processes(_worker, args=(2, _free_port(), P, str(tmp_path)), nprocs=2, start_method="spawn")
    merged = np.load(tmp_path / "merged.npy")
    d = synthetic.make(400, 16, 12, P, seed=9, n_class_b=8, set_min=5, set_max=40)
    es_full, st_full = oracle.gsea(8, d.exprs, d.labels, d.set_offsets, d.set_genes, P)
    np.testing.assert_array_equal(merged, es_full)
    np.testing.assert_array_equal(oracle.stats(merged), st_full)


def _merge_worker(rank, world, port, P, out_dir):
    import torch.distributed as dist
    import oracle
    from oracle.shard import OracleOps
    from cudagsea_gb300 import synthetic
    from cudagsea_gb300.shard import merge_stats, shard_range
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    d = synthetic.make(400, 16, 12, P, seed=9, n_class_b=8, set_min=5, set_max=40)
    first, count = shard_range(P, rank, world)
    keys = oracle.metric(8, d.exprs, d.labels, count, shift=first)
    sk, order = oracle.sort(keys)
    es_local = oracle.es(sk, order, d.set_offsets, d.set_genes)
    st = merge_stats(OracleOps(32), es_local, first, P)
    np.save(os.path.join(out_dir, f"stats{rank}.npy"), st)
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("world,P", [(2, 64), (3, 50)])
def test_partial_statistics_merge_equals_single_run(tmp_path, world, P):
    """O(K) merge over gloo ranks (sequential |ES| sum chained rank to rank,
    counts and FDR histograms summed): every rank gets the single run's
    statistics bit for bit."""
    import oracle
    from cudagsea_gb300 import synthetic
    mp.start_processes(_merge_worker, args=(world, _free_port(), P, str(tmp_path)), nprocs=world,
                       start_method="spawn")
    d = synthetic.make(400, 16, 12, P, seed=9, n_class_b=8, set_min=5, set_max=40)
    _, st_full = oracle.gsea(8, d.exprs, d.labels, d.set_offsets, d.set_genes, P)
    for r in range(world):
        st = np.load(tmp_path / f"stats{r}.npy")
        np.testing.assert_array_equal(st.view(np.uint32), st_full.view(np.uint32))
