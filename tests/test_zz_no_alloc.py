"""gsea_stats_device_noalloc: the statistics step for callers that cannot
allocate device memory (a host whose memory belongs to its own pool
allocator, or a loop that must not call cudaMalloc/cudaFree because they can
synchronise the device).  It must give the same statistics as the regular
pipeline, call after call, even though every call reuses the same fixed
scratch array inside the library.

Kept in a file of its own that pytest collects last."""
import ctypes

import numpy as np
import pytest

from cudagsea_gb300 import api, synthetic
from cudagsea_gb300 import _native as N

pytestmark = pytest.mark.gpu


def _plan(d, P, precision):
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P, "twopass_signal2noise", precision=precision)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    plan.synchronize()
    return plan


@pytest.mark.parametrize("precision", [32, 64])
def test_noalloc_statistics_match_regular_pipeline(gpu, precision):
    """Three calls in a row (data set 1, 2, 1 again) reproduce the pipeline's
    statistics bit for bit; the device's free memory does not change after
    the first call; the last call runs on a caller's own stream."""
    import torch
    L = N.lib()
    stream = torch.cuda.Stream()
    d1 = synthetic.make(1500, 30, 40, 200, seed=21, n_class_b=15, set_min=10, set_max=120)
    d2 = synthetic.make(1500, 30, 40, 333, seed=22, n_class_b=12, set_min=10, set_max=120)
    a = _plan(d1, d1.num_perms, precision)          # ES and statistics of data set 1
    b = _plan(d2, d2.num_perms, precision)          # ES and statistics of data set 2
    sink = _plan(d1, 4, precision)                  # its STATS buffer receives the results
    K = d1.num_sets
    dt = np.float64 if precision == 64 else np.float32
    out_ptr, out_bytes = sink.buffer(N.BUF_STATS)
    assert out_bytes >= 5 * K * np.dtype(dt).itemsize
    free_after_first = None
    for i, (src, d) in enumerate(((a, d1), (b, d2), (a, d1))):  # consecutive calls reuse the scratch
        es_ptr, _ = src.buffer(N.BUF_ES)
        st = ctypes.c_void_p(stream.cuda_stream) if i == 2 else None
        rc = L.gsea_stats_device_noalloc(ctypes.c_void_p(es_ptr), K, d.num_perms, precision,
                                         ctypes.c_void_p(out_ptr), st)
        N.check(rc)
        if i == 2:
            stream.synchronize()
        else:
            torch.cuda.synchronize()
        free_now = torch.cuda.mem_get_info()[0]
        if free_after_first is None:
            free_after_first = free_now
        assert free_now == free_after_first, "a call allocated device memory"
        got = sink.read_buffer(N.BUF_STATS, dt, (5 * K,))
        want = src.read_buffer(N.BUF_STATS, dt, (5 * K,))
        np.testing.assert_array_equal(got, want)
    for p in (a, b, sink):
        p.close()


def test_noalloc_rejects_sizes_beyond_fixed_scratch(gpu):
    L = N.lib()
    d = synthetic.tiny()
    p = _plan(d, d.num_perms, 32)
    es_ptr, _ = p.buffer(N.BUF_ES)
    st_ptr, _ = p.buffer(N.BUF_STATS)
    rc = L.gsea_stats_device_noalloc(ctypes.c_void_p(es_ptr), d.num_sets, 10_000_000, 32,
                                     ctypes.c_void_p(st_ptr), None)
    assert rc == 1
    assert b"4 MiB" in L.gsea_last_error()
    p.close()
