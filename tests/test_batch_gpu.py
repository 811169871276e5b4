"""Batched instances: uneven GSEA problems run together (one launch per
stage over every instance, one persistent enrichment launch per size class,
one CUDA graph) give exactly the results of running each instance on its own
plan; the graph replays; the batch autotuner keeps the results."""
import numpy as np
import pytest

from cudagsea_gb300 import api, synthetic
from cudagsea_gb300 import _native as N

pytestmark = pytest.mark.gpu


def instances():
    shapes = [  # genes, samples, sets, perms: every enrichment size class, G > 20,480 too
        (3000, 24, 40, 300), (7000, 60, 150, 257), (12000, 33, 90, 400), (16000, 100, 60, 128),
        (20000, 48, 200, 300), (25000, 40, 120, 200), (5000, 500, 30, 64), (900, 20, 12, 500),
    ]
    out = []
    for i, (G, S, K, P) in enumerate(shapes):
        out.append(synthetic.make(G, S, K, P, seed=100 + i, n_class_b=S // 2 - 3 * (i % 3), sd_range=(0.5, 2.0),
                                  n_shift=max(20, G // 100), shift_range=(0.3, 1.0), set_min=15,
                                  set_max=min(400, G // 4), enriched_frac=0.2))
    return out


METRICS = ["twopass_signal2noise", "naive_diff_of_classes", "onepass_t_test", "stable_signal2noise",
           "overkill_t_test", "twopass_t_test", "onepass_signal2noise", "stable_diff_of_classes"]


def solo(d, metric, precision, form):
    p = api.Plan(d.num_genes, d.num_samples, d.num_sets, d.num_perms, metric, precision=precision, form=form)
    p.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    p.execute()
    es, st = p.read()
    p.close()
    return es, st


def same(a, b):
    u = np.uint64 if a.dtype == np.float64 else np.uint32
    return np.array_equal(a.view(u), b.view(u))


@pytest.mark.parametrize("precision,form", [(32, N.FORM_PLAIN), (64, N.FORM_PLAIN), (32, N.FORM_CHOSEN),
                                            (32, N.FORM_CHOSEN_FP64)])
def test_batch_matches_solo_plans(gpu, precision, form):
    ds = instances()
    metrics = METRICS if form == N.FORM_PLAIN else ["twopass_signal2noise"] * len(ds)
    if form == N.FORM_CHOSEN_FP64:  # every metric family of the tensor-core form in one batch
        metrics = ["twopass_signal2noise", "naive_diff_of_classes", "onepass_t_test", "naive_ratio_of_classes",
                   "stable_signal2noise", "naive_log2_ratio_of_classes", "overkill_t_test", "stable_t_test"]
    ref = [solo(d, m, precision, form) for d, m in zip(ds, metrics)]
    b = api.Batch(ds, metrics, precision=precision, form=form, streams=4)
    for rep in range(2):  # the second execute replays the captured graph
        b.execute()
        b.synchronize()
        for i in range(len(ds)):
            es, st = b.read(i)
            assert same(es, ref[i][0]), (rep, i)
            assert same(st, ref[i][1]), (rep, i)
    info = b.info()
    assert info["es_classes"] >= 5
    assert info["launches"] > 0
    if form == N.FORM_CHOSEN:
        # permute 1 + metric 3 + sort classes + ES classes + statistics 9
        assert info["launches"] <= 1 + 3 + 7 + info["es_classes"] + 9, info
    elif form == N.FORM_CHOSEN_FP64:
        # the metric: 3 launches per metric family (5 families)
        assert info["launches"] <= 1 + 3 * 5 + 7 + info["es_classes"] + 9, info
    else:
        # permute 1 + one metric launch per metric + sort classes (+ the fp64
        # instance beyond the register sort) + ES classes + statistics 9
        assert info["launches"] <= 1 + len(set(metrics)) + 7 + 1 + info["es_classes"] + 9, info
    b.close()


@pytest.mark.parametrize("form", [N.FORM_CHOSEN, N.FORM_PLAIN])
def test_batch_of_40_uneven_instances_matches_solo_plans(gpu, form):
    """40 instances with genes U[1,000, 30,000], samples U[20, 200], sets
    U[10, 300] and permutations U[64, 600] (one metric): the batched execute
    equals every solo plan bit for bit, and issues a handful of launches --
    one per stage (and per sort / enrichment class), not one per instance."""
    ds = synthetic.batch_instances(40, seed=5, num_perms=64, genes=(1000, 30000), samples=(20, 200),
                                   sets=(10, 300), set_size=(15, 200))
    rs = np.random.RandomState(9)
    for d in ds:
        d.num_perms = int(rs.randint(64, 601))
    ref = [solo(d, "twopass_signal2noise", 32, form) for d in ds]
    b = api.Batch(ds, "twopass_signal2noise", precision=32, form=form)
    for rep in range(2):
        b.execute()
        b.synchronize()
        for i in range(len(ds)):
            es, st = b.read(i)
            assert same(es, ref[i][0]), (rep, i)
            assert same(st, ref[i][1]), (rep, i)
    info = b.info()
    assert info["launches"] <= 1 + 3 + 7 + info["es_classes"] + 9, info
    b.close()


def test_batch_autotune_keeps_results(gpu):
    ds = instances()[:5]
    ref = [solo(d, "twopass_signal2noise", 32, N.FORM_PLAIN) for d in ds]
    b = api.Batch(ds, precision=32)
    b.autotune(128)
    t = b.tuning(0)
    assert t["sort_variant"] in (1, 2) and t["metric_pb"] in (4, 8)
    b.execute()
    b.synchronize()
    for i in range(len(ds)):
        es, st = b.read(i)
        assert same(es, ref[i][0]) and same(st, ref[i][1])
    b.close()


def test_batch_rejects_mixed_precision(gpu):
    ds = instances()[:2]
    L = N.lib()
    import ctypes
    cfgs = (N.Config * 2)()
    for i, d in enumerate(ds):
        L.gsea_config_init(ctypes.byref(cfgs[i]))
        cfgs[i].num_samples, cfgs[i].num_genes = d.exprs.shape
        cfgs[i].num_sets, cfgs[i].num_perms = d.num_sets, d.num_perms
    cfgs[1].precision = 64
    h = ctypes.c_void_p()
    assert L.gsea_batch_create(2, cfgs, 0, ctypes.byref(h)) == 1


@pytest.mark.parametrize("form", [N.FORM_PLAIN, N.FORM_CHOSEN])
def test_batch_mixed_sort_directions(gpu, form):
    """Instances sorting in ascending and descending order in one batch (the
    reference's `-order ascending`): each equals its solo plan bit for bit."""
    ds = instances()[:6]
    asc = [i % 2 == 1 for i in range(len(ds))]
    metric = "twopass_signal2noise"
    ref = []
    for d, a in zip(ds, asc):
        p = api.Plan(d.num_genes, d.num_samples, d.num_sets, d.num_perms, metric, form=form, ascending=a)
        p.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        p.execute()
        ref.append(p.read())
        p.close()
    b = api.Batch(ds, metric, precision=32, form=form, ascending=asc)
    b.execute()
    b.synchronize()
    for i in range(len(ds)):
        es, st = b.read(i)
        assert same(es, ref[i][0]) and same(st, ref[i][1]), i
    b.close()


def test_batch_single_instance_and_single_permutation(gpu):
    d1 = synthetic.make(4000, 30, 25, 1, seed=3, n_class_b=15, set_min=15, set_max=100)
    d2 = synthetic.make(1500, 22, 7, 33, seed=4, n_class_b=11, set_min=15, set_max=100)
    for ds in ([d1], [d1, d2]):
        ref = [solo(d, "twopass_signal2noise", 32, N.FORM_PLAIN) for d in ds]
        b = api.Batch(ds, precision=32)
        b.execute()
        b.synchronize()
        for i in range(len(ds)):
            es, st = b.read(i)
            assert same(es, ref[i][0]) and same(st, ref[i][1])
        b.close()
