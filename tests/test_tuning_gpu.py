"""Launch configurations: every tuning choice of the metric, sort and
enrichment kernels (and the tensor-core tile) computes the same results as the
automatic one; the autotuner returns a configuration that runs and keeps the
results unchanged."""
import numpy as np
import pytest

from cudagsea_gb300 import api, synthetic
from cudagsea_gb300 import _native as N

pytestmark = pytest.mark.gpu


def run(d, form=N.FORM_PLAIN, precision=32, **tuning):
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, d.num_perms, "twopass_signal2noise",
                    precision=precision, form=form)
    plan.set_debug(True)
    if tuning:
        plan.set_tuning(**tuning)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es, st = plan.read()
    dt = np.float64 if precision == 64 else np.float32
    keys = plan.read_buffer(N.BUF_KEYS, dt, (plan.perm_batch, d.num_genes))
    plan.close()
    return keys, es, st


def same(a, b):
    u = np.uint64 if a.dtype == np.float64 else np.uint32
    return np.array_equal(a.view(u), b.view(u))


@pytest.fixture(scope="module")
def data():
    return synthetic.make(6000, 48, 120, 600, seed=31, n_class_b=20, sd_range=(0.5, 2.0), n_shift=100,
                          shift_range=(0.3, 1.0), set_min=15, set_max=300, enriched_frac=0.2)


@pytest.mark.parametrize("precision", [32, 64])
def test_plain_tunings_are_bit_identical(gpu, data, precision):
    ref = run(data, precision=precision)
    variants = [dict(sort_variant=2), dict(es_warps=8, es_stage=1), dict(es_warps=16, es_stage=0),
                dict(es_warps=32, es_stage=0)]
    if precision == 32:
        variants += [dict(metric_pb=4), dict(sort_variant=1)]
    for v in variants:
        got = run(data, precision=precision, **v)
        for a, b in zip(ref, got):
            assert same(a, b), v


def test_tensor_core_tiles_are_bit_identical(gpu, data):
    ref = run(data, form=N.FORM_CHOSEN, chosen_tile=256)
    got = run(data, form=N.FORM_CHOSEN, chosen_tile=128)
    for a, b in zip(ref, got):
        assert same(a, b)


@pytest.mark.parametrize("G,S,P", [(130, 7, 1), (257, 33, 129), (1000, 200, 300), (5000, 11, 2000)])
@pytest.mark.parametrize("form", [N.FORM_CHOSEN, N.FORM_CHOSEN_FP64])
def test_persistent_tensor_core_kernel_on_ragged_shapes(gpu, G, S, P, form):
    """The persistent warp-specialised class statistics (the 128-permutation
    tile: tiles of 128 genes x 128 permutations walked by one CTA per SM,
    copies, MMAs and epilogue on separate warps) against the one-tile kernel
    of the 256-permutation tile: partial gene and permutation tiles, a single
    permutation, more tiles than SMs, K chunks not filled by the samples."""
    d = synthetic.make(G, S, 5, P, seed=G + S, n_class_b=max(1, S // 3), set_min=1, set_max=min(60, G))
    ref = run(d, form=form, chosen_tile=256)
    got = run(d, form=form, chosen_tile=128)
    for a, b in zip(ref, got):
        assert same(a, b)


def test_invalid_tuning_is_rejected(gpu, data):
    plan = api.Plan(data.num_genes, data.num_samples, data.num_sets, 64, 8)
    with pytest.raises(N.GseaError):
        plan.set_tuning(es_warps=12)
    with pytest.raises(N.GseaError):
        plan.set_tuning(chosen_tile=64)
    # fp64 keys take the register sort up to 20,480 genes (one CTA, then a
    # two-CTA cluster), not beyond
    big = synthetic.make(20481, 8, 3, 4, seed=3, n_class_b=4)
    p64 = api.Plan(big.num_genes, big.num_samples, big.num_sets, 4, 8, precision=64)
    p64.set_tuning(sort_variant=1)
    p64.set_inputs(big.exprs, big.labels, big.set_offsets, big.set_genes)
    with pytest.raises(N.GseaError):
        p64.execute()
        p64.synchronize()
    plan.close()
    p64.close()


def test_fp64_register_sort_equals_tiled(gpu, data):
    """fp64 at this size: the register / cluster sort (variant 1) and the
    tiled sort (variant 2) give the same ranks, hence the same ES bit for bit."""
    out = []
    for v in (1, 2):
        plan = api.Plan(data.num_genes, data.num_samples, data.num_sets, data.num_perms, 8, precision=64)
        plan.set_tuning(sort_variant=v)
        plan.set_inputs(data.exprs, data.labels, data.set_offsets, data.set_genes)
        plan.execute()
        out.append(plan.read())
        plan.close()
    assert np.array_equal(out[0][0].view(np.uint64), out[1][0].view(np.uint64))
    assert np.array_equal(out[0][1].view(np.uint64), out[1][1].view(np.uint64))


@pytest.mark.parametrize("form", [N.FORM_PLAIN, N.FORM_CHOSEN])
def test_autotune_keeps_results(gpu, data, form):
    ref = run(data, form=form)
    plan = api.Plan(data.num_genes, data.num_samples, data.num_sets, data.num_perms, "twopass_signal2noise",
                    form=form)
    plan.set_debug(True)
    plan.set_inputs(data.exprs, data.labels, data.set_offsets, data.set_genes)
    best, ms = plan.autotune(128)
    assert best["es_warps"] in (8, 16, 24, 32) and best["es_stage"] in (0, 1, 2, 3)
    assert best["sort_variant"] in (1, 2)
    assert (best["chosen_tile"] in (128, 256)) if form == N.FORM_CHOSEN else (best["metric_pb"] in (4, 8))
    assert all(v > 0 for v in ms.values())
    assert plan.get_tuning() == best
    plan.execute()
    es, st = plan.read()
    assert same(es, ref[1]) and same(st, ref[2])
    plan.close()


def test_graph_replay_matches_direct_launches(gpu, data):
    """An execute is captured into a CUDA graph and replayed (profiling off);
    replays, re-captures after a tuning change and direct launches (profiling
    on) all give the same results bit for bit."""
    import torch
    plan = api.Plan(data.num_genes, data.num_samples, data.num_sets, data.num_perms, "twopass_signal2noise")
    plan.set_inputs(data.exprs, data.labels, data.set_offsets, data.set_genes)
    outs = []
    plan.execute()
    outs.append(plan.read())
    s = torch.cuda.Stream()
    plan.execute(s.cuda_stream)  # replay on another stream
    outs.append(plan.read())
    plan.set_tuning(es_warps=16)  # re-capture
    plan.execute()
    outs.append(plan.read())
    plan.set_profiling(True)      # direct launches
    plan.execute()
    outs.append(plan.read())
    assert plan.last_launches() > 5
    plan.close()
    for es, st in outs[1:]:
        assert same(es, outs[0][0]) and same(st, outs[0][1])


@pytest.mark.parametrize("precision", [32, 64])
def test_large_g_enrichment_stagings_identical(precision):
    """24,000 genes (24 bitmap words per lane): every enrichment launch that
    fits -- ranks and weights staged at 16 warps, weights only or ranks only
    at 32 / 24 (/ 16) warps, nothing staged at 32 / 24 warps -- gives the
    automatic choice's ES bit for bit."""
    d = synthetic.make(24000, 24, 40, 16, seed=5, n_class_b=12, n_shift=200, set_min=15, set_max=400)
    _, es0, st0 = run(d, precision=precision)
    configs = [(16, 1), (32, 3), (24, 3), (32, 2), (24, 2), (16, 2), (32, 0), (24, 0)]
    ran = 0
    for w, stage in configs:
        try:
            _, es, st = run(d, precision=precision, es_warps=w, es_stage=stage)
        except N.GseaError:
            # fp64 staging of 24,000 weights (192 KB) does not fit beside 32 bitmaps
            assert precision == 64 and stage in (1, 3), (w, stage)
            continue
        assert same(es, es0), (w, stage)
        assert same(st, st0), (w, stage)
        ran += 1
    assert ran == (8 if precision == 32 else 5), ran
