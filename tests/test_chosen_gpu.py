"""The chosen form: class statistics as tcgen05 tensor-core GEMMs.

Its keys are the metric of the fp32 inputs computed with higher internal
precision than the reference's own summation order, so it is judged against
the FP64 oracle: keys to 2e-5 relative, NES to 1e-4, and every difference in
the rank order must be between near-tied genes."""
import numpy as np
import pytest

import oracle
from cudagsea_gb300 import api, synthetic
from cudagsea_gb300 import _native as N
from tests import helpers as H
from tests.golden import make_golden as MG

pytestmark = pytest.mark.gpu

KEY_RTOL = 1e-4
NES_ATOL = 1e-4


def chosen_run(d, metric, P=None, debug=True, form=N.FORM_CHOSEN):
    P = P or d.num_perms
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P, metric, precision=32, form=form)
    if debug:
        plan.set_debug(True)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es, st = plan.read()
    out = {"es": es, "stats": st}
    if debug:
        out["keys"] = plan.read_buffer(N.BUF_KEYS, np.float32, (plan.perm_batch, d.num_genes))
        out["order"] = plan.read_buffer(N.BUF_ORDER, np.uint32, (plan.perm_batch, d.num_genes))
    plan.close()
    return out


def key_close(k, k64):
    """Relative to the key, with a floor of 5% of the permutation's largest
    |key|: FP32 accumulation leaves an absolute error of ~1e-6 on keys of
    order one, so keys near zero are compared on the row's scale."""
    k = k.astype(np.float64)
    scale = np.maximum(np.abs(k64), np.abs(k64).max(axis=1, keepdims=True) * 0.05)
    return np.abs(k - k64) <= KEY_RTOL * scale


def flips_are_near_ties(keys64, order_a, order_b, rel=1e-4):
    """Positions where two rank orders differ hold genes whose FP64 keys are close."""
    P, G = order_a.shape
    bad = 0
    for p in range(P):
        diff = np.flatnonzero(order_a[p] != order_b[p])
        if diff.size == 0:
            continue
        ka = keys64[p, order_a[p, diff]]
        kb = keys64[p, order_b[p, diff]]
        tol = rel * np.maximum(np.abs(keys64[p]).max(), 1e-12)
        bad += int(np.sum(np.abs(ka - kb) > tol))
    return bad


@pytest.mark.parametrize("form", [N.FORM_CHOSEN, N.FORM_CHOSEN_FP64], ids=["fp32eft", "fp64"])
@pytest.mark.parametrize("metric", [0, 1, 2, 6, 8, 9, 12])
def test_chosen_keys_match_fp64(gpu, metric, form):
    d = MG.metrics_case()
    r = chosen_run(d, metric, form=form)
    k64 = oracle.metric(metric, d.exprs.astype(np.float64), d.labels, d.num_perms, double=True)
    ok = key_close(r["keys"], k64)
    assert ok.all(), (metric, np.abs(r["keys"] - k64)[~ok][:5])


@pytest.mark.parametrize("shape", [(37, 5, 3, 3), (300, 16, 10, 40), (1000, 77, 12, 300), (20000, 200, 50, 64)])
def test_chosen_sizes(gpu, shape):
    G, S, K, P = shape
    d = synthetic.make(G, S, K, P, seed=G + S, n_class_b=S // 2, set_min=min(3, G), set_max=min(60, G))
    r = chosen_run(d, 8)
    k64 = oracle.metric(8, d.exprs.astype(np.float64), d.labels, P, double=True)
    assert key_close(r["keys"], k64).all(), np.abs(r["keys"] - k64).max()
    _, o64 = oracle.sort(k64)
    assert flips_are_near_ties(k64, r["order"], o64) == 0


@pytest.mark.parametrize("form", [N.FORM_CHOSEN, N.FORM_CHOSEN_FP64], ids=["fp32eft", "fp64"])
def test_chosen_pipeline_vs_fp64_oracle(gpu, form):
    """2,000 x 40, 50 sets, 1,024 permutations: |dNES| <= 1e-4 against FP64."""
    d = synthetic.small()
    r = chosen_run(d, 8, debug=False, form=form)
    es64, st64 = oracle.gsea(8, d.exprs.astype(np.float64), d.labels, d.set_offsets, d.set_genes, d.num_perms,
                             double=True)
    K = d.num_sets
    dnes = np.abs(r["stats"][K:2 * K].astype(np.float64) - st64[K:2 * K])
    assert dnes.max() <= NES_ATOL, dnes.max()
    des = np.abs(r["es"].astype(np.float64) - es64)
    assert np.median(des) < 1e-5
