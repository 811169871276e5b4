"""The learned permutation allocator on the GPU: the network's kernels against
the numpy oracle (loss, gradient, prediction), its training on null scores
the permutation kernels produce, the ragged statistics, and the adaptive test
judged against the full permutation test (bit-identical scores for every
permutation a set received; the same calls at FDR < 0.25 except sets whose
full-test q lies within 0.03 of the level)."""
import numpy as np
import pytest

from cudagsea_gb300 import allocator, api, synthetic
from cudagsea_gb300 import _native as N
from oracle import model as M
from tests.test_model_oracle import random_problem

pytestmark = pytest.mark.gpu

Q_CALL = 0.25
Q_BAND = 0.03
P_MAX = 4000
QUERIES = 24


def f32(a):
    return np.ascontiguousarray(a, np.float32)


def test_model_loss_gradient_and_prediction_match_oracle(gpu):
    p, norms, x, t = random_problem(rows=1000, seed=11)  # 1000 rows: a partial last tile
    p, norms, x, t = f32(p), f32(norms), f32(x), f32(t)
    m = allocator.Model(seed=1)
    m.set(p, norms)
    g, l = m.loss_grad(x, t)
    lo, go = M.loss_grad(M.bf16(p), norms, x, t)
    assert abs(l - lo) <= 2e-6 * abs(lo) + 1e-7
    scale = np.abs(go).max()
    assert np.abs(g - go).max() <= 1e-4 * scale, np.abs(g - go).max() / scale
    # every parameter block, relative to its own size
    for a, b in ((M.OFF_W1, M.OFF_B1), (M.OFF_B1, M.OFF_W2), (M.OFF_W2, M.OFF_B2), (M.OFF_B2, M.OFF_W3),
                 (M.OFF_W3, M.OFF_B3), (M.OFF_B3, M.NPARAM)):
        blk = np.abs(go[a:b]).max()
        assert np.abs(g[a:b] - go[a:b]).max() <= 1e-4 * blk + 1e-7, (a, b)
    y = m.predict(x).cpu().numpy()
    yo = M.predict(p, norms, x)
    np.testing.assert_allclose(y, yo, rtol=1e-4, atol=1e-6)
    # the master parameters are FP32, the computing copies BF16
    assert np.array_equal(m.get()[0], p)
    m.close()


def case(seed, K=400):
    return synthetic.make(3000, 60, K, P_MAX, seed=seed, n_class_b=30, sd_range=(0.5, 2.5), n_shift=150,
                          shift_range=(0.2, 0.8), set_min=15, set_max=250, enriched_frac=0.1)


def full_run(d, P=P_MAX):
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P, "twopass_signal2noise")
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es, st = plan.read()
    return plan, es, st.reshape(5, -1)


_MODEL = {}


def trained_model():
    """A model trained on the null scores of a calibration data set (another
    seed of the same shape) by the library's own kernels."""
    if "m" not in _MODEL:
        plan, _, _ = full_run(case(seed=901))
        x, t, xv, tv = allocator.model_samples(plan, queries=QUERIES, holdout=10)
        m = allocator.Model(seed=5)
        curve = m.train(x, t, steps=3000, batch=4096, lr=3e-3)
        sig = m.calibrate(xv, tv)
        _MODEL["m"], _MODEL["curve"], _MODEL["sig"] = m, curve, sig
        _MODEL["samples"] = (x.cpu().numpy(), t.cpu().numpy(), plan.read()[0], plan)
    return _MODEL["m"]


def test_training_samples_follow_their_definition(gpu):
    trained_model()
    x, t, es, plan = _MODEL["samples"]
    d = case(seed=901)
    sizes = np.diff(d.set_offsets)
    q = QUERIES
    for k in (0, 1, 5, 12):  # training sets (k % 10 != 9): rows k - k // 10 ...
        r0 = (k - k // 10) * (q + 1)
        a = np.abs(es[k].astype(np.float64))
        m = a.mean()
        assert np.isclose(t[r0, 1], np.log(m), rtol=1e-6)
        for j in (0, 3, q - 1):
            f = M.query_factor(k, j, q)
            assert 0.25 <= f < 9.0
            assert np.isclose(x[r0 + j, 1], f, rtol=1e-6)
            assert t[r0 + j, 0] == np.float32(np.count_nonzero(a >= m * f) / a.size)
        assert t[r0 + q, 0] == np.float32(np.count_nonzero(a >= a[0]) / a.size)
        assert np.isclose(x[r0 + q, 1], a[0] / m, rtol=1e-6)
        assert np.isclose(x[r0, 0], np.log(sizes[k]), rtol=1e-6)


def test_training_lowers_loss_and_calibrates(gpu):
    trained_model()
    curve, (s_tail, s_mean) = _MODEL["curve"], _MODEL["sig"]
    assert np.all(np.isfinite(curve))
    assert curve[-100:].mean() < 0.75 * curve[:20].mean()
    # held-out sets: tail within ~0.3 logit, null mean within ~5 %
    assert s_tail < 0.3, s_tail
    assert s_mean < 0.05, s_mean


def test_ragged_statistics_match_oracle(gpu):
    import torch
    rs = np.random.RandomState(7)
    K, ld = 37, 900
    es = rs.normal(0, 0.3, (K, ld)).astype(np.float32)
    es[:, 0] += rs.normal(0, 0.6, K).astype(np.float32)
    es[5, 0] = np.nan  # a set without hits
    counts = rs.randint(40, ld + 1, K).astype(np.int64)
    counts[0] = ld
    p_fwer = int(counts.min())
    got = allocator.stats_ragged(torch.as_tensor(es).cuda(), counts, p_fwer).cpu().numpy().reshape(5, -1)
    ref = M.stats_ragged(es, counts, p_fwer).reshape(5, -1)
    assert np.array_equal(np.isnan(got), np.isnan(ref))
    ok = ~np.isnan(ref)
    assert np.array_equal(got[:4][ok[:4]].view(np.uint32), ref[:4][ok[:4]].view(np.uint32))
    np.testing.assert_allclose(got[4], ref[4], rtol=1e-6)
    # full counts: the ragged form is the dense one, bit for bit
    d = synthetic.small(num_perms=512)
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, 512, 8)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es_d, st_d = plan.read()
    got = allocator.stats_ragged(torch.as_tensor(es_d).cuda(), np.full(d.num_sets, 512), 512).cpu().numpy()
    assert np.array_equal(got.view(np.uint32), st_d.view(np.uint32))


def check_against_full(d, res, es_full, st_full, plan):
    es_a, st_a = plan.read()
    st_a = st_a.reshape(5, -1)
    counts = res.counts
    assert counts.min() >= 250 and counts.max() <= d.num_perms
    # every score a set received is the full run's score of that permutation
    for k in range(d.num_sets):
        assert np.array_equal(es_a[k, :counts[k]].view(np.uint32), es_full[k, :counts[k]].view(np.uint32)), k
    # sets run to completion: ES, NES, NP identical to the full test
    full = counts == d.num_perms
    assert full.any()
    for r in (0, 1, 2):
        assert np.array_equal(st_a[r, full].view(np.uint32), st_full[r, full].view(np.uint32))
    # the calls at FDR < 0.25 are the full test's outside the FDR estimator's
    # noise band: a stopped set adds only its own permutations to the pooled
    # null, which moves the q-values of the other sets by a few per cent
    calls_full = set(np.where(st_full[4] < Q_CALL)[0])
    calls = set(np.where(st_a[4] < Q_CALL)[0])
    assert calls_full
    flips = sorted(calls ^ calls_full)
    for k in flips:
        assert abs(st_full[4][k] - Q_CALL) <= Q_BAND, (k, st_full[4][k], st_a[4][k])
    assert len(flips) <= max(1, d.num_sets // 100), flips
    # every called set ran the full test or stopped as clearly significant
    short_calls = [k for k in sorted(calls) if counts[k] < d.num_perms]
    assert len(short_calls) <= res.report["stopped_sig"], (short_calls, res.report)
    return res.report["scores"]


def test_adaptive_without_model_matches_full_test(gpu):
    d = case(seed=77)
    plan_f, es_f, st_f = full_run(d)
    plan_f.close()
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P_MAX, "twopass_signal2noise")
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    res = allocator.execute_adaptive(plan, None, pilot_perms=250)
    assert res.report["model_used"] == 0
    scores = check_against_full(d, res, es_f, st_f, plan)
    assert scores < 0.8 * d.num_sets * P_MAX
    assert res.report["scores"] == int(res.counts.sum())
    assert res.report["stopped_pilot"] > 0


def test_learned_prior_saves_permutations_with_identical_calls(gpu):
    """What the trained network gains: the same calls as the full test and as
    the rule without it, with fewer enrichment scores computed."""
    m = trained_model()
    d = case(seed=77)
    plan_f, es_f, st_f = full_run(d)
    plan_f.close()
    out = {}
    for name, model in (("empirical", None), ("learned", m)):
        plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P_MAX, "twopass_signal2noise")
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        res = allocator.execute_adaptive(plan, model, pilot_perms=250)
        out[name] = (check_against_full(d, res, es_f, st_f, plan), res.report)
        plan.close()
    assert out["learned"][1]["model_used"] == 1
    assert out["learned"][1]["model_mean_err"] < 0.1
    assert out["learned"][0] < out["empirical"][0], out
    assert out["learned"][1]["stopped_pilot"] > out["empirical"][1]["stopped_pilot"]


def test_model_fallback_on_mismatched_model(gpu):
    """A model whose null means are far off is dropped: the run is the
    empirical rule's, call for call and count for count."""
    m = trained_model()
    p, n = m.get()
    bad = allocator.Model(seed=2)
    n2 = n.copy()
    n2[10] += 3.0  # every predicted null mean x e^3
    bad.set(p, n2)
    d = case(seed=77)
    counts = {}
    for name, model in (("none", None), ("bad", bad)):
        plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P_MAX, "twopass_signal2noise")
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        res = allocator.execute_adaptive(plan, model, pilot_perms=250)
        counts[name] = (res.counts, res.report)
        plan.close()
    assert counts["bad"][1]["model_used"] == 0
    assert counts["bad"][1]["model_mean_err"] > 2.0
    assert np.array_equal(counts["bad"][0], counts["none"][0])


def test_adaptive_with_pilot_covering_every_permutation_is_the_full_test(gpu):
    """pilot >= num_perms: one round, every set full -- the statistics are the
    dense statistics bit for bit (FWER over all permutations, unit FDR weights)."""
    d = synthetic.small(num_perms=512)
    plan_f = api.Plan(d.num_genes, d.num_samples, d.num_sets, 512, 8)
    plan_f.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan_f.execute()
    es_f, st_f = plan_f.read()
    plan_f.close()
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, 512, 8)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    res = allocator.execute_adaptive(plan, None, pilot_perms=2000)
    es, st = plan.read()
    plan.close()
    assert res.report["rounds"] == 1 and np.all(res.counts == 512)
    assert np.array_equal(es.view(np.uint32), es_f.view(np.uint32))
    assert np.array_equal(st.view(np.uint32), st_f.view(np.uint32))


def test_adaptive_single_set_and_invalid_parameters(gpu):
    d = synthetic.make(500, 20, 1, 300, seed=9, n_class_b=10, set_min=30, set_max=60)
    plan = api.Plan(d.num_genes, d.num_samples, 1, 300, 8)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    res = allocator.execute_adaptive(plan, None, pilot_perms=50)
    assert 50 <= res.counts[0] <= 300
    with pytest.raises(N.GseaError):
        allocator.execute_adaptive(plan, None, pilot_perms=1)
    with pytest.raises(N.GseaError):
        allocator.execute_adaptive(plan, None, growth=1.0)
    plan.close()


def test_fdr_bound_matches_oracle(gpu):
    """gsea_fdr_lower_bound against the numpy restatement: ragged counts,
    z = 0 (the FDR q itself) and z = 3."""
    import torch
    rs = np.random.RandomState(3)
    K, ld = 40, 300
    es = rs.normal(0, 0.3, (K, ld)).astype(np.float32)
    es[:, 0] += rs.normal(0, 0.6, K).astype(np.float32)
    counts = rs.randint(50, ld + 1, K).astype(np.int64)
    counts[0] = ld
    a = np.abs(es.astype(np.float64))
    sums = np.concatenate([[a[k, :counts[k]].sum() for k in range(K)],
                           [(a[k, :counts[k]] ** 2).sum() for k in range(K)]])
    p_fwer = int(counts.min())
    for dt in (np.float32, np.float64):
        e = es.astype(dt)
        for z in (0.0, 3.0):
            st, q = allocator.fdr_lower_bound(torch.as_tensor(e).cuda(), counts, p_fwer, sums, z)
            st_o, q_o = M.fdr_bound(e, counts, p_fwer, sums, z, dtype=dt)
            np.testing.assert_allclose(q.cpu().numpy(), q_o, rtol=1e-5, atol=1e-7)
            if z == 0.0:
                np.testing.assert_allclose(q.cpu().numpy(), st.cpu().numpy().reshape(5, -1)[4], rtol=1e-6)


def test_fdr_rule_saves_scores_with_the_full_tests_calls(gpu):
    """Stopping sets whose FDR q is clearly above the call level: the full
    test's calls, fewer scores than the p rule alone."""
    d = case(seed=77)
    plan_f, es_f, st_f = full_run(d)
    plan_f.close()
    scores, reports = {}, {}
    for qm in (0.0, 1.5):
        plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P_MAX, "twopass_signal2noise")
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        res = allocator.execute_adaptive(plan, None, pilot_perms=250, q_margin=qm)
        scores[qm] = check_against_full(d, res, es_f, st_f, plan)
        reports[qm] = res.report
        plan.close()
    assert reports[0.0]["stopped_q"] == 0
    assert reports[1.5]["stopped_q"] > 0
    assert scores[1.5] < scores[0.0], scores


def test_adaptive_double_precision_matches_full_test(gpu):
    """doublePrecision: the adaptive test (both rules) in FP64 -- every score a
    set received is the full FP64 run's, sets run to completion keep their
    ES / NES / NP, and the calls are the full test's outside the band."""
    d = case(seed=91, K=200)
    x = d.exprs.astype(np.float64)
    full = api.Plan(d.num_genes, d.num_samples, d.num_sets, P_MAX, "twopass_signal2noise", precision=64)
    full.set_inputs(x, d.labels, d.set_offsets, d.set_genes)
    full.execute()
    es_f, st_f = full.read()
    st_f = st_f.reshape(5, -1)
    full.close()
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P_MAX, "twopass_signal2noise", precision=64)
    plan.set_inputs(x, d.labels, d.set_offsets, d.set_genes)
    res = allocator.execute_adaptive(plan, None, pilot_perms=250)
    es_a, st_a = plan.read()
    st_a = st_a.reshape(5, -1)
    plan.close()
    counts = res.counts
    assert counts.min() >= 250 and counts.max() <= P_MAX and res.report["scores"] < d.num_sets * P_MAX
    for k in range(d.num_sets):
        assert np.array_equal(es_a[k, :counts[k]].view(np.uint64), es_f[k, :counts[k]].view(np.uint64)), k
    fullk = counts == P_MAX
    for r in (0, 1, 2):
        assert np.array_equal(st_a[r, fullk].view(np.uint64), st_f[r, fullk].view(np.uint64))
    calls_f = set(np.where(st_f[4] < Q_CALL)[0])
    calls = set(np.where(st_a[4] < Q_CALL)[0])
    for k in sorted(calls ^ calls_f):
        assert abs(st_f[4][k] - Q_CALL) <= Q_BAND, (k, st_f[4][k], st_a[4][k])
    short_calls = [k for k in sorted(calls) if counts[k] < P_MAX]
    assert len(short_calls) <= res.report["stopped_sig"], (short_calls, res.report)


def test_adaptive_graph_replays_and_matches_the_host_rule(gpu):
    """The adaptive test runs as one captured CUDA graph: the decisions are
    kernels, the set counts read on the device.  A replay gives the same
    counts and statistics bit for bit, a parameter change records a new graph,
    and the final decisions equal the host-side rule (gsea_adaptive_decide)
    applied to the final counts and exceedances."""
    d = case(seed=91)
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P_MAX, "twopass_signal2noise")
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    a = allocator.execute_adaptive(plan, None, pilot_perms=250, q_margin=0.0, sig_margin=0.0)
    st_a = plan.read(es=False)[1]
    b = allocator.execute_adaptive(plan, None, pilot_perms=250, q_margin=0.0, sig_margin=0.0)
    st_b = plan.read(es=False)[1]
    assert np.array_equal(a.counts, b.counts)
    assert all(a.report[k] == b.report[k] or (a.report[k] != a.report[k] and b.report[k] != b.report[k])
               for k in a.report)  # NaN (no model error) on both sides counts as equal
    assert np.array_equal(st_a.view(np.uint32), st_b.view(np.uint32))
    c = allocator.execute_adaptive(plan, None, pilot_perms=500, q_margin=0.0, sig_margin=0.0)
    assert c.counts.min() >= 500 and not np.array_equal(c.counts, a.counts)
    a2 = allocator.execute_adaptive(plan, None, pilot_perms=250, q_margin=0.0, sig_margin=0.0)
    assert np.array_equal(a2.counts, a.counts)
    # the host rule on the final state: every set that stopped short of P_MAX
    # is one the rule stops, given the run's own stop_p
    es, _ = plan.read(stats=False)
    exceed = np.array([int(np.sum(np.abs(es[k, :a.counts[k]]) >= np.abs(es[k, 0]))) for k in range(d.num_sets)])
    stop = allocator.decide(a.counts, exceed, a.report["stop_p"])
    short = a.counts < P_MAX
    assert np.all(stop[short] == 1)
    plan.close()


def test_significance_rule_saves_scores_with_the_full_tests_calls(gpu):
    """Stopping sets whose q is clearly below the call level (and whose p is
    clearly below every pilot non-call's): the full test's calls, strictly
    fewer scores than without the rule, every early-stopped call counted in
    the report; with the learned prior on top, the calls stay the full
    test's.  16,000 permutations and strongly enriched sets (whose pilot
    sees no null above them): the rule acts on the Jeffreys posterior alone
    after a few rounds."""
    P = 16000
    d = synthetic.make(3000, 60, 400, P, seed=77, n_class_b=30, sd_range=(0.5, 2.5), n_shift=150,
                       shift_range=(0.8, 1.5), set_min=15, set_max=250, enriched_frac=0.1)
    plan_f, es_f, st_f = full_run(d, P)
    plan_f.close()
    scores, reports = {}, {}
    for name, sm, model in (("off", 0.0, None), ("on", 2.0, None), ("learned", 2.0, trained_model())):
        plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P, "twopass_signal2noise")
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        res = allocator.execute_adaptive(plan, model, pilot_perms=250, sig_margin=sm)
        scores[name] = check_against_full(d, res, es_f, st_f, plan)
        reports[name] = res.report
        plan.close()
    assert reports["off"]["stopped_sig"] == 0 and reports["off"]["p_sig"] == 0.0
    assert reports["on"]["stopped_sig"] > 0 and reports["on"]["p_sig"] > 0.0
    assert scores["on"] < scores["off"], scores


def test_learned_allocator_at_full_scale(gpu):
    """The allocator workload itself: 20,000 genes x 200 samples, 20,000 sets
    (5 % enriched, the rest null), up to 100,000 permutations per set, the
    network trained on a 2,000-set calibration run.  Judged against the full
    tensor-core test: the same FDR < 0.25 calls (flips only within the
    estimator's band), ES / NES / NP bit-identical for every set that ran all
    permutations, every score a sampled set received equal to the full test's
    score of that permutation, and the learned prior computing fewer scores
    than the same rules without it."""
    from cudagsea_gb300.precision_check import _DeviceRows
    d = synthetic.learned()
    K, P = d.num_sets, d.num_perms
    full = api.Plan(d.num_genes, d.num_samples, K, P, "twopass_signal2noise", form=N.FORM_CHOSEN)
    full.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    full.execute()
    st_f = full.read(es=False)[1].reshape(5, -1)
    rows_f = _DeviceRows(full, N.BUF_ES, np.float32, P)
    cal = synthetic.learned(seed=6262, num_sets=2000, num_perms=4000)
    cp = api.Plan(cal.num_genes, cal.num_samples, cal.num_sets, cal.num_perms, "twopass_signal2noise",
                  form=N.FORM_CHOSEN)
    cp.set_inputs(cal.exprs, cal.labels, cal.set_offsets, cal.set_genes)
    cp.execute()
    model, _ = allocator.train_model(cp, seed=5, queries=24, steps=3000)
    cp.close()
    calls_full = set(np.where(st_f[4] < Q_CALL)[0])
    assert len(calls_full) > 100
    sample = np.random.RandomState(3).choice(K, 300, replace=False)
    reports = {}
    for name, m in (("rules", None), ("learned", model)):
        plan = api.Plan(d.num_genes, d.num_samples, K, P, "twopass_signal2noise", form=N.FORM_CHOSEN)
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        res = allocator.execute_adaptive(plan, m, pilot_perms=1000)
        st_a = plan.read(es=False)[1].reshape(5, -1)
        counts = res.counts
        assert counts.min() >= 1000 and counts.max() <= P
        calls = set(np.where(st_a[4] < Q_CALL)[0])
        flips = sorted(calls ^ calls_full)
        for k in flips:
            assert abs(st_f[4][k] - Q_CALL) <= Q_BAND, (name, k, st_f[4][k], st_a[4][k])
        assert len(flips) <= K // 100, (name, flips)
        done = counts == P
        assert done.any()
        for r in (0, 1, 2):
            assert np.array_equal(st_a[r, done].view(np.uint32), st_f[r, done].view(np.uint32)), (name, r)
        got = _DeviceRows(plan, N.BUF_ES, np.float32, P).rows(sample)
        ref = rows_f.rows(sample)
        for i, k in enumerate(sample):
            n = counts[k]
            assert np.array_equal(got[i, :n].view(np.uint32), ref[i, :n].view(np.uint32)), (name, k)
        short_calls = [k for k in sorted(calls) if counts[k] < P]
        assert len(short_calls) <= res.report["stopped_sig"], (name, res.report)
        assert res.report["scores"] < 0.1 * K * P, (name, res.report)
        reports[name] = res.report
        plan.close()
    model.close()
    full.close()
    assert reports["learned"]["model_used"] == 1
    assert reports["learned"]["scores"] < reports["rules"]["scores"], reports
