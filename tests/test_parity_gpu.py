"""Parity of the CUDA path (through the C ABI) with the oracle and with the
reference's golden outputs.  Stage by stage:

  permutations   label masks == oracle permutations (bit-exact)
  metric         keys == oracle keys bit-exact (log2 metrics: <= 2 ulp);
                 == the reference's keys (SHA-256 of the golden fixture)
  sort           order == oracle's stable order of the GPU's own keys; ranks
                 are its inverse; sorted weights == |keys| in that order
  ES             within 1e-5 relative (fp32) / 1e-12 (fp64) of the oracle's
                 dense Kahan running sum over the same order
  statistics     bit-identical to the oracle's final_statistics + FDR for
                 the GPU's own ES
"""
import os

import numpy as np
import pytest

import oracle
from cudagsea_gb300 import api, synthetic
from cudagsea_gb300 import _native as N
from tests import helpers as H
from tests.golden import make_golden as MG

pytestmark = pytest.mark.gpu


def run_plan(d, metric, double=False, P=None, perm_offset=0, perm_batch=0, ascending=False, debug=True,
             tuning=None):
    P = P or d.num_perms
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P, metric, precision=64 if double else 32,
                    ascending=ascending, perm_offset=perm_offset, perm_batch=perm_batch)
    if tuning:
        plan.set_tuning(**tuning)
    if debug:
        plan.set_debug(True)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es, st = plan.read()
    out = {"es": es, "stats": st, "plan": plan}
    if debug:
        pb, G = plan.perm_batch, d.num_genes
        dt = plan.dtype
        out["keys"] = plan.read_buffer(N.BUF_KEYS, dt, (pb, G))
        out["order"] = plan.read_buffer(N.BUF_ORDER, np.uint32, (pb, G))
        out["ranks"] = plan.read_buffer(N.BUF_RANKS, np.uint16 if plan.ranks16 else np.uint32, (pb, G))
        out["sorted"] = plan.read_buffer(N.BUF_SORTED, dt, (pb, G))
        words = (d.num_samples + 31) // 32
        out["masks"] = plan.read_buffer(N.BUF_LABEL_MASKS, np.uint32, (pb, words))
    return out


def decode_masks(masks, S):
    bits = np.unpackbits(masks.view(np.uint8), bitorder="little").reshape(masks.shape[0], -1)[:, :S]
    return np.where(bits == 1, 0, 1).astype(np.uint8)  # bit set = class A = label 0


def check_sort(keys, order, ranks, sorted_abs, ascending=False):
    sk, ref_order = oracle.sort(keys, ascending=ascending)
    np.testing.assert_array_equal(order, ref_order)
    P, G = keys.shape
    inv = np.empty_like(order)
    inv[np.arange(P)[:, None], order] = np.arange(G, dtype=order.dtype)[None, :]
    np.testing.assert_array_equal(ranks.astype(np.uint32), inv)
    np.testing.assert_array_equal(sorted_abs, np.where(sk < 0, -sk, sk))
    return sk, ref_order


def test_permutation_masks(gpu):
    g = H.load("perm_labels.npz")
    labels = g["labels"]
    S = labels.size
    d = synthetic.make(64, S, 2, 17, seed=5, n_class_b=int(labels.sum()))
    d.labels = labels
    r = run_plan(d, "naive_diff_of_classes")
    np.testing.assert_array_equal(decode_masks(r["masks"], S), g["perm_labels"])
    # counter-based stream: a shifted plan reproduces the same global permutations
    r2 = run_plan(d, "naive_diff_of_classes", P=8, perm_offset=1000)
    np.testing.assert_array_equal(decode_masks(r2["masks"], S), oracle.perm_labels(labels, 8, shift=1000))


@pytest.mark.parametrize("double", [False, True], ids=["f32", "f64"])
def test_all_metrics_stagewise(gpu, double):
    g = H.load(f"metrics_{'f64' if double else 'f32'}.npz")
    d = MG.metrics_case()
    for m in range(14):
        name = api.METRICS[m]
        r = run_plan(d, m, double=double)
        ok = oracle.metric(m, d.exprs, d.labels, d.num_perms, double=double)
        if m in H.LOG_METRICS:
            assert H.ulp_diff(r["keys"], ok).max() <= 2, name
        else:
            np.testing.assert_array_equal(r["keys"].view(np.uint8), ok.view(np.uint8), err_msg=name)
            assert H.sha(r["keys"]) == str(g[f"keys_sha_{m}"]), name
        sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"])
        es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
        assert H.es_close(r["es"], es_o, double).all(), (name, np.nanmax(np.abs(r["es"] - es_o)))
        st_o = oracle.stats(r["es"])
        np.testing.assert_array_equal(r["stats"].view(np.uint8), st_o.view(np.uint8), err_msg=name)
        # against the reference's own ES: equal within tolerance unless a tie
        # explains the difference (the reference CPU sort is unstable)
        ref_es = g[f"es_{m}"]
        for kk, p in np.argwhere(~H.es_close(r["es"], ref_es, double)):
            members = d.set_genes[d.set_offsets[kk]:d.set_offsets[kk + 1]]
            if m in H.LOG_METRICS:
                continue  # near-tie rank flips are allowed for the log metrics
            assert H.tie_explained(sk[p], order[p], members), (name, kk, p)


@pytest.mark.parametrize("double", [False, True], ids=["f32", "f64"])
def test_config1_vs_reference(gpu, double):
    """2,000 x 40, 50 sets, 1,024 permutations, twopass_signal2noise."""
    g = H.load(f"small_{'f64' if double else 'f32'}.npz")
    d = synthetic.small()
    es, st = api.gsea(d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, "twopass_signal2noise",
                      precision=64 if double else 32)
    K = d.num_sets
    assert H.es_close(es[:, :128], g["es_head"], double).mean() > 0.999
    ref = g["stats"]
    assert H.es_close(st[:K], ref[:K], double).all()          # ES
    assert H.es_close(st[K:2 * K], ref[K:2 * K], double).all()  # NES
    np.testing.assert_allclose(st[2 * K:4 * K], ref[2 * K:4 * K], atol=2.0 / d.num_perms)  # NP, FWER
    # the oracle on the GPU's ES reproduces the GPU's statistics bit for bit
    np.testing.assert_array_equal(oracle.stats(es).view(np.uint8), st.view(np.uint8))


@pytest.mark.parametrize("G", [30000, 50000])
@pytest.mark.parametrize("double", [False, True], ids=["f32", "f64"])
def test_large_genes_against_reference(gpu, G, double):
    """30,000 and 50,000 genes -- the two-CTA cluster sort (fp32, 30,000) and
    the tiled sort (the rest), the ES kernel's large size classes -- against
    the reference's own CPU build (fixtures written by make_golden.py from
    it): ES matrix, ES and NES within the tolerance, NP and FWER within 2/P."""
    g = H.load(f"large_{G}.npz")
    d = MG.large_case(G)
    assert MG.input_hash(d) == str(g["input_sha"])
    prec = "f64" if double else "f32"
    es, st = api.gsea(d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, "twopass_signal2noise",
                      precision=64 if double else 32)
    K = d.num_sets
    ref_es, ref = g[f"es_{prec}"], g[f"stats_{prec}"]
    # the reference's CPU sort is unstable: a member tied with a non-member may
    # take the other order in a rare permutation
    assert H.es_close(es, ref_es, double).mean() > 0.999
    assert H.es_close(st[:K], ref[:K], double).all()            # ES
    assert H.es_close(st[K:2 * K], ref[K:2 * K], double).all()  # NES
    np.testing.assert_allclose(st[2 * K:4 * K], ref[2 * K:4 * K], atol=2.0 / d.num_perms)  # NP, FWER


@pytest.mark.parametrize("double", [False, True], ids=["f32", "f64"])
def test_tie_heavy_data(gpu, double):
    g = H.load(f"ties_{'f64' if double else 'f32'}.npz")
    d = MG.ties_case()
    for m in (0, 8):
        r = run_plan(d, m, double=double)
        assert H.sha(r["keys"]) == str(g[f"keys_sha_{m}"])
        sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"])
        es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
        assert H.es_close(r["es"], es_o, double).all()


def test_tiny_shapes_all_metrics(gpu):
    d = synthetic.tiny()
    for double in (False, True):
        for m in range(14):
            r = run_plan(d, m, double=double)
            ok = oracle.metric(m, d.exprs, d.labels, d.num_perms, double=double)
            assert H.ulp_diff(r["keys"], ok).max() <= (2 if m in H.LOG_METRICS else 0)
            sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"])
            es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
            assert H.es_close(r["es"], es_o, double).all(), (m, double)


@pytest.mark.parametrize("G", [1, 31, 4097, 20480, 20481, 30000, 40000, 49152, 65536, 70000, 150001])
@pytest.mark.parametrize("double", [False, True], ids=["f32", "f64"])
def test_sort_sizes(gpu, G, double):
    """Register-resident sort up to 20,480 genes (fp32), two-CTA clusters up to
    40,960, tiled sort beyond and for fp64; the ES register procedure up to
    65,536 genes (partial staging above ~20,000); beyond, 32-bit ranks and the
    general two-walk procedure (16 warps at 70,000 genes, 8 at 150,001, whose
    last bitmap word is partly used)."""
    d = synthetic.make(G, 12, 3, 5, seed=G, n_class_b=6, n_shift=min(10, G), set_min=1, set_max=min(40, G))
    r = run_plan(d, "twopass_signal2noise", double=double)
    assert r["ranks"].dtype == (np.uint16 if G <= 65536 else np.uint32)
    sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"])
    es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
    assert H.es_close(r["es"], es_o, double).all()


@pytest.mark.parametrize("G", [4095, 4097, 8194, 12289, 41003])
@pytest.mark.parametrize("double", [False, True], ids=["f32", "f64"])
def test_tiled_sort_edge_keys(gpu, G, double):
    """The tiled sort (tiles of 4,096 keys staged in shared memory by bulk
    copies, one digit count for every pass) on tied, infinite and NaN keys,
    with tile boundaries and rows whose length is not a multiple of 4, and 160
    permutations so that each CTA sorts several permutations in turn: order,
    ranks and weights equal the oracle's stable sort, ES the oracle's."""
    d = synthetic.make(G, 10, 4, 160, seed=G, n_class_b=5, set_min=5, set_max=min(300, G))
    t = G // 3
    d.exprs[:, :t] = d.exprs[:, [t + 100]]  # a third of the genes tie
    d.exprs[:, t:t + 40] = 0.0              # 0 / 0
    d.exprs[:4, t + 40:t + 80] = 0.0        # zero means in some permutations' classes
    for metric in ("naive_ratio_of_classes", "twopass_signal2noise"):
        r = run_plan(d, metric, double=double, tuning=dict(sort_variant=2))
        sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"])
        es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
        assert H.es_close(r["es"], es_o, double).all(), metric


@pytest.mark.parametrize("G,double", [(41003, False), (8194, True)], ids=["f32", "f64"])
def test_tiled_sort_ascending(gpu, G, double):
    """The tiled sort in ascending order (the reference's `-order ascending`),
    ties and 160 permutations: the oracle's stable ascending order."""
    d = synthetic.make(G, 10, 4, 160, seed=G + 1, n_class_b=5, set_min=5, set_max=300)
    d.exprs[:, : G // 4] = d.exprs[:, [G // 2]]
    r = run_plan(d, "twopass_t_test", double=double, ascending=True, tuning=dict(sort_variant=2))
    sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"], ascending=True)
    es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
    assert H.es_close(r["es"], es_o, double).all()


@pytest.mark.parametrize("double", [False, True], ids=["f32", "f64"])
def test_tiled_sort_all_keys_equal(gpu, double):
    """Every gene identical: every radix digit is uniform, no pass moves a key,
    and the order is the identity (stable)."""
    d = synthetic.make(9000, 10, 3, 20, seed=4, n_class_b=5, set_min=5, set_max=200)
    d.exprs[:] = d.exprs[:, [0]]
    r = run_plan(d, "twopass_signal2noise", double=double, tuning=dict(sort_variant=2))
    sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"])
    assert (order == np.arange(d.num_genes)[None, :]).all()


def test_ascending_order(gpu):
    d = MG.metrics_case()
    r = run_plan(d, "twopass_t_test", ascending=True)
    sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"], ascending=True)
    es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
    assert H.es_close(r["es"], es_o, False).all()


def test_edge_sets(gpu):
    """Empty overlap, all genes, duplicates, out-of-range ids, single-gene sets."""
    d = synthetic.make(200, 10, 1, 16, seed=11, n_class_b=5)
    G = d.num_genes
    sets = [np.array([], np.int32), np.arange(G, dtype=np.int32), np.array([3, 3, 3, 7, 7], np.int32),
            np.array([-5, 10**6, 4], np.int32), np.array([0], np.int32), np.array([G - 1], np.int32)]
    d.set_offsets = np.r_[0, np.cumsum([s.size for s in sets])].astype(np.int64)
    d.set_genes = np.concatenate(sets).astype(np.int32)
    for double in (False, True):
        r = run_plan(d, "twopass_signal2noise", double=double)
        sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"])
        es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
        assert H.es_close(r["es"], es_o, double).all(), (r["es"], es_o)
        np.testing.assert_array_equal(oracle.stats(r["es"]).view(np.uint8), r["stats"].view(np.uint8))


def test_nonfinite_keys(gpu):
    """Zeros in class means make the ratio metrics produce inf/NaN keys."""
    d = synthetic.make(300, 8, 6, 16, seed=3, n_class_b=4, set_min=5, set_max=60)
    d.exprs[:, :40] = 0.0
    d.exprs[:4, 40:60] = 0.0
    for m in (1, 2, 4):
        for double in (False, True):
            r = run_plan(d, m, double=double)
            ok = oracle.metric(m, d.exprs, d.labels, d.num_perms, double=double)
            assert H.ulp_diff(r["keys"], ok).max() <= (2 if m in H.LOG_METRICS else 0)
            sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"])
            es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
            assert H.es_close(r["es"], es_o, double).all(), (m, double)


def test_perm_batches_and_shards_agree(gpu):
    d = MG.metrics_case()
    full = run_plan(d, "twopass_signal2noise", P=64, debug=False)
    batched = run_plan(d, "twopass_signal2noise", P=64, perm_batch=7, debug=False)
    np.testing.assert_array_equal(full["es"], batched["es"])
    np.testing.assert_array_equal(full["stats"], batched["stats"])
    a = run_plan(d, "twopass_signal2noise", P=40, debug=False)
    b = run_plan(d, "twopass_signal2noise", P=24, perm_offset=40, debug=False)
    np.testing.assert_array_equal(np.concatenate([a["es"], b["es"]], axis=1), full["es"])


def test_proxy_symbol_mapping(gpu, tmp_path):
    """GSEA() through gsea_proxy_run: unknown symbols dropped, duplicates collapse."""
    d = MG.metrics_case()
    genes = [f"G{g}" for g in range(d.num_genes)]
    table = api.ExpressionTable(d.exprs.T.astype(np.float64), genes, [f"p{s}" for s in range(d.num_samples)])
    sets = {}
    for k in range(d.num_sets):
        mem = [genes[g] for g in d.set_genes[d.set_offsets[k]:d.set_offsets[k + 1]]]
        sets[f"set{k}"] = mem + mem[:2] + ["NOT_A_GENE", "ALSO_MISSING"]
    prefix = str(tmp_path / "dump")
    res = api.GSEA(table, d.labels.tolist(), sets, d.num_perms, "twopass_signal2noise", dumpFileName=prefix)
    es, st = api.gsea(d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, "twopass_signal2noise")
    K = d.num_sets
    np.testing.assert_array_equal(res.ES, st[:K])
    np.testing.assert_array_equal(res.NES, st[K:2 * K])
    np.testing.assert_array_equal(res.FWER, st[3 * K:4 * K])
    dumped = np.fromfile(f"{prefix}_{K}_{d.num_perms}_32.es", np.float32).reshape(K, -1)
    np.testing.assert_array_equal(dumped, es)
    with pytest.raises(N.GseaError) as e:
        api.GSEA(table, d.labels.tolist(), sets, 8, "no_such_metric")
    assert e.value.status == 2


def test_injected_launch_failure_keeps_context(gpu, monkeypatch):
    d = synthetic.tiny()
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, d.num_perms, "twopass_signal2noise")
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    monkeypatch.setenv("GSEA_FAULT", "launch")
    with pytest.raises(N.GseaError) as e:
        plan.execute()
    assert e.value.status == 8
    monkeypatch.delenv("GSEA_FAULT")
    plan.execute()
    es, st = plan.read()
    es2, st2 = api.gsea(d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, "twopass_signal2noise")
    np.testing.assert_array_equal(es, es2)


@pytest.mark.parametrize("double", [False, True], ids=["f32", "f64"])
@pytest.mark.parametrize("metric", range(14), ids=api.METRICS)
def test_full_size_properties(gpu, metric, double):
    """20,000 x 200, 1,000 sets, 1,000 permutations, every metric in fp32 and
    fp64: size-independent checks (finite |ES| <= 1, statistics bit-identical
    to the oracle's for the GPU's ES) and spot permutations against the
    oracle (keys bit-exact -- log2 metrics <= 2 ulp --, order equal to the
    oracle's stable order of the GPU's keys, ES within tolerance); and the
    statistics against the reference's own CPU build on the same inputs
    (`full_<prec>.npz`).  The packed metric unroll at 200 samples, the
    register sort (fp32) / the two-CTA cluster sort (fp64) at 20,000 genes
    and the 32-warp enrichment staging all run at this size."""
    from cudagsea_gb300.precision_check import _DeviceRows
    d = synthetic.full()
    dt = np.float64 if double else np.float32
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, d.num_perms, metric, precision=64 if double else 32,
                    perm_batch=d.num_perms)
    plan.set_debug(True)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es, st = plan.read()
    assert np.isfinite(es).all() and (np.abs(es) <= 1.0 + 1e-6).all()
    keys = _DeviceRows(plan, N.BUF_KEYS, dt, d.num_genes)
    order = _DeviceRows(plan, N.BUF_ORDER, np.uint32, d.num_genes)
    perms = [0, 1, 499, d.num_perms - 1]
    kg, og = keys.rows(perms), order.rows(perms)
    x = d.exprs.astype(np.float64) if double else d.exprs
    for i, p in enumerate(perms):
        k1 = oracle.metric(metric, x, d.labels, 1, shift=p, double=double)
        if metric in H.LOG_METRICS:
            assert H.ulp_diff(kg[i], k1[0]).max() <= 2, p
        else:
            np.testing.assert_array_equal(kg[i].view(np.uint8), k1[0].view(np.uint8), err_msg=str(p))
        sk, o = oracle.sort(kg[i:i + 1])
        np.testing.assert_array_equal(og[i], o[0])
        e1 = oracle.es(sk, o, d.set_offsets, d.set_genes)
        assert H.es_close(es[:, p], e1[:, 0], double).all(), p
    np.testing.assert_array_equal(oracle.stats(es).view(np.uint8), st.view(np.uint8))
    plan.close()
    # the reference's own statistics: its CPU sort is unstable, so a set
    # member tied with a non-member (and the log2 metrics' keys, <= 2 ulp
    # apart) can move a set's ES by a step of the running sum; ties are
    # common for the fp32 ratio metrics (quotients near 1 take few distinct
    # float values: ~60 tied pairs among 20,000 keys)
    g = H.load(f"full_{'f64' if double else 'f32'}.npz")
    assert str(g["input_sha"]) == MG.input_hash(d)
    ref = g[f"stats_{metric}"]
    K = d.num_sets
    for lo in (0, K):  # ES, NES: at least 97% of the sets within the tolerance,
        # the rest within a few steps of the running sum (~5e-5 of ES each;
        # NES: times the set's normalising factor)
        assert H.es_close(st[lo:lo + K], ref[lo:lo + K], double).mean() >= 0.97
        bound = 5e-3 * (np.maximum(1.0, np.abs(ref[lo:lo + K])) if lo else 1.0)
        assert (np.abs(st[lo:lo + K] - ref[lo:lo + K]) <= bound).all()
    np.testing.assert_allclose(st[2 * K:4 * K], ref[2 * K:4 * K], atol=2.0 / d.num_perms)  # NP, FWER
    assert H.es_close(es[:, :4], g[f"es_head_{metric}"], double).mean() >= 0.97
    if metric == 8 and not double:
        # a sharded plan reproduces the columns
        tail = api.Plan(d.num_genes, d.num_samples, d.num_sets, 100, metric, perm_offset=900)
        tail.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        tail.execute()
        np.testing.assert_array_equal(tail.read()[0], es[:, 900:])
        tail.close()


@pytest.mark.parametrize("value", [np.inf, -np.inf, np.nan, 3e18], ids=["inf", "-inf", "nan", "huge"])
def test_packed_metric_falls_back_on_special_inputs(gpu, value):
    """Inputs the packed fp32 form cannot reproduce send the kernel to the
    exact predicated form: keys stay bit-identical to the oracle."""
    d = MG.metrics_case()
    d.exprs = d.exprs.copy()
    d.exprs[3, 17] = value
    d.exprs[10, 400] = value
    for m in (6, 8, 9, 0):
        r = run_plan(d, m)
        ok = oracle.metric(m, d.exprs, d.labels, d.num_perms)
        np.testing.assert_array_equal(r["keys"].view(np.uint32), ok.view(np.uint32), err_msg=str(m))
        sk, order = check_sort(r["keys"], r["order"], r["ranks"], r["sorted"])
        es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
        assert H.es_close(r["es"], es_o, False).all()


def test_run_sharded_single_rank(gpu, tmp_path):
    """The shard driver on a one-rank gloo group equals the plain run."""
    import socket
    import torch.distributed as dist
    from cudagsea_gb300.shard import run_sharded
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        d = MG.metrics_case()
        es, st = run_sharded(d, d.num_perms)
        es2, st2 = api.gsea(d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms)
        np.testing.assert_array_equal(es, es2)
        np.testing.assert_array_equal(st, st2)
    finally:
        dist.destroy_process_group()


def test_null_distribution_compliance(gpu, tmp_path):
    """The GPU null ES against the oracle's (the reference's arithmetic), 4,096
    permutations of the 2,000 x 40 workload, read back from .es dumps: every
    set's KS distance is a few 1/(P-1) steps at most (the permutations are the
    reference's; only ulp-level differences reorder near-equal nulls); and a
    fp32 run against a fp64 run stays far below the 1% critical distance."""
    from cudagsea_gb300 import compliance
    d = synthetic.small(num_perms=4096)
    P = d.num_perms
    api.gsea(d.exprs, d.labels, d.set_offsets, d.set_genes, P, dump_prefix=str(tmp_path / "g32"))
    api.gsea(d.exprs, d.labels, d.set_offsets, d.set_genes, P, precision=64, dump_prefix=str(tmp_path / "g64"))
    es32 = compliance.read_es_dump(str(tmp_path / f"g32_{d.num_sets}_{P}_32.es"))
    es64 = compliance.read_es_dump(str(tmp_path / f"g64_{d.num_sets}_{P}_64.es"))
    es_o, _ = oracle.gsea(8, d.exprs, d.labels, d.set_offsets, d.set_genes, P)
    # fp32 ES agree with the oracle to a few ulp: ties in the sorted nulls may
    # swap, which moves the empirical CDF by a couple of 1 / (P - 1) steps
    assert compliance.null_distances(es32, es_o).max() <= 3.0 / (P - 1)
    crit = compliance.critical_value(P - 1, P - 1)
    assert compliance.null_distances(es32, es64).max() < 0.1 * crit


def test_device_set_mapping_matches_host_rules(gpu):
    """gsea_map_sets on the device = the host rules of create_bitmaps: unknown
    symbols dropped, duplicates collapsed, ascending genes, a repeated gene
    symbol mapped to its first gene; empty and all-unknown sets."""
    rs = np.random.RandomState(5)
    G = 3000
    genes = [f"G{g}" for g in range(G)]
    genes[17] = "G5"  # a repeated gene symbol
    sets = []
    for k in range(200):
        n = int(rs.randint(0, 300))
        members = [f"G{int(x)}" for x in rs.randint(0, G, n)]
        members += [f"X{int(x)}" for x in rs.randint(0, 50, int(rs.randint(0, 5)))]  # unknown
        members += members[: n // 10]  # duplicates
        rs.shuffle(members)
        sets.append(members)
    sets.append([])
    sets.append(["nope", "X1"])
    off, gs = api.map_sets(genes, sets)
    first = {}
    for g, s in enumerate(genes):
        first.setdefault(s, g)
    exp_off, exp = [0], []
    for st in sets:
        idx = sorted({first[m] for m in st if m in first})
        exp += idx
        exp_off.append(len(exp))
    assert np.array_equal(off, np.array(exp_off))
    assert np.array_equal(gs, np.array(exp, np.int32))


@pytest.mark.parametrize("precision,shards", [(32, 3), (64, 2)])
def test_shard_partial_statistics_on_device(gpu, precision, shards):
    """The library's shard kernels, ranks emulated in one process (the
    exchange replaced by passing tensors on): the merged statistics equal the
    single plan's bit for bit."""
    import torch
    from cudagsea_gb300.shard import DeviceOps, shard_range
    d = synthetic.make(3000, 30, 60, 700, seed=12, n_class_b=14, sd_range=(0.5, 2.0), n_shift=40,
                       shift_range=(0.3, 1.0), set_min=10, set_max=200, enriched_frac=0.2)
    P = d.num_perms
    ref = api.Plan(d.num_genes, d.num_samples, d.num_sets, P, 8, precision=precision)
    ref.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    ref.execute()
    _, st_ref = ref.read(es=False)
    ref.close()
    ops = DeviceOps(precision)
    parts = []
    for r in range(shards):
        first, count = shard_range(P, r, shards)
        plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, count, 8, precision=precision, perm_offset=first)
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        plan.execute()
        es, _ = plan.read(stats=False)
        plan.close()
        parts.append((first, torch.from_numpy(es).cuda()))
    total = None
    for _, es in parts:
        total = ops.chain_sum(es, total)
    head = ops.head(ops.observed(parts[0][1]), total, P)
    counts = hist = None
    for first, es in parts:
        c, h = ops.partial(es, first, head)
        counts = c if counts is None else counts + c
        hist = h if hist is None else hist + h
    st = ops.finish(head, P, counts, hist).cpu().numpy()
    u = np.uint64 if precision == 64 else np.uint32
    assert np.array_equal(st.view(u), st_ref.view(u))


def test_run_sharded_statistics_beyond_fixed_scratch(gpu):
    """The gather driver computes the merged statistics with torch-allocated
    scratch (gsea_stats_device): a size whose statistics need more than the
    allocation-free entry point's fixed 4 MiB (20 sets x 600,000
    permutations in fp32: ~4.8 MB) goes through and equals a single plan's
    statistics bit for bit."""
    import ctypes
    import socket
    import torch.distributed as dist
    from cudagsea_gb300.shard import run_sharded
    d = synthetic.make(300, 12, 20, 600_000, seed=31, n_class_b=6, set_min=5, set_max=60)
    need = ctypes.c_size_t(0)
    N.check(N.lib().gsea_stats_scratch_bytes(d.num_sets, d.num_perms, 32, ctypes.byref(need)))
    assert need.value > 4 << 20
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=0, world_size=1)
    try:
        es, st = run_sharded(d, d.num_perms)
    finally:
        dist.destroy_process_group()
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, d.num_perms, "twopass_signal2noise")
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es2, st2 = plan.read()
    plan.close()
    np.testing.assert_array_equal(es, es2)
    np.testing.assert_array_equal(st.view(np.uint32), st2.view(np.uint32))


def test_null_distribution_compliance_at_reference_scale(gpu):
    """The reference's compliance scale: 2^20 permutations of the 2,000 x 40
    workload, 50 sets.  fp32 against fp64 nulls: every set's KS distance far
    below the 1% critical distance; the GPU's fp32 scores against the oracle
    (the reference's arithmetic) on 2,048 columns at each end of the range."""
    from cudagsea_gb300 import compliance
    P = 1 << 20
    d = synthetic.small(num_perms=P)
    runs = {}
    for prec in (32, 64):
        plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P, "twopass_signal2noise", precision=prec)
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        plan.execute()
        runs[prec] = plan.read(stats=False)[0]
        plan.close()
    crit = compliance.critical_value(P - 1, P - 1)
    dist = compliance.null_distances(runs[32], runs[64])
    assert dist.max() < 0.1 * crit, (dist.max(), crit)
    n = 2048
    for s in (0, P - n):
        k1 = oracle.metric(8, d.exprs, d.labels, n, shift=s)
        sk, o = oracle.sort(k1)
        e1 = oracle.es(sk, o, d.set_offsets, d.set_genes)
        assert H.es_close(runs[32][:, s:s + n], e1, False).all(), s
