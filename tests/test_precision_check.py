"""Host logic of the headline precision check (cudagsea_gb300/precision_check.py),
on the CPU: its FP64 enrichment score in a given rank order equals the
oracle's; its tracing calls a near-tie swap at the running sum's extremum
tie-explained and a planted wrong score not."""
import numpy as np

import oracle
from cudagsea_gb300 import precision_check as PC
from cudagsea_gb300 import synthetic


class _Rows:
    def __init__(self, a):
        self.a = a

    def rows(self, idx):
        return self.a[np.asarray(idx)]


class _Run:
    def __init__(self, es, stats, keys, order):
        self.es, self.stats, self.keys, self.order = es, stats.reshape(5, -1), _Rows(keys), _Rows(order)


def test_es_in_order_matches_oracle():
    d = synthetic.make(500, 12, 20, 6, seed=9, n_class_b=6, set_min=1, set_max=80)
    keys = oracle.metric(8, d.exprs.astype(np.float64), d.labels, d.num_perms, double=True)
    sk, order = oracle.sort(keys)
    es_o = oracle.es(sk, order, d.set_offsets, d.set_genes)
    for p in range(d.num_perms):
        for k in range(d.num_sets):
            m = d.set_genes[d.set_offsets[k]:d.set_offsets[k + 1]]
            e = PC.es_in_order(order[p].astype(np.int64), np.abs(keys[p]), m, d.num_genes)
            assert abs(e - es_o[k, p]) <= 1e-12, (k, p, e, es_o[k, p])


def _case():
    """A workload, its FP64 run (oracle) and a copy to perturb."""
    d = synthetic.make(400, 10, 12, 64, seed=3, n_class_b=5, set_min=10, set_max=60)
    keys = oracle.metric(8, d.exprs.astype(np.float64), d.labels, d.num_perms, double=True)
    sk, order = oracle.sort(keys)
    es = oracle.es(sk, order, d.set_offsets, d.set_genes)
    st = oracle.stats(es)
    return d, keys, order, es, st


def _swap_at_extremum(d, keys, order, k):
    """Permutation 0's order with one of set k's hits swapped with the
    non-member right after it, chosen so that set k's score moves (the swap
    sits at the running sum's extremum)."""
    G = d.num_genes
    members = d.set_genes[d.set_offsets[k]:d.set_offsets[k + 1]]
    mem = np.zeros(G, bool)
    mem[members] = True
    o = order[0].astype(np.int64)
    base = PC.es_in_order(o, np.abs(keys[0]), members, G)
    for i in np.flatnonzero(mem[o]):
        if i + 1 < G and not mem[o[i + 1]]:
            t = o.copy()
            t[i], t[i + 1] = t[i + 1], t[i]
            if abs(PC.es_in_order(t, np.abs(keys[0]), members, G) - base) > 10 * PC.ES_ROUND:
                return t
    raise AssertionError("no swap moves the score")


def test_compare_explains_a_near_tie_swap_and_flags_a_wrong_score():
    d, keys, order, es, st = _case()
    K = d.num_sets
    ref = _Run(es, st, keys, order)
    # (1) a near-tie swap in the observed permutation of set 0
    k = 0
    o_sw = _swap_at_extremum(d, keys, order, k)
    order_c = order.copy()
    order_c[0] = o_sw
    es_c = es.copy()
    for kk in range(K):
        mm = d.set_genes[d.set_offsets[kk]:d.set_offsets[kk + 1]]
        es_c[kk, 0] = PC.es_in_order(o_sw, np.abs(keys[0]), mm, d.num_genes)
    st_c = oracle.stats(es_c)
    moved = np.abs(es_c[:, 0] - es[:, 0]) > PC.ES_ROUND
    rep = PC.compare(d, _Run(es_c, st_c, keys, order_c), ref, nes_tol=1e-9)
    assert moved[k] and rep["sets_over_tol"] >= 1
    traced = {e["set"]: e for e in rep["exceedances"]}
    for kk in np.flatnonzero(moved):
        assert traced[int(kk)]["observed_moved"] and traced[int(kk)]["order_explained"]
    assert rep["all_tie_explained"]
    # (2) a planted wrong score (no reorder behind it) is not explained
    es_bad = es.copy()
    es_bad[3, 7] += 0.01
    rep2 = PC.compare(d, _Run(es_bad, oracle.stats(es_bad), keys, order), ref)
    assert rep2["sets_over_tol"] >= 1 and not rep2["all_tie_explained"]
    bad = {e["set"]: e for e in rep2["exceedances"]}
    assert bad[3]["moved_perms"] == 1 and not bad[3]["order_explained"]


def test_sign_tie_of_the_extrema_is_explained():
    """A score whose maximum and minimum tie in magnitude may come out with
    either sign; a moved score of the same magnitude and the other sign is
    explained, a different magnitude is not."""
    d, keys, order, es, st = _case()
    ref = _Run(es, st, keys, order)
    k, p = 2, 0  # the observed score: its sign is the NES's
    es_flip = es.copy()
    es_flip[k, p] = -es[k, p]
    rep = PC.compare(d, _Run(es_flip, oracle.stats(es_flip), keys, order), ref, nes_tol=1e-9)
    tr = {e["set"]: e for e in rep["exceedances"]}
    assert tr[k]["order_explained"] and tr[k]["sign_ties"] == 1
    es_bad = es.copy()
    es_bad[k, p] = -0.5 * es[k, p]
    rep2 = PC.compare(d, _Run(es_bad, oracle.stats(es_bad), keys, order), ref, nes_tol=1e-9)
    assert not {e["set"]: e for e in rep2["exceedances"]}[k]["order_explained"]
