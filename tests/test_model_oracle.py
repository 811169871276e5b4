"""CPU checks of the learned allocator's oracle and host logic: the oracle's
backpropagation against central finite differences, the library's stopping
rule (a host function) against the oracle's, and the ragged statistics oracle
against the C oracle's dense statistics when every set holds the same count."""
import numpy as np
import pytest

import oracle
from oracle import model as M
from cudagsea_gb300 import allocator, synthetic


def random_problem(rows=300, seed=0):
    rs = np.random.RandomState(seed)
    p = np.zeros(M.NPARAM)
    p[M.OFF_W1:M.OFF_B1] = rs.uniform(-0.6, 0.6, M.H * M.IN)
    p[M.OFF_B1:M.OFF_W2] = rs.uniform(-0.1, 0.1, M.H)
    p[M.OFF_W2:M.OFF_B2] = rs.uniform(-0.2, 0.2, M.H * M.H)
    p[M.OFF_B2:M.OFF_W3] = rs.uniform(-0.1, 0.1, M.H)
    p[M.OFF_W3:M.OFF_B3] = rs.uniform(-0.3, 0.3, M.OUT * M.H)
    p[M.OFF_B3:] = rs.uniform(-0.1, 0.1, M.OUT)
    x = rs.normal(size=(rows, M.IN)) * [1.0, 0.5, 2.0, 0.3, 1.5] + [4.0, 1.0, 0.2, 0.0, 0.7]
    norms = np.zeros(15)
    norms[:5] = x.mean(0)
    norms[5:10] = 1 / x.std(0)
    t = np.stack([rs.uniform(0, 1, rows), rs.normal(-1.5, 0.4, rows)], axis=1)
    norms[10], norms[11] = t[:, 1].mean(), t[:, 1].std()
    return p, norms, x, t


def test_oracle_backprop_matches_finite_differences():
    p, norms, x, t = random_problem()
    _, g = M.loss_grad(p, norms, x, t)
    rs = np.random.RandomState(1)
    idx = np.concatenate([rs.choice(M.NPARAM, 150, replace=False), np.arange(M.OFF_B3, M.NPARAM)])
    h = 1e-6
    for i in idx:
        e = np.zeros(M.NPARAM)
        e[i] = h
        fd = (M.loss(p + e, norms, x, t) - M.loss(p - e, norms, x, t)) / (2 * h)
        assert abs(fd - g[i]) <= 1e-7 + 1e-5 * abs(g[i]), (i, fd, g[i])


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.00390625, 1.005859375, -2.0009765625, 3.14159265], np.float32)
    r = M.bf16(v)
    # bf16 keeps 8 significant bits: 1 + k/128
    assert r[0] == 1.0
    assert r[1] == 1.0                      # 1 + 2^-8 is a tie -> even (1.0)
    assert r[2] == np.float32(1.0078125)    # above the tie -> up
    assert r[3] == -2.0
    assert abs(r[4] - 3.140625) < 1e-7


def test_library_stopping_rule_matches_oracle():
    rs = np.random.RandomState(3)
    K = 5000
    counts = rs.choice([250, 500, 1000, 4000], K).astype(np.int64)
    exceed = (rs.beta(0.7, 3.0, K) * counts).astype(np.int64) + 1
    pm = rs.uniform(0, 1, K).astype(np.float32)
    prior = rs.uniform(0, 2000, K).astype(np.float32)
    for stop_p in (0.01, 0.05, 0.2):
        a = allocator.decide(counts, exceed, stop_p, 3.0)
        b = M.decide(counts, exceed, stop_p, 3.0)
        assert np.array_equal(a, b)
        a = allocator.decide(counts, exceed, stop_p, 2.5, pm, prior)
        b = M.decide(counts, exceed, stop_p, 2.5, pm, prior)
        assert np.array_equal(a, b)
        assert 0 < a.sum() < K


def test_stopping_rule_properties():
    # more evidence never un-stops a clearly null set; a zero count never stops
    n = np.array([100, 1000, 10000], np.int64)
    assert list(M.decide(n, n // 2, 0.1)) == [1, 1, 1]
    assert list(M.decide(n, np.ones(3, np.int64), 0.01)) == [0, 0, 0]
    # a prior at p~ = 0.5 with many pseudo-counts stops a set the data alone cannot
    c, e = np.array([100], np.int64), np.array([12], np.int64)
    assert M.decide(c, e, 0.06)[0] == 0
    assert M.decide(c, e, 0.06, 3.0, np.array([0.14], np.float32), np.array([400.0], np.float32))[0] == 1
    # ... but a prior that the permutations contradict is dropped
    assert M.decide(c, np.array([1], np.int64), 0.06, 3.0, np.array([0.3], np.float32),
                    np.array([1000.0], np.float32))[0] == 0


@pytest.mark.parametrize("double", [False, True])
def test_ragged_oracle_reduces_to_dense_statistics(double):
    d = synthetic.tiny()
    d = synthetic.make(300, 16, 12, 64, seed=5, n_class_b=8, sd=2.0, n_shift=20, shift=1.0, set_min=8, set_max=40)
    dt = np.float64 if double else np.float32
    es, st = oracle.gsea(8, d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, double=double)
    r = M.stats_ragged(es, np.full(d.num_sets, d.num_perms), d.num_perms, dtype=dt).reshape(5, -1)
    st = st.reshape(5, -1)
    assert np.array_equal(r[:4].view(np.uint64 if double else np.uint32), st[:4].view(np.uint64 if double else np.uint32))
    np.testing.assert_allclose(r[4], st[4], rtol=1e-6 if not double else 1e-12)


def _ragged_case(seed=3, K=40, ld=300):
    rs = np.random.RandomState(seed)
    es = rs.normal(0, 0.3, (K, ld)).astype(np.float32)
    es[:, 0] += rs.normal(0, 0.6, K).astype(np.float32)
    counts = rs.randint(50, ld + 1, K).astype(np.int64)
    counts[0] = ld
    a = np.abs(es.astype(np.float64))
    sums = np.concatenate([[a[k, :counts[k]].sum() for k in range(K)],
                           [(a[k, :counts[k]] ** 2).sum() for k in range(K)]])
    return es, counts, sums


def test_fdr_bound_oracle_is_q_at_z0_and_below_q_otherwise():
    """The adaptive test's FDR stopping bound: at z = 0 it is the set's own
    FDR q (no ties here); a wider interval only lowers it, and it never
    exceeds q at any |NES| inside the interval (checked at the observed keys
    the interval covers)."""
    es, counts, sums = _ragged_case()
    p_fwer = int(counts.min())
    st, q0 = M.fdr_bound(es, counts, p_fwer, sums, 0.0)
    q = st.reshape(5, -1)[4]
    np.testing.assert_allclose(q0, q, rtol=1e-6)
    _, q1 = M.fdr_bound(es, counts, p_fwer, sums, 1.0)
    _, q3 = M.fdr_bound(es, counts, p_fwer, sums, 3.0)
    assert np.all(q1 <= q0) and np.all(q3 <= q1)
    assert np.any(q3 < q0)
    # q(x) at every observed key x inside [|NES_k|, key_k] is >= the bound
    K = es.shape[0]
    nes = st.reshape(5, -1)[1].astype(np.float64)
    for k in range(K):
        n = counts[k]
        m = sums[k] / n
        cv = np.sqrt(max(sums[K + k] / n - m * m, 0.0)) / m
        key = abs(nes[k]) * (1 + 3.0 * cv / np.sqrt(n))
        same = [j for j in range(K) if np.sign(nes[j]) == np.sign(nes[k]) and abs(nes[k]) <= abs(nes[j]) <= key]
        for j in same:
            assert q3[k] <= q[j] + 1e-6, (k, j, q3[k], q[j])
