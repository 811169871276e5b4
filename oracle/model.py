"""Oracle of the learned permutation allocator and of the ragged statistics:
numpy restatements in float64, test infrastructure only (imported by tests/,
never by the product).

These components have no counterpart in the reference (every set gets the same
number of permutations there), so nothing here is pinned to a reference
output: the network's gradient is pinned by central finite differences of
this restatement (tests/test_model_oracle.py); the ragged statistics reduce to
the reference's final_statistics (src/include/statistics.cuh:46-117) when
every set holds the same count, which the tests check against the C oracle.
"""
from __future__ import annotations

import numpy as np

IN, H, OUT = 5, 64, 2
OFF_W1 = 0
OFF_B1 = OFF_W1 + H * IN
OFF_W2 = OFF_B1 + H
OFF_B2 = OFF_W2 + H * H
OFF_W3 = OFF_B2 + H
OFF_B3 = OFF_W3 + OUT * H
NPARAM = OFF_B3 + OUT


def bf16(a) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest, ties to even), as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return (r & 0xFFFFFFFF).astype(np.uint32).view(np.float32)


def unpack(p):
    p = np.asarray(p, np.float64)
    return (p[OFF_W1:OFF_B1].reshape(H, IN), p[OFF_B1:OFF_W2], p[OFF_W2:OFF_B2].reshape(H, H), p[OFF_B2:OFF_W3],
            p[OFF_W3:OFF_B3].reshape(OUT, H), p[OFF_B3:NPARAM])


INPUT_CLAMP = 8.0  # standardised inputs are clamped to +-8 (k_model.cu kInputClamp)


def normalise(x, norms):
    n = np.asarray(norms, np.float64)
    return np.clip((np.asarray(x, np.float64) - n[:IN]) * n[IN:2 * IN], -INPUT_CLAMP, INPUT_CLAMP)


def forward(p, norms, x):
    """Raw outputs z [n][2] for parameters p (used as given)."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    xn = normalise(x, norms)
    h1 = np.tanh(xn @ W1.T + b1)
    h2 = np.tanh(h1 @ W2.T + b2)
    return h2 @ W3.T + b3, (xn, h1, h2)


def predict(params, norms, x):
    """(tail probability, null mean) with the BF16-rounded parameters."""
    z, _ = forward(bf16(params), norms, x)
    n = np.asarray(norms, np.float64)
    return np.stack([1.0 / (1.0 + np.exp(-z[:, 0])), np.exp(z[:, 1] * n[2 * IN + 1] + n[2 * IN])], axis=1)


def loss(p, norms, x, t) -> float:
    """Mean loss for parameters p (used as given)."""
    z, _ = forward(p, norms, x)
    t = np.asarray(t, np.float64)
    n = np.asarray(norms, np.float64)
    u1 = (t[:, 1] - n[2 * IN]) / n[2 * IN + 1]
    lt, w = tail_target(t[:, 0])
    return float(np.mean(0.5 * w * (z[:, 0] - lt) ** 2 + 0.5 * (z[:, 1] - u1) ** 2))


def tail_target(t0):
    """logit of the clamped tail target and its weight (k_model.cu)."""
    tc = np.clip(np.asarray(t0, np.float64), 1e-4, 1 - 1e-4)
    return np.log(tc / (1 - tc)), np.minimum(1.0, 400.0 * tc * (1 - tc))


def loss_grad(p, norms, x, t):
    """(mean loss, gradient) for parameters p (used as given), by backpropagation."""
    W1, b1, W2, b2, W3, b3 = unpack(p)
    z, (xn, h1, h2) = forward(p, norms, x)
    t = np.asarray(t, np.float64)
    n = np.asarray(norms, np.float64)
    u1 = (t[:, 1] - n[2 * IN]) / n[2 * IN + 1]
    rows = x.shape[0]
    lt, w = tail_target(t[:, 0])
    dy = np.stack([w * (z[:, 0] - lt), z[:, 1] - u1], axis=1)
    dz2 = (dy @ W3) * (1 - h2 * h2)
    dz1 = (dz2 @ W2) * (1 - h1 * h1)
    g = np.zeros(NPARAM)
    g[OFF_W1:OFF_B1] = (dz1.T @ xn).ravel()
    g[OFF_B1:OFF_W2] = dz1.sum(0)
    g[OFF_W2:OFF_B2] = (dz2.T @ h1).ravel()
    g[OFF_B2:OFF_W3] = dz2.sum(0)
    g[OFF_W3:OFF_B3] = (dy.T @ h2).ravel()
    g[OFF_B3:NPARAM] = dy.sum(0)
    return loss(p, norms, x, t), g / rows


def query_factor(k, j, queries):
    """Multiplier of training threshold j of set k: 0.25 * 36^((j + h) / queries)
    with h in [0, 1) from an integer hash of (k, j) (k_adaptive.cu)."""
    M64 = (1 << 64) - 1
    h = (k * 0x9E3779B97F4A7C15 + j * 0xC2B2AE3D27D4EB4F + 0x165667B19E3779F9) & M64
    h ^= h >> 33
    h = (h * 0xFF51AFD7ED558CCD) & M64
    h ^= h >> 33
    u = (h >> 11) * (1.0 / 9007199254740992.0)
    return 0.25 * np.exp(np.log(36.0) * (j + u) / queries)


def decide(counts, exceed, stop_p, z=3.0, p_model=None, prior=None):
    """The sequential stopping rule (Beta posterior lower bound vs stop_p; the
    model's prior is dropped for a set whose observed fraction lies more than
    z sd from the prior predictive)."""
    n = np.asarray(counts, np.float64)
    c = np.asarray(exceed, np.float64)
    a = 0.5 + c
    b = 0.5 + (n - c)
    if p_model is not None and prior is not None:
        pm = np.clip(np.asarray(p_model, np.float32).astype(np.float64), 1e-6, 1 - 1e-6)
        w = np.asarray(prior, np.float32).astype(np.float64)
        ok = np.isfinite(pm) & np.isfinite(w) & (w > 0)
        with np.errstate(divide="ignore", invalid="ignore"):
            sd_pp = np.sqrt(pm * (1 - pm) * (w + n) / (n * (w + 1)))
            ok &= np.abs(c / n - pm) <= z * sd_pp
        a = a + np.where(ok, pm * w, 0)
        b = b + np.where(ok, (1 - pm) * w, 0)
    s = a + b
    lb = a / s - z * np.sqrt(a * b / (s * s * (s + 1)))
    valid = (n > 0) & (c >= 0) & (c <= n)
    return (valid & (lb >= stop_p)).astype(np.uint8)


def stats_ragged(es, counts, p_fwer, dtype=np.float32):
    """Ragged ES / NES / NP / FWER / FDR (see cudagsea_gb300/csrc/k_stats.cu).

    Row k of es holds counts[k] scores; sums run sequentially in `dtype` as
    the reference's host loop does; FDR weights every null score of set k by
    (ld - 1) / (n_k - 1)."""
    T = dtype
    es = np.asarray(es, T)
    K, ld = es.shape
    counts = np.asarray(counts, np.int64)
    out = np.zeros((5, K), T)
    fac = np.zeros(K, T)
    for k in range(K):
        n = counts[k]
        row = es[k, :n]
        s = np.cumsum(np.abs(row), dtype=T)[-1]
        fac[k] = T(n) / s
        out[0, k] = row[0]
        out[1, k] = row[0] * fac[k]
        out[2, k] = T(np.count_nonzero(np.abs(row) >= np.abs(row[0]))) / T(n)
    norm = es[:, :p_fwer] * fac[:, None]
    with np.errstate(invalid="ignore"):
        mx = np.nanmax(np.where(np.isnan(norm), -np.inf, norm), axis=0)
        mn = np.nanmin(np.where(np.isnan(norm), np.inf, norm), axis=0)
    for k in range(K):
        s = out[1, k]
        if s > 0:
            out[3, k] = T(np.count_nonzero(mx >= s)) / T(p_fwer)
        else:
            out[3, k] = T(np.count_nonzero(mn <= s)) / T(p_fwer)
    # FDR
    obs = out[1].astype(np.float64)
    vals, wts = [], []
    for k in range(K):
        n = counts[k]
        if n < 2:
            continue
        vals.append((es[k, 1:n] * fac[k]).astype(np.float64))
        wts.append(np.full(n - 1, (ld - 1) / (n - 1)))
    v = np.concatenate(vals) if vals else np.zeros(0)
    w = np.concatenate(wts) if wts else np.zeros(0)
    null_pos, null_neg = w[v >= 0].sum(), w[v <= 0].sum()
    opos, oneg = obs[obs >= 0], obs[obs <= 0]
    for k in range(K):
        s = obs[k]
        if np.isnan(s):
            out[4, k] = T(np.nan)
            continue
        if s > 0:
            c_null = w[v >= s].sum()
            fn = c_null / null_pos if null_pos > 0 else 0.0
            fo = np.count_nonzero(opos >= s) / opos.size
        else:
            c_null = w[v <= s].sum()
            fn = c_null / null_neg if null_neg > 0 else 0.0
            fo = np.count_nonzero(oneg <= s) / oneg.size
        out[4, k] = T(min(fn / fo, 1.0))
    return out.ravel()


def fdr_bound(es, counts, p_fwer, sums, z, dtype=np.float32):
    """Lower bound of every set's FDR q over |NES| in [|NES|, key], key =
    |NES| (1 + z cv / sqrt(n)) (k_stats.cu stats_fdr_bound_kernel), cv from
    sums (sum |S| then sum S^2 per set): the null weight at or above the
    observed key next above key (i_up keys below key) over the side's null
    weight, divided by max(m - i_lo, 1) / m (i_lo keys below |NES|), capped at
    1.  NaN or zero NES: 0.  Returns (statistics, bounds float32)."""
    T = dtype
    es = np.asarray(es, T)
    K, ld = es.shape
    counts = np.asarray(counts, np.int64)
    sums = np.asarray(sums, np.float64)
    st = stats_ragged(es, counts, p_fwer, dtype).reshape(5, K)
    fac = np.zeros(K, T)
    for k in range(K):
        n = counts[k]
        fac[k] = T(n) / np.cumsum(np.abs(es[k, :n]), dtype=T)[-1]
    vals, wts = [], []
    for k in range(K):
        n = counts[k]
        if n >= 2:
            vals.append((es[k, 1:n] * fac[k]).astype(np.float64))
            wts.append(np.full(n - 1, (ld - 1) / (n - 1)))
    v = np.concatenate(vals) if vals else np.zeros(0)
    w = np.concatenate(wts) if wts else np.zeros(0)
    obs = st[1].astype(np.float64)
    sides = {True: (np.sort(obs[obs >= 0]), v >= 0, v), False: (np.sort(-obs[obs <= 0]), v <= 0, -v)}
    q = np.zeros(K, np.float32)
    for k in range(K):
        s, n = obs[k], float(counts[k])
        if not (s == s) or s == 0.0 or n <= 0:
            continue
        m = sums[k] / n
        var = max(sums[K + k] / n - m * m, 0.0)
        cv = np.sqrt(var) / m if m > 0 else np.inf
        key = abs(s) * (1.0 + z * cv / np.sqrt(n))
        keys, on_side, nv = sides[s > 0]
        mc = keys.size
        if not np.isfinite(key) or mc == 0:
            continue
        i_up = int(np.count_nonzero(keys < key))
        i_lo = int(np.count_nonzero(keys < abs(s)))
        c_null = w[on_side & (nv >= keys[i_up])].sum() if i_up < mc else 0.0
        wtot = w[on_side].sum()
        fn = c_null / wtot if wtot > 0 else 0.0
        q[k] = np.float32(min(fn / (max(mc - i_lo, 1) / mc), 1.0))
    return st.ravel(), q
