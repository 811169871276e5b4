"""Oracle of the O(K) statistics merge over permutation shards: the steps of
gsea_shard_sum / _head / _partial / _finish (cudagsea_gb300/csrc/shard_stats.cu)
restated with numpy on CPU arrays, test infrastructure only.  Driven by
cudagsea_gb300.shard.merge_stats on gloo ranks, the merged statistics must
equal the single run's final_statistics (src/include/statistics.cuh:46-117)
bit for bit."""
from __future__ import annotations

import numpy as np


class OracleOps:
    def __init__(self, precision: int = 32):
        import torch
        self.torch = torch
        self.T = np.float64 if precision == 64 else np.float32

    # es arrays: numpy [K][count]
    def chain_sum(self, es, init):
        T = self.T
        out = np.empty(es.shape[0], T)
        for k in range(es.shape[0]):
            seq = np.abs(es[k].astype(T))
            start = T(0) if init is None else T(init[k])
            out[k] = np.cumsum(np.concatenate([[start], seq]).astype(T), dtype=T)[-1]
        return out

    def observed(self, es):
        return np.ascontiguousarray(es[:, 0].astype(self.T))

    def head(self, es_obs, total, num_perms):
        T = self.T
        fac = (T(num_perms) / total.astype(T)).astype(T)
        return np.concatenate([es_obs.astype(T), (es_obs.astype(T) * fac).astype(T), fac])

    def partial(self, es, first, head):
        T = self.T
        K, count = es.shape
        es = es.astype(T)
        obs, nes, fac = head[:K], head[K:2 * K], head[2 * K:]
        np_c = np.count_nonzero(np.abs(es) >= np.abs(obs)[:, None], axis=1)
        norm = (es * fac[:, None]).astype(T)
        with np.errstate(invalid="ignore"):
            mx = np.where(np.isnan(norm), -np.inf, norm).max(axis=0) if count else np.zeros(0, T)
            mn = np.where(np.isnan(norm), np.inf, norm).min(axis=0) if count else np.zeros(0, T)
        fw = np.array([np.count_nonzero(mx >= s) if s > 0 else np.count_nonzero(mn <= s) for s in nes])
        sorted_pos, sorted_neg = np.sort(nes[nes >= 0]), np.sort(-nes[nes <= 0])
        hist = np.zeros(2 * (K + 2) + 2)
        c0 = 1 if first == 0 else 0
        v = norm[:, c0:].ravel().astype(np.float64)
        pos, neg = v[v >= 0], v[v <= 0]
        np.add.at(hist, np.searchsorted(sorted_pos.astype(np.float64), pos, side="right"), 1.0)
        np.add.at(hist, (K + 2) + np.searchsorted(sorted_neg.astype(np.float64), -neg, side="right"), 1.0)
        hist[2 * (K + 2)] = pos.size
        hist[2 * (K + 2) + 1] = neg.size
        return np.concatenate([np_c, fw]).astype(np.int64), hist

    def finish(self, head, num_perms, counts, hist):
        T = self.T
        K = head.shape[0] // 3
        obs, nes = head[:K], head[K:2 * K]
        out = np.zeros(5 * K, T)
        out[:K] = obs
        out[K:2 * K] = nes
        out[2 * K:3 * K] = (counts[:K].astype(T) / T(num_perms)).astype(T)
        out[3 * K:4 * K] = (counts[K:].astype(T) / T(num_perms)).astype(T)
        hpos = hist[:K + 2][::-1].cumsum()[::-1]
        hneg = hist[K + 2:2 * (K + 2)][::-1].cumsum()[::-1]
        npos, nneg = hist[2 * (K + 2)], hist[2 * (K + 2) + 1]
        opos, oneg = nes[nes >= 0], nes[nes <= 0]
        for k in range(K):
            s = nes[k]
            if np.isnan(s):
                out[4 * K + k] = s
                continue
            if s > 0:
                L = np.count_nonzero(opos < s)
                c_null = hpos[L + 1] if L + 1 <= opos.size else 0.0
                fn = c_null / npos if npos > 0 else 0.0
                fo = np.count_nonzero(opos >= s) / opos.size
            else:
                L = np.count_nonzero(-oneg < -s)
                c_null = hneg[L + 1] if L + 1 <= oneg.size else 0.0
                fn = c_null / nneg if nneg > 0 else 0.0
                fo = np.count_nonzero(oneg <= s) / oneg.size
            out[4 * K + k] = T(min(fn / fo, 1.0))
        return out

    def empty_like_sum(self, K, like):
        return np.zeros(K, self.T)

    def to_comm(self, x, device):
        return self.torch.from_numpy(np.ascontiguousarray(x))

    def from_comm(self, t, like):
        return t.numpy()
