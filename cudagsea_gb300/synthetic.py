"""Seeded synthetic GSEA inputs with the shapes of the benchmark workloads.

There is no public dataset behind the benchmark: expression tables, labels and
gene sets are generated from a seed with numpy's legacy ``RandomState``, whose
streams are stable across numpy versions, so the same seed gives the same
inputs on every machine.

Workloads (all expression values are log2-like, ~N(8, sd)):

* ``small``   2,000 genes x 40 samples (20/20), sd 2, 50 genes shifted +1.0 in
              class 1; 50 sets of size U[15,200]; 1,024 permutations.
* ``full``    20,000 genes x 200 samples (100/100), per-gene sd ~ U[0.3,3],
              500 genes shifted +/-U[0.5,2] in class 1; 1,000 sets of size
              U[15,500], 20% of them enriched with shifted genes; 1,000
              permutations.  Values are clamped at 1e-3 so that the ratio
              metrics stay finite.
* ``precision`` 20,000 x 600 (300/300), 2,000 sets, 10,000 permutations.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import List, Optional

import numpy as np


@dataclass
class GseaInput:
    exprs: np.ndarray          # patient-major [S][G] float32
    labels: np.ndarray         # uint8 [S], 0 = class A, 1 = class B
    set_offsets: np.ndarray    # int64 [K+1]
    set_genes: np.ndarray      # int32 [sum n_k], gene indices
    num_perms: int
    name: str = ""

    @property
    def num_genes(self) -> int:
        return int(self.exprs.shape[1])

    @property
    def num_samples(self) -> int:
        return int(self.exprs.shape[0])

    @property
    def num_sets(self) -> int:
        return int(self.set_offsets.size - 1)

    def gene_symbols(self) -> List[str]:
        return [f"G{g}" for g in range(self.num_genes)]

    def set_lists(self) -> List[List[str]]:
        out = []
        for k in range(self.num_sets):
            a, b = self.set_offsets[k], self.set_offsets[k + 1]
            out.append([f"G{g}" for g in self.set_genes[a:b]])
        return out


def _csr(sets: List[np.ndarray]):
    off = np.zeros(len(sets) + 1, np.int64)
    off[1:] = np.cumsum([len(s) for s in sets])
    genes = np.concatenate(sets).astype(np.int32) if sets else np.zeros(0, np.int32)
    return off, genes


def make(num_genes: int, num_samples: int, num_sets: int, num_perms: int, *, seed: int = 1234,
         n_class_b: Optional[int] = None, sd=2.0, sd_range=None, n_shift: int = 50,
         shift=1.0, shift_range=None, set_min: int = 15, set_max: int = 200,
         enriched_frac: float = 0.0, clamp: Optional[float] = None, null_background: bool = False,
         name: str = "") -> GseaInput:
    rs = np.random.RandomState(seed)
    G, S = num_genes, num_samples
    nB = S // 2 if n_class_b is None else n_class_b
    labels = np.zeros(S, np.uint8)
    labels[rs.permutation(S)[:nB]] = 1
    if sd_range is not None:
        gene_sd = rs.uniform(sd_range[0], sd_range[1], size=G)
    else:
        gene_sd = np.full(G, float(sd))
    x = 8.0 + rs.standard_normal((S, G)) * gene_sd[None, :]
    shifted = rs.choice(G, size=min(n_shift, G), replace=False)
    if shift_range is not None:
        amount = rs.uniform(shift_range[0], shift_range[1], size=shifted.size)
        amount *= np.where(rs.uniform(size=shifted.size) < 0.5, -1.0, 1.0)
    else:
        amount = np.full(shifted.size, float(shift))
    x[np.ix_(labels == 1, shifted)] += amount[None, :]
    if clamp is not None:
        x = np.maximum(x, clamp)
    exprs = np.ascontiguousarray(x.astype(np.float32))
    sets = []
    unshifted = np.setdiff1d(np.arange(G), shifted) if null_background else None
    hi = min(set_max, G)
    lo = min(set_min, hi)
    for k in range(num_sets):
        n = int(rs.randint(lo, hi + 1))
        if enriched_frac > 0 and rs.uniform() < enriched_frac:
            n_enr = min(n // 2, shifted.size)
            enr = rs.choice(shifted, size=n_enr, replace=False)
            rest = rs.choice(np.setdiff1d(np.arange(G), enr), size=n - n_enr, replace=False)
            members = np.concatenate([enr, rest])
        elif null_background:  # a null set: unshifted genes only
            members = rs.choice(unshifted, size=n, replace=False)
        else:
            members = rs.choice(G, size=n, replace=False)
        sets.append(np.sort(members))
    off, genes = _csr(sets)
    return GseaInput(exprs, labels, off, genes, num_perms, name)


def learned(seed: int = 5150, num_sets: int = 20000, num_perms: int = 100000) -> GseaInput:
    """20,000 genes x 200 samples (100/100) as full(), 20,000 sets U[15,500]
    of which 5 % are enriched for the shifted genes and the other 95 % are
    null sets drawn from the unshifted genes; up to 100,000 permutations per
    set."""
    return make(20000, 200, num_sets, num_perms, seed=seed, n_class_b=100, sd_range=(0.3, 3.0),
                n_shift=500, shift_range=(0.5, 2.0), set_min=15, set_max=500, enriched_frac=0.05,
                clamp=1e-3, null_background=True, name=f"learned_20000x200_K{num_sets}_P{num_perms}")


def small(seed: int = 1234, num_perms: int = 1024) -> GseaInput:
    """2,000 genes x 40 samples (20/20), 50 sets U[15,200], 1,024 permutations."""
    return make(2000, 40, 50, num_perms, seed=seed, n_class_b=20, sd=2.0, n_shift=50, shift=1.0,
                set_min=15, set_max=200, name="small_2000x40_K50_P1024")


def full(seed: int = 4321, num_perms: int = 1000) -> GseaInput:
    """20,000 genes x 200 samples (100/100), 1,000 sets U[15,500], 1,000 permutations."""
    return make(20000, 200, 1000, num_perms, seed=seed, n_class_b=100, sd_range=(0.3, 3.0),
                n_shift=500, shift_range=(0.5, 2.0), set_min=15, set_max=500, enriched_frac=0.2,
                clamp=1e-3, name="full_20000x200_K1000_P1000")


def precision(seed: int = 777, num_perms: int = 10000) -> GseaInput:
    """20,000 genes x 600 samples (300/300), 2,000 sets U[15,500], 10,000 permutations."""
    return make(20000, 600, 2000, num_perms, seed=seed, n_class_b=300, sd_range=(0.3, 3.0),
                n_shift=500, shift_range=(0.5, 2.0), set_min=15, set_max=500, enriched_frac=0.2,
                clamp=1e-3, name="precision_20000x600_K2000_P10000")


def tiny(seed: int = 7, G: int = 37, S: int = 5, K: int = 3, P: int = 3, n_class_b: int = 2) -> GseaInput:
    """Exhaustive-check shapes (default 37 genes x 5 samples, 3 sets, 3 permutations)."""
    return make(G, S, K, P, seed=seed, n_class_b=n_class_b, sd=2.0, n_shift=min(5, G), shift=1.0,
                set_min=min(3, G), set_max=min(12, G), name=f"tiny_{G}x{S}_K{K}_P{P}")


def batch_instances(n: int = 256, seed: int = 77, num_perms: int = 1000, genes=(5000, 30000), samples=(20, 500),
                    sets=(50, 5000), set_size=(15, 500)):
    """`n` uneven instances: genes ~ U[5,000, 30,000], samples ~ U[20, 500] with
    class B a U[30 %, 70 %] share, K ~ U[50, 5,000] sets of size U[15, 500],
    expression 8 + N(0, sd_g^2) with sd_g ~ U[0.3, 3] and 2.5 % of the genes
    shifted by +-U[0.5, 2] in class B, `num_perms` permutations each.  Drawn
    with numpy's PCG64 generator (fast enough for 256 instances)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n):
        G = int(rng.integers(genes[0], genes[1] + 1))
        S = int(rng.integers(samples[0], samples[1] + 1))
        nB = int(np.clip(round(S * rng.uniform(0.3, 0.7)), 1, S - 1))
        K = int(rng.integers(sets[0], sets[1] + 1))
        labels = np.zeros(S, np.uint8)
        labels[rng.permutation(S)[:nB]] = 1
        sd = rng.uniform(0.3, 3.0, G).astype(np.float32)
        x = rng.standard_normal((S, G), dtype=np.float32) * sd[None, :] + np.float32(8.0)
        shifted = rng.choice(G, size=max(1, G // 40), replace=False)
        amount = (rng.uniform(0.5, 2.0, shifted.size) * rng.choice([-1.0, 1.0], shifted.size)).astype(np.float32)
        x[np.ix_(labels == 1, shifted)] += amount[None, :]
        hi = min(set_size[1], G)
        members = [np.sort(rng.choice(G, size=int(rng.integers(set_size[0], hi + 1)), replace=False))
                   for _ in range(K)]
        off, gs = _csr(members)
        out.append(GseaInput(np.ascontiguousarray(x), labels, off, gs, num_perms, f"batch{i}_{G}x{S}_K{K}"))
    return out
