"""Null-distribution compliance: compare the permutation null of two runs.

The reference checks its null ES distributions against Broad GSEA by plotting
per-set CDFs (results/compliance/histograms.py:66-134).  Here the comparison
is numeric: for every gene set the two-sample Kolmogorov-Smirnov distance
between the null ES (permutations 1..P-1) of two `.es` matrices, e.g. this
library against the reference or a fp32 run against a fp64 run.
"""
from __future__ import annotations

import os
import re
from typing import Tuple

import numpy as np


def read_es_dump(path: str) -> np.ndarray:
    """Read `<prefix>_<K>_<P>_<32|64>.es` (row-major [K][P])."""
    m = re.search(r"_(\d+)_(\d+)_(32|64)\.es$", os.path.basename(path))
    if not m:
        raise ValueError(f"not an .es dump name: {path}")
    K, P, bits = int(m.group(1)), int(m.group(2)), int(m.group(3))
    data = np.fromfile(path, np.float64 if bits == 64 else np.float32)
    if data.size != K * P:
        raise ValueError(f"{path}: {data.size} values, expected {K * P}")
    return data.reshape(K, P)


def ks_distance(a: np.ndarray, b: np.ndarray) -> float:
    """Two-sample Kolmogorov-Smirnov statistic sup |F_a - F_b| (NaNs dropped)."""
    a = np.sort(a[~np.isnan(a)].astype(np.float64))
    b = np.sort(b[~np.isnan(b)].astype(np.float64))
    if a.size == 0 or b.size == 0:
        return 0.0 if a.size == b.size else 1.0
    v = np.concatenate([a, b])
    fa = np.searchsorted(a, v, side="right") / a.size
    fb = np.searchsorted(b, v, side="right") / b.size
    return float(np.max(np.abs(fa - fb)))


def null_distances(es_a: np.ndarray, es_b: np.ndarray) -> np.ndarray:
    """Per-set KS distance between the null columns (1..) of two ES matrices."""
    if es_a.shape[0] != es_b.shape[0]:
        raise ValueError("different numbers of gene sets")
    return np.array([ks_distance(es_a[k, 1:], es_b[k, 1:]) for k in range(es_a.shape[0])])


def critical_value(n: int, m: int, alpha: float = 0.01) -> float:
    """Asymptotic KS critical distance for sample sizes n, m at level alpha."""
    c = np.sqrt(-0.5 * np.log(alpha / 2.0))
    return float(c * np.sqrt((n + m) / (n * m)))
