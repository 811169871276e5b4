"""Comparison helpers shared by the parity tests."""
from __future__ import annotations

import hashlib
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")

# metric ids whose keys pass through logf/log: the device's log and glibc's
# may differ by one unit in the last place, so their keys are compared to
# 2 ulp and their rank orders with the near-tie rule
LOG_METRICS = (2, 5)

# ES / NES tolerance of the plain form against the oracle (relative to the
# magnitude, with an absolute floor for scores near zero)
ES_RTOL_F32 = 1e-5
ES_ATOL_F32 = 2e-6
ES_RTOL_F64 = 1e-12
ES_ATOL_F64 = 1e-13


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def load(name: str):
    return np.load(os.path.join(GOLDEN, name))


def input_hash(d) -> str:
    return sha(d.exprs, d.labels, d.set_offsets, d.set_genes)


def ulp_diff(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Distance in units in the last place between same-typed float arrays."""
    it = np.int32 if a.dtype == np.float32 else np.int64
    ai = a.view(it).astype(np.int64)
    bi = b.view(it).astype(np.int64)
    big = np.int64(1) << (31 if a.dtype == np.float32 else 63)
    ai = np.where(ai < 0, -(ai + big), ai)  # sign-magnitude -> two's complement order
    bi = np.where(bi < 0, -(bi + big), bi)
    return np.abs(ai - bi)


def es_close(a, b, double: bool):
    rtol, atol = (ES_RTOL_F64, ES_ATOL_F64) if double else (ES_RTOL_F32, ES_ATOL_F32)
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    both_nan = np.isnan(a) & np.isnan(b)
    ok = np.abs(a - b) <= atol + rtol * np.maximum(np.abs(a), np.abs(b))
    return ok | both_nan


def tie_explained(sorted_keys_row: np.ndarray, order_row: np.ndarray, members: np.ndarray) -> bool:
    """True if some group of equal keys holds both a member and a non-member of the
    set, i.e. an unstable sort could legitimately order this permutation differently."""
    k = sorted_keys_row
    mem = np.zeros(order_row.max() + 1, bool)
    mem[members] = True
    hit = mem[order_row]
    start = np.flatnonzero(np.r_[True, k[1:] != k[:-1]])
    end = np.r_[start[1:], k.size]
    for s, e in zip(start, end):
        if e - s > 1 and hit[s:e].any() and not hit[s:e].all():
            return True
    return False


def near_tie_ok(keys_row: np.ndarray, order_a: np.ndarray, order_b: np.ndarray, max_ulp: int = 4) -> bool:
    """Rank orders may differ only between genes whose keys are within max_ulp."""
    if np.array_equal(order_a, order_b):
        return True
    diff = np.flatnonzero(order_a != order_b)
    ka = keys_row[order_a[diff]]
    kb = keys_row[order_b[diff]]
    return bool(np.all(ulp_diff(ka, kb) <= max_ulp))
