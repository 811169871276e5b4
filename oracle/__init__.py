"""CPU oracle for the GSEA permutation pipeline -- TEST INFRASTRUCTURE ONLY.

Two oracles live here:

* ``gsea_oracle.cpp`` -- our own C++ restatement of the reference algorithm
  (each stage cites the cudaGSEA file:line it follows), built into
  ``oracle/_build/libgsea_oracle.so``.  It is pinned against the reference's
  own CPU build (``oracle/_ref``) and the committed golden fixtures.
* ``_ref/libgsea_ref.so`` -- the reference's own CPU stages compiled from the
  cudaGSEA sources by ``build_ref.sh`` (only where those sources exist).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline legs of
``bench.py`` may import this package.  The product library never does.
"""
from __future__ import annotations

import ctypes
import os
import platform
import subprocess
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
REF_DIR = os.path.join(HERE, "_ref")
ORACLE_SO = os.path.join(BUILD_DIR, "libgsea_oracle.so")
REF_SO = os.path.join(REF_DIR, "libgsea_ref.so")

METRICS = [
    "naive_diff_of_classes",
    "naive_ratio_of_classes",
    "naive_log2_ratio_of_classes",
    "stable_diff_of_classes",
    "stable_ratio_of_classes",
    "stable_log2_ratio_of_classes",
    "onepass_signal2noise",
    "onepass_t_test",
    "twopass_signal2noise",
    "twopass_t_test",
    "stable_signal2noise",
    "stable_t_test",
    "overkill_signal2noise",
    "overkill_t_test",
]
PERMUTATION_SEED = 42


def build(force: bool = False) -> str:
    """Compile gsea_oracle.cpp (g++, -ffp-contract=off, OpenMP)."""
    src = os.path.join(HERE, "gsea_oracle.cpp")
    os.makedirs(BUILD_DIR, exist_ok=True)
    if (not force and os.path.exists(ORACLE_SO) and _elf_machine(ORACLE_SO) == platform.machine()
            and os.path.getmtime(ORACLE_SO) >= os.path.getmtime(src)):
        return ORACLE_SO
    tmp = ORACLE_SO + f".tmp{os.getpid()}"
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-fopenmp",
           "-ffp-contract=off", "-o", tmp, src]
    subprocess.check_call(cmd)
    os.replace(tmp, ORACLE_SO)
    return ORACLE_SO


STAGED_REF = os.path.join(os.path.dirname(HERE), "baseline", "_ref")


def stage_ref() -> None:
    """Stage the reference's CPU-path sources into baseline/_ref/ (git-ignored)
    where they exist on this machine, so that they travel to the GPU host and
    build_ref() can compile them there (oracle/stage_ref.sh)."""
    subprocess.check_call(["bash", os.path.join(HERE, "stage_ref.sh")])


def _ref_root(reference_root: Optional[str]) -> Optional[str]:
    for root in (reference_root, os.environ.get("GSEA_REFERENCE_ROOT"), STAGED_REF):
        if root and os.path.isdir(os.path.join(root, "cudaGSEA", "src", "include")):
            return root
    return None


def build_ref(reference_root: Optional[str] = None, wait: bool = True):
    """Build the reference's CPU stages (oracle/build_ref.sh) from
    `reference_root`, $GSEA_REFERENCE_ROOT or the staged copy, whichever
    exists first; None when there are no sources.  wait=False starts the
    build and returns its process (or REF_SO when it is up to date)."""
    root = _ref_root(reference_root)
    if root is None:
        return None
    script = os.path.join(HERE, "build_ref.sh")
    if ref_available() and os.path.getmtime(REF_SO) >= max(
            os.path.getmtime(script), os.path.getmtime(os.path.join(HERE, "ref_harness.cu"))):
        return REF_SO
    proc = subprocess.Popen(["bash", script, root])
    if not wait:
        return proc
    if proc.wait() != 0:
        raise subprocess.CalledProcessError(proc.returncode, script)
    return REF_SO


def _elf_machine(path: str) -> Optional[str]:
    try:
        with open(path, "rb") as f:
            head = f.read(20)
    except OSError:
        return None
    if head[:4] != b"\x7fELF":
        return None
    mach = int.from_bytes(head[18:20], "little")
    return {62: "x86_64", 183: "aarch64"}.get(mach, str(mach))


def ref_available() -> bool:
    """True when the reference CPU build exists and runs on this machine."""
    return os.path.exists(REF_SO) and _elf_machine(REF_SO) == platform.machine()


_lib = None
_ref = None

_p = ctypes.c_void_p
_sz = ctypes.c_size_t


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(ORACLE_SO)
        for name in ("orc_metric_f32", "orc_metric_f64"):
            getattr(L, name).argtypes = [ctypes.c_int, _p, _p, _sz, _sz, _sz, _sz, ctypes.c_uint32, _p]
            getattr(L, name).restype = ctypes.c_int
        for name in ("orc_sort_f32", "orc_sort_f64"):
            getattr(L, name).argtypes = [_p, _sz, _sz, ctypes.c_int, _p, _p]
        for name in ("orc_es_f32", "orc_es_f64"):
            getattr(L, name).argtypes = [_p, _p, _sz, _sz, _p, _p, _sz, _p]
        for name in ("orc_stats_f32", "orc_stats_f64"):
            getattr(L, name).argtypes = [_p, _sz, _sz, _p]
        for name in ("orc_gsea_f32", "orc_gsea_f64"):
            getattr(L, name).argtypes = [ctypes.c_int, _p, _p, _sz, _sz, _p, _p, _sz, _sz,
                                         ctypes.c_int, ctypes.c_uint32, _p, _p]
            getattr(L, name).restype = ctypes.c_int
        L.orc_perm_labels.argtypes = [_p, _sz, _sz, _sz, ctypes.c_uint32, _p]
        L.orc_kiss_stream.argtypes = [ctypes.c_uint32, _sz, _p]
        L.orc_kiss_stream.restype = ctypes.c_uint32
        _lib = L
    return _lib


def ref():
    global _ref
    if _ref is None:
        if not ref_available():
            raise RuntimeError("reference CPU build (oracle/_ref) is not available here")
        R = ctypes.CDLL(REF_SO)
        for name in ("ref_correlate_f32", "ref_correlate_f64"):
            getattr(R, name).argtypes = [ctypes.c_char_p, _p, _p, _sz, _sz, _sz, _sz, _p]
        for name in ("ref_sort_f32", "ref_sort_f64"):
            getattr(R, name).argtypes = [_p, _sz, _sz, _p, ctypes.c_int]
        for name in ("ref_scores_f32", "ref_scores_f64"):
            getattr(R, name).argtypes = [_p, _p, _sz, _sz, _p, _p, _sz, _p]
        for name in ("ref_final_statistics_f32", "ref_final_statistics_f64"):
            getattr(R, name).argtypes = [_p, _sz, _sz, _p]
        for name in ("ref_pipeline_f32", "ref_pipeline_f64"):
            getattr(R, name).argtypes = [ctypes.c_char_p, _p, _p, _sz, _sz, _p, _p, _sz, _sz,
                                         ctypes.c_int, _p, _p]
        _ref = R
    return _ref


def _dt(double: bool):
    return np.float64 if double else np.float32


def _sfx(double: bool) -> str:
    return "f64" if double else "f32"


# ------------------------------------------------------------------ oracle API
def kiss_stream(seed: int, n: int) -> np.ndarray:
    out = np.zeros(n, np.uint32)
    lib().orc_kiss_stream(seed, n, _ptr(out))
    return out


def perm_labels(labels: np.ndarray, P: int, shift: int = 0, seed: int = PERMUTATION_SEED) -> np.ndarray:
    labels = np.ascontiguousarray(labels, np.uint8)
    out = np.zeros((P, labels.size), np.uint8)
    lib().orc_perm_labels(_ptr(labels), labels.size, P, shift, seed, _ptr(out))
    return out


def metric(metric_id: int, exprs_pm: np.ndarray, labels: np.ndarray, P: int, shift: int = 0,
           double: bool = False, seed: int = PERMUTATION_SEED) -> np.ndarray:
    """keys[P][G]; exprs_pm is patient-major [S][G]."""
    x = np.ascontiguousarray(exprs_pm, _dt(double))
    S, G = x.shape
    labels = np.ascontiguousarray(labels, np.uint8)
    out = np.zeros((P, G), _dt(double))
    rc = getattr(lib(), "orc_metric_" + _sfx(double))(metric_id, _ptr(x), _ptr(labels), G, S, P,
                                                     shift, seed, _ptr(out))
    if rc:
        raise ValueError(f"unknown metric id {metric_id}")
    return out


def sort(keys: np.ndarray, ascending: bool = False):
    double = keys.dtype == np.float64
    k = np.ascontiguousarray(keys)
    P, G = k.shape
    sk = np.zeros_like(k)
    idx = np.zeros((P, G), np.uint32)
    getattr(lib(), "orc_sort_" + _sfx(double))(_ptr(k), G, P, int(ascending), _ptr(sk), _ptr(idx))
    return sk, idx


def es(sorted_keys: np.ndarray, idx: np.ndarray, set_offsets: np.ndarray, set_genes: np.ndarray) -> np.ndarray:
    double = sorted_keys.dtype == np.float64
    sk = np.ascontiguousarray(sorted_keys)
    ix = np.ascontiguousarray(idx, np.uint32)
    off = np.ascontiguousarray(set_offsets, np.int64)
    gs = np.ascontiguousarray(set_genes, np.int32)
    P, G = sk.shape
    K = off.size - 1
    out = np.zeros((K, P), sk.dtype)
    getattr(lib(), "orc_es_" + _sfx(double))(_ptr(sk), _ptr(ix), G, P, _ptr(off), _ptr(gs), K, _ptr(out))
    return out


def stats(es_mat: np.ndarray) -> np.ndarray:
    double = es_mat.dtype == np.float64
    e = np.ascontiguousarray(es_mat)
    K, P = e.shape
    out = np.zeros(5 * K, e.dtype)
    getattr(lib(), "orc_stats_" + _sfx(double))(_ptr(e), K, P, _ptr(out))
    return out


def gsea(metric_id: int, exprs_pm: np.ndarray, labels: np.ndarray, set_offsets: np.ndarray,
         set_genes: np.ndarray, P: int, double: bool = False, ascending: bool = False,
         seed: int = PERMUTATION_SEED):
    """Full pipeline; returns (es[K][P], stats[5K])."""
    x = np.ascontiguousarray(exprs_pm, _dt(double))
    S, G = x.shape
    labels = np.ascontiguousarray(labels, np.uint8)
    off = np.ascontiguousarray(set_offsets, np.int64)
    gs = np.ascontiguousarray(set_genes, np.int32)
    K = off.size - 1
    e = np.zeros((K, P), _dt(double))
    st = np.zeros(5 * K, _dt(double))
    rc = getattr(lib(), "orc_gsea_" + _sfx(double))(metric_id, _ptr(x), _ptr(labels), G, S, _ptr(off),
                                                   _ptr(gs), K, P, int(ascending), seed, _ptr(e), _ptr(st))
    if rc:
        raise ValueError(f"unknown metric id {metric_id}")
    return e, st


# ------------------------------------------------------------------ reference API
def ref_metric(metric_id: int, exprs_pm: np.ndarray, labels: np.ndarray, P: int, shift: int = 0,
               double: bool = False) -> np.ndarray:
    x = np.ascontiguousarray(np.asarray(exprs_pm, _dt(double)).T)  # gene-major for the CPU path
    G, S = x.shape
    labels = np.ascontiguousarray(labels, np.uint8)
    out = np.zeros((P, G), _dt(double))
    getattr(ref(), "ref_correlate_" + _sfx(double))(METRICS[metric_id].encode(), _ptr(x), _ptr(labels),
                                                   G, S, P, shift, _ptr(out))
    return out


def ref_sort(keys: np.ndarray, ascending: bool = False):
    k = np.array(keys, copy=True, order="C")
    P, G = k.shape
    idx = np.zeros((P, G), np.uint32)
    getattr(ref(), "ref_sort_" + _sfx(k.dtype == np.float64))(_ptr(k), G, P, _ptr(idx), int(ascending))
    return k, idx


def ref_es(sorted_keys, idx, set_offsets, set_genes):
    double = sorted_keys.dtype == np.float64
    sk = np.ascontiguousarray(sorted_keys)
    ix = np.ascontiguousarray(idx, np.uint32)
    off = np.ascontiguousarray(set_offsets, np.int64)
    gs = np.ascontiguousarray(set_genes, np.int32)
    P, G = sk.shape
    K = off.size - 1
    out = np.zeros((K, P), sk.dtype)
    getattr(ref(), "ref_scores_" + _sfx(double))(_ptr(sk), _ptr(ix), G, P, _ptr(off), _ptr(gs), K, _ptr(out))
    return out


def ref_stats(es_mat):
    e = np.ascontiguousarray(es_mat)
    K, P = e.shape
    out = np.zeros(5 * K, e.dtype)
    getattr(ref(), "ref_final_statistics_" + _sfx(e.dtype == np.float64))(_ptr(e), K, P, _ptr(out))
    return out


def ref_gsea(metric_id, exprs_pm, labels, set_offsets, set_genes, P, double=False, ascending=False):
    x = np.ascontiguousarray(np.asarray(exprs_pm, _dt(double)).T)
    G, S = x.shape
    labels = np.ascontiguousarray(labels, np.uint8)
    off = np.ascontiguousarray(set_offsets, np.int64)
    gs = np.ascontiguousarray(set_genes, np.int32)
    K = off.size - 1
    e = np.zeros((K, P), _dt(double))
    st = np.zeros(5 * K, _dt(double))
    getattr(ref(), "ref_pipeline_" + _sfx(double))(METRICS[metric_id].encode(), _ptr(x), _ptr(labels), G, S,
                                                  _ptr(off), _ptr(gs), K, P, int(ascending), _ptr(e), _ptr(st))
    return e, st
