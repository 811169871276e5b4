"""Python host API of the GB300 GSEA pipeline.

Mirrors cudaGSEA's R interface (cudaGSEA/R/GSEA.R:1-5, cudaGSEA/R/CUDA.R:1-11)
on top of the C ABI of libgsea103.so:

* ``GSEA(exprsData, labelList, geneSets, numPermutations, metricString="",
  dumpFileName="", checkInput=True, doublePrecision=False)`` -- same
  arguments, same input checks and messages as the Rcpp layer
  (src/cudaGSEA_wrapper.cpp:86-280), returns a table with ES, NES, NP, FWER
  (and FDR) per gene set, or ``False`` when a check fails.
* ``listCudaDevices()``, ``getCudaDevice()``, ``setCudaDevice(id)``.
* ``Plan`` -- device-resident inputs for repeated execution (benchmarks,
  sharded permutation ranges), and ``gsea()`` for array inputs.
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field
from typing import Dict, List, Mapping, Optional, Sequence, Tuple, Union

import numpy as np

from . import _native as N

METRICS = [
    "naive_diff_of_classes", "naive_ratio_of_classes", "naive_log2_ratio_of_classes",
    "stable_diff_of_classes", "stable_ratio_of_classes", "stable_log2_ratio_of_classes",
    "onepass_signal2noise", "onepass_t_test", "twopass_signal2noise", "twopass_t_test",
    "stable_signal2noise", "stable_t_test", "overkill_signal2noise", "overkill_t_test",
]


def metric_id(metric: Union[str, int]) -> int:
    if isinstance(metric, (int, np.integer)):
        return int(metric)
    mid = N.lib().gsea_metric_id(metric.encode())
    if mid < 0:
        raise N.GseaError(2, f"unknown metric: {metric}")
    return mid


# ------------------------------------------------------------------ devices
def listCudaDevices() -> List[str]:
    n = ctypes.c_int(0)
    N.check(N.lib().gsea_device_count(ctypes.byref(n)))
    out = []
    buf = ctypes.create_string_buffer(512)
    for d in range(n.value):
        N.check(N.lib().gsea_device_string(d, buf, 512))
        out.append(buf.value.decode())
    return out


def getCudaDevice() -> int:
    d = ctypes.c_int(0)
    N.check(N.lib().gsea_get_device(ctypes.byref(d)))
    return d.value


def setCudaDevice(device_id: int) -> int:
    """Select a device; like the reference, an invalid id warns and keeps the current one."""
    active = ctypes.c_int(0)
    rc = N.lib().gsea_set_device(int(device_id), ctypes.byref(active))
    if rc != N.GSEA_OK:
        print(f"WARNING: invalid device id, fallback to device {active.value}.")
    return active.value


# ------------------------------------------------------------------ plans
class Plan:
    """A device-resident GSEA problem (gsea_plan in the C ABI)."""

    def __init__(self, num_genes: int, num_samples: int, num_sets: int, num_perms: int,
                 metric: Union[str, int] = "twopass_signal2noise", precision: int = 32,
                 ascending: bool = False, form: int = N.FORM_PLAIN, perm_offset: int = 0,
                 perm_batch: int = 0, seed: int = 42, device: int = -1):
        L = N.lib()
        cfg = N.Config()
        L.gsea_config_init(ctypes.byref(cfg))
        cfg.num_genes, cfg.num_samples = num_genes, num_samples
        cfg.num_sets, cfg.num_perms = num_sets, num_perms
        cfg.metric = metric_id(metric)
        cfg.precision = precision
        cfg.ascending = int(bool(ascending))
        cfg.form = form
        cfg.perm_offset, cfg.perm_batch = perm_offset, perm_batch
        cfg.seed, cfg.device = seed, device
        self.cfg = cfg
        self.dtype = np.float64 if precision == 64 else np.float32
        h = ctypes.c_void_p()
        N.check(L.gsea_plan_create(ctypes.byref(cfg), ctypes.byref(h)))
        self._h = h
        pb = ctypes.c_int64(0)
        r16 = ctypes.c_int(0)
        N.check(L.gsea_plan_info(h, ctypes.byref(pb), ctypes.byref(r16)))
        self.perm_batch = pb.value
        self.ranks16 = bool(r16.value)
        self._keep = []

    # ---- inputs
    def _prep(self, exprs, labels, set_offsets, set_genes):
        x = np.ascontiguousarray(exprs, self.dtype)
        if x.shape != (self.cfg.num_samples, self.cfg.num_genes):
            raise ValueError(f"exprs must be patient-major [{self.cfg.num_samples}][{self.cfg.num_genes}]")
        lab = np.ascontiguousarray(labels, np.uint8)
        off = np.ascontiguousarray(set_offsets, np.int64)
        gs = np.ascontiguousarray(set_genes, np.int32)
        if off.size != self.cfg.num_sets + 1:
            raise ValueError("set_offsets must have num_sets + 1 entries")
        return x, lab, off, gs

    def set_inputs(self, exprs, labels, set_offsets, set_genes) -> None:
        x, lab, off, gs = self._prep(exprs, labels, set_offsets, set_genes)
        N.check(N.lib().gsea_plan_set_inputs(self._h, N.ptr(x), N.ptr(lab), N.ptr(off), N.ptr(gs)))

    def execute(self, stream: Optional[int] = None) -> None:
        N.check(N.lib().gsea_plan_execute(self._h, ctypes.c_void_p(stream) if stream else None))

    def synchronize(self) -> None:
        N.check(N.lib().gsea_plan_synchronize(self._h))

    def read(self, es: bool = True, stats: bool = True) -> Tuple[Optional[np.ndarray], Optional[np.ndarray]]:
        K, P = self.cfg.num_sets, self.cfg.num_perms
        e = np.empty((K, P), self.dtype) if es else None
        s = np.empty(5 * K, self.dtype) if stats else None
        N.check(N.lib().gsea_plan_read(self._h, N.ptr(e), N.ptr(s)))
        return e, s

    def run_host(self, exprs, labels, set_offsets, set_genes, es_out=None, stats_out=None):
        """Upload + execute + download in one call (host buffers; pinned ones copy asynchronously)."""
        x, lab, off, gs = self._prep(exprs, labels, set_offsets, set_genes)
        N.check(N.lib().gsea_plan_run_host(self._h, N.ptr(x), N.ptr(lab), N.ptr(off), N.ptr(gs),
                                           N.ptr(es_out), N.ptr(stats_out)))
        return es_out, stats_out

    # ---- introspection
    def set_debug(self, keep: bool = True) -> None:
        N.check(N.lib().gsea_plan_set_debug(self._h, int(keep)))

    def buffer(self, which: int) -> Tuple[int, int]:
        p = ctypes.c_void_p()
        n = ctypes.c_size_t(0)
        N.check(N.lib().gsea_plan_buffer(self._h, which, ctypes.byref(p), ctypes.byref(n)))
        return (p.value or 0), n.value

    def read_buffer(self, which: int, dtype, shape) -> np.ndarray:
        out = np.empty(shape, dtype)
        N.check(N.lib().gsea_plan_read_buffer(self._h, which, N.ptr(out), out.nbytes))
        return out

    # ---- launch configuration
    def set_tuning(self, **kw) -> None:
        """metric_pb, chosen_tile, sort_variant, es_warps, es_stage (0 / -1 = automatic)."""
        t = N.Tuning()
        N.lib().gsea_tuning_init(ctypes.byref(t))
        for k, v in kw.items():
            if not hasattr(t, k):
                raise TypeError(f"unknown tuning field {k}")
            setattr(t, k, v)
        N.check(N.lib().gsea_plan_set_tuning(self._h, ctypes.byref(t)))

    def get_tuning(self) -> Dict[str, int]:
        t = N.Tuning()
        N.check(N.lib().gsea_plan_get_tuning(self._h, ctypes.byref(t)))
        return {name: getattr(t, name) for name, _ in N.Tuning._fields_}

    def autotune(self, sample_perms: int = 0) -> Tuple[Dict[str, int], Dict[str, float]]:
        """Time every launch configuration on the plan's inputs and keep the fastest."""
        t = N.Tuning()
        ms = (ctypes.c_double * 3)()
        N.check(N.lib().gsea_plan_autotune(self._h, sample_perms, ctypes.byref(t), ms))
        return ({name: getattr(t, name) for name, _ in N.Tuning._fields_},
                {"metric": ms[0], "sort": ms[1], "es": ms[2]})

    def set_profiling(self, on: bool = True) -> None:
        N.check(N.lib().gsea_plan_set_profiling(self._h, int(on)))

    def stage_times(self) -> Dict[str, float]:
        """Device milliseconds per stage of the last execute (profiling on)."""
        ms = (ctypes.c_double * len(N.STAGES))()
        N.check(N.lib().gsea_plan_stage_times(self._h, ms))
        return dict(zip(N.STAGES, list(ms)))

    def last_launches(self) -> int:
        n = ctypes.c_int64(0)
        N.check(N.lib().gsea_plan_last_launches(self._h, ctypes.byref(n)))
        return n.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().gsea_plan_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def map_sets(gene_symbols: Sequence[str], gene_sets: Sequence[Sequence[str]]) -> Tuple[np.ndarray, np.ndarray]:
    """Gene-set symbols -> CSR (offsets int64[K+1], genes int32) on the device
    (gsea_map_sets): unknown symbols dropped, duplicates collapsed, ascending."""
    L = N.lib()
    gs = [s.encode() for s in gene_symbols]
    garr = (ctypes.c_char_p * len(gs))(*gs)
    members = [m.encode() for st in gene_sets for m in st]
    marr = (ctypes.c_char_p * max(1, len(members)))(*members)
    soff = np.zeros(len(gene_sets) + 1, np.int64)
    soff[1:] = np.cumsum([len(st) for st in gene_sets]) if len(gene_sets) else []
    off = np.empty(len(gene_sets) + 1, np.int64)
    genes = np.empty(max(1, len(members)), np.int32)
    nnz = ctypes.c_int64(0)
    N.check(L.gsea_map_sets(len(gs), garr, len(gene_sets), N.ptr(soff), marr, N.ptr(off), N.ptr(genes),
                            genes.size, ctypes.byref(nnz)))
    return off, genes[:nnz.value].copy()


class Batch:
    """Many independent GSEA instances run together in one CUDA graph
    (gsea_batch in the C ABI).  `instances`: GseaInput-like objects (exprs,
    labels, set_offsets, set_genes, num_perms); one metric / precision / form
    for all, or a metric (and a sort direction) per instance."""

    def __init__(self, instances, metric: Union[str, int, Sequence] = "twopass_signal2noise", precision: int = 32,
                 form: int = N.FORM_PLAIN, streams: int = 0, seed: int = 42, device: int = -1,
                 ascending: Union[bool, Sequence[bool]] = False):
        L = N.lib()
        n = len(instances)
        cfgs = (N.Config * n)()
        metrics = list(metric) if isinstance(metric, (list, tuple)) else [metric] * n
        asc = list(ascending) if isinstance(ascending, (list, tuple)) else [ascending] * n
        for i, d in enumerate(instances):
            c = cfgs[i]
            L.gsea_config_init(ctypes.byref(c))
            c.num_samples, c.num_genes = d.exprs.shape
            c.num_sets = len(d.set_offsets) - 1
            c.num_perms = d.num_perms
            c.metric = metric_id(metrics[i])
            c.precision, c.form, c.seed, c.device = precision, form, seed, device
            c.ascending = 1 if asc[i] else 0
        h = ctypes.c_void_p()
        N.check(L.gsea_batch_create(n, cfgs, streams, ctypes.byref(h)))
        self._h = h
        self.cfgs = cfgs
        self.dtype = np.float64 if precision == 64 else np.float32
        for i, d in enumerate(instances):
            x = np.ascontiguousarray(d.exprs, self.dtype)
            lab = np.ascontiguousarray(d.labels, np.uint8)
            off = np.ascontiguousarray(d.set_offsets, np.int64)
            gs = np.ascontiguousarray(d.set_genes, np.int32)
            N.check(L.gsea_batch_set_inputs(h, i, N.ptr(x), N.ptr(lab), N.ptr(off), N.ptr(gs)))

    def __len__(self):
        return len(self.cfgs)

    def autotune(self, sample_perms: int = 0) -> None:
        N.check(N.lib().gsea_batch_autotune(self._h, sample_perms))

    def execute(self, stream: Optional[int] = None) -> None:
        N.check(N.lib().gsea_batch_execute(self._h, ctypes.c_void_p(stream) if stream else None))

    def synchronize(self) -> None:
        N.check(N.lib().gsea_batch_synchronize(self._h))

    def read(self, i: int, es: bool = True, stats: bool = True):
        c = self.cfgs[i]
        e = np.empty((c.num_sets, c.num_perms), self.dtype) if es else None
        s = np.empty(5 * c.num_sets, self.dtype) if stats else None
        N.check(N.lib().gsea_batch_read(self._h, i, N.ptr(e), N.ptr(s)))
        return e, s

    def info(self) -> Dict[str, int]:
        a, b, c = ctypes.c_int64(0), ctypes.c_int64(0), ctypes.c_int64(0)
        N.check(N.lib().gsea_batch_info(self._h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c)))
        return {"graph_nodes": a.value, "es_classes": b.value, "launches": c.value}

    def tuning(self, i: int) -> Dict[str, int]:
        p = ctypes.c_void_p()
        N.check(N.lib().gsea_batch_plan(self._h, i, ctypes.byref(p)))
        t = N.Tuning()
        N.check(N.lib().gsea_plan_get_tuning(p, ctypes.byref(t)))
        return {name: getattr(t, name) for name, _ in N.Tuning._fields_}

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().gsea_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def gsea(exprs_pm: np.ndarray, labels: np.ndarray, set_offsets: np.ndarray, set_genes: np.ndarray,
         num_perms: int, metric: Union[str, int] = "twopass_signal2noise", precision: int = 32,
         ascending: bool = False, dump_prefix: Optional[str] = None) -> Tuple[np.ndarray, np.ndarray]:
    """One-shot pipeline on arrays (gsea_run): returns es[K][P], stats[5K]."""
    dt = np.float64 if precision == 64 else np.float32
    x = np.ascontiguousarray(exprs_pm, dt)
    S, G = x.shape
    lab = np.ascontiguousarray(labels, np.uint8)
    off = np.ascontiguousarray(set_offsets, np.int64)
    gs = np.ascontiguousarray(set_genes, np.int32)
    K = off.size - 1
    cfg = N.Config()
    N.lib().gsea_config_init(ctypes.byref(cfg))
    cfg.num_genes, cfg.num_samples, cfg.num_sets, cfg.num_perms = G, S, K, num_perms
    cfg.metric, cfg.precision, cfg.ascending = metric_id(metric), precision, int(bool(ascending))
    es = np.empty((K, num_perms), dt)
    st = np.empty(5 * K, dt)
    N.check(N.lib().gsea_run(ctypes.byref(cfg), N.ptr(x), N.ptr(lab), N.ptr(off), N.ptr(gs), N.ptr(es),
                             N.ptr(st), dump_prefix.encode() if dump_prefix else None))
    return es, st


# ------------------------------------------------------------------ R-style API
@dataclass
class ExpressionTable:
    """The R data.frame argument: rows = genes (row.names), columns = patients."""
    values: np.ndarray                  # [genes][patients]
    genes: Sequence[str]
    patients: Sequence[str]


@dataclass
class GseaResult:
    """data.frame(ES, NES, NP, FWER) with row.names = gene-set names, plus FDR."""
    names: List[str]
    ES: np.ndarray
    NES: np.ndarray
    NP: np.ndarray
    FWER: np.ndarray
    FDR: np.ndarray = field(default_factory=lambda: np.zeros(0))

    def as_dict(self) -> Dict[str, np.ndarray]:
        return {"ES": self.ES, "NES": self.NES, "NP": self.NP, "FWER": self.FWER, "FDR": self.FDR}


def _as_table(exprsData) -> ExpressionTable:
    if isinstance(exprsData, ExpressionTable):
        return exprsData
    if isinstance(exprsData, Mapping):
        return ExpressionTable(np.asarray(exprsData["values"]), list(exprsData["genes"]),
                               list(exprsData["patients"]))
    values, genes, patients = exprsData
    return ExpressionTable(np.asarray(values), list(genes), list(patients))


def GSEA(exprsData, labelList: Sequence[int], geneSets: Mapping[str, Sequence[str]], numPermutations: int,
         metricString: str = "", dumpFileName: str = "", checkInput: bool = True,
         doublePrecision: bool = False) -> Union[GseaResult, bool]:
    """R's GSEA(); see the module docstring.  Returns False when an input check fails."""
    table = _as_table(exprsData)
    values = np.asarray(table.values, np.float64)
    names = list(geneSets.keys())
    sets = [list(geneSets[n]) for n in names]
    if any(n in ("", "NA", None) for n in names):
        names = [str(i + 1) for i in range(len(sets))]
        print("WARNING: We enumerated your gene set names from 1 to n.")
    labels = [int(x) for x in labelList]
    if checkInput:
        if values.ndim != 2 or values.shape[0] != len(table.genes):
            print("INVALID DATA: the vertical dimension and the number of row names do not comply.")
            return False
        if values.shape[1] != len(table.patients):
            print("INVALID DATA: the horizontal dimension and the number of column names do not comply.")
            return False
        if len(labels) != values.shape[1]:
            print("INVALID DATA: Your label list has a different amount of entries as the number of "
                  "columns in your gene  expression data frame.")
            return False
        if any(l not in (0, 1) for l in labels):
            print("INVALID DATA: Label vector may only contain zeros and ones since cudaGSEA only "
                  "supports two classes of phenotypes.")
            return False
        if np.isnan(values).any():
            print("INVALID DATA: expression table has NaN entries that cannot be handled by the GSEA algorithm.")
            return False
        if values.size and values.min() < 0:
            print("WARNING: There are negative expression values in the provided table. Some metrics "
                  "cannot handle negative amplitudes e.g. the log2_ratio_of_classes family.")
        if len(sets) == 0:
            print("INVALID DATA: you must at least specify one gene set.")
            return False
        if any(len(s) == 0 for s in sets):
            print("INVALID DATA: There is an empty gene set (no gene identifiers) in your list of gene sets.")
            return False
    precision = 64 if doublePrecision else 32
    dt = np.float64 if doublePrecision else np.float32
    exprs_pm = np.ascontiguousarray(values.T, dt)  # R's column-major matrix = patient-major
    G, S = len(table.genes), len(table.patients)
    gene_syms = [str(g).encode() for g in table.genes]
    set_syms = [str(s).encode() for ss in sets for s in ss]
    sym_off = np.zeros(len(sets) + 1, np.int64)
    sym_off[1:] = np.cumsum([len(s) for s in sets])
    c_genes = (ctypes.c_char_p * max(1, G))(*gene_syms)
    c_sets = (ctypes.c_char_p * max(1, len(set_syms)))(*set_syms)
    lab = np.ascontiguousarray(labels, np.uint8)
    K = len(sets)
    out = np.empty(5 * K, dt)
    rc = N.lib().gsea_proxy_run(precision, N.ptr(exprs_pm), G, S, c_genes, N.ptr(lab), K, N.ptr(sym_off),
                                c_sets, metricString.encode(), int(numPermutations), 1, 0,
                                dumpFileName.encode() if dumpFileName else None, N.ptr(out))
    N.check(rc)
    return GseaResult(names, out[0:K].copy(), out[K:2 * K].copy(), out[2 * K:3 * K].copy(),
                      out[3 * K:4 * K].copy(), out[4 * K:5 * K].copy())
