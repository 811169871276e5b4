"""ctypes binding of libgsea103.so (include/gsea103.h).

The library is the product: every compute call goes through it.  If the
shared object is missing or cannot be loaded, importing the bindings raises --
there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
from typing import Optional

import numpy as np

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "_lib", "libgsea103.so")

GSEA_OK = 0
STATUS = {
    0: "GSEA_OK", 1: "GSEA_ERR_INVALID_ARGUMENT", 2: "GSEA_ERR_UNKNOWN_METRIC", 3: "GSEA_ERR_CUDA",
    4: "GSEA_ERR_OUT_OF_MEMORY", 5: "GSEA_ERR_NO_DEVICE", 6: "GSEA_ERR_IO", 7: "GSEA_ERR_UNSUPPORTED",
    8: "GSEA_ERR_INJECTED", 9: "GSEA_ERR_INVALID_INPUT",
}

BUF_EXPRS, BUF_LABEL_MASKS, BUF_KEYS, BUF_RANKS, BUF_ORDER, BUF_ES, BUF_STATS, BUF_SORTED = range(8)
FORM_PLAIN, FORM_CHOSEN, FORM_CHOSEN_FP64 = 0, 1, 2
STAGES = ("permute", "metric", "sort", "es", "stats")


class GseaError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Config(ctypes.Structure):
    _fields_ = [
        ("num_genes", ctypes.c_int64),
        ("num_samples", ctypes.c_int64),
        ("num_sets", ctypes.c_int64),
        ("num_perms", ctypes.c_int64),
        ("metric", ctypes.c_int32),
        ("precision", ctypes.c_int32),
        ("ascending", ctypes.c_int32),
        ("form", ctypes.c_int32),
        ("perm_offset", ctypes.c_int64),
        ("perm_batch", ctypes.c_int64),
        ("seed", ctypes.c_uint32),
        ("device", ctypes.c_int32),
    ]


class Tuning(ctypes.Structure):
    _fields_ = [
        ("metric_pb", ctypes.c_int32),
        ("chosen_tile", ctypes.c_int32),
        ("sort_variant", ctypes.c_int32),
        ("es_warps", ctypes.c_int32),
        ("es_stage", ctypes.c_int32),
    ]


class AdaptiveParams(ctypes.Structure):
    _fields_ = [
        ("pilot_perms", ctypes.c_int64),
        ("growth", ctypes.c_double),
        ("z", ctypes.c_double),
        ("q_call", ctypes.c_double),
        ("margin", ctypes.c_double),
        ("p_floor", ctypes.c_double),
        ("prior_cap", ctypes.c_double),
        ("fallback_tol", ctypes.c_double),
        ("q_margin", ctypes.c_double),
        ("sig_margin", ctypes.c_double),
    ]


class AdaptiveReport(ctypes.Structure):
    _fields_ = [
        ("rounds", ctypes.c_int64),
        ("scores", ctypes.c_int64),
        ("stopped_pilot", ctypes.c_int64),
        ("full_sets", ctypes.c_int64),
        ("stop_p", ctypes.c_double),
        ("model_used", ctypes.c_int32),
        ("model_mean_err", ctypes.c_double),
        ("prior_sets", ctypes.c_int64),
        ("prior_agreed", ctypes.c_int64),
        ("stopped_q", ctypes.c_int64),
        ("stopped_sig", ctypes.c_int64),
        ("p_sig", ctypes.c_double),
    ]


MODEL_INPUTS, MODEL_HIDDEN, MODEL_OUTPUTS, MODEL_PARAMS, MODEL_NORMS = 5, 64, 2, 4674, 15

_lib: Optional[ctypes.CDLL] = None
_p = ctypes.c_void_p
_i64 = ctypes.c_int64
_sz = ctypes.c_size_t

# (name, restype, argtypes) of every symbol include/gsea103.h declares
SIGNATURES = [
    ("gsea_status_string", ctypes.c_char_p, [ctypes.c_int]),
    ("gsea_last_error", ctypes.c_char_p, []),
    ("gsea_metric_id", ctypes.c_int, [ctypes.c_char_p]),
    ("gsea_metric_name", ctypes.c_char_p, [ctypes.c_int]),
    ("gsea_config_init", None, [ctypes.POINTER(Config)]),
    ("gsea_device_count", ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    ("gsea_device_string", ctypes.c_int, [ctypes.c_int, ctypes.c_char_p, _sz]),
    ("gsea_get_device", ctypes.c_int, [ctypes.POINTER(ctypes.c_int)]),
    ("gsea_set_device", ctypes.c_int, [ctypes.c_int, ctypes.POINTER(ctypes.c_int)]),
    ("gsea_run", ctypes.c_int, [ctypes.POINTER(Config), _p, _p, _p, _p, _p, _p, ctypes.c_char_p]),
    ("gsea_run_f32", ctypes.c_int, [_p, _i64, _i64, _p, _p, _p, _i64, _i64, ctypes.c_int, ctypes.c_int, _p, _p,
                                    ctypes.c_char_p]),
    ("gsea_run_f64", ctypes.c_int, [_p, _i64, _i64, _p, _p, _p, _i64, _i64, ctypes.c_int, ctypes.c_int, _p, _p,
                                    ctypes.c_char_p]),
    ("gsea_proxy_run", ctypes.c_int, [ctypes.c_int, _p, _i64, _i64, _p, _p, _i64, _p, _p, ctypes.c_char_p, _i64,
                                      ctypes.c_int, ctypes.c_int, ctypes.c_char_p, _p]),
    ("gsea_shard_sum", ctypes.c_int, [_p, _i64, _i64, _i64, ctypes.c_int, _p, _p, _p]),
    ("gsea_shard_head", ctypes.c_int, [_p, _p, _i64, _i64, ctypes.c_int, _p, _p]),
    ("gsea_shard_partial", ctypes.c_int, [_p, _i64, _i64, _i64, ctypes.c_int, _i64, _p, _p, _p, _p]),
    ("gsea_shard_finish", ctypes.c_int, [_p, _i64, _i64, ctypes.c_int, _p, _p, _p, _p]),
    ("gsea_map_sets", ctypes.c_int, [_i64, _p, _i64, _p, _p, _p, _p, _i64, ctypes.POINTER(_i64)]),
    ("gsea_plan_create", ctypes.c_int, [ctypes.POINTER(Config), ctypes.POINTER(_p)]),
    ("gsea_plan_destroy", ctypes.c_int, [_p]),
    ("gsea_plan_set_inputs", ctypes.c_int, [_p, _p, _p, _p, _p]),
    ("gsea_plan_execute", ctypes.c_int, [_p, _p]),
    ("gsea_plan_run_host", ctypes.c_int, [_p, _p, _p, _p, _p, _p, _p]),
    ("gsea_plan_read", ctypes.c_int, [_p, _p, _p]),
    ("gsea_plan_synchronize", ctypes.c_int, [_p]),
    ("gsea_plan_buffer", ctypes.c_int, [_p, ctypes.c_int, ctypes.POINTER(_p), ctypes.POINTER(_sz)]),
    ("gsea_plan_read_buffer", ctypes.c_int, [_p, ctypes.c_int, _p, _sz]),
    ("gsea_plan_info", ctypes.c_int, [_p, ctypes.POINTER(_i64), ctypes.POINTER(ctypes.c_int)]),
    ("gsea_plan_set_debug", ctypes.c_int, [_p, ctypes.c_int]),
    ("gsea_plan_last_launches", ctypes.c_int, [_p, ctypes.POINTER(_i64)]),
    ("gsea_plan_set_profiling", ctypes.c_int, [_p, ctypes.c_int]),
    ("gsea_plan_stage_times", ctypes.c_int, [_p, ctypes.POINTER(ctypes.c_double)]),
    ("gsea_stats_scratch_bytes", ctypes.c_int, [_i64, _i64, ctypes.c_int, ctypes.POINTER(_sz)]),
    ("gsea_stats_device", ctypes.c_int, [_p, _i64, _i64, ctypes.c_int, _p, _p, _sz, _p]),
    ("gsea_stats_device_noalloc", ctypes.c_int, [_p, _i64, _i64, ctypes.c_int, _p, _p]),
    ("gsea_tuning_init", None, [ctypes.POINTER(Tuning)]),
    ("gsea_plan_set_tuning", ctypes.c_int, [_p, ctypes.POINTER(Tuning)]),
    ("gsea_plan_get_tuning", ctypes.c_int, [_p, ctypes.POINTER(Tuning)]),
    ("gsea_plan_autotune", ctypes.c_int, [_p, _i64, ctypes.POINTER(Tuning), ctypes.POINTER(ctypes.c_double)]),
    ("gsea_batch_create", ctypes.c_int, [_i64, ctypes.POINTER(Config), ctypes.c_int, ctypes.POINTER(_p)]),
    ("gsea_batch_destroy", ctypes.c_int, [_p]),
    ("gsea_batch_set_inputs", ctypes.c_int, [_p, _i64, _p, _p, _p, _p]),
    ("gsea_batch_autotune", ctypes.c_int, [_p, _i64]),
    ("gsea_batch_execute", ctypes.c_int, [_p, _p]),
    ("gsea_batch_synchronize", ctypes.c_int, [_p]),
    ("gsea_batch_read", ctypes.c_int, [_p, _i64, _p, _p]),
    ("gsea_batch_plan", ctypes.c_int, [_p, _i64, ctypes.POINTER(_p)]),
    ("gsea_batch_info", ctypes.c_int, [_p, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i64)]),
    ("gsea_model_create", ctypes.c_int, [ctypes.c_uint32, ctypes.c_int, ctypes.POINTER(_p)]),
    ("gsea_model_destroy", ctypes.c_int, [_p]),
    ("gsea_model_get", ctypes.c_int, [_p, _p, _p]),
    ("gsea_model_set", ctypes.c_int, [_p, _p, _p]),
    ("gsea_model_predict", ctypes.c_int, [_p, _p, _i64, _p, _p]),
    ("gsea_model_loss_grad", ctypes.c_int, [_p, _p, _p, _i64, _p, _p, _p]),
    ("gsea_model_train", ctypes.c_int, [_p, _p, _p, _i64, ctypes.c_int, ctypes.c_int, ctypes.c_float, _p]),
    ("gsea_model_calibrate", ctypes.c_int, [_p, _p, _p, _i64]),
    ("gsea_plan_model_samples", ctypes.c_int, [_p, ctypes.c_int, ctypes.c_int, _p, _p, ctypes.POINTER(_i64), _p, _p,
                                               ctypes.POINTER(_i64)]),
    ("gsea_adaptive_params_init", None, [ctypes.POINTER(AdaptiveParams)]),
    ("gsea_plan_execute_adaptive", ctypes.c_int, [_p, _p, ctypes.POINTER(AdaptiveParams), _p,
                                                  ctypes.POINTER(AdaptiveReport)]),
    ("gsea_adaptive_decide", ctypes.c_int, [_i64, _p, _p, _p, _p, ctypes.c_double, ctypes.c_double, _p]),
    ("gsea_stats_ragged", ctypes.c_int, [_p, _i64, _i64, _p, _i64, ctypes.c_int, _p, _p]),
    ("gsea_fdr_lower_bound", ctypes.c_int, [_p, _i64, _i64, _p, _i64, _p, ctypes.c_double, ctypes.c_int, _p, _p, _p]),
    ("gsea_dataset_load", ctypes.c_int, [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(_p)]),
    ("gsea_dataset_dims", ctypes.c_int, [_p, ctypes.POINTER(_i64), ctypes.POINTER(_i64), ctypes.POINTER(_i64),
                                         ctypes.POINTER(_i64)]),
    ("gsea_dataset_arrays", ctypes.c_int, [_p, ctypes.c_int, _p, _p, _p, _p]),
    ("gsea_dataset_gene", ctypes.c_char_p, [_p, _i64]),
    ("gsea_dataset_set_name", ctypes.c_char_p, [_p, _i64]),
    ("gsea_dataset_free", None, [_p]),
    ("gsea_host_alloc", ctypes.c_int, [_sz, ctypes.POINTER(_p)]),
    ("gsea_host_free", ctypes.c_int, [_p]),
    ("gsea_write_es_dump", ctypes.c_int, [ctypes.c_char_p, _p, _i64, _i64, ctypes.c_int, ctypes.c_char_p, _sz]),
]


def lib() -> ctypes.CDLL:
    """Load libgsea103.so; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError(f"{LIB_PATH} is missing: build it with cudagsea_gb300.build.build()")
        L = ctypes.CDLL(LIB_PATH)
        for name, res, args in SIGNATURES:
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def check(status: int) -> None:
    if status != GSEA_OK:
        msg = lib().gsea_last_error()
        raise GseaError(status, msg.decode() if msg else "")


def ptr(a: Optional[np.ndarray]):
    return None if a is None else ctypes.c_void_p(a.ctypes.data)
