"""cudagsea_gb300 -- GB300-native GSEA permutation pipeline.

A from-scratch sm_103a implementation of cudaGSEA's permutation path
(label permutation -> class statistics and ranking metric -> per-permutation
sort -> running-sum enrichment score -> NES / nominal p / FWER / FDR) behind the
reference's own interfaces: the C++ proxies of include/gsea103_proxy.hpp, the
C ABI of include/gsea103.h and, here, a Python mirror of the R functions.

Compute runs only in libgsea103.so: every compute call raises if the library
has not been built (``cudagsea_gb300.build.build()``); there is no CPU
fallback.
"""
from .api import (METRICS, GSEA, Batch, ExpressionTable, GseaResult, Plan, getCudaDevice, gsea,
                  listCudaDevices, metric_id, setCudaDevice)
from ._native import GseaError, FORM_CHOSEN, FORM_CHOSEN_FP64, FORM_PLAIN

__all__ = ["METRICS", "GSEA", "Batch", "ExpressionTable", "GseaResult", "Plan", "getCudaDevice", "gsea",
           "listCudaDevices", "metric_id", "setCudaDevice", "GseaError", "FORM_PLAIN", "FORM_CHOSEN",
           "FORM_CHOSEN_FP64"]
