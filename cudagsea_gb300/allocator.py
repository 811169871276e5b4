"""Learned permutation allocator: the network, its training on a plan's null
scores, and the adaptive permutation test (include/gsea103.h, "learned
permutation allocator").  No counterpart in the reference, which gives every
gene set the same number of permutations (src/cudaGSEA_wrapper.cu:300-372).

Device arrays are torch CUDA tensors (plumbing only: every computation runs in
libgsea103.so's kernels).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Dict, Optional, Tuple

import numpy as np

from . import _native as N

IN, H, OUT, NPARAM, NNORM = N.MODEL_INPUTS, N.MODEL_HIDDEN, N.MODEL_OUTPUTS, N.MODEL_PARAMS, N.MODEL_NORMS


def _torch():
    import torch
    return torch


def _dev_f32(a, device=None):
    """float32 contiguous CUDA tensor of `a` (numpy array or tensor)."""
    torch = _torch()
    if isinstance(a, torch.Tensor):
        t = a.to(dtype=torch.float32)
        if not t.is_cuda:
            t = t.cuda(device)
        return t.contiguous()
    return torch.as_tensor(np.ascontiguousarray(a, np.float32)).cuda(device)


def _vp(t) -> ctypes.c_void_p:
    return ctypes.c_void_p(t.data_ptr())


class Model:
    """The allocator's network (gsea_model): 5 -> 64 -> 64 -> 2, tanh, BF16
    parameters, FP32 accumulation; trained and evaluated by the library's own
    kernels."""

    def __init__(self, seed: int = 0, device: int = -1):
        h = ctypes.c_void_p()
        N.check(N.lib().gsea_model_create(seed, device, ctypes.byref(h)))
        self._h = h

    @property
    def handle(self):
        return self._h

    def get(self) -> Tuple[np.ndarray, np.ndarray]:
        p = np.empty(NPARAM, np.float32)
        n = np.empty(NNORM, np.float32)
        N.check(N.lib().gsea_model_get(self._h, N.ptr(p), N.ptr(n)))
        return p, n

    def set(self, params: Optional[np.ndarray] = None, norms: Optional[np.ndarray] = None) -> None:
        p = None if params is None else np.ascontiguousarray(params, np.float32)
        n = None if norms is None else np.ascontiguousarray(norms, np.float32)
        if p is not None and p.size != NPARAM:
            raise ValueError(f"params must have {NPARAM} entries")
        if n is not None and n.size != NNORM:
            raise ValueError(f"norms must have {NNORM} entries")
        N.check(N.lib().gsea_model_set(self._h, N.ptr(p), N.ptr(n)))

    @property
    def trained(self) -> bool:
        return bool(self.get()[1][14])

    def predict(self, x):
        """x [n][5] raw features -> [n][2] (tail probability, null mean), CUDA tensor."""
        torch = _torch()
        xd = _dev_f32(x)
        y = torch.empty((xd.shape[0], 2), dtype=torch.float32, device=xd.device)
        N.check(N.lib().gsea_model_predict(self._h, _vp(xd), xd.shape[0], _vp(y), None))
        torch.cuda.synchronize(xd.device)
        return y

    def loss_grad(self, x, t) -> Tuple[np.ndarray, float]:
        """Mean loss and its gradient over all samples (the kernels' backward pass)."""
        torch = _torch()
        xd, td = _dev_f32(x), _dev_f32(t)
        g = torch.empty(NPARAM, dtype=torch.float32, device=xd.device)
        l = torch.empty(1, dtype=torch.float32, device=xd.device)
        N.check(N.lib().gsea_model_loss_grad(self._h, _vp(xd), _vp(td), xd.shape[0], _vp(g), _vp(l), None))
        return g.cpu().numpy(), float(l.cpu()[0])

    def train(self, x, t, steps: int = 1500, batch: int = 4096, lr: float = 3e-3) -> np.ndarray:
        """Adam on the samples; returns the loss of every step."""
        xd, td = _dev_f32(x), _dev_f32(t)
        curve = np.empty(steps, np.float32)
        N.check(N.lib().gsea_model_train(self._h, _vp(xd), _vp(td), xd.shape[0], steps, batch, lr, N.ptr(curve)))
        return curve

    def calibrate(self, x, t) -> Tuple[float, float]:
        xd, td = _dev_f32(x), _dev_f32(t)
        N.check(N.lib().gsea_model_calibrate(self._h, _vp(xd), _vp(td), xd.shape[0]))
        n = self.get()[1]
        return float(n[12]), float(n[13])

    def save(self, path: str) -> None:
        p, n = self.get()
        np.savez(path, params=p, norms=n)

    def load(self, path: str) -> None:
        z = np.load(path)
        self.set(z["params"], z["norms"])

    def close(self) -> None:
        if getattr(self, "_h", None):
            N.lib().gsea_model_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def model_samples(plan, queries: int = 16, holdout: int = 10):
    """Training / held-out samples from the plan's last execute: (x, t, x_val, t_val) CUDA tensors."""
    torch = _torch()
    K = plan.cfg.num_sets
    rows = K * (queries + 1)
    dev = torch.device("cuda", torch.cuda.current_device())
    x = torch.empty((rows, IN), dtype=torch.float32, device=dev)
    t = torch.empty((rows, 2), dtype=torch.float32, device=dev)
    xv = torch.empty((rows, IN), dtype=torch.float32, device=dev)
    tv = torch.empty((rows, 2), dtype=torch.float32, device=dev)
    nt, nv = ctypes.c_int64(0), ctypes.c_int64(0)
    N.check(N.lib().gsea_plan_model_samples(plan._h, queries, holdout, _vp(x), _vp(t), ctypes.byref(nt), _vp(xv),
                                            _vp(tv), ctypes.byref(nv)))
    return x[:nt.value], t[:nt.value], xv[:nv.value], tv[:nv.value]


def train_model(plan, seed: int = 0, queries: int = 16, holdout: int = 10, steps: int = 1500, batch: int = 4096,
                lr: float = 3e-3) -> Tuple[Model, np.ndarray]:
    """Train a model on the null scores of `plan` (executed, all sets, perm_offset 0)."""
    x, t, xv, tv = model_samples(plan, queries, holdout)
    m = Model(seed)
    curve = m.train(x, t, steps=steps, batch=batch, lr=lr)
    if xv.shape[0]:
        m.calibrate(xv, tv)
    return m, curve


@dataclass
class AdaptiveResult:
    counts: np.ndarray
    report: Dict[str, float]


def params(**kw) -> N.AdaptiveParams:
    ap = N.AdaptiveParams()
    N.lib().gsea_adaptive_params_init(ctypes.byref(ap))
    for k, v in kw.items():
        if not hasattr(ap, k):
            raise TypeError(f"unknown adaptive parameter {k}")
        setattr(ap, k, v)
    return ap


def execute_adaptive(plan, model: Optional[Model] = None, **kw) -> AdaptiveResult:
    """Adaptive permutation test on the plan (see gsea_plan_execute_adaptive)."""
    ap = params(**kw)
    counts = np.empty(plan.cfg.num_sets, np.int64)
    rep = N.AdaptiveReport()
    N.check(N.lib().gsea_plan_execute_adaptive(plan._h, model.handle if model is not None else None,
                                               ctypes.byref(ap), N.ptr(counts), ctypes.byref(rep)))
    report = {name: getattr(rep, name) for name, _ in N.AdaptiveReport._fields_}
    return AdaptiveResult(counts, report)


def decide(counts, exceed, stop_p: float, z: float = 3.0, p_model=None, prior=None) -> np.ndarray:
    """The stopping rule alone, on host arrays (gsea_adaptive_decide)."""
    c = np.ascontiguousarray(counts, np.int64)
    e = np.ascontiguousarray(exceed, np.int64)
    pm = None if p_model is None else np.ascontiguousarray(p_model, np.float32)
    pr = None if prior is None else np.ascontiguousarray(prior, np.float32)
    out = np.empty(c.size, np.uint8)
    N.check(N.lib().gsea_adaptive_decide(c.size, N.ptr(c), N.ptr(e), N.ptr(pm), N.ptr(pr), stop_p, z, N.ptr(out)))
    return out


def stats_ragged(es, counts, p_fwer: int):
    """Ragged statistics of a CUDA ES tensor [K][ld] whose row k holds counts[k] scores."""
    torch = _torch()
    K, ld = es.shape
    prec = 64 if es.dtype == torch.float64 else 32
    c = torch.as_tensor(np.ascontiguousarray(counts, np.int64)).to(es.device)
    out = torch.empty(5 * K, dtype=es.dtype, device=es.device)
    N.check(N.lib().gsea_stats_ragged(_vp(es.contiguous()), K, ld, _vp(c), p_fwer, prec, _vp(out), None))
    return out


def fdr_lower_bound(es, counts, p_fwer: int, sums, z: float):
    """(statistics [5K], q lower bounds [K]) of a CUDA ES tensor [K][ld] whose
    row k holds counts[k] scores; sums [2K]: sum |S| then sum S^2 per set
    (gsea_fdr_lower_bound)."""
    torch = _torch()
    K, ld = es.shape
    prec = 64 if es.dtype == torch.float64 else 32
    c = torch.as_tensor(np.ascontiguousarray(counts, np.int64)).to(es.device)
    sm = torch.as_tensor(np.ascontiguousarray(sums, np.float64)).to(es.device)
    out = torch.empty(5 * K, dtype=es.dtype, device=es.device)
    q = torch.empty(K, dtype=torch.float32, device=es.device)
    N.check(N.lib().gsea_fdr_lower_bound(_vp(es.contiguous()), K, ld, _vp(c), p_fwer, _vp(sm), z, prec, _vp(out),
                                         _vp(q), None))
    return out, q
