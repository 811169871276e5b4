"""NES of the tensor-core forms against FP64, with every exceedance traced.

The accuracy condition of the tensor-core forms is |dNES| <= 1e-4 against an
FP64 evaluation, with identical FDR < 0.25 calls.  The FP64
evaluation here is the plain form in double precision (every stage in FP64,
pinned bit for bit to the FP64 oracle by the parity tests), run on the same
inputs and the same label permutations.

No evaluation that is not bit-identical to FP64 can meet 1e-4 for every set
of every workload: where a set member and a non-member have metric keys
closer than the form's key error, either order is a correct rounding, and a
swap at the running sum's extremum moves ES by one miss step 1/(G - n) or one
hit step w/N_R (src/include/enrichment_scores.cuh:178-195), i.e. NES by ~1e-4
at 20,000 genes.  `compare` therefore reports, for every set above the
tolerance, which permutations' scores moved and why:

* a permutation's score has *moved* when |dES| exceeds the rounding
  tolerance of the fp32 path (`ES_ROUND`);
* a moved score is *order-explained* when the enrichment score recomputed in
  FP64 from the FP64 keys, but walking the tensor-core form's rank order,
  reproduces the tensor-core score: the weights are then not the cause, only
  the order is, and the two orders differ only where keys are within the
  form's key error of each other (near ties); or when that recomputation
  gives the same magnitude with the other sign -- the running sum's maximum
  and minimum tie in magnitude, and which one the score reports is decided
  by roundings (a sign tie, src/include/enrichment_scores.cuh:192-195);
* the set's exceedance is *tie-explained* when every moved score is
  order-explained and its NES, recomputed with the moved scores replaced by
  their FP64 values, is back within the tolerance.

Package code: it calls the library (plans, buffers) and numpy only.
"""
from __future__ import annotations

from dataclasses import dataclass
from typing import Dict, List, Optional

import numpy as np

from . import api
from . import _native as N

NES_TOL = 1e-4      # the |dNES| bound of the tensor-core forms
ES_ROUND = 2e-5     # |dES| below this is rounding of the fp32 path (scores are O(0.1-1))
FDR_CALL = 0.25


class _DeviceRows:
    """A plan buffer [rows][G] on the device, gathered row by row through
    torch (the buffer is wrapped in place through __cuda_array_interface__)."""

    def __init__(self, plan: api.Plan, which: int, dtype, G: int):
        import torch
        ptr, nbytes = plan.buffer(which)
        itemsize = np.dtype(dtype).itemsize
        rows = nbytes // (itemsize * G)
        # unsigned 32-bit words travel as int32 (torch's unsigned support is partial)
        typestr = np.dtype(np.int32 if np.dtype(dtype) == np.uint32 else dtype).str

        class _Iface:
            __cuda_array_interface__ = {"shape": (rows, G), "typestr": typestr, "data": (ptr, False),
                                        "version": 2, "strides": None}

        self.t = torch.as_tensor(_Iface(), device="cuda")
        self.dtype = dtype

    def rows(self, idx) -> np.ndarray:
        import torch
        sel = torch.as_tensor(np.asarray(idx, np.int64), device=self.t.device)
        out = self.t.index_select(0, sel).cpu().numpy()
        return out.view(self.dtype)


@dataclass
class FormRun:
    """One executed plan with all permutations in one device batch."""
    plan: api.Plan
    es: np.ndarray
    stats: np.ndarray  # [5][K]
    keys: _DeviceRows
    order: _DeviceRows

    def close(self):
        self.plan.close()


def run_form(d, metric, precision: int, form: int) -> FormRun:
    P = d.num_perms
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, P, metric, precision=precision, form=form,
                    perm_batch=P)
    plan.set_debug(True)  # materialises the rank order (GSEA_BUF_ORDER)
    x = d.exprs.astype(np.float64) if precision == 64 else d.exprs
    plan.set_inputs(x, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es, st = plan.read()
    dt = np.float64 if precision == 64 else np.float32
    return FormRun(plan, es, st.reshape(5, -1), _DeviceRows(plan, N.BUF_KEYS, dt, d.num_genes),
                   _DeviceRows(plan, N.BUF_ORDER, np.uint32, d.num_genes))


def es_in_order(order: np.ndarray, weights: np.ndarray, members: np.ndarray, G: int) -> float:
    """Enrichment score of one set in FP64 for the ranked list `order` (gene
    at each position) with per-gene weights `weights` (|key|): the running
    sum of enrichment_scores.cuh:143-195 (hit: +w/N_R, miss: -1/(G - N_H);
    first value of largest magnitude, sign kept), evaluated at its extrema
    (just before and just after each hit)."""
    members = np.unique(members[(members >= 0) & (members < G)])
    n = members.size
    if n == 0:
        return float("nan")
    pos_of = np.empty(G, np.int64)
    pos_of[order] = np.arange(G)
    pos = np.sort(pos_of[members])
    w = np.asarray(weights, np.float64)[order[pos]]
    W = np.cumsum(w)
    NR = W[-1]
    dec = 1.0 / (G - n) if n < G else 0.0
    j = np.arange(n)
    miss = (pos - j) * dec
    before = np.r_[0.0, W[:-1]] / NR - miss
    after = W / NR - miss
    end = 1.0 - (G - n) * dec
    vals = np.concatenate([np.stack([before, after], 1).ravel(), [end]])
    where = np.concatenate([np.stack([pos - 1, pos], 1).ravel(), [G - 1]])
    mag = np.abs(vals)
    best = mag.max()
    if best == 0.0:
        return 0.0
    cand = np.flatnonzero(mag == best)
    return float(vals[cand[np.argmin(where[cand])]])


def _nes(row: np.ndarray) -> float:
    s = np.abs(row).sum()
    return float(row[0] * row.size / s)


def compare(d, cur: FormRun, ref: FormRun, nes_tol: float = NES_TOL, max_sets: int = 200) -> Dict:
    """Report of one tensor-core run against the FP64 run (see the module
    docstring).  Traces at most `max_sets` exceeding sets (largest first)."""
    K, P, G = d.num_sets, d.num_perms, d.num_genes
    nes_c = cur.stats[1].astype(np.float64)
    nes_r = ref.stats[1]
    ok = np.isfinite(nes_c) & np.isfinite(nes_r)
    dnes = np.where(ok, np.abs(nes_c - nes_r), 0.0)
    over = np.flatnonzero(dnes > nes_tol)
    over = over[np.argsort(-dnes[over])]
    calls_c = set(np.flatnonzero(cur.stats[4] < FDR_CALL).tolist())
    calls_r = set(np.flatnonzero(ref.stats[4] < FDR_CALL).tolist())
    es_c = cur.es.astype(np.float64)
    es_r = ref.es
    des = np.abs(es_c - es_r)
    traced: List[Dict] = []
    explained_all = True
    moved_total = 0
    for k in over[:max_sets]:
        moved = np.flatnonzero(des[k] > ES_ROUND)
        moved_total += moved.size
        members = d.set_genes[d.set_offsets[k]:d.set_offsets[k + 1]]
        order_ok = True
        rank_moves = 0
        mix_err = 0.0
        sign_ties = 0
        if moved.size:
            orders = cur.order.rows(moved)
            w64 = np.abs(ref.keys.rows(moved))
            orders_r = ref.order.rows(moved)
            for i, p in enumerate(moved):
                e_mix = es_in_order(orders[i], w64[i], members, G)
                err = abs(e_mix - es_c[k, p])
                if err > ES_ROUND and abs(abs(e_mix) - abs(es_c[k, p])) <= ES_ROUND:
                    err = abs(abs(e_mix) - abs(es_c[k, p]))  # a sign tie of the extrema
                    sign_ties += 1
                mix_err = max(mix_err, err)
                if not err <= ES_ROUND:
                    order_ok = False
                pc = np.empty(G, np.int64)
                pc[orders[i]] = np.arange(G)
                pr = np.empty(G, np.int64)
                pr[orders_r[i]] = np.arange(G)
                rank_moves += int(np.count_nonzero(pc[members] != pr[members]))
        row = es_c[k].copy()
        row[moved] = es_r[k, moved]
        residual = abs(_nes(row) - nes_r[k])
        explained = bool(order_ok and residual <= nes_tol)
        explained_all &= explained
        traced.append({"set": int(k), "dNES": float(dnes[k]), "moved_perms": int(moved.size),
                       "observed_moved": bool(0 in moved), "member_rank_moves": rank_moves,
                       "order_explained": bool(order_ok), "residual_dNES": float(residual),
                       "max_order_mismatch": float(mix_err), "sign_ties": sign_ties,
                       "tie_explained": explained})
    if over.size > max_sets:
        explained_all = False  # untraced sets count as unexplained
    return {"max_abs_dNES": float(dnes.max()) if dnes.size else 0.0,
            "sets_over_tol": int(over.size), "nes_tol": nes_tol,
            "all_tie_explained": bool(explained_all),
            "max_abs_dES": float(np.nanmax(des)) if des.size else 0.0,
            "moved_scores": int(np.count_nonzero(des > ES_ROUND)),
            "fdr_calls_fp64": len(calls_r), "fdr_calls": len(calls_c),
            "fdr_call_diffs": len(calls_c ^ calls_r),
            "exceedances": traced}


def check_forms(d, metric="twopass_signal2noise", forms=(N.FORM_CHOSEN, N.FORM_CHOSEN_FP64),
                nes_tol: float = NES_TOL) -> Dict[str, Dict]:
    """FP64 plain run + each tensor-core form on `d`; one report per form."""
    names = {N.FORM_CHOSEN: "chosen", N.FORM_CHOSEN_FP64: "chosen_fp64", N.FORM_PLAIN: "plain_fp32"}
    ref = run_form(d, metric, 64, N.FORM_PLAIN)
    out = {}
    try:
        for f in forms:
            cur = run_form(d, metric, 32, f)
            try:
                out[names[f]] = compare(d, cur, ref, nes_tol)
            finally:
                cur.close()
    finally:
        ref.close()
    return out


def summary(rep: Dict) -> Dict:
    """The bench line's compact form of one report."""
    keys = ("max_abs_dNES", "sets_over_tol", "all_tie_explained", "fdr_call_diffs", "fdr_calls", "fdr_calls_fp64",
            "moved_scores", "max_abs_dES")
    out = {k: rep[k] for k in keys}
    out["exceedances"] = [{k: e[k] for k in ("set", "dNES", "moved_perms", "observed_moved", "tie_explained")}
                          for e in rep["exceedances"][:10]]
    return out
