"""Error of the tensor-core forms against FP64, per metric, at the precision
workload (20,000 genes x 600 samples, 300/300, 2,000 sets).

The FP64 reference is the plain form in double precision (every stage in
FP64, bit-identical to the FP64 oracle on the parity cases).  For every
metric the two forms run the same permutations; reported: the largest key
error relative to the permutation's largest |key|, the largest |dES| and
|dNES|, the FDR < 0.25 calls of both, and the rank flips of the sampled
permutations -- positions where the tensor-core order differs from the FP64
order -- split into near-ties (FP64 keys within 1e-4 of the permutation's key
scale) and the rest.  The same comparison for the plain form in fp32 (the
reference's own single-precision arithmetic) shows what any FP32 evaluation
of the path loses against FP64.  Both tensor-core forms are reported: the
error-free FP32 variance (GSEA_FORM_CHOSEN) and the FP64 variance
finalisation (GSEA_FORM_CHOSEN_FP64); for each, every set above
|dNES| = 1e-4 is traced to its moved scores (precision_check.compare: a
moved score is order-explained when the FP64 keys walked in the form's own
rank order reproduce it).

    python -m cudagsea_gb300.precision_report [--perms 10000] [--sample 64] [--json out.json]
"""
from __future__ import annotations

import argparse
import json

import numpy as np

from . import api, build, synthetic
from . import _native as N

NEAR_TIE = 1e-4


def workload(num_perms: int):
    return synthetic.make(20000, 600, 2000, num_perms, seed=6060, n_class_b=300, sd_range=(0.3, 3.0),
                          n_shift=500, shift_range=(0.5, 2.0), set_min=15, set_max=500, enriched_frac=0.2,
                          clamp=1e-3, name=f"precision_20000x600_K2000_P{num_perms}")


def run(d, metric, precision, form, sample):
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, d.num_perms, metric, precision=precision, form=form,
                    perm_batch=d.num_perms)
    plan.set_debug(True)
    x = d.exprs.astype(np.float64) if precision == 64 else d.exprs
    plan.set_inputs(x, d.labels, d.set_offsets, d.set_genes)
    plan.execute()
    es, st = plan.read()
    dt = np.float64 if precision == 64 else np.float32
    keys = plan.read_buffer(N.BUF_KEYS, dt, (sample, d.num_genes))   # the first `sample` permutations
    order = plan.read_buffer(N.BUF_ORDER, np.uint32, (sample, d.num_genes))
    plan.close()
    return es, st.reshape(5, -1), keys, order


def flips(order_c, order_r, keys_r):
    """(near-tie flips, other flips) of the sampled permutations."""
    near = other = 0
    for oc, orr, kr in zip(order_c, order_r, keys_r):
        diff = np.nonzero(oc != orr)[0]
        if diff.size == 0:
            continue
        scale = np.nanmax(np.abs(kr))
        kc = kr[oc[diff]]   # FP64 key of the gene the tensor-core form put there
        kf = kr[orr[diff]]  # FP64 key of the gene FP64 put there
        tie = np.abs(kc - kf) <= NEAR_TIE * scale
        near += int(np.count_nonzero(tie))
        other += int(np.count_nonzero(~tie))
    return near, other


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--perms", type=int, default=10000)
    ap.add_argument("--sample", type=int, default=64, help="permutations whose rank orders are compared")
    ap.add_argument("--json", default="")
    ap.add_argument("--metrics", default="", help="comma-separated metric names (default: all 14)")
    a = ap.parse_args(argv)
    build.build()
    d = workload(a.perms)
    rows = []
    def compare(es_c, st_c, k_c, o_c, es_r, st_r, k_r, o_r):
        fin = np.isfinite(k_r) & np.isfinite(k_c)
        scale = np.nanmax(np.abs(np.where(np.isfinite(k_r), k_r, np.nan)), axis=1, keepdims=True)
        kerr = float(np.nanmax(np.where(fin, np.abs(k_c - k_r) / scale, 0.0)))
        ok = np.isfinite(es_r) & np.isfinite(es_c)
        d_es = np.abs(es_c[ok] - es_r[ok])
        okn = np.isfinite(st_r[1]) & np.isfinite(st_c[1])
        d_nes = np.abs(st_c[1][okn] - st_r[1][okn])
        calls_c = set(np.nonzero(st_c[4] < 0.25)[0])
        calls_r = set(np.nonzero(st_r[4] < 0.25)[0])
        near, other = flips(o_c, o_r, k_r)
        return {"key_rel_err": kerr, "max_abs_dES": float(d_es.max()) if d_es.size else 0.0,
                "es_sign_flips": int(np.count_nonzero(d_es > 0.1)),
                "max_abs_dNES": float(d_nes.max()) if d_nes.size else 0.0,
                "sets_dNES_over_1e-4": int(np.count_nonzero(d_nes > 1e-4)),
                "calls_fp64": len(calls_r), "calls": len(calls_c), "call_diff": len(calls_c ^ calls_r),
                "rank_flips_near_tie": near, "rank_flips_other": other}

    from . import precision_check as PC

    def traced(form, ref_run):
        cur = PC.run_form(d, m, 32, form)
        try:
            rep = PC.compare(d, cur, ref_run)
        finally:
            cur.close()
        return {"sets_dNES_over_1e-4": rep["sets_over_tol"], "all_tie_explained": rep["all_tie_explained"],
                "traced_not_explained": sum(1 for e in rep["exceedances"] if not e["tie_explained"]),
                "not_explained": [e for e in rep["exceedances"] if not e["tie_explained"]][:5],
                "fdr_call_diffs": rep["fdr_call_diffs"]}

    chosen_names = [x for x in a.metrics.split(",") if x] or api.METRICS
    for m, name in enumerate(api.METRICS):
        if name not in chosen_names:
            continue
        ref = run(d, m, 64, N.FORM_PLAIN, a.sample)
        tensor = compare(*run(d, m, 32, N.FORM_CHOSEN, a.sample), *ref)
        tensor64 = compare(*run(d, m, 32, N.FORM_CHOSEN_FP64, a.sample), *ref)
        plain32 = compare(*run(d, m, 32, N.FORM_PLAIN, a.sample), *ref)
        ref_run = PC.run_form(d, m, 64, N.FORM_PLAIN)
        try:
            tensor["trace"] = traced(N.FORM_CHOSEN, ref_run)
            tensor64["trace"] = traced(N.FORM_CHOSEN_FP64, ref_run)
        finally:
            ref_run.close()
        row = {"metric": name, "tensor_core_fp32": tensor, "tensor_core_fp64_variance": tensor64,
               "plain_fp32": plain32}
        rows.append(row)
        print(json.dumps(row), flush=True)
    if a.json:
        with open(a.json, "w") as f:
            json.dump({"workload": d.name, "sample_perms": a.sample, "near_tie": NEAR_TIE, "rows": rows}, f, indent=1)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
