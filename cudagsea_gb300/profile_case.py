"""A profiling-size run of the pipeline: the headline shapes (20,000 genes x
200 samples, 1,000 sets) with fewer permutations, so that an ncu capture of
one kernel stays small.  Used by the commands recorded under profiles/.

    python -m cudagsea_gb300.profile_case [--perms 152] [--reps 2]
        [--precision 32|64] [--form plain|chosen|chosen64] [--batch 0]
        [--model 0] [--genes 20000] [--adaptive 0] [--sort-variant 0]

--batch N   runs N uneven instances through gsea_batch instead (the
            persistent multi-instance enrichment kernel)
--model N   runs N training steps of the allocator network on samples of the
            run (the model kernels)
--genes G   the same data with G genes (the large-G sort and enrichment
            variants: two-CTA cluster sort, ranks-only staging)
--sort-variant V
            1 register / cluster sort, 2 tiled sort (0: the automatic choice)
--adaptive P0
            one adaptive test (both stopping rules, no model) with a pilot of
            P0 permutations on the allocator workload (20,000 sets, 100,000
            permutations)
"""
from __future__ import annotations

import argparse

from . import api, build, synthetic
from . import _native as N

FORMS = {"plain": N.FORM_PLAIN, "chosen": N.FORM_CHOSEN, "chosen64": N.FORM_CHOSEN_FP64}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--perms", type=int, default=152)
    ap.add_argument("--reps", type=int, default=2)
    ap.add_argument("--precision", type=int, default=32)
    ap.add_argument("--form", choices=sorted(FORMS), default="plain")
    ap.add_argument("--batch", type=int, default=0)
    ap.add_argument("--model", type=int, default=0)
    ap.add_argument("--genes", type=int, default=20000)
    ap.add_argument("--adaptive", type=int, default=0)
    ap.add_argument("--sort-variant", type=int, default=0)
    a = ap.parse_args(argv)
    build.build()
    if a.adaptive:
        from . import allocator
        d = synthetic.learned()
        plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, d.num_perms, "twopass_signal2noise",
                        form=N.FORM_CHOSEN)
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        r = allocator.execute_adaptive(plan, None, pilot_perms=a.adaptive)
        print("adaptive", r.report)
        plan.close()
        return 0
    if a.batch:
        ds = synthetic.batch_instances(a.batch, num_perms=a.perms)
        b = api.Batch(ds, precision=a.precision, form=FORMS[a.form])
        for _ in range(a.reps):
            b.execute()
        b.synchronize()
        print("batch", b.info())
        b.close()
        return 0
    if a.genes == 20000:
        d = synthetic.full(num_perms=a.perms)
    else:
        d = synthetic.make(a.genes, 200, 1000, a.perms, seed=4321, n_class_b=100, sd_range=(0.3, 3.0),
                           n_shift=500, shift_range=(0.5, 2.0), set_min=15, set_max=500, enriched_frac=0.2,
                           clamp=1e-3, name=f"full_{a.genes}x200_K1000_P{a.perms}")
    plan = api.Plan(d.num_genes, d.num_samples, d.num_sets, a.perms, "twopass_signal2noise",
                    precision=a.precision, form=FORMS[a.form])
    if a.sort_variant:
        plan.set_tuning(sort_variant=a.sort_variant)
    plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
    plan.set_profiling(True)
    for i in range(a.reps):
        plan.execute()
        print(i, plan.stage_times(), flush=True)
    if a.model:
        from . import allocator
        m, curve = allocator.train_model(plan, steps=a.model)
        print("model loss", float(curve[0]), "->", float(curve[-1]))
        m.close()
    plan.close()
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
