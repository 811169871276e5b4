"""Generate the golden fixtures of tests/golden/ from the REFERENCE's own CPU
pipeline (oracle/_ref/libgsea_ref.so, built by oracle/build_ref.sh from the
cudaGSEA sources).  Run here, where the reference sources exist:

    python tests/golden/make_golden.py

Inputs are regenerated from seeds by cudagsea_gb300.synthetic (numpy legacy
RandomState streams, stable across numpy versions); a SHA-256 of each input is
stored so a drifting generator is detected instead of silently compared.

Fixtures (compressed .npz):
  perm_labels.npz      permuted labels of permutations 0..16 (S=40), read back
                       from the reference's naive_diff metric on an identity
                       expression table (key = 1/nA for class A, -1/nB for B)
  metrics_<prec>.npz   G=500, S=24, K=20, P=32, all 14 metrics: SHA-256 of the
                       reference's metric keys (all permutations), its ES
                       matrix and final statistics
  small_<prec>.npz     2,000 x 40 (20/20), 50 sets, 1,024 permutations,
                       twopass_signal2noise: statistics, ES of the first 128
                       permutations, SHA-256 of the full ES matrix
  ties_<prec>.npz      integer-valued expressions (many tied metrics),
                       G=300, S=16, K=10, P=32, naive_diff and twopass_s2n
  tiny.npz             37 genes x 5 samples, 3 sets, 3 permutations
  full_<prec>.npz      the 20,000 x 200 workload (1,000 sets, 1,000
                       permutations), all 14 metrics: the reference's final
                       statistics and the ES of its first 4 permutations
                       (`python tests/golden/make_golden.py full` writes these
                       alone: ~30 s of the reference per metric and precision)
  large_<G>.npz        G = 30,000 / 50,000 genes x 24 samples, 20 sets, 64
                       permutations, twopass_signal2noise: the reference's ES
                       matrix and statistics in fp32 and fp64
                       (`python tests/golden/make_golden.py large` writes
                       these alone)
  cli_result_*.txt     "RESULT:" lines of the reference CLI (-cpu) on .gct /
                       .cls / .gmt files of the 2,000 x 40 workload (256
                       permutations, twopass_signal2noise; single, double and
                       single with -order ascending)
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from cudagsea_gb300 import synthetic  # noqa: E402


def sha(*arrays) -> str:
    h = hashlib.sha256()
    for a in arrays:
        h.update(np.ascontiguousarray(a).tobytes())
    return h.hexdigest()


def input_hash(d) -> str:
    return sha(d.exprs, d.labels, d.set_offsets, d.set_genes)


def metrics_case():
    return synthetic.make(500, 24, 20, 32, seed=2024, n_class_b=12, sd=2.0, n_shift=25, shift=1.0,
                          set_min=10, set_max=60, name="metrics_500x24_K20_P32")


def ties_case():
    d = synthetic.make(300, 16, 10, 32, seed=99, n_class_b=8, sd=2.0, n_shift=20, shift=1.0,
                       set_min=8, set_max=40, name="ties_300x16_K10_P32")
    d.exprs = np.round(d.exprs).astype(np.float32)
    return d


def large_case(G):
    """G genes x 24 samples, 20 sets, 64 permutations: the sizes of the two-CTA
    cluster sort (30,000 genes, fp32) and of the tiled sort (50,000 genes;
    fp64 at both sizes)."""
    return synthetic.make(G, 24, 20, 64, seed=G + 7, n_class_b=12, sd_range=(0.5, 2.0), n_shift=200,
                          shift_range=(0.5, 1.5), set_min=15, set_max=400, enriched_frac=0.3,
                          name=f"large_{G}x24_K20_P64")


def write_large():
    """The cluster and tiled sort paths against the reference itself."""
    for G in (30000, 50000):
        d = large_case(G)
        out = {"input_sha": input_hash(d)}
        for double in (False, True):
            prec = "f64" if double else "f32"
            es, st = oracle.ref_gsea(8, d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, double=double)
            out[f"es_{prec}"] = es
            out[f"stats_{prec}"] = st
        np.savez_compressed(os.path.join(HERE, f"large_{G}.npz"), **out)


def write_full():
    """The headline workload, every metric, both precisions."""
    d = synthetic.full()
    for double in (False, True):
        prec = "f64" if double else "f32"
        out = {"input_sha": input_hash(d)}
        for m in range(14):
            es, st = oracle.ref_gsea(m, d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, double=double)
            out[f"stats_{m}"] = st
            out[f"es_head_{m}"] = np.ascontiguousarray(es[:, :4])
        np.savez_compressed(os.path.join(HERE, f"full_{prec}.npz"), **out)


def main():
    oracle.build_ref()
    if not oracle.ref_available():
        raise SystemExit("reference build not available")
    if sys.argv[1:] == ["large"]:
        write_large()
        print("large fixtures written to", HERE)
        return
    if sys.argv[1:] == ["full"]:
        write_full()
        print("full-size fixtures written to", HERE)
        return
    # --- permutation KAT
    S, nA = 40, 20
    labels = np.array([0] * nA + [1] * (S - nA), np.uint8)
    ident = np.eye(S, dtype=np.float64)  # patient-major [S][G=S]: gene g is sample g's indicator
    keys = oracle.ref_metric(0, ident, labels, 17, double=True)
    perm = np.where(keys > 0, 0, 1).astype(np.uint8)
    np.savez_compressed(os.path.join(HERE, "perm_labels.npz"), labels=labels, perm_labels=perm)

    for double in (False, True):
        prec = "f64" if double else "f32"
        dt = np.float64 if double else np.float32
        # --- all metrics
        d = metrics_case()
        out = {"input_sha": input_hash(d)}
        for m in range(14):
            k = oracle.ref_metric(m, d.exprs, d.labels, d.num_perms, double=double)
            es, st = oracle.ref_gsea(m, d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, double=double)
            out[f"keys_sha_{m}"] = sha(k)
            out[f"keys0_{m}"] = k[:2].astype(dt)
            out[f"es_{m}"] = es.astype(dt)
            out[f"stats_{m}"] = st.astype(dt)
        np.savez_compressed(os.path.join(HERE, f"metrics_{prec}.npz"), **out)
        # --- config-1 sized run
        d = synthetic.small()
        es, st = oracle.ref_gsea(8, d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, double=double)
        np.savez_compressed(os.path.join(HERE, f"small_{prec}.npz"), input_sha=input_hash(d), stats=st,
                            es_head=es[:, :128], es_sha=sha(es))
        # --- tie-heavy data
        d = ties_case()
        out = {"input_sha": input_hash(d)}
        for m in (0, 8):
            k = oracle.ref_metric(m, d.exprs, d.labels, d.num_perms, double=double)
            es, st = oracle.ref_gsea(m, d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, double=double)
            out[f"keys_sha_{m}"] = sha(k)
            out[f"es_{m}"] = es
            out[f"stats_{m}"] = st
        np.savez_compressed(os.path.join(HERE, f"ties_{prec}.npz"), **out)
    write_large()
    write_full()
    # --- tiny shapes
    d = synthetic.tiny()
    out = {"input_sha": input_hash(d)}
    for double in (False, True):
        prec = "f64" if double else "f32"
        for m in range(14):
            es, st = oracle.ref_gsea(m, d.exprs, d.labels, d.set_offsets, d.set_genes, d.num_perms, double=double)
            out[f"es_{prec}_{m}"] = es
            out[f"stats_{prec}_{m}"] = st
    np.savez_compressed(os.path.join(HERE, "tiny.npz"), **out)
    # --- the reference CLI on Broad files of the 2,000 x 40 workload (CPU mode)
    import subprocess
    import tempfile
    from cudagsea_gb300 import broad
    d = synthetic.small(num_perms=256)
    with tempfile.TemporaryDirectory() as tmp:
        gct, cls, gmt = broad.write_dataset(os.path.join(tmp, "small"), d)
        runs = [("single", [], "cli_result_single.txt"), ("double", [], "cli_result_double.txt"),
                ("single", ["-order", "ascending"], "cli_result_ascending_single.txt")]
        for prec, extra, fname in runs:
            out = subprocess.run([os.path.join(oracle.REF_DIR, "cudaGSEA_cpu"), "-res", gct, "-cls", cls, "-gmx",
                                  gmt, "-nperm", "256", "-metric", "twopass_signal2noise", "-precision", prec,
                                  "-cpu"] + extra, capture_output=True, text=True, check=True).stdout
            lines = [l for l in out.splitlines() if l.startswith("RESULT:")]
            with open(os.path.join(HERE, fname), "w") as f:
                f.write("\n".join(lines) + "\n")
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
