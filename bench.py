#!/usr/bin/env python
"""Benchmark of the GSEA permutation pipeline on GB300.

Metric: enrichment scores per second (gene sets x permutations) on the
20,000 genes x 200 samples x 1,000 gene sets x 1,000 permutations workload
(twopass_signal2noise, fp32), synthetic seeded data.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

One step = one pass of the pipeline (permutation -> metric -> sort -> ES ->
statistics) over the whole workload.

* value          K*P / device time of one step, inputs resident in HBM, CUDA
                 events on the launching stream, L2 flushed (256 MB write)
                 between steps, outside the timed events.  A step replays the
                 plan's captured CUDA graph (its ~12 kernels); the stage times
                 come from three separate, untimed profiled executes.
* e2e            the same metric through the C ABI from pinned host buffers:
                 gsea_plan_run_host copies the inputs in, runs the pipeline
                 and copies ES + statistics out, every step.
* roofline       the dominant stage's algorithmic bytes per launch / its
                 average device time, against MEASURED_PEAKS.json; `limiter`
                 adds the kernel's issue-slot utilisation from its ncu summary
                 under profiles/ (the stage is instruction bound: its data
                 stay in shared memory, so the HBM fraction is small by
                 construction).
* pipeline_roofline
                 the whole step against its compulsory HBM bytes, e*G*S +
                 P*(2*e*G + 8*G + e*K): the expression table once, per
                 permutation the metric keys and u32 ranks written and read
                 back and the ES column written.
* forms.adaptive / forms.learned
                 the adaptive permutation test (tensor-core form) without
                 and with the learned prior: wall time of the whole adaptive
                 run (host decisions between rounds included), the fraction
                 of the K*P scores it computed, and its FDR < 0.25 calls
                 against the full test's.  Reported beside the headline; the
                 headline value always computes all K*P scores.  The prior's
                 network is trained beforehand (untimed) on the null scores of
                 another seed of the same workload.
* cpu_baseline   the reference's CPU path (its own build where it runs on
                 this machine, else the oracle port of it) on a bounded sample
                 of permutations, all host cores.
Under torchrun (N > 1) every rank runs the same workload on its own GPU over a
distinct permutation range (weak scaling, no collective on the data path); the
time is the maximum over ranks and the value the sum of all ranks' scores.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC_NAME = "enrichment scores/sec (sets x perms)"
UNIT = "ES/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--metric", default="twopass_signal2noise")
    ap.add_argument("--precision", type=int, default=32)
    ap.add_argument("--form", choices=["both", "plain-only"], default="both",
                    help="measure the plain and the chosen (tensor-core) form, or the plain one only")
    ap.add_argument("--workload", choices=["full", "small", "learned", "batched"], default="full",
                    help="learned: the 20,000-set / 100,000-permutation allocator workload; batched: 256 uneven "
                         "instances in one CUDA graph (each its own JSON line)")
    ap.add_argument("--instances", type=int, default=256, help="instances of the batched workload")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-precision-check", action="store_true",
                    help="skip the NES check of the tensor-core forms against the plain form in FP64 (outside the "
                         "timed region)")
    ap.add_argument("--no-learned", action="store_true",
                    help="skip the adaptive forms (sequential rule with and without the learned prior)")
    ap.add_argument("--pilot", type=int, default=250, help="pilot permutations of the adaptive forms")
    ap.add_argument("--growth", type=float, default=4.0,
                    help="growth of the permutation count between rounds of the headline's adaptive forms (4: the "
                         "pilot, then one round to all 1,000 permutations); the learned workload keeps the "
                         "library's doubling")
    ap.add_argument("--no-autotune", action="store_true",
                    help="keep the automatic launch configuration (by default each form's plan is autotuned on a "
                         "sample of its permutations before the warm-up, outside the timed region)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0, help="target CPU-baseline sample time")
    ap.add_argument("--ref-seconds", type=float, default=150.0,
                    help="reference arm: target time of all warm-up and timed steps together")
    return ap.parse_args()


def workload(name):
    from cudagsea_gb300 import synthetic
    return synthetic.full() if name == "full" else synthetic.small()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class _Nvml:
    """Read-only clock queries through the driver's NVML library (ctypes):
    SM clock, maximum SM clock, power draw and the active clock event
    reasons of one device.  Raises OSError where the library or the device
    is not available."""

    SM = 1  # NVML_CLOCK_SM
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown",
               0x40: "hw_thermal_slowdown"}

    def __init__(self, device: int):
        import ctypes
        self.c = ctypes
        self.lib = ctypes.CDLL("libnvidia-ml.so.1")
        if self.lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.h = ctypes.c_void_p()
        rc = 1
        try:  # the CUDA device's own UUID: NVML and CUDA may number devices differently
            import torch
            uuid = "GPU-" + str(torch.cuda.get_device_properties(device).uuid)
            rc = self.lib.nvmlDeviceGetHandleByUUID(uuid.encode(), ctypes.byref(self.h))
        except Exception:
            pass
        if rc != 0 and self.lib.nvmlDeviceGetHandleByIndex_v2(device, ctypes.byref(self.h)) != 0:
            raise OSError("no NVML handle")
        try:
            self.reasons_fn = self.lib.nvmlDeviceGetCurrentClocksEventReasons
        except AttributeError:
            self.reasons_fn = self.lib.nvmlDeviceGetCurrentClocksThrottleReasons
        self.max_sm = self._uint(self.lib.nvmlDeviceGetMaxClockInfo, self.SM)

    def _uint(self, fn, *args):
        v = self.c.c_uint()
        if fn(self.h, *args, self.c.byref(v)) != 0:
            raise OSError(fn.__name__)
        return v.value

    def sample(self):
        sm = self._uint(self.lib.nvmlDeviceGetClockInfo, self.SM)
        bits = self.c.c_ulonglong()
        self.reasons_fn(self.h, self.c.byref(bits))
        try:
            watts = self._uint(self.lib.nvmlDeviceGetPowerUsage) / 1e3
        except OSError:
            watts = None
        return sm, self.max_sm, watts, sorted(n for b, n in self.REASONS.items() if bits.value & b)

    def close(self):
        self.lib.nvmlShutdown()


class Clocks:
    """Clock samples during the timed region: NVML every 10 ms (one sample
    on entry, before the region's first launch, and one on exit), else
    nvidia-smi every 200 ms, started before the region begins."""

    def __init__(self, device: int, period_s: float = 0.01):
        self.device = device
        self.period = period_s
        self.proc = None
        self.nvml = None
        self.samples = []  # (sm_mhz, max_sm_mhz, watts, reasons)
        self.stop = threading.Event()

    def __enter__(self):
        try:
            self.nvml = _Nvml(self.device)
        except Exception:
            self.nvml = None
        if self.nvml is not None:
            self.samples.append(self.nvml.sample())
            self.t = threading.Thread(target=self._poll, daemon=True)
            self.t.start()
            return self
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.first = threading.Event()
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            self.first.wait(timeout=5.0)
        except Exception:
            self.proc = None
        return self

    def _poll(self):
        while not self.stop.wait(self.period):
            try:
                self.samples.append(self.nvml.sample())
            except OSError:
                return

    def _read(self):
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.proc.stdout:
            f = [x.strip() for x in line.split(",")]
            if len(f) >= 9:
                try:
                    watts = float(f[3])
                except ValueError:
                    watts = None
                try:
                    self.samples.append((float(f[1]), float(f[2]), watts,
                                         sorted(n for n, v in zip(names, f[5:9]) if v.lower() == "active")))
                except ValueError:
                    pass
            self.first.set()
        self.first.set()  # nvidia-smi ended without a sample

    def __exit__(self, *exc):
        if self.nvml is not None:
            self.stop.set()
            self.t.join(timeout=5)
            try:
                self.samples.append(self.nvml.sample())
            except OSError:
                pass
            self.nvml.close()
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        sm = [x[0] for x in self.samples]
        watts = [x[2] for x in self.samples if x[2] is not None]
        return {"sm_mhz": statistics.median(sm), "sm_min_mhz": min(sm),
                "sm_max_mhz": max(x[1] for x in self.samples),
                "reasons": sorted({r for x in self.samples for r in x[3]}),
                "power_w": statistics.median(watts) if watts else None,
                "samples": len(sm), "source": "nvml" if self.nvml is not None else "nvidia-smi"}


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# the stage's kernel profile and what bounds it (read off that profile)
STAGE_PROFILES = {"es": ("es_kernel_full_20000x200_K1000_152perms.md", "instruction issue"),
                  "sort": ("sort_regs_kernel_full_20000x200_152perms.md", "latency (barriers, ballots)"),
                  ("metric", "chosen"): ("class_stats_persistent_full_20000x200_152perms.md",
                                         "latency (epilogue)"),
                  ("metric", "plain"): ("metric_fast_kernel_full_20000x200_152perms.md", "latency (L2 loads)")}


def issue_limiter(stage, form):
    """Issue-slot utilisation of the stage's kernel (in `form`) from its
    committed ncu summary (the `issue active %` row), or None."""
    entry = STAGE_PROFILES.get(stage) or STAGE_PROFILES.get((stage, form))
    if not entry:
        return None
    name, kind = entry
    path = os.path.join(ROOT, "profiles", name)
    try:
        for line in open(path):
            cells = [c.strip() for c in line.strip().strip("|").split("|")]
            if len(cells) == 2 and cells[0] == "issue active %":
                return {"kind": kind, "issue_active": float(cells[1]) / 100.0, "source": "profiles/" + name}
    except Exception:
        return None
    return None


def traffic_record():
    path = os.path.join(ROOT, "profiles", "ncu_traffic_full_20000x200.json")
    try:
        with open(path) as f:
            return json.load(f)
    except Exception:
        return {}


def stage_bytes(d, P, esize, ranks16):
    """Algorithmic (compulsory) bytes of each stage for P permutations."""
    G, S, K = d.num_genes, d.num_samples, d.num_sets
    nnz = int(d.set_offsets[-1])
    rb = 2 if ranks16 else 4
    words = (S + 31) // 32
    return {
        "permute": S + 4 * words * P,
        "metric": esize * G * S + 4 * words * P + esize * G * P,
        "sort": esize * G * P + (rb + esize) * G * P,
        "es": (rb + esize) * G * P + 8 * (K + 1) + 4 * nnz + esize * K * P,
        "stats": 4 * esize * K * P,
    }


def cpu_sample(d, metric_id, double, target_s, use_ref, max_s=10.0):
    """Time the CPU path on a sample of the permutations; returns (ES/s, sample P, seconds, kind).

    Two pilot calls (2n and 4n permutations on n threads: the stages run in
    parallel over permutations, so fewer than n permutations hide the cost
    of one) split a call's time into a fixed part and a part per permutation.  The reference's own build has a large
    fixed part: its CPU pipeline matches gene symbols to every 32-set batch
    (create_bitmaps) once per call, ~0.85 s at 20,000 genes x 1,000 sets on
    8 x86 cores, which a full run pays once.  The sample is sized to at least
    `target_s` of work and to keep the fixed part at most a tenth of it,
    within `max_s` and the workload's permutation count."""
    import oracle
    kind = "reference" if use_ref else "port"
    fn = oracle.ref_gsea if use_ref else oracle.gsea

    def run(P):
        t0 = time.perf_counter()
        fn(metric_id, d.exprs, d.labels, d.set_offsets, d.set_genes, P, double=double)
        return time.perf_counter() - t0

    n = int(os.environ.get("OMP_NUM_THREADS") or os.cpu_count() or 1)
    p1 = max(1, min(2 * n, d.num_perms // 4))
    t1, t2 = run(p1), run(2 * p1)
    per = max((t2 - t1) / p1, 1e-6)
    fixed = max(2 * t1 - t2, 0.0)
    want = max(target_s - fixed, 9 * fixed) / per
    P = int(min(d.num_perms, max(2 * p1, want), max((max_s - fixed) / per, 2 * p1)))
    dt = run(P)
    return d.num_sets * P / dt, P, dt, kind


def headline_config(d, args, world):
    """The `config` of both arms' lines (identical, so that the two are
    compared on the same workload)."""
    return {"workload": d.name, "metric_string": args.metric, "precision": args.precision,
            "l2": "256 MB write between timed GPU steps", "parallelism": f"perm-shard x{world}"}


def run_reference(args):
    """The reference's own CPU pipeline (its build from the cudaGSEA sources,
    oracle/_ref, where it exists on this machine; else the oracle's port of
    it) on all host cores.  A step is a bounded sample of the workload's
    permutations -- all sets -- sized so that the warm-up and timed steps
    together take about `--ref-seconds`."""
    world, rank, _ = dist_env()
    if rank != 0:
        return 0
    import oracle
    from cudagsea_gb300.api import METRICS
    oracle.build()
    oracle.build_ref()
    d = workload(args.workload)
    mid = METRICS.index(args.metric)
    double = args.precision == 64
    use_ref = oracle.ref_available()
    ncores = os.cpu_count() or 1
    os.environ.setdefault("OMP_NUM_THREADS", str(ncores))
    fn = oracle.ref_gsea if use_ref else oracle.gsea
    per_step = min(10.0, max(1.0, args.ref_seconds / max(1, args.steps + args.warmup)))
    _, P, dt, kind = cpu_sample(d, mid, double, per_step, use_ref, max_s=1.5 * per_step)
    for _ in range(args.warmup):
        fn(mid, d.exprs, d.labels, d.set_offsets, d.set_genes, P, double=double)
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        fn(mid, d.exprs, d.labels, d.set_offsets, d.set_genes, P, double=double)
        times.append(time.perf_counter() - t0)
    mean = sum(times) / len(times)
    value = d.num_sets * P / mean
    sample = (f"{P} of {d.num_perms} permutations per step (one call: metric, sort, scores and statistics), "
              f"all {d.num_sets} sets, {d.name}; {'the reference build' if use_ref else 'the oracle port'}")
    out = {
        "impl": "reference", "metric": METRIC_NAME, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64" if double else "f32", "data": "synthetic",
        "config": headline_config(d, args, world),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]),
                         "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(out), flush=True)
    return 0


def run_adaptive(args, d, full_plan, stream, flush, local):
    """The adaptive forms on the tensor-core plan's workload: the sequential
    rule alone ("adaptive") and with the learned prior ("learned")."""
    import numpy as np
    import torch
    from cudagsea_gb300 import allocator, api, synthetic
    from cudagsea_gb300 import _native as N
    K, P = d.num_sets, d.num_perms
    _, st_full = full_plan.read(es=False)
    calls_full = set(np.where(st_full.reshape(5, -1)[4] < 0.25)[0])
    # the prior's network: trained on the null scores of another seed
    t0 = time.perf_counter()
    cal = synthetic.full(seed=4322) if args.workload == "full" else synthetic.small(seed=4322)
    cp = api.Plan(cal.num_genes, cal.num_samples, cal.num_sets, cal.num_perms, args.metric, form=N.FORM_CHOSEN,
                  device=local)
    cp.set_inputs(cal.exprs, cal.labels, cal.set_offsets, cal.set_genes)
    cp.execute()
    cp.synchronize()
    model, curve = allocator.train_model(cp, seed=5, queries=24, steps=3000)
    cp.close()
    train_s = time.perf_counter() - t0
    out = {}
    for name, m in (("adaptive", None), ("learned", model)):
        plan = api.Plan(d.num_genes, d.num_samples, K, P, args.metric, form=N.FORM_CHOSEN, device=local)
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        for _ in range(args.warmup):
            allocator.execute_adaptive(plan, m, pilot_perms=args.pilot, growth=args.growth)
        times = []
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            torch.cuda.synchronize()
            t1 = time.perf_counter()
            res = allocator.execute_adaptive(plan, m, pilot_perms=args.pilot, growth=args.growth)  # after its last copy
            times.append(time.perf_counter() - t1)
        _, st = plan.read(es=False)
        calls = set(np.where(st.reshape(5, -1)[4] < 0.25)[0])
        mean_s = sum(times) / len(times)
        out[name] = {"ms_per_step": mean_s * 1e3, "value_equivalent": K * P / mean_s,
                     "scores_per_s": res.report["scores"] / mean_s,
                     "scores_fraction": res.report["scores"] / (K * P), "pilot_perms": args.pilot,
                     "growth": args.growth,
                     "rounds": res.report["rounds"], "stop_p": res.report["stop_p"],
                     "stopped_after_pilot": res.report["stopped_pilot"], "stopped_by_fdr_bound": res.report["stopped_q"],
                     "full_sets": res.report["full_sets"],
                     "model_used": res.report["model_used"], "calls": len(calls), "calls_full": len(calls_full),
                     "call_flips": len(calls ^ calls_full)}
        plan.close()
    out["learned"]["training_s"] = train_s
    out["learned"]["held_out_sigma_tail"] = float(model.get()[1][12])
    model.close()
    return out


def run_learned(args):
    """The learned-allocator workload: 20,000 x 200, 20,000 sets (5 % enriched),
    100,000 permutations.  Times the full test (plain and tensor-core forms,
    every score computed) and the adaptive test (tensor-core form) without and
    with the learned prior, and counts the FDR < 0.25 calls that differ."""
    import numpy as np
    import torch
    from cudagsea_gb300 import allocator, api, build, synthetic
    from cudagsea_gb300 import _native as N
    build.build()
    d = synthetic.learned()
    K, P = d.num_sets, d.num_perms
    steps = max(1, min(args.steps, 2))
    res = {}
    full_stats = None
    for name, form in (("plain", N.FORM_PLAIN), ("chosen", N.FORM_CHOSEN)):
        plan = api.Plan(d.num_genes, d.num_samples, K, P, args.metric, form=form)
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        plan.execute()
        plan.synchronize()
        times = []
        for _ in range(steps):
            t0 = time.perf_counter()
            plan.execute()
            plan.synchronize()
            times.append(time.perf_counter() - t0)
        mean = sum(times) / len(times)
        res[name] = {"s_per_run": mean, "value": K * P / mean}
        if name == "chosen":
            full_stats = plan.read(es=False)[1].reshape(5, -1)
        plan.close()
    calls_full = set(np.where(full_stats[4] < 0.25)[0])
    t0 = time.perf_counter()
    cal = synthetic.learned(seed=6262, num_sets=2000, num_perms=4000)
    cp = api.Plan(cal.num_genes, cal.num_samples, cal.num_sets, cal.num_perms, args.metric, form=N.FORM_CHOSEN)
    cp.set_inputs(cal.exprs, cal.labels, cal.set_offsets, cal.set_genes)
    cp.execute()
    cp.synchronize()
    model, _ = allocator.train_model(cp, seed=5, queries=24, steps=3000)
    cp.close()
    train_s = time.perf_counter() - t0
    for name, m in (("adaptive", None), ("learned", model)):
        plan = api.Plan(d.num_genes, d.num_samples, K, P, args.metric, form=N.FORM_CHOSEN)
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        allocator.execute_adaptive(plan, m, pilot_perms=args.pilot)
        times = []
        for _ in range(steps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            r = allocator.execute_adaptive(plan, m, pilot_perms=args.pilot)
            times.append(time.perf_counter() - t0)
        st = plan.read(es=False)[1].reshape(5, -1)
        calls = set(np.where(st[4] < 0.25)[0])
        flips = sorted(calls ^ calls_full)
        mean = sum(times) / len(times)
        res[name] = {"s_per_run": mean, "value_equivalent": K * P / mean, "scores_per_s": r.report["scores"] / mean,
                     "scores_fraction": r.report["scores"] / (K * P), "rounds": r.report["rounds"],
                     "stop_p": r.report["stop_p"], "stopped_after_pilot": r.report["stopped_pilot"],
                     "stopped_by_fdr_bound": r.report["stopped_q"], "full_sets": r.report["full_sets"],
                     "model_used": r.report["model_used"], "prior_sets_agreed": r.report["prior_agreed"],
                     "calls": len(calls), "calls_full": len(calls_full), "call_flips": len(flips),
                     "flip_q_full": [float(full_stats[4][k]) for k in flips[:10]]}
        plan.close()
    res["learned"]["training_s"] = train_s
    res["learned"]["held_out_sigma_tail"] = float(model.get()[1][12])
    model.close()
    out = {"metric": METRIC_NAME + ", adaptive (equivalent: K*P / wall time of the whole test)",
           "value": res["learned"]["value_equivalent"], "unit": UNIT, "n_gpus": 1, "steps": steps,
           "higher_is_better": True, "dtype": "f32", "data": "synthetic",
           "config": {"workload": d.name, "metric_string": args.metric, "pilot_perms": args.pilot,
                      "timing": "host wall clock, synchronised, whole test incl. statistics"},
           "forms": res,
           "learned_over_plain_full": res["learned"]["value_equivalent"] / res["plain"]["value"],
           "learned_over_chosen_full": res["learned"]["value_equivalent"] / res["chosen"]["value"]}
    print(json.dumps(out), flush=True)
    return 0


def run_batched(args):
    """256 uneven instances (genes U[5k, 30k], samples U[20, 500], sets
    U[50, 5,000], 1,000 permutations each, fp32, tensor-core form) in one
    CUDA graph, autotuned; against the same instances executed one plan after
    another on one stream (same buffers, same tuning)."""
    import ctypes
    import torch
    from cudagsea_gb300 import api, build, synthetic
    from cudagsea_gb300 import _native as N
    build.build()
    t0 = time.perf_counter()
    ds = synthetic.batch_instances(args.instances)
    gen_s = time.perf_counter() - t0
    total = sum(d.num_sets * d.num_perms for d in ds)
    t0 = time.perf_counter()
    b = api.Batch(ds, args.metric, precision=32, form=N.FORM_CHOSEN)
    setup_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    b.autotune()
    tune_s = time.perf_counter() - t0
    stream = torch.cuda.Stream()
    for _ in range(max(1, args.warmup)):  # the first execute captures the graph
        b.execute(stream.cuda_stream)
    b.synchronize()
    steps = max(1, min(args.steps, 5))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    with Clocks(0) as clk:
        for s0, s1 in ev:
            s0.record(stream)
            b.execute(stream.cuda_stream)
            s1.record(stream)
        torch.cuda.synchronize()
    b.synchronize()
    graph_ms = sum(a.elapsed_time(c) for a, c in ev) / steps
    # the same instances one plan after another on one stream
    L = N.lib()
    handles = []
    for i in range(len(ds)):
        h = ctypes.c_void_p()
        N.check(L.gsea_batch_plan(b._h, i, ctypes.byref(h)))
        handles.append(h)
    for h in handles:
        N.check(L.gsea_plan_execute(h, ctypes.c_void_p(stream.cuda_stream)))
    torch.cuda.synchronize()
    s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s0.record(stream)
    for h in handles:
        N.check(L.gsea_plan_execute(h, ctypes.c_void_p(stream.cuda_stream)))
    s1.record(stream)
    torch.cuda.synchronize()
    seq_ms = s0.elapsed_time(s1)
    info = b.info()
    b.close()
    out = {"metric": METRIC_NAME + f", {len(ds)} batched instances", "value": total / (graph_ms / 1e3), "unit": UNIT,
           "n_gpus": 1, "steps": steps, "warmup": args.warmup, "ms_per_step": graph_ms, "higher_is_better": True,
           "dtype": "f32", "data": "synthetic",
           "config": {"workload": f"batched_{len(ds)}_instances_P1000", "form": "chosen", "metric_string": args.metric,
                      "instances": len(ds), "scores_per_step": total,
                      "genes": [min(d.num_genes for d in ds), max(d.num_genes for d in ds)],
                      "samples": [min(d.num_samples for d in ds), max(d.num_samples for d in ds)],
                      "sets": [min(d.num_sets for d in ds), max(d.num_sets for d in ds)]},
           "forms": {"batched_graph": {"value": total / (graph_ms / 1e3), "ms_per_step": graph_ms},
                     "sequential_plans": {"value": total / (seq_ms / 1e3), "ms_per_step": seq_ms}},
           "batched_over_sequential": seq_ms / graph_ms,
           "graph": info, "setup_s": {"generate": gen_s, "plans": setup_s, "autotune": tune_s},
           "clocks": clk.summary()}
    print(json.dumps(out), flush=True)
    return 0


def run_ours(args):
    import numpy as np
    world, rank, local = dist_env()
    import torch
    if world > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    from cudagsea_gb300 import api, build
    from cudagsea_gb300 import _native as N
    if world > 1 and rank != 0:
        torch.distributed.barrier()  # rank 0 brings the in-tree build up to date first
    build.build()
    if world > 1 and rank == 0:
        torch.distributed.barrier()
    torch.cuda.set_device(local)
    d = workload(args.workload)
    P, K = d.num_perms, d.num_sets
    double = args.precision == 64
    esize = 8 if double else 4
    forms = ["plain"] if (double or args.form == "plain-only") else ["plain", "chosen", "chosen_fp64"]
    form_ids = {"plain": N.FORM_PLAIN, "chosen": N.FORM_CHOSEN, "chosen_fp64": N.FORM_CHOSEN_FP64}
    stream = torch.cuda.Stream(device=local)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{local}")
    measured = {}
    plans = {}
    clk = None
    for form_name in forms:
        form = form_ids[form_name]
        plan = api.Plan(d.num_genes, d.num_samples, K, P, args.metric, precision=args.precision, form=form,
                        perm_offset=rank * P, device=local)
        plan.set_inputs(d.exprs, d.labels, d.set_offsets, d.set_genes)
        tuning = plan.autotune() if not args.no_autotune else (plan.get_tuning(), None)
        # stage times from three profiled executes (untimed: profiling records
        # events between the stages, so it runs the launches one by one)
        plan.set_profiling(True)
        stage_sum = {s: 0.0 for s in N.STAGES}
        for _ in range(3):
            plan.execute(stream.cuda_stream)
            for k, v in plan.stage_times().items():
                stage_sum[k] += v / 3
        plan.set_profiling(False)  # the timed executes replay the plan's captured CUDA graph
        for _ in range(args.warmup):
            plan.execute(stream.cuda_stream)
        torch.cuda.synchronize()
        if world > 1:
            torch.distributed.barrier()
        starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
        launches = 0
        with Clocks(local) as c:
            torch.cuda.synchronize()
            for i in range(args.steps):
                with torch.cuda.stream(stream):
                    flush.zero_()  # evict L2 between timed steps (outside the events)
                starts[i].record(stream)
                plan.execute(stream.cuda_stream)
                ends[i].record(stream)
                launches += plan.last_launches()
            torch.cuda.synchronize()
        plan.synchronize()  # surfaces a kernel error flag, if any
        if world > 1:
            torch.distributed.barrier()
        step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
        mean_ms = sum(step_ms) / len(step_ms)
        if world > 1:
            t = torch.tensor([mean_ms], dtype=torch.float64, device=f"cuda:{local}")
            torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
            mean_ms = float(t.item())
        measured[form_name] = {"mean_ms": mean_ms, "value": world * K * P / (mean_ms / 1e3),
                               "stages": dict(stage_sum), "launches": launches,
                               "tuning": tuning[0], "clocks": c.summary()}
        plans[form_name] = plan
    if "chosen" in measured and world == 1 and not args.no_learned:
        measured.update(run_adaptive(args, d, plans["chosen"], stream, flush, local))
    # the headline: the tensor-core form with the error-free FP32 variance when
    # measured (the fastest form computing every score), else the plain form
    head = "chosen" if "chosen" in measured else "plain"
    clk = measured[head]["clocks"]
    plan = plans[head]
    mean_ms = measured[head]["mean_ms"]
    value = measured[head]["value"]
    launches = measured[head]["launches"]
    stage_avg = measured[head]["stages"]

    # ---- end to end through the C ABI, pinned host buffers
    hx = N.lib()
    import ctypes

    def pinned(nbytes):
        p = ctypes.c_void_p()
        N.check(hx.gsea_host_alloc(nbytes, ctypes.byref(p)))
        return p

    dt = np.float64 if double else np.float32
    arrs = {"x": np.ascontiguousarray(d.exprs, dt), "l": d.labels, "o": d.set_offsets, "g": d.set_genes}
    pins = {}
    for k, a in arrs.items():
        p = pinned(a.nbytes)
        ctypes.memmove(p, a.ctypes.data, a.nbytes)
        pins[k] = p
    es_b = pinned(esize * K * P)
    st_b = pinned(esize * 5 * K)
    plan.set_profiling(False)

    def e2e_step():  # through the C ABI, on the headline form's plan
        N.check(hx.gsea_plan_run_host(plan._h, pins["x"], pins["l"], pins["o"], pins["g"], es_b, st_b))

    for _ in range(args.warmup):
        e2e_step()
    if world > 1:
        torch.distributed.barrier()
    e2e_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        e2e_step()
        e2e_t.append(time.perf_counter() - t0)
    e2e_mean = sum(e2e_t) / len(e2e_t)
    if world > 1:
        t = torch.tensor([e2e_mean], dtype=torch.float64, device=f"cuda:{local}")
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_mean = float(t.item())
    e2e_value = world * K * P / e2e_mean
    h2d = sum(a.nbytes for a in arrs.values())
    d2h = esize * K * P + esize * 5 * K
    for p in list(pins.values()) + [es_b, st_b]:
        hx.gsea_host_free(p)

    # ---- roofline of the dominant stage
    dominant = max(stage_avg, key=stage_avg.get)
    sb = stage_bytes(d, P, esize, plan.ranks16)
    peak, peak_kind = peaks()
    achieved = sb[dominant] / (stage_avg[dominant] / 1e3) / 1e9
    tr = traffic_record().get(dominant)
    roof = {"bound": "hbm", "kernel": dominant, "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "traffic": tr, "peak_source": peak_kind,
            "algorithmic_bytes": sb[dominant], "avg_ms": stage_avg[dominant]}
    lim = issue_limiter(dominant, head)
    if lim is not None:
        roof["limiter"] = lim
    # the whole pipeline against its compulsory bytes: X once, then per
    # permutation the metric keys written + read, the u32 ranks written +
    # read and the ES column written
    Gd, Sd = d.num_genes, d.num_samples
    pipe_bytes = esize * Gd * Sd + P * (2 * esize * Gd + 8 * Gd + esize * K)
    pipe_gbs = pipe_bytes / (mean_ms / 1e3) / 1e9
    pipeline_roof = {"bound": "hbm", "algorithmic_bytes": pipe_bytes, "achieved": pipe_gbs, "peak": peak,
                     "unit": "GB/s", "frac": pipe_gbs / peak}

    # ---- issue-slot roofline of the dominant stage: its warp instructions
    # per launch (ncu count per (set, permutation) or per permutation, from
    # the committed profile record) over its event time, against the issue
    # slots of the SMs at the sampled median SM clock
    issue_roof = None
    cnt = traffic_record().get("warp_instructions", {}).get(dominant)
    if cnt and clk.get("sm_mhz"):
        units = K * P if cnt.get("per") == "set_perm" else P
        inst = cnt["value"] * units
        sms = torch.cuda.get_device_properties(local).multi_processor_count
        slots = sms * 4 * clk["sm_mhz"] * 1e6
        ach = inst / (stage_avg[dominant] / 1e3)
        issue_roof = {"bound": "issue", "kernel": dominant, "warp_instructions": inst,
                      "achieved": ach, "peak": slots, "unit": "warp-inst/s", "frac": ach / slots,
                      "source": cnt.get("source")}

    # ---- the headline's accuracy condition, outside every timed region:
    # both tensor-core forms against the plain form in FP64 on this workload
    nes_check = None
    if rank == 0 and "chosen" in measured and not args.no_precision_check:
        from cudagsea_gb300 import precision_check as PC
        t0 = time.perf_counter()
        reps = PC.check_forms(d, args.metric)
        nes_check = {name: PC.summary(r) for name, r in reps.items()}
        nes_check["reference"] = "plain form in FP64, same inputs and permutations"
        nes_check["seconds"] = time.perf_counter() - t0

    out = None
    if rank == 0:
        cpu = None
        if world == 1 and not args.no_cpu_baseline:
            import oracle
            oracle.build()
            use_ref = oracle.ref_available()
            os.environ.setdefault("OMP_NUM_THREADS", str(os.cpu_count() or 1))
            v, Ps, secs, kind = cpu_sample(d, api.METRICS.index(args.metric), double, args.cpu_seconds, use_ref)
            cpu = {"value": v, "unit": UNIT, "cores": int(os.environ["OMP_NUM_THREADS"]), "kind": kind,
                   "sample": f"{Ps} of {P} permutations, all {K} sets, {secs:.1f} s"}
        out = {
            "metric": METRIC_NAME, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64" if double else "f32", "data": "synthetic",
            "config": headline_config(d, args, world),
            "form": head,
            "forms": {k: ({"value": v["value"], "ms_per_step": v["mean_ms"], "stages_ms": v["stages"],
                           "tuning": v["tuning"]} if "stages" in v else v) for k, v in measured.items()},
            "chosen_over_plain": (measured["chosen"]["value"] / measured["plain"]["value"]
                                  if "chosen" in measured else None),
            "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
            "roofline": roof,
            "pipeline_roofline": pipeline_roof,
            "issue_roofline": issue_roof,
            "nes_vs_fp64": nes_check,
            "stages_ms": stage_avg,
            "cpu_baseline": cpu,
            "clocks": clk,
            "gpu_launches": launches,
        }
        print(json.dumps(out), flush=True)
    for pl in plans.values():
        pl.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "learned":
        return run_learned(args)
    if args.workload == "batched":
        return run_batched(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
