"""Host side of bench.py that needs no GPU: the clock sampler around the
timed region, driven by a fake NVML device."""
import time

import pytest

import bench


class FakeNvml:
    """Scripted NVML answers: the SM clock falls from 2070 to 1980 MHz and
    the power cap becomes active after the first two samples."""

    def __init__(self, device):
        self.n = 0
        self.closed = False

    def sample(self):
        self.n += 1
        capped = self.n > 2
        return (1980.0 if capped else 2070.0), 2070.0, 1100.0, (["sw_power_cap"] if capped else [])

    def close(self):
        self.closed = True


def test_clock_sampler_samples_before_during_and_after(monkeypatch):
    monkeypatch.setattr(bench, "_Nvml", FakeNvml)
    with bench.Clocks(0, period_s=0.002) as c:
        assert len(c.samples) == 1  # taken before the region's first launch
        time.sleep(0.05)
    s = c.summary()
    assert c.nvml.closed
    assert s["source"] == "nvml"
    assert s["samples"] >= 4
    assert s["sm_max_mhz"] == 2070.0 and s["sm_min_mhz"] == 1980.0
    assert s["reasons"] == ["sw_power_cap"]
    assert s["power_w"] == 1100.0


def test_clock_sampler_without_nvml_or_nvidia_smi(monkeypatch):
    def no_nvml(device):
        raise OSError("no library")

    monkeypatch.setattr(bench, "_Nvml", no_nvml)
    monkeypatch.setenv("PATH", "/nonexistent")
    with bench.Clocks(0) as c:
        pass
    assert c.summary() == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


class FakeClock:
    def __init__(self):
        self.t = 0.0

    def perf_counter(self):
        return self.t


def test_cpu_sample_amortises_a_fixed_per_call_cost(monkeypatch):
    """A CPU path with a fixed cost per call (0.8 s) and 30 ms per permutation
    on 8 threads, run in waves of 8 permutations: the sample keeps the fixed
    part at most a tenth of the timed call and stays within the step limit."""
    import types
    import oracle
    clock = FakeClock()
    calls = []

    def fake_gsea(metric_id, exprs, labels, off, genes, P, double=False):
        calls.append(P)
        clock.t += 0.8 + 0.03 * 8 * -(-P // 8)  # whole waves of 8 permutations

    monkeypatch.setattr(bench, "time", types.SimpleNamespace(perf_counter=clock.perf_counter))
    monkeypatch.setattr(oracle, "ref_gsea", fake_gsea)
    monkeypatch.setenv("OMP_NUM_THREADS", "8")
    d = types.SimpleNamespace(exprs=None, labels=None, set_offsets=None, set_genes=None, num_sets=1000,
                              num_perms=1000)
    value, P, secs, kind = bench.cpu_sample(d, 8, False, 2.0, True)
    assert kind == "reference" and calls[:2] == [16, 32]
    assert 0.8 <= 0.1 * secs + 1e-9 and secs <= 10.0
    assert value == pytest.approx(1000 * P / secs)
    # without a fixed cost the sample is just the target time
    calls.clear()
    monkeypatch.setattr(oracle, "gsea", lambda *a, **k: (calls.append(a[5]),
                                                         setattr(clock, "t", clock.t + 0.03 * a[5])))
    value, P, secs, kind = bench.cpu_sample(d, 8, False, 2.0, False)
    assert kind == "port" and secs == pytest.approx(2.0, rel=0.05)
