"""Host side of bench.py that needs no GPU: the clock sampler around the
timed region, driven by a fake NVML device."""
import time

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
