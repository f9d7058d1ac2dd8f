"""The bench's clock record: NVML polled during the timed region, the GPU
found by the CUDA device's UUID, reason bits named as nvidia-smi names them.
A fake NVML stands in for libnvidia-ml (no GPU here); only read-only queries
are made."""
import time
from types import SimpleNamespace

import bench


class FakeNvml:
    def __init__(self, mhz, bits):
        self.mhz, self.bits = list(mhz), list(bits)
        self.calls = 0
        self.uuid = None
        self.shut = False

    def nvmlInit_v2(self):
        return 0

    def nvmlShutdown(self):
        self.shut = True
        return 0

    def nvmlDeviceGetHandleByUUID(self, uuid, handle):
        self.uuid = uuid
        return 0 if uuid == b"GPU-1234" else 13

    def nvmlDeviceGetHandleByPciBusId_v2(self, bus, handle):
        return 13

    def nvmlDeviceGetMaxClockInfo(self, h, kind, out):
        out._obj.value = 2070
        return 0

    def nvmlDeviceGetClockInfo(self, h, kind, out):
        out._obj.value = self.mhz[min(self.calls, len(self.mhz) - 1)]
        return 0

    def nvmlDeviceGetCurrentClocksEventReasons(self, h, out):
        out._obj.value = self.bits[min(self.calls, len(self.bits) - 1)]
        self.calls += 1
        return 0

    def nvmlDeviceGetPowerUsage(self, h, out):
        out._obj.value = 900_000
        return 0


def test_sampler_polls_during_the_region_and_names_reasons():
    fake = FakeNvml(mhz=[2070, 2055, 1980], bits=[0x0, 0x4, 0x4])
    reader = bench.NvmlReader(0, lib=fake, props=SimpleNamespace(uuid="1234"))
    assert fake.uuid == b"GPU-1234"
    with bench.ClockSampler(0, reader=reader) as clk:
        time.sleep(0.1)
    s = clk.summary()
    assert fake.shut
    assert s["source"] == "nvml"
    assert s["samples"] >= 5          # entry, exit and the 2 ms polls between
    assert s["sm_max_mhz"] == 2070.0
    assert s["sm_mhz"] == 1980.0      # the median of the samples
    assert s["reasons"] == ["sw_power_cap"]
    assert s["power_w_median"] == 900.0


def test_thermal_and_hw_slowdown_bits_are_reported():
    fake = FakeNvml(mhz=[1500], bits=[0x8 | 0x20 | 0x40])
    reader = bench.NvmlReader(0, lib=fake, props=SimpleNamespace(uuid="GPU-1234"))
    with bench.ClockSampler(0, reader=reader) as clk:
        pass
    assert clk.summary()["reasons"] == ["hw_slowdown", "hw_thermal_slowdown",
                                        "sw_thermal_slowdown"]


def test_unknown_device_is_refused():
    fake = FakeNvml(mhz=[2070], bits=[0])
    try:
        bench.NvmlReader(0, lib=fake, props=SimpleNamespace(uuid="other"))
    except OSError:
        assert fake.shut
    else:
        raise AssertionError("a device NVML does not know must not be sampled")


def test_nvidia_smi_lines_are_parsed():
    clk = bench.ClockSampler(0)
    clk.source = "nvidia-smi"
    clk.lines = ["0, 2070, 2070, 850.1, 0x4, Not Active, Not Active, Not Active, Active",
                 "0, 2040, 2070, 860.3, 0x4, Not Active, Not Active, Not Active, Active"]
    s = clk.summary()
    assert s["samples"] == 2 and s["sm_mhz"] == 2055.0 and s["reasons"] == ["sw_power_cap"]
