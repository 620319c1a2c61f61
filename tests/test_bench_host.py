"""Host logic of bench.py that needs no GPU: the clock record's decoding of
NVML clock-event reasons and of nvidia-smi lines (fake samples, no NVML)."""
import bench


def test_nvml_samples_decode_median_max_and_reasons():
    s = bench.ClockSampler(0)
    # (sm MHz, max MHz, nvmlClocksEventReason bits): sw power cap, then idle bit only, then hw thermal
    s.samples = [(2070.0, 2070.0, 0x4), (1950.0, 2070.0, 0x1), (2010.0, 2070.0, 0x40 | 0x8)]
    out = s.summary()
    assert out["sm_mhz"] == 2010.0 and out["sm_max_mhz"] == 2070.0 and out["samples"] == 3
    assert out["reasons"] == ["hw_slowdown", "hw_thermal_slowdown", "sw_power_cap"]
    assert out["source"] == "nvml"


def test_nvidia_smi_lines_decode_and_empty_record():
    s = bench.ClockSampler(0)
    s.lines = ["0, 2070, 2070, 900.5, 0x0, Not Active, Not Active, Not Active, Active",
               "0, 2065, 2070, 910.0, 0x0, Not Active, Not Active, Active, Not Active",
               "garbage"]
    out = s.summary()
    assert out["samples"] == 2 and out["sm_mhz"] == 2067.5
    assert out["reasons"] == ["sw_power_cap", "sw_thermal_slowdown"]
    assert out["source"] == "nvidia-smi"
    empty = bench.ClockSampler(0).summary()
    assert empty == {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}


def test_sampler_enters_and_exits_on_any_host():
    # with or without NVML and nvidia-smi, sampling starts, stops and yields a record
    s = bench.ClockSampler(0)
    with s:
        pass
    out = s.summary()
    assert {"sm_mhz", "sm_max_mhz", "reasons", "samples"} <= set(out)
    assert out["samples"] <= len(s.samples) + len(s.lines)
