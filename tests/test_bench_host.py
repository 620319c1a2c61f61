"""Host logic of bench.py that needs no GPU: the clock record's decoding of
NVML clock-event reasons and of nvidia-smi lines (fake samples, no NVML),
and the reference arm's JSON line (the CPU oracle, one step)."""
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


def test_reference_arm_prints_one_contract_line():
    """`bench.py --impl reference` (the CPU oracle on the host's threads, no
    GPU) prints one JSON line with the reference arm's keys: its own value as
    the CPU baseline and an e2e record without device copies."""
    import json
    import pathlib
    import subprocess
    import sys
    root = pathlib.Path(bench.__file__).resolve().parent
    out = subprocess.run([sys.executable, str(root / "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], cwd=root, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, out.stdout[-2000:]
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["metric"] == bench.METRIC
    assert d["value"] > 0 and d["unit"] == "cell-stage/s" and d["higher_is_better"] is True
    assert d["steps"] == 1 and d["n_gpus"] == 1
    assert d["config"]["workload"] == bench.HEADLINE["workload"]
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference") and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
