"""bench.py without a GPU: its command line parses and every library
function it calls exists (the GPU runs of the benchmark cannot catch a
misspelt name before the section that uses it)."""
import os
import re
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_bench_help():
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--help"], capture_output=True, text=True,
                         timeout=120)
    assert out.returncode == 0 and "--impl" in out.stdout


def test_bench_api_names_exist():
    from tokura_zgeev_batched_gb300 import api

    src = open(os.path.join(ROOT, "bench.py")).read()
    names = set(re.findall(r"\bapi\.([A-Za-z_]\w*)", src))
    assert names and not [n for n in names if not hasattr(api, n)]
    lib = api.lib()
    syms = set(re.findall(r"\bapi\.lib\(\)\.([A-Za-z_]\w*)", src))
    assert not [s for s in syms if not hasattr(lib, s)]


def test_reference_arm_json_line():
    """`bench.py --impl reference` (the LAPACK CPU path) prints one JSON line with the
    contract's keys; it needs no GPU."""
    import json

    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "1"], capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["cores"] >= 1
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0


def test_clock_record_summary():
    """The `clocks` object of the JSON line: median SM clock, max clock and power, and the
    throttle reasons seen Active during the timed region (nvidia-smi csv, noheader, nounits)."""
    sys.path.insert(0, ROOT)
    import bench

    lines = [
        "2070, 2070, 612.5, 0x0000000000000000, Not Active, Not Active, Not Active, Not Active",
        "2055, 2070, 640.1, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "1980, 2070, 655.0, 0x0000000000000004, Not Active, Not Active, Not Active, Active",
        "garbage line",
        "[N/A], 2070, 600.0, 0x0, Not Active, Not Active, Not Active, Not Active",
    ]
    s = bench.ClockSampler.summarize(lines)
    assert s["sm_mhz"] == 2055 and s["sm_max_mhz"] == 2070 and s["samples"] == 3
    assert s["power_w_max"] == 655.0 and s["reasons"] == ["sw_power_cap"]
    hot = bench.ClockSampler.summarize(["1500, 2070, 700, 0x8, Not Active, Active, Not Active, Not Active"])
    assert hot["reasons"] == ["hw_thermal_slowdown"]
    assert bench.ClockSampler.summarize([]) is None
