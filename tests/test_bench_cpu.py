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
