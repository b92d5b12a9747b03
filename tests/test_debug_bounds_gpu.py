"""Bounds-checked build (the stand-in for a memory checker): every matrix-element access of
every entry point's kernels stays inside its matrix, and the plain kernels' per-matrix QR sweep
counts equal those of the CPU model of the same iteration (oracle/model_qr.c)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def debug_run(cuda):
    from tokura_zgeev_batched_gb300 import build

    build.build(debug=True)
    env = dict(os.environ, TOKURA_ZGEEV_DEBUG_BOUNDS="1")
    res = subprocess.run([sys.executable, os.path.join(HERE, "debug_bounds_run.py")], env=env,
                         capture_output=True, text=True, timeout=900)
    assert res.returncode == 0, res.stderr[-4000:]
    return json.loads(res.stdout.strip().splitlines()[-1])


def test_release_library_reports_no_checking():
    from tokura_zgeev_batched_gb300 import api

    assert api.lib().tokuraDebugAttach(None) == -2


def test_no_out_of_bounds_access(debug_run):
    bad = {k: v for k, v in debug_run["cases"].items() if v["violations"] != 0}
    assert len(debug_run["cases"]) >= 20
    assert not bad, bad


@pytest.mark.parametrize("n", [33, 64])
@pytest.mark.parametrize("scaled", [65, 1])
def test_sweeps_equal_the_cpu_model(debug_run, n, scaled):
    rec = debug_run[f"sweeps_n{n}_s{scaled}"]
    A = wl.gaussian(rec["batch"], n, seed=rec["A_seed"])
    gpu = np.array(rec["gpu"])
    assert (gpu > 0).all() and not any(rec["flags"])
    if scaled == 65:
        _, flag, model = lo.model_qr(A)
    else:
        _, flag, model, _, _ = lo.model_qr_variant(A, scaled=True)
    assert not flag.any()
    same = float(np.mean(gpu == model))
    # The GPU contracts multiply-adds (FMA), the model rounds each operation: a sweep more or
    # less on a few matrices is rounding; the totals agree closely.
    assert same >= 0.9, (same, np.abs(gpu - model).max())
    assert abs(gpu.sum() - model.sum()) <= 0.01 * model.sum(), (gpu.sum(), model.sum())
