"""Runtime autotuner: picks valid shapes, results unchanged, tuning file round trip and device keying."""
import os

import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import api
from tokura_zgeev_batched_gb300 import workloads as wl

pytestmark = pytest.mark.gpu


def test_autotune_plain_and_roundtrip(cuda, tmp_path):
    import torch

    h = api.Handle()
    assert h.autotune(6, 9, 3000) == 0
    shapes = {n: h.plain_config(n, 3000) for n in range(6, 10)}
    for lanes, threads in shapes.values():
        assert lanes in (1, 2, 4, 8) and threads in (32, 64, 128, 256)
    A = wl.gaussian(500, 7, seed=21)
    w, f = api.zgeev_batched(torch.from_numpy(A).cuda(), handle=h)
    rep = lo.parity_report(A, w.cpu().numpy(), f.cpu().numpy(), with_cond=False)
    assert rep["max_rel_err"] <= lo.TOL_REL_FRO and rep["flag_mismatch"] == 0

    path = str(tmp_path / "tuning.txt")
    assert h.autotune_ragged(2000, 1, 16) == 0
    assert h.save_tuning(path) == 0
    text = open(path).read()
    assert text.startswith("tokura_zgeev_gb300_tuning 1") and "ragged" in text
    h2 = api.Handle()
    assert h2.load_tuning(path) == 0
    for n, shape in shapes.items():
        assert h2.plain_config(n, 3000) == shape

    # Another device's file is refused and leaves the handle unchanged.
    other = str(tmp_path / "other.txt")
    with open(other, "w") as fo:
        fo.write(text.replace("sms ", "sms 1"))
    h3 = api.Handle()
    before = h3.plain_config(7, 3000)
    assert h3.load_tuning(other) == 3
    assert h3.plain_config(7, 3000) == before
    bad = str(tmp_path / "bad.txt")
    with open(bad, "w") as fb:
        fb.write(text + "plain 7 3 128\n")
    assert h3.load_tuning(bad) == 2
    assert h3.load_tuning(str(tmp_path / "missing.txt")) == 1


def test_tuning_file_from_environment(cuda, tmp_path):
    h = api.Handle()
    assert h.set_plain_config(11, 2, 64) == 0
    path = str(tmp_path / "env_tuning.txt")
    assert h.save_tuning(path) == 0
    os.environ["TOKURA_ZGEEV_TUNING_FILE"] = path
    try:
        h2 = api.Handle()
        assert h2.plain_config(11, 100000) == (2, 64)
    finally:
        del os.environ["TOKURA_ZGEEV_TUNING_FILE"]
