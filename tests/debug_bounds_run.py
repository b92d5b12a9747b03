"""Runs the bounds-checked library (TOKURA_ZGEEV_DEBUG_BOUNDS=1) over every entry point and
prints one JSON object: violations per case and per-matrix QR sweep counts. Started as a
subprocess by tests/test_debug_bounds_gpu.py, so the checking library never replaces the
release one in the test process."""
import json
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def main():
    assert os.environ.get("TOKURA_ZGEEV_DEBUG_BOUNDS") == "1"
    import numpy as np
    import torch

    from tokura_zgeev_batched_gb300 import api, build
    from tokura_zgeev_batched_gb300 import workloads as wl

    lib = api.lib()
    assert lib._name == build.DEBUG_LIB_PATH, lib._name
    dev = torch.device("cuda", 0)
    cap = 4096
    sweeps = torch.full((cap,), -1, dtype=torch.int32, device=dev)
    rec = torch.zeros(6, dtype=torch.int64, device=dev)
    rec[4] = sweeps.data_ptr()
    rec[5] = cap
    assert lib.tokuraDebugAttach(ctypes_ptr(rec)) == 0
    out = {"cases": {}}

    def check(name, fn):
        rec[0] = 0
        sweeps.fill_(-1)
        torch.cuda.synchronize()
        res = fn()
        torch.cuda.synchronize()
        r = rec.cpu().tolist()
        out["cases"][name] = {"violations": int(r[0]), "first": r[1:4]}
        return res

    def plain(n, batch, seed, mode=1, scaled=16, lanes=0, balance=0):
        h = api.Handle()
        assert h.set_shift_hints(mode) == 0 and h.set_scaled_rotations(scaled) == 0
        assert h.set_balancing(balance) == 0
        if lanes:
            assert h.set_plain_config(n, lanes, 64) == 0
        A = torch.from_numpy(wl.gaussian(batch, n, seed=seed)).to(dev)
        w, f = api.zgeev_batched(A, handle=h)
        return A, w, f

    for n in (1, 2, 3, 17, 33, 64):
        for lanes in (1, 4, 32):
            check(f"plain_n{n}_L{lanes}", lambda: plain(n, 96, 10 + n, lanes=lanes))
    check("plain_balance_n40", lambda: plain(40, 64, 7, balance=3))
    # sweeps against the CPU model of the iteration: no hints, plain and scaled rotations
    for n in (33, 64):
        for scaled in (65, 1):
            A, w, f = check(f"sweeps_n{n}_s{scaled}", lambda: plain(n, 256, 500 + n, mode=0, scaled=scaled))
            out[f"sweeps_n{n}_s{scaled}"] = {"A_seed": 500 + n, "batch": 256,
                                             "gpu": sweeps[:256].cpu().tolist(), "flags": f.cpu().tolist()}
    # ragged (hints for orders >= 48), backward, vectors, real, other layouts
    def ragged():
        ns = wl.ragged_sizes(600, 1, 64, seed=3)
        mats = [wl.gaussian(1, int(k), seed=1000 + j)[0] for j, k in enumerate(ns)]
        buf, ns_, offs, eoffs = wl.pack_ragged(mats)
        return api.zgeev_ragged(torch.from_numpy(buf).to(dev), torch.from_numpy(ns))
    check("ragged", ragged)

    def backward(n):
        A, _ = wl.torch_vdv_separated(64, n, seed=9, min_sep=0.05, device="cuda")
        lam, f = api.zgeev_batched(A)
        gbar = (torch.exp(lam.real) + 2 * lam).contiguous()
        return api.zgeev_backward(A, lam, gbar)
    for n in (5, 24):
        check(f"backward_n{n}", lambda: backward(n))
    for n in (6, 40):
        check(f"vectors_n{n}", lambda: api.zgeev_vectors(torch.from_numpy(wl.gaussian(64, n, seed=4)).to(dev)))
    for n in (3, 16, 45):
        check(f"real_n{n}", lambda: api.dgeev_batched(torch.randn(96, n, n, dtype=torch.float64, device=dev)))
    big = torch.from_numpy(wl.gaussian(40, 48, seed=8)).to(dev)
    check("strided", lambda: api.zgeev_strided(big[:, 5:37, 3:35]))
    check("pointers", lambda: api.zgeev_pointers([big[k] for k in range(40)]))
    check("complex64", lambda: api.cgeev_batched(big.to(torch.complex64)))

    def noalloc():
        h = api.Handle()
        A = torch.from_numpy(wl.gaussian(200, 30, seed=5)).to(dev)
        eig = torch.empty(200, 30, dtype=torch.complex128, device=dev)
        flag = torch.empty(200, dtype=torch.int8, device=dev)
        assert api.lib().tokura_zgeev_batched_gpu_noalloc(h.value, 30, 200, A.data_ptr(), eig.data_ptr(),
                                                          flag.data_ptr(), torch.cuda.current_stream().cuda_stream) == 0
    check("noalloc", noalloc)
    assert lib.tokuraDebugAttach(None) == 0
    print(json.dumps(out))


def ctypes_ptr(t):
    return t.data_ptr()


if __name__ == "__main__":
    main()
