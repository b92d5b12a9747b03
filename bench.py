"""Benchmark of the batched eigenvalue-only ZGEEV path on GB300.

Default workload (one "step"): one call of the plain entry point
``tokura_zgeev_batched_gpu`` on 65,536 complex128 64x64 matrices
(4 GiB, Re/Im i.i.d. N(0,1), fixed seed) — the n=64 case of the size sweep,
the order at which the throughput target is stated. Inputs are resident in
HBM for ``value``; ``e2e`` times the same call with the input copied from
pinned host memory and the eigenvalues/flags copied back inside every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

``--impl reference`` times the reference's CPU comparison path (LAPACK zgeev
per matrix over all host cores, stream_test_with_MKL/get_eig_MKL.c:27-47) on
a bounded sample of the same workload. Under torchrun every rank processes its
own batch (weak scaling, no collective on the data path); rank 0 prints the
JSON line with the max time over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "matrices/s eigvals (n=32,64; ragged 1-64), fwd+bwd matrices/s, % FP64 peak"
N = 64
BATCH = (4 << 30) // (16 * N * N)  # 65,536 matrices = 4 GiB of input
SEED = 20261203
SWEEP_NS = (4, 8, 16, 32, 48)  # the size sweep's other orders (n = 64 is the timed workload)


# Orders from which the plain entry point runs with FP32 shift hints by default
# (three kernels per call: estimator, Hessenberg phase, QR phase).
SHIFT_HINT_MIN_N = 12


def set_workload(n: int, batch: int = 0) -> None:
    """Overrides the timed workload (used for small profiling captures)."""
    global N, BATCH
    N = int(n)
    BATCH = int(batch) if batch > 0 else (4 << 30) // (16 * N * N)


def flops_per_matrix(n: int) -> float:
    """Algorithmic work convention: 40 n^3 real FP64 flops per matrix (Hessenberg + QR, complex)."""
    return 40.0 * n ** 3


# Real FP64 flops of the backward per matrix, in units of n^3 (FMA = 2 flops), counted from
# its steps (tokura_zgeev_batched_gb300/csrc/zgeev_backward.cuh) at leading order:
#   Householder Hessenberg keeping tau        16 * sum_m m (m + n)        = 40/3
#   Q from the reflectors                     16 * sum_m m^2              = 16/3
#   Schur QR, full-width updates, Q rotated   20 flops per element pair, ~2n pairs per rotation,
#     one sweep per eigenvalue (perfect shifts; CPU model ~1.0)  20 * 2n * n^2/2 = 20
#   X and Y by back-substitution              8 * 2 * sum_k k^2/2         = 8/3
#   M = Y Z, P = Q M, Abar = P Q^H            8 * (n^3/6 + n^3/2 + n^3)   = 40/3
BWD_FLOPS_PER_N3 = 40.0 / 3 + 16.0 / 3 + 20.0 + 8.0 / 3 + 40.0 / 3


def bytes_per_matrix(n: int) -> int:
    return 16 * n * n + 16 * n + 1


# ----------------------------------------------------------------------------- helpers

def max_over_ranks(x: float, dist, device) -> float:
    """Max of a per-rank scalar over all ranks (identity without torch.distributed)."""
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def rank_seed(seed: int, rank: int) -> int:
    """Each rank solves its own batch (weak scaling: no data is exchanged)."""
    return seed + 1000 * rank


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class ClockSampler:
    """Samples nvidia-smi clocks/throttle reasons in the background."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_id: str | None):
        self.proc = None
        self.lines: list[str] = []
        cmd = ["nvidia-smi", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits", "-lms", "200"]
        if gpu_id:
            cmd += ["-i", gpu_id]
        try:
            self.proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        return self.summarize(self.lines)

    @staticmethod
    def summarize(lines: list[str]) -> dict | None:
        """Median SM clock, max SM clock, max power and the throttle reasons seen as Active in
        `nvidia-smi --format=csv,noheader,nounits` lines of FIELDS (malformed lines skipped)."""
        sm, smax, power, reasons = [], [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                smax.append(float(parts[1]))
                power.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "samples": len(sm),
                "power_w_max": max(power), "reasons": sorted(reasons)}


def gpu_uuid(dev) -> str | None:
    import torch

    try:
        u = str(torch.cuda.get_device_properties(dev).uuid)
        return u if u.startswith("GPU-") else "GPU-" + u
    except Exception:
        return None


def read_profile_traffic() -> dict | None:
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as f:
            return json.load(f)
    except (OSError, ValueError):
        return None


def guarded(fn):
    """Runs one optional configuration: a failure is reported in its place (and its traceback on
    stderr) instead of ending the run before the JSON line."""
    try:
        return fn()
    except Exception as exc:  # noqa: BLE001
        import traceback

        traceback.print_exc(file=sys.stderr)
        return {"error": f"{type(exc).__name__}: {exc}"[:500]}


def cpu_baseline(n: int, seconds: float = 8.0) -> dict:
    """LAPACK zgeev per matrix over all host cores on a bounded sample of the workload."""
    import numpy as np

    from oracle import lapack_oracle as lo
    from tokura_zgeev_batched_gb300 import workloads

    threads = lo.default_threads()
    probe = workloads.gaussian(max(threads * 4, 64), n, seed=SEED + 99)
    _, _, t = lo.zgeev(probe, threads)
    rate = probe.shape[0] / max(t, 1e-6)
    count = int(min(max(rate * seconds, threads * 8), 200000))
    sample = workloads.gaussian(count, n, seed=SEED + 100)
    _, info, t = lo.zgeev(sample, threads)
    return {"value": count / t, "unit": "matrices/s", "cores": threads, "kind": "port",
            "sample": f"{count} complex Gaussian {n}x{n} matrices (seeded), LAPACK zgeev('N','N') from scipy's "
                      f"OpenBLAS 0.3.34, one call per matrix, {threads} threads, {t:.2f} s",
            "lapack_info_nonzero": int(np.count_nonzero(info))}


# ----------------------------------------------------------------------------- reference arm

def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return
    import numpy as np

    from oracle import lapack_oracle as lo
    from tokura_zgeev_batched_gb300 import workloads

    threads = lo.default_threads()
    sample_n = max(threads * 32, 256)
    mats = workloads.gaussian(sample_n, N, seed=SEED + 7)
    for _ in range(args.warmup):
        lo.zgeev(mats[: threads * 4], threads)
    times = []
    for _ in range(args.steps):
        _, info, t = lo.zgeev(mats, threads)
        times.append(t)
    total = sum(times)
    value = sample_n * args.steps / total
    out = {
        "metric": METRIC, "value": value, "unit": "matrices/s", "impl": "reference",
        "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "c128 (f64)", "data": "synthetic",
        "config": {"workload": f"plain zgeev eigenvalues, n={N}, complex Gaussian; each step a {sample_n}-matrix "
                               f"sample of the {BATCH}-matrix batch", "n": N, "batch": sample_n},
        "cpu_baseline": {"value": value, "unit": "matrices/s", "cores": threads, "kind": "port",
                         "sample": f"{sample_n} matrices per step, LAPACK zgeev('N','N') (scipy's OpenBLAS "
                                   f"0.3.34) over {threads} threads; the reference's own CPU path "
                                   f"(get_eig_MKL.c) needs MKL, which is absent"},
        "e2e": {"value": value, "unit": "matrices/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "lapack_info_nonzero": int(np.count_nonzero(info)),
    }
    print(json.dumps(out), flush=True)


# ----------------------------------------------------------------------------- our arm

def phase(name: str) -> None:
    """Progress marker on stderr (the JSON line is the only stdout output)."""
    print(f"[bench {time.strftime('%H:%M:%S')}] {name}", file=sys.stderr, flush=True)


# Parity at configuration scale: LAPACK zgeev on every matrix of a batch for flag parity
# (CHECK_FULL_FLAGS) and the matched eigenvalue error, with zgeevx condition numbers, on a
# seeded random subset of CHECK_SUBSET matrices (the whole batch when it is smaller).
CHECK_SUBSET = 10000
CHECK_FULL_FLAGS = True


def _parity_fields(rep: dict, seconds: float) -> dict:
    return {"checked": rep["checked"], "flags_checked": rep["flags_checked"],
            "max_rel_err_fro": rep["max_rel_err"], "p99_rel_err_fro": rep["p99_rel_err"],
            "flag_mismatch": rep["flag_mismatch"], "lapack_fail": rep["lapack_fail"],
            "gpu_flagged": rep["gpu_flagged"], "cond_le_1e3": rep.get("well_conditioned"),
            "max_rel_err_fro_cond_le_1e3": rep.get("max_rel_err_well"),
            "p99_rel_err_fro_cond_le_1e3": rep.get("p99_rel_err_well"), "cpu_seconds": seconds}


def scale_check(A, eig, flag, seed: int, subset: int | None = None, full_flags: bool | None = None) -> dict:
    """Parity of a whole uniform batch against LAPACK zgeev (flags of every matrix, matched
    errors on a seeded subset); max/p99 of max|dlambda|/||A||_F."""
    from oracle import lapack_oracle as lo

    t0 = time.perf_counter()
    rep = lo.batch_parity(A.cpu().numpy(), eig.cpu().numpy(), flag.cpu().numpy(),
                          subset=CHECK_SUBSET if subset is None else subset, seed=seed,
                          full_flags=CHECK_FULL_FLAGS if full_flags is None else full_flags)
    return _parity_fields(rep, time.perf_counter() - t0)


def time_ms(fn, reps: int, stream) -> float:
    """Average CUDA-event time of fn() on `stream` over reps calls (after one warm-up call)."""
    import torch

    fn()
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def measure_config1(h, dev, stream, peak, call) -> dict:
    """10,000 complex Gaussian 32x32 matrices, one plain call (the small-batch configuration)."""
    import torch

    from tokura_zgeev_batched_gb300 import api, workloads

    n, batch = 32, 10000
    A = workloads.torch_gaussian(batch, n, seed=SEED + 1, device=str(dev))
    eig = torch.empty(batch, n, dtype=torch.complex128, device=dev)
    flag = torch.empty(batch, dtype=torch.int8, device=dev)
    work = torch.empty(api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch), dtype=torch.uint8, device=dev)
    ms = time_ms(lambda: call(n, batch, A, eig, flag, work), 5, stream)
    rate = batch / (ms * 1e-3)
    out = {"n": n, "batch": batch, "ms": ms, "matrices_per_s": rate, "fp64_frac": flops_per_matrix(n) * rate / peak,
           "lanes_per_matrix": h.plain_config(n, batch)[0], "flagged": int((flag != 0).sum().item()),
           "parity": scale_check(A, eig, flag, seed=SEED + 1, subset=batch)}
    # The same call on a handle tuned for this order and batch (tokuraAutotune).
    ht = api.Handle()
    if ht.autotune(n, n, batch, stream.cuda_stream) == 0:
        def tuned_call():
            st = api.tokura_zgeev_batched_gpu(ht, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(),
                                              flag.data_ptr(), stream.cuda_stream)
            if st != 0:
                raise RuntimeError(f"tokura_zgeev_batched_gpu returned {st}")

        ms_t = time_ms(tuned_call, 5, stream)
        lanes, threads = ht.plain_config(n, batch)
        out["autotuned"] = {"ms": ms_t, "matrices_per_s": batch / (ms_t * 1e-3),
                            "fp64_frac": flops_per_matrix(n) * batch / (ms_t * 1e-3) / peak,
                            "lanes_per_matrix": lanes, "threads_per_block": threads,
                            "flagged": int((flag != 0).sum().item())}
    return out


def measure_real(h, dev, stream, peak, n: int = 64, batch: int = 65536, cpu_seconds: float = 2.0) -> dict:
    """Real-input path (tokura_dgeev_batched_gpu): real Gaussian n x n matrices.

    Convention: 10 n^3 flop per real matrix (Hessenberg + double-shift QR,
    eigenvalues only). Parity against LAPACK dgeev on an evenly spaced sample,
    including LAPACK's conjugate-pair convention; LAPACK dgeev over the host
    cores on a bounded sample for comparison.
    """
    import torch

    from oracle import lapack_oracle as lo
    from tokura_zgeev_batched_gb300 import api

    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 5)
    A = torch.randn(batch, n, n, generator=g, device=dev, dtype=torch.float64)
    wr = torch.empty(batch, n, dtype=torch.float64, device=dev)
    wi = torch.empty_like(wr)
    flag = torch.empty(batch, dtype=torch.int8, device=dev)
    work = torch.empty(api.tokura_get_dgeev_workspacesize(n, batch), dtype=torch.uint8, device=dev)

    def call():
        st = api.tokura_dgeev_batched_gpu(h, n, batch, A.data_ptr(), wr.data_ptr(), wi.data_ptr(), work.data_ptr(),
                                          flag.data_ptr(), stream.cuda_stream)
        if st != 0:
            raise RuntimeError(f"tokura_dgeev_batched_gpu returned {st}")

    ms = time_ms(call, 3, stream)
    rate = batch / (ms * 1e-3)
    idx = torch.arange(0, batch, max(1, batch // 256), device=dev)[:256]
    rep = lo.real_parity_report(A[idx].cpu().numpy(), wr[idx].cpu().numpy(), wi[idx].cpu().numpy(),
                                flag[idx].cpu().numpy())
    threads = lo.default_threads()
    sample = A[: max(threads * 16, 64)].cpu().numpy()
    _, _, _, t = lo.dgeev(sample, threads)
    cpu_count = int(min(max(sample.shape[0] / max(t, 1e-6) * cpu_seconds, threads * 8), batch))
    _, _, _, t = lo.dgeev(A[:cpu_count].cpu().numpy(), threads)
    return {"n": n, "batch": batch, "ms": ms, "matrices_per_s": rate,
            "fp64_frac_10n3": 10.0 * n ** 3 * rate / peak, "flagged": int((flag != 0).sum().item()),
            "parity": {"checked": int(idx.numel()), "max_rel_err_fro": rep["max_rel_err"],
                       "max_rel_err_fro_cond_le_1e3": rep["max_rel_err_well"], "cond_le_1e3": rep["well_conditioned"],
                       "flag_mismatch": rep["flag_mismatch"], "conjugate_pairs_exact": rep["pairs_ok"]},
            "cpu_lapack_dgeev": {"matrices_per_s": cpu_count / t, "threads": threads, "sample": cpu_count}}


def measure_vectors(h, dev, stream, n: int = 64, batch: int = 65536, cpu_seconds: float = 2.0) -> dict:
    """Eigenvalues with left and right eigenvectors (tokura_zgeev_vectors_batched_gpu) on 65,536 complex
    Gaussian 64x64 matrices (the eigenvalue workload's batch; about 13 GiB of A, VL and VR): matrices/s (raw C-ABI call on device buffers), residuals
    ||A VR - VR diag(w)|| / ||A|| and ||VL^H A - diag(w) VL^H|| / ||A|| on a sample, and LAPACK
    zgeev('V','V') over the host cores on a bounded sample for comparison."""
    import torch

    from oracle import lapack_oracle as lo
    from tokura_zgeev_batched_gb300 import api, workloads

    A = workloads.torch_gaussian(batch, n, seed=SEED + 9, device=str(dev))
    w = torch.empty(batch, n, dtype=torch.complex128, device=dev)
    VL = torch.empty(batch, n, n, dtype=torch.complex128, device=dev)
    VR = torch.empty(batch, n, n, dtype=torch.complex128, device=dev)
    flag = torch.empty(batch, dtype=torch.int8, device=dev)
    work = torch.empty(api.tokura_get_zgeev_vectors_workspacesize(n, batch), dtype=torch.uint8, device=dev)

    def call():
        st = api.lib().tokura_zgeev_vectors_batched_gpu(h.value, n, batch, A.data_ptr(), w.data_ptr(), VL.data_ptr(),
                                                        VR.data_ptr(), work.data_ptr(), flag.data_ptr(),
                                                        stream.cuda_stream)
        if st != 0:
            raise RuntimeError(f"tokura_zgeev_vectors_batched_gpu returned {st}")

    ms = time_ms(call, 3, stream)
    k = 64
    # Buffers are column-major per matrix: the row-major views are the transposes.
    Ak = A[:k].transpose(-1, -2)
    VRk = VR[:k].transpose(-1, -2)
    VLk = VL[:k].transpose(-1, -2)
    wk = w[:k]
    nA = torch.linalg.matrix_norm(Ak)
    res_r = torch.linalg.matrix_norm(Ak @ VRk - VRk * wk[:, None, :]) / nA
    res_l = torch.linalg.matrix_norm(VLk.conj().transpose(-1, -2) @ Ak - wk[:, :, None] * VLk.conj().transpose(-1, -2)) / nA
    threads = lo.default_threads()
    sample = A[: max(threads * 4, 32)].cpu().numpy()
    t0 = time.perf_counter()
    lo.zgeev_vectors(sample, threads)
    t = time.perf_counter() - t0
    count = int(min(max(sample.shape[0] / max(t, 1e-6) * cpu_seconds, threads * 4), batch))
    big = A[:count].cpu().numpy()
    t0 = time.perf_counter()
    lo.zgeev_vectors(big, threads)
    t = time.perf_counter() - t0
    return {"n": n, "batch": batch, "ms": ms, "matrices_per_s": batch / (ms * 1e-3),
            "flagged": int((flag != 0).sum().item()), "max_residual_right": float(res_r.max()),
            "max_residual_left": float(res_l.max()),
            "cpu_lapack_zgeev_vv": {"matrices_per_s": count / t, "threads": threads, "sample": count}}


def measure_config4(h, dev, stream, peak, batch: int = 50000, orders=(16, 48)) -> dict:
    """Differentiable eigenvalues: 50,000 separated-spectrum matrices each at n=16 and n=48.

    Loss L = sum_i exp(Re lambda_i) + |lambda_i|^2, so gbar = exp(Re lambda) + 2 lambda
    (torch's convention). Times the forward call and the backward call separately
    (CUDA events); a 16-matrix sample of the gradient is checked against
    torch.linalg.eigvals' backward on the CPU.
    """
    import numpy as np
    import torch

    from tokura_zgeev_batched_gb300 import api, workloads

    out = {}
    s = stream.cuda_stream
    for n in orders:
        A, _ = workloads.torch_vdv_separated(batch, n, seed=SEED + 40 + n, min_sep=0.05, device=str(dev))
        eig = torch.empty(batch, n, dtype=torch.complex128, device=dev)
        flag = torch.empty(batch, dtype=torch.int8, device=dev)
        work = torch.empty(api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch), dtype=torch.uint8, device=dev)
        gA = torch.empty_like(A)
        bflag = torch.empty(batch, dtype=torch.int8, device=dev)
        bwork = torch.empty(api.tokura_get_zgeev_backward_workspacesize(n, batch), dtype=torch.uint8, device=dev)

        def fwd():
            assert api.tokura_zgeev_batched_gpu(h, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(),
                                                flag.data_ptr(), s) == 0

        fwd()
        fwd_parity = scale_check(A, eig, flag, seed=SEED + 40 + n)
        gbar = (torch.exp(eig.real) + 2 * eig).contiguous()

        def bwd():
            assert api.tokura_zgeev_backward_gpu(h, n, batch, A.data_ptr(), eig.data_ptr(), gbar.data_ptr(),
                                                 gA.data_ptr(), bwork.data_ptr(), bflag.data_ptr(), s) == 0

        ms_f = time_ms(fwd, 3, stream)
        ms_b = time_ms(bwd, 3, stream)
        # gradient spot check against torch.linalg.eigvals backward (CPU, FP64)
        idx = torch.arange(0, batch, max(1, batch // 16), device=dev)[:16]
        Ac = A[idx].cpu().requires_grad_(True)
        lam = torch.linalg.eigvals(Ac)
        torch.sum(torch.exp(lam.real) + lam.real ** 2 + lam.imag ** 2).backward()
        ref = Ac.grad.numpy()
        got = gA[idx].cpu().numpy()
        rel = float(np.max(np.linalg.norm(got - ref, axis=(1, 2)) / np.linalg.norm(ref, axis=(1, 2))))
        f_fwd = 40.0 * n ** 3
        f_bwd = BWD_FLOPS_PER_N3 * n ** 3
        out[str(n)] = {
            "batch": batch, "ms_forward": ms_f, "ms_backward": ms_b,
            "matrices_per_s_forward": batch / (ms_f * 1e-3),
            "matrices_per_s_fwd_bwd": batch / ((ms_f + ms_b) * 1e-3),
            "fwd_bwd_over_fwd": (ms_f + ms_b) / ms_f,
            "fp64_frac_fwd_bwd": (f_fwd + f_bwd) * batch / ((ms_f + ms_b) * 1e-3) / peak,
            "fp64_frac_backward": f_bwd * batch / (ms_b * 1e-3) / peak,
            "grad_rel_err_vs_torch_cpu_16": rel,
            "flagged_forward": int((flag != 0).sum().item()), "flagged_backward": int((bflag != 0).sum().item()),
            "forward_parity": fwd_parity,
        }
        del A, eig, flag, work, gA, bflag, bwork, gbar
        torch.cuda.empty_cache()
    out["convention"] = (f"F_fwd = 40 n^3, F_bwd = {BWD_FLOPS_PER_N3:.2f} n^3 flop per matrix (the backward's "
                         f"operation count with one perfect-shift sweep per eigenvalue)")
    return out


def measure_config5(h, dev, stream, peak, batch: int = 20000, steps: int = 100) -> dict:
    """Ragged fwd+bwd optimisation loop in one CUDA graph.

    20,000 matrices, n ~ U{8..64}, separated spectra (min gap 0.05) shifted by +0.5;
    per matrix the smoothed spectral abscissa tau*logsumexp(Re lambda / tau),
    tau = 0.05, summed over matrices; 100 gradient-descent steps (lr 1e-2).
    One step (ragged forward, loss, ragged backward, update) is captured in a
    CUDA graph and replayed.
    """
    import numpy as np
    import torch

    from tokura_zgeev_batched_gb300 import api, workloads
    from tokura_zgeev_batched_gb300.autograd import eigvals_ragged

    tau, lr = 0.05, 1e-2
    ns = workloads.ragged_sizes(batch, 8, 64, seed=SEED + 5)
    order = np.argsort(ns, kind="stable")
    sizes_sorted = ns[order].astype(np.int64) ** 2
    start_sorted = np.concatenate([[0], np.cumsum(sizes_sorted)[:-1]])
    offsets = np.empty(batch, np.int64)
    offsets[order] = start_sorted
    total = int(sizes_sorted.sum())
    A0 = torch.empty(total, dtype=torch.complex128, device=dev)
    pos = 0
    for k in range(8, 65):
        c = int(np.count_nonzero(ns == k))
        if c == 0:
            continue
        Ak, _ = workloads.torch_vdv_separated(c, k, seed=SEED + 500 + k, min_sep=0.05, shift=0.5, device=str(dev))
        A0[pos:pos + c * k * k] = Ak.reshape(-1)
        pos += c * k * k
    n_d = torch.from_numpy(ns).to(dev)
    o_d = torch.from_numpy(offsets).to(dev)
    total_eig = int(ns.sum())
    seg = torch.repeat_interleave(torch.arange(batch, device=dev), n_d.to(torch.int64))
    work_f = torch.empty(api.tokura_get_zgeev_ragged_workspacesize(batch, total), dtype=torch.uint8, device=dev)
    work_b = torch.empty(api.tokura_get_zgeev_ragged_backward_workspacesize(batch, total), dtype=torch.uint8,
                         device=dev)
    A = A0.clone().requires_grad_(True)

    def eig_of(X):
        return eigvals_ragged(X, n_d, o_d, handle=h, work_fwd=work_f, work_bwd=work_b, total_eigenvalues=total_eig)

    def class_max(lam):
        """Per size class: max, mean and median over matrices of max Re lambda."""
        re = lam.real
        m = torch.full((batch,), -float("inf"), dtype=torch.float64, device=dev).scatter_reduce(
            0, seg, re, reduce="amax")
        res = {}
        for lo_, hi_ in ((8, 16), (16, 32), (32, 48), (48, 65)):
            sel = m[(n_d >= lo_) & (n_d < hi_)]
            res[f"{lo_}-{min(hi_, 64)}"] = {"max": float(sel.max().item()), "mean": float(sel.mean().item()),
                                            "median": float(sel.median().item())}
        return res

    def step():
        lam = eig_of(A)
        x = lam.real / tau
        m = torch.full((batch,), -float("inf"), dtype=torch.float64, device=dev).scatter_reduce(
            0, seg, x.detach(), reduce="amax")
        ssum = torch.zeros(batch, dtype=torch.float64, device=dev).index_add(0, seg, torch.exp(x - m[seg]))
        loss = (tau * (torch.log(ssum) + m)).sum()
        (g,) = torch.autograd.grad(loss, A)
        with torch.no_grad():
            A.sub_(lr * g)
        return loss

    def per_matrix(lam):
        """Per matrix: max Re lambda and the smoothed abscissa tau*logsumexp(Re lambda / tau)."""
        x = lam.real / tau
        m = torch.full((batch,), -float("inf"), dtype=torch.float64, device=dev).scatter_reduce(
            0, seg, x, reduce="amax")
        ssum = torch.zeros(batch, dtype=torch.float64, device=dev).index_add(0, seg, torch.exp(x - m[seg]))
        return m * tau, tau * (torch.log(ssum) + m)

    with torch.no_grad():
        lam0 = api.zgeev_ragged(A.detach(), n_d, offsets=o_d, handle=h, work=work_f, total_eigenvalues=total_eig)[0]
        before = class_max(lam0)
        maxre0, abscissa0 = per_matrix(lam0)
    side = torch.cuda.Stream(dev)
    side.wait_stream(stream)
    with torch.cuda.stream(side):
        for _ in range(2):
            step()
    stream.wait_stream(side)
    graph = torch.cuda.CUDAGraph()
    with torch.cuda.graph(graph):
        static_loss = step()
    with torch.no_grad():
        A.copy_(A0)
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(steps):
        graph.replay()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    final_loss = float(static_loss.item())
    with torch.no_grad():
        lam_final, flag = api.zgeev_ragged(A.detach(), n_d, offsets=o_d, handle=h, work=work_f,
                                           total_eigenvalues=total_eig)
        after = class_max(lam_final)
        maxre1, abscissa1 = per_matrix(lam_final)
    ms_fwd = time_ms(lambda: api.zgeev_ragged(A.detach(), n_d, offsets=o_d, handle=h, work=work_f,
                                              total_eigenvalues=total_eig), 3, stream)
    del graph
    diagnosis = guarded(lambda: diagnose_config5(A0, A.detach(), ns, offsets, maxre0, maxre1, tau, lr, steps))
    rose = (maxre1 > maxre0)
    rose_by_class = {}
    for lo_, hi_ in ((8, 16), (16, 32), (32, 48), (48, 65)):
        sel = (n_d >= lo_) & (n_d < hi_)
        rose_by_class[f"{lo_}-{min(hi_, 64)}"] = {"matrices": int(sel.sum().item()),
                                                   "max_re_lambda_rose": int((rose & sel).sum().item())}
    return {"batch": batch, "steps": steps, "ms_total": ms, "ms_per_step": ms / steps,
            "matrices_per_s_fwd_bwd": batch * steps / (ms * 1e-3), "ms_forward_only": ms_fwd,
            "fwd_bwd_over_fwd": (ms / steps) / ms_fwd, "max_re_lambda_before": before,
            "max_re_lambda_after": after, "initial_loss": float(abscissa0.sum().item()),
            "loss_after_last_step": float(abscissa1.sum().item()),
            "loss_at_last_step_start": final_loss, "rose_by_class": rose_by_class,
            "diagnosis": diagnosis, "flagged_after": int((flag != 0).sum().item())}


def diagnose_config5(A0, A1, ns, offsets, maxre0, maxre1, tau, lr, steps, worst: int = 10) -> dict:
    """The matrices whose max Re lambda rose most over the GD run: their largest eigenvalue
    condition number (LAPACK zgeevx on the initial matrix); the same `steps` GD steps repeated on
    the CPU with torch.linalg.eigvals (FP64) and autograd, per matrix (the loss is a sum over
    matrices, so each matrix's trajectory is independent), once from the same start and once from
    a start perturbed by 1e-14 relative (the trajectory's sensitivity to rounding); and the CPU's
    max Re lambda of the GPU's final matrix (the forward at the end point)."""
    import numpy as np
    import torch

    from oracle import lapack_oracle as lo

    def run_cpu(M):
        X = torch.from_numpy(M.copy()).requires_grad_(True)
        for _ in range(steps):
            lam = torch.linalg.eigvals(X)
            loss = tau * torch.logsumexp(lam.real / tau, 0)
            (g,) = torch.autograd.grad(loss, X)
            with torch.no_grad():
                X -= lr * g
        X = X.detach()
        return X.numpy(), float(torch.linalg.eigvals(X).real.max())

    rng = np.random.default_rng(5)
    rise = (maxre1 - maxre0).cpu().numpy()
    idx = np.argsort(-rise)[:worst]
    out = []
    for j in idx:
        k = int(ns[j])
        o = int(offsets[j])
        M0 = A0[o:o + k * k].cpu().numpy().reshape(k, k)  # the column-major buffer read row-major: A^T
        _, rc, _ = lo.zgeevx_rconde(M0[None])
        X, cpu_final = run_cpu(M0)
        pert = M0 + 1e-14 * np.linalg.norm(M0) / k * (rng.standard_normal(M0.shape) + 1j * rng.standard_normal(M0.shape))
        Xp, cpu_pert_final = run_cpu(pert)
        gpu_final_A = A1[o:o + k * k].cpu().numpy().reshape(k, k)
        nrm = np.linalg.norm(gpu_final_A)
        out.append({"n": k, "max_re_lambda_before": float(maxre0[j]), "max_re_lambda_after_gpu": float(maxre1[j]),
                    "cpu_max_re_lambda_of_gpu_final_matrix": float(np.linalg.eigvals(gpu_final_A).real.max()),
                    "max_re_lambda_after_cpu": cpu_final, "max_re_lambda_after_cpu_perturbed_1e-14": cpu_pert_final,
                    "max_eig_condition": float(1.0 / max(float(np.min(rc)), 1e-300)),
                    "rel_diff_final_matrix_gpu_vs_cpu": float(np.linalg.norm(gpu_final_A - X) / nrm),
                    "rel_diff_final_matrix_cpu_vs_cpu_perturbed": float(np.linalg.norm(Xp - X) / nrm)})
    rises = np.array([d["max_re_lambda_after_gpu"] - d["max_re_lambda_before"] for d in out])
    cpu_rises = np.array([d["max_re_lambda_after_cpu"] - d["max_re_lambda_before"] for d in out])
    fwd_ok = all(abs(d["cpu_max_re_lambda_of_gpu_final_matrix"] - d["max_re_lambda_after_gpu"]) <= 1e-8 * max(
        1.0, abs(d["max_re_lambda_after_gpu"])) for d in out)
    return {"worst": out, "cpu_reproduces_rise": bool(np.all((cpu_rises > 0) == (rises > 0))),
            "gpu_forward_matches_cpu_at_final_matrices": bool(fwd_ok),
            "median_rel_diff_gpu_vs_cpu": float(np.median([d["rel_diff_final_matrix_gpu_vs_cpu"] for d in out])),
            "median_rel_diff_cpu_vs_perturbed_cpu": float(np.median(
                [d["rel_diff_final_matrix_cpu_vs_cpu_perturbed"] for d in out])),
            "method": f"{worst} largest rises; CPU: torch.linalg.eigvals FP64 + autograd, {steps} steps, lr {lr}; "
                      f"a rounding-size (1e-14) perturbation of the start tests the trajectory's sensitivity"}


def measure_ragged(h, dev, stream, peak, batch: int = 200000) -> dict:
    """Ragged configuration: 200,000 complex Gaussian matrices, n ~ U{1..64} (seeded).

    The same matrices are solved (a) by one ragged call (persistent launch,
    replayed from a CUDA graph) and (b) by per-size plain launches on the same
    data grouped by n. Matrices sit in one buffer grouped by n; the ragged call
    sees them in the random order of their sizes through its offsets array.
    """
    import numpy as np
    import torch

    from tokura_zgeev_batched_gb300 import api, workloads

    ns = workloads.ragged_sizes(batch, 1, 64, seed=SEED + 3)
    order = np.argsort(ns, kind="stable")
    sizes_sorted = ns[order].astype(np.int64) ** 2
    start_sorted = np.concatenate([[0], np.cumsum(sizes_sorted)[:-1]])
    offsets = np.empty(batch, np.int64)
    offsets[order] = start_sorted
    total = int(sizes_sorted.sum())
    g = torch.Generator(device=dev)
    g.manual_seed(SEED + 4)
    A = torch.complex(torch.randn(total, generator=g, device=dev, dtype=torch.float64),
                      torch.randn(total, generator=g, device=dev, dtype=torch.float64))
    n_d = torch.from_numpy(ns).to(dev)
    o_d = torch.from_numpy(offsets).to(dev)
    total_eig = int(ns.sum())
    eig = torch.empty(total_eig, dtype=torch.complex128, device=dev)
    flag = torch.empty(batch, dtype=torch.int8, device=dev)
    work = torch.empty(api.tokura_get_zgeev_ragged_workspacesize(batch, total), dtype=torch.uint8, device=dev)
    s = stream.cuda_stream

    def ragged_call():
        st = api.tokura_zgeev_ragged_gpu(h, batch, n_d.data_ptr(), o_d.data_ptr(), None, total, A.data_ptr(),
                                         eig.data_ptr(), work.data_ptr(), flag.data_ptr(), s)
        assert st == 0

    ms_ragged = time_ms(ragged_call, 3, stream)
    flagged = int((flag != 0).sum().item())
    # Parity at full scale: LAPACK on every matrix (flags), matched errors on a seeded subset.
    from oracle import lapack_oracle as lo

    eoffs = np.concatenate([[0], np.cumsum(ns.astype(np.int64))[:-1]])
    t_chk = time.perf_counter()
    rep = lo.ragged_batch_parity(A.cpu().numpy(), ns, offsets, eig.cpu().numpy(), eoffs, flag.cpu().numpy(),
                                 subset=CHECK_SUBSET, seed=SEED + 3, full_flags=CHECK_FULL_FLAGS)
    parity = _parity_fields(rep, time.perf_counter() - t_chk)
    # CUDA graph of the ragged call (planning kernels + persistent solver).
    graph_ms = None
    try:
        gs = torch.cuda.Stream(dev)
        gs.wait_stream(stream)
        cg = torch.cuda.CUDAGraph()
        with torch.cuda.graph(cg, stream=gs):
            st = api.tokura_zgeev_ragged_gpu(h, batch, n_d.data_ptr(), o_d.data_ptr(), None, total, A.data_ptr(),
                                             eig.data_ptr(), work.data_ptr(), flag.data_ptr(),
                                             torch.cuda.current_stream().cuda_stream)
            assert st == 0
        graph_ms = time_ms(cg.replay, 3, stream)
        del cg
    except RuntimeError as exc:  # pragma: no cover - reported, not fatal
        graph_ms = f"capture failed: {exc}"
    # Per-size plain launches on the same data (grouped by n).
    counts = np.bincount(ns, minlength=65)
    starts = {}
    pos = 0
    epos = 0
    for k in range(1, 65):
        starts[k] = (pos, epos)
        pos += int(counts[k]) * k * k
        epos += int(counts[k]) * k
    eig2 = torch.empty(total_eig, dtype=torch.complex128, device=dev)
    flag2 = torch.empty(batch, dtype=torch.int8, device=dev)
    wmax = max(api.tokura_get_zgeeveigenvaluesgetworspacesize(k, int(counts[k])) for k in range(1, 65) if counts[k])
    work2 = torch.empty(wmax, dtype=torch.uint8, device=dev)
    fbase = np.concatenate([[0], np.cumsum(counts[1:])])

    def per_size_calls():
        for k in range(1, 65):
            c = int(counts[k])
            if c == 0:
                continue
            p0, e0 = starts[k]
            st = api.tokura_zgeev_batched_gpu(h, k, c, A.data_ptr() + 16 * p0, eig2.data_ptr() + 16 * e0,
                                              work2.data_ptr(), flag2.data_ptr() + int(fbase[k - 1]), s)
            assert st == 0

    ms_plain = time_ms(per_size_calls, 2, stream)
    flag2_serial = flag2.clone()
    eig2_serial = eig2.clone()

    # The same 64 plain launches spread over CONC_STREAMS streams, each stream with its own
    # handle (so each has its own estimator stream) and its own workspace; sizes are dealt
    # largest work first to the stream with the least work so far.
    CONC_STREAMS = 8
    streams = [torch.cuda.Stream(dev) for _ in range(CONC_STREAMS)]
    handles = [api.Handle() for _ in range(CONC_STREAMS)]
    works = [torch.empty(wmax, dtype=torch.uint8, device=dev) for _ in range(CONC_STREAMS)]
    load = [0.0] * CONC_STREAMS
    plan = [[] for _ in range(CONC_STREAMS)]
    for k in sorted((k for k in range(1, 65) if counts[k]), key=lambda k: -float(counts[k]) * k ** 3):
        i = min(range(CONC_STREAMS), key=lambda i: load[i])
        plan[i].append(k)
        load[i] += float(counts[k]) * k ** 3

    def per_size_concurrent(hs):
        for i in range(CONC_STREAMS):
            streams[i].wait_stream(stream)
            for k in plan[i]:
                p0, e0 = starts[k]
                st = api.tokura_zgeev_batched_gpu(hs[i], k, int(counts[k]), A.data_ptr() + 16 * p0,
                                                  eig2.data_ptr() + 16 * e0, works[i].data_ptr(),
                                                  flag2.data_ptr() + int(fbase[k - 1]), streams[i].cuda_stream)
                assert st == 0
        for i in range(CONC_STREAMS):
            stream.wait_stream(streams[i])

    ms_conc_default = time_ms(lambda: per_size_concurrent(handles), 2, stream)
    conc_same = bool(torch.equal(flag2, flag2_serial) and torch.equal(eig2, eig2_serial))
    # The library's shapes assume a launch has the GPU to itself and widen small batches to up to
    # 32 lanes per matrix; eight launches sharing the GPU do better with at most 4 lanes. The
    # stronger of the two concurrent variants is the comparator.
    want = torch.cuda.get_device_properties(dev).multi_processor_count * 4 * 2 * 32
    capped = [api.Handle() for _ in range(CONC_STREAMS)]
    for i in range(CONC_STREAMS):
        for k in plan[i]:
            c = int(counts[k])
            lanes = 1 if (k <= 2 or c >= want) else (2 if 2 * c >= want else 4)
            assert capped[i].set_plain_config(k, lanes, 32) == 0
    ms_conc_capped = time_ms(lambda: per_size_concurrent(capped), 2, stream)
    capped_flags_same = bool(torch.equal(flag2, flag2_serial))
    ms_conc = min(ms_conc_default, ms_conc_capped)
    del works, handles, capped
    work_flops = float(np.sum(40.0 * ns.astype(np.float64) ** 3))
    best = graph_ms if isinstance(graph_ms, float) else ms_ragged
    return {"batch": batch, "total_elements": total, "ms_ragged": ms_ragged, "ms_ragged_graph": graph_ms,
            "ms_per_size_plain": ms_plain, "matrices_per_s_ragged": batch / (best * 1e-3),
            "matrices_per_s_per_size_plain": batch / (ms_plain * 1e-3), "speedup_vs_per_size": ms_plain / best,
            "ms_per_size_plain_concurrent": ms_conc, "speedup_vs_per_size_concurrent": ms_conc / best,
            "per_size_concurrent": f"the 64 plain launches over {CONC_STREAMS} streams, one handle and one "
                                   f"workspace each, sizes dealt largest work first to the least-loaded stream; "
                                   f"the faster of the library's launch shapes ({ms_conc_default:.1f} ms, results "
                                   f"bitwise equal to the serial launches: {conc_same}) and at most 4 lanes per "
                                   f"matrix ({ms_conc_capped:.1f} ms, flags equal: {capped_flags_same})",
            "fp64_frac": work_flops / (best * 1e-3) / peak, "flagged": flagged,
            "plain_launches": int(np.count_nonzero(counts)), "parity": parity,
            "shift_hints": "FP32 estimates for orders >= 48 (the default); the per-size plain launches use them "
                           "for n >= 12"}

def measure_reference_gpu(h, dev, stream, peak) -> dict:
    """The reference library itself (tokura_zgeev_batched_library, unmodified, built for sm_103a
    with the three host functions it declares but never defines restated in
    oracle/ref_gpu_glue.cu) beside this library, on the same device-resident inputs.

    Its kernels keep block barriers in control flow that diverges between the 32 matrices of a
    thread block, so they run only on batches where each block of 32 consecutive matrices holds
    copies of one matrix, and only on matrices that the CPU restatement of its algorithm
    converges (oracle/ref_gpu.py). Such batches flatter both libraries a little (no divergence
    between the matrices of a warp); configuration 1 and the main workload are this library's
    figures on distinct matrices. Orders 32 (313 x 32 = 10,016 matrices, configuration 1's size)
    and 64 (2,048 x 32 = 65,536, the main workload's size)."""
    import numpy as np
    import torch

    from oracle import lapack_oracle as lo
    from oracle import ref_gpu
    from tokura_zgeev_batched_gb300 import api, workloads

    if not os.path.exists(ref_gpu.LIB_PATH):
        return {"unavailable": "reference library not built (its sources were not staged with the tree)"}
    out = {"method": "each thread block of the reference = 32 copies of one seeded complex Gaussian matrix; "
                     "CUDA events around one tokura_zgeev_batched_gpu call of each library on the same device batch "
                     "(the reference overwrites A, so it is re-copied before its call, outside the timing)"}
    for n, d in ((32, 313), (64, 2048)):
        cand = workloads.gaussian(d + d // 8 + 8, n, seed=SEED + 60 + n)
        ok, passes = ref_gpu.safe_matrices(cand, 20)
        distinct = cand[ok[:d]]
        d = distinct.shape[0]
        ref_gpu.solve_uniform(distinct[:8], stream)  # warm-up (module load)
        # a quarter of the batch first: the full batch only if it is projected to take under a minute
        q = max(8, d // 4)
        _, _, ms_q = ref_gpu.solve_uniform(distinct[:q], stream)
        if ms_q * d / q > 60e3:
            distinct = distinct[:q]
            d = q
        eig_r, flag_r, ms_r = ref_gpu.solve_uniform(distinct, stream)
        batch = d * 32
        e = eig_r.view(d, 32, n)
        copies_identical = bool((e == e[:, :1]).all().item())
        f = flag_r.view(d, 32)
        rep = lo.batch_parity(distinct, e[:, 0].cpu().numpy(), f[:, 0].cpu().numpy(), subset=d)
        # this library on the same batch
        A = torch.from_numpy(distinct).to(dev).repeat_interleave(32, dim=0)
        eig = torch.empty(batch, n, dtype=torch.complex128, device=dev)
        flag = torch.empty(batch, dtype=torch.int8, device=dev)
        work = torch.empty(api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch), dtype=torch.uint8, device=dev)

        def ours():
            assert api.tokura_zgeev_batched_gpu(h, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(),
                                                flag.data_ptr(), stream.cuda_stream) == 0

        ms_o = time_ms(ours, 3, stream)
        rep_o = lo.batch_parity(distinct, eig.view(d, 32, n)[:, 0].cpu().numpy(),
                                flag.view(d, 32)[:, 0].cpu().numpy(), subset=d)
        out[str(n)] = {
            "batch": batch, "distinct_matrices": d,
            "cpu_restatement_passes_max": int(passes[ok[:d]].max()),
            "reference_ms": ms_r, "reference_matrices_per_s": batch / (ms_r * 1e-3),
            "reference_fp64_frac": flops_per_matrix(n) * batch / (ms_r * 1e-3) / peak,
            "reference_flagged": int((flag_r != 0).sum().item()), "reference_copies_identical": copies_identical,
            "reference_parity": {"max_rel_err_fro": rep["max_rel_err"], "p99_rel_err_fro": rep["p99_rel_err"],
                                 "max_rel_err_fro_cond_le_1e3": rep["max_rel_err_well"],
                                 "flag_mismatch": rep["flag_mismatch"], "checked": rep["checked"]},
            "ours_ms": ms_o, "ours_matrices_per_s": batch / (ms_o * 1e-3),
            "ours_parity": {"max_rel_err_fro": rep_o["max_rel_err"], "flag_mismatch": rep_o["flag_mismatch"]},
            "speedup_ours_vs_reference": ms_r / ms_o,
        }
        del A, eig, flag, work, eig_r, flag_r
        torch.cuda.empty_cache()
    return out


def run_ours(args):
    import numpy as np
    import torch

    from tokura_zgeev_batched_gb300 import api, build, workloads

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    if rank == 0:
        build.build()
    if dist is not None:
        dist.barrier()
    api.lib()

    def barrier():
        if dist is not None:
            dist.barrier()

    peak = api.probe_fp64_peak(dev)
    h = api.Handle()
    if args.lanes:  # profiling cases: the full-size launch shape on a smaller batch
        assert h.set_plain_config(N, args.lanes, 32) == 0
    stream = torch.cuda.current_stream(dev)
    s = stream.cuda_stream

    def alloc(n, batch, gen="gaussian", seed=SEED):
        A = workloads.TORCH_GENERATORS[gen](batch, n, seed=rank_seed(seed, rank), device=str(dev))
        eig = torch.empty(batch, n, dtype=torch.complex128, device=dev)
        flag = torch.empty(batch, dtype=torch.int8, device=dev)
        work = torch.empty(api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch), dtype=torch.uint8, device=dev)
        return A, eig, flag, work

    def call(n, batch, A, eig, flag, work):
        st = api.tokura_zgeev_batched_gpu(h, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(),
                                          flag.data_ptr(), s)
        if st != 0:
            raise RuntimeError(f"tokura_zgeev_batched_gpu returned {st}")

    # ---- main workload: n = 64, 4 GiB
    A, eig, flag, work = alloc(N, BATCH)
    for _ in range(args.warmup):
        call(N, BATCH, A, eig, flag, work)
    torch.cuda.synchronize()
    sampler = ClockSampler(gpu_uuid(dev))
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    barrier()
    torch.cuda.synchronize()
    t0 = torch.cuda.Event(enable_timing=True)
    t1 = torch.cuda.Event(enable_timing=True)
    t0.record(stream)
    for k in range(args.steps):
        ev[k][0].record(stream)
        call(N, BATCH, A, eig, flag, work)
        ev[k][1].record(stream)
    t1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = sampler.stop()
    ms_total = max_over_ranks(t0.elapsed_time(t1), dist, dev)
    kern_ms = [a.elapsed_time(b) for a, b in ev]
    ms_step = ms_total / args.steps
    value = ws * BATCH / (ms_step * 1e-3)
    flagged = int((flag != 0).sum().item())

    phase("main timed region done")
    # Config 3 (ragged) next, while the process state matches a fresh run.
    ragged = None
    if not args.no_ragged:
        # The main buffers stay allocated; the ragged batch needs ~9 GB more.
        ragged = guarded(lambda: measure_ragged(h, dev, stream, peak))
        phase("ragged done")

    # Parity spot check of the timed output against LAPACK (rank 0, outside timing).
    parity = None
    if rank == 0 and not args.no_check:
        parity = scale_check(A, eig, flag, seed=SEED)

    kern_avg = statistics.mean(kern_ms)
    achieved = flops_per_matrix(N) * BATCH / (kern_avg * 1e-3)
    # DRAM bytes of one call: the per-matrix traffic of an ncu capture (profiles/traffic.json)
    # times this batch; the capture's conditions and the scaling are stated there.
    prof = read_profile_traffic()
    traffic = traffic_note = None
    if prof and prof.get("n") == N and prof.get("dram_bytes_per_matrix"):
        traffic = prof["dram_bytes_per_matrix"] * BATCH
        traffic_note = prof.get("scaling")
    roofline = {
        "bound": "fp64", "achieved": achieved / 1e12, "peak": peak / 1e12, "unit": "TFLOP/s",
        "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_note,
        "peak_source": "FP64 FMA-loop probe run in this process (MEASURED_PEAKS.json has no FP64 figure)",
        "algorithmic": f"40*n^3 flops and 16*n^2+16*n+1 bytes per matrix x {BATCH} matrices per launch",
        "kernel_ms_avg": kern_avg,
    }
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            hbm_peak = json.load(f).get("hbm_gbs")
    except (OSError, ValueError):
        hbm_peak = None
    alg_gbs = bytes_per_matrix(N) * BATCH / (kern_avg * 1e-3) / 1e9
    roofline["hbm"] = {"achieved": alg_gbs, "peak": hbm_peak, "unit": "GB/s",
                       "frac": (alg_gbs / hbm_peak) if hbm_peak else None}

    phase("parity spot check done")
    # ---- end to end: host buffers through the public API, copies inside every step.
    # tokura_zgeev_batched_host takes host pointers, pipelines chunked H2D copies,
    # solves and D2H copies over the handle's streams and returns when the
    # eigenvalues and flags are in host memory (wall-clock timed). The same
    # steps on one stream without chunking (copy in, solve, copy out, wait)
    # are reported as "single_stream".
    e2e = None
    if not args.no_e2e:
        # Pinned host buffers from the library's allocator (tokuraHostAlloc: huge pages, so the
        # host link keeps its full rate after the idle gaps between steps); torch's pinned memory
        # if that allocator fails.
        try:
            A_host = api.host_empty(A.shape, A.dtype)
            eig_host = api.host_empty(eig.shape, eig.dtype)
            flag_host = api.host_empty(flag.shape, flag.dtype)
            host_buffers = "tokuraHostAlloc (pinned, huge pages)"
        except RuntimeError as exc:
            A_host = torch.empty(A.shape, dtype=A.dtype, pin_memory=True)
            eig_host = torch.empty(eig.shape, dtype=eig.dtype, pin_memory=True)
            flag_host = torch.empty(flag.shape, dtype=flag.dtype, pin_memory=True)
            host_buffers = f"torch pinned memory ({exc})"
        A_host.copy_(A)
        torch.cuda.synchronize()

        def huge_page_share(t) -> float | None:
            """Share of a host tensor's mapping backed by transparent huge pages (/proc/self/smaps);
            without them the host link's rate after idle periods depends on the box."""
            addr, inside, size, huge = t.data_ptr(), False, 0, 0
            try:
                with open("/proc/self/smaps") as f:
                    for line in f:
                        head = line.split(None, 1)[0]
                        if "-" in head and not head.endswith(":"):
                            lo, hi = (int(x, 16) for x in head.split("-"))
                            inside = lo <= addr < hi
                        elif inside and head == "Size:":
                            size = int(line.split()[1])
                        elif inside and head == "AnonHugePages:":
                            huge = int(line.split()[1])
            except (OSError, ValueError):
                return None
            return huge / size if size else None

        host_huge = huge_page_share(A_host)

        def h2d_rate():
            """The host link's rate now (one pinned copy of the whole input), GB/s."""
            c0 = torch.cuda.Event(enable_timing=True)
            c1 = torch.cuda.Event(enable_timing=True)
            c0.record(stream)
            A.copy_(A_host, non_blocking=True)
            c1.record(stream)
            torch.cuda.synchronize()
            return A_host.numel() * 16 / (c0.elapsed_time(c1) * 1e6)

        h2d_start = h2d_rate()

        def host_call():
            st = api.tokura_zgeev_batched_host(h, N, BATCH, A_host.data_ptr(), eig_host.data_ptr(),
                                               flag_host.data_ptr(), 0)
            if st != 0:
                raise RuntimeError(f"tokura_zgeev_batched_host returned {st}")

        for _ in range(max(1, args.warmup)):
            host_call()
        barrier()
        t_start = time.perf_counter()
        for _ in range(args.steps):
            host_call()
        t_host = time.perf_counter() - t_start
        barrier()
        e_ms = max_over_ranks(1e3 * t_host / args.steps, dist, dev)
        host_flagged = int((flag_host != 0).sum().item())

        def e2e_step():
            # One caller-side step on one stream, waiting for its results like the host-buffer call
            # does (five steps queued back to back without a wait made later copies from this
            # memory slow, 5-7 GB/s instead of 211, on the boxes measured; cause unknown).
            A.copy_(A_host, non_blocking=True)
            call(N, BATCH, A, eig, flag, work)
            eig_host.copy_(eig, non_blocking=True)
            flag_host.copy_(flag, non_blocking=True)
            torch.cuda.synchronize()

        e2e_step()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(max(1, args.steps // 2)):
            e2e_step()
        e1.record(stream)
        torch.cuda.synchronize()
        single_ms = max_over_ranks(e0.elapsed_time(e1) / max(1, args.steps // 2), dist, dev)
        # The host link's rate on this machine before and after the steps: it sets how much of the
        # copy the chunked host-buffer call can hide.
        h2d_gbs = {"start": h2d_start, "end": h2d_rate()}
        e2e = {"value": ws * BATCH / (e_ms * 1e-3), "unit": "matrices/s",
               "h2d_bytes_per_step": A_host.numel() * 16,
               "d2h_bytes_per_step": eig_host.numel() * 16 + flag_host.numel(),
               "ms_per_step": e_ms,
               "api": "tokura_zgeev_batched_host (pinned host buffers, wall clock)", "host_buffers": host_buffers,
               "flagged": host_flagged,
               "single_stream": {"value": ws * BATCH / (single_ms * 1e-3), "ms_per_step": single_ms},
               "h2d_gbs": h2d_gbs, "host_input_huge_page_share": host_huge}
        del A_host, eig_host, flag_host
    del A, eig, flag, work
    torch.cuda.empty_cache()

    phase("e2e done")
    # ---- size sweep (the other orders of the 4 GiB size-sweep configuration)
    def run_sweep():
        sweep = {}
        for cls in ("gaussian", "vdv", "companion"):
            res = {}
            for n in SWEEP_NS + (N,):
                if cls == "gaussian" and n == N:
                    res[str(n)] = {"batch": BATCH, "matrices_per_s": value / ws, "fp64_frac": achieved / peak,
                                   "flagged": flagged, "parity": parity}
                    continue
                batch = (4 << 30) // (16 * n * n)
                A, eig, flag, work = alloc(n, batch, gen=cls, seed=SEED + 17 * n)
                ms = time_ms(lambda: call(n, batch, A, eig, flag, work), 2, stream)
                rate = batch / (ms * 1e-3)
                res[str(n)] = {"batch": batch, "matrices_per_s": rate,
                               "fp64_frac": flops_per_matrix(n) * rate / peak,
                               "flagged": int((flag != 0).sum().item())}
                if rank == 0 and not args.no_check:
                    res[str(n)]["parity"] = scale_check(A, eig, flag, seed=SEED + 17 * n)
                del A, eig, flag, work
                torch.cuda.empty_cache()
            sweep[cls] = res
        return sweep

    sweep = {}
    config1 = None
    if not args.no_sweep:
        sweep = guarded(run_sweep)
        torch.cuda.empty_cache()
        config1 = guarded(lambda: measure_config1(h, dev, stream, peak, call))
    phase("sweep and config 1 done")
    config4 = config5 = None
    if not args.no_grad:
        config4 = guarded(lambda: measure_config4(h, dev, stream, peak))
        torch.cuda.empty_cache()
        phase("config 4 done")
        config5 = guarded(lambda: measure_config5(h, dev, stream, peak))
        phase("config 5 done")
    real = None
    if not args.no_real:
        real = guarded(lambda: measure_real(h, dev, stream, peak))
        torch.cuda.empty_cache()
        phase("real path done")
    vectors = None
    if not args.no_vectors:
        vectors = guarded(lambda: measure_vectors(h, dev, stream))
        torch.cuda.empty_cache()
        phase("eigenvectors done")

    reference_gpu = None
    if rank == 0 and not args.no_reference_gpu:
        reference_gpu = guarded(lambda: measure_reference_gpu(h, dev, stream, peak))
        torch.cuda.empty_cache()
        phase("reference library on the GPU done")

    cpu = None
    if rank == 0 and not args.no_cpu:
        cpu = guarded(lambda: cpu_baseline(N))

    if rank == 0:
        out = {
            "metric": METRIC, "value": value, "unit": "matrices/s", "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_step, "ms_per_step_median": statistics.median(kern_ms),
            "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128 (f64)", "data": "synthetic",
            "config": {"workload": f"plain zgeev eigenvalues (tokura_zgeev_batched_gpu), n={N}, {BATCH} complex "
                                   f"Gaussian matrices per GPU ({16 * N * N * BATCH / 2 ** 30:.2f} GiB), seed {SEED}",
                       "n": N, "global_batch": ws * BATCH,
                       "l2": f"inputs ({16 * N * N * BATCH / 2 ** 20:.0f} MiB) "
                             f"{'larger' if 16 * N * N * BATCH > 129 * 2 ** 20 else 'smaller'} than L2 (129 MB)",
                       "lanes_per_matrix": h.plain_config(N, BATCH)[0],
                       "shift_hints": "FP32 estimator on a second stream beside the FP64 Hessenberg kernel, then "
                                      "the FP64 QR kernel" if N >= SHIFT_HINT_MIN_N else "off (n < 12)"},
            "roofline": roofline, "cpu_baseline": cpu, "e2e": e2e, "clocks": clocks,
            "gpu_launches": args.steps * (3 if N >= SHIFT_HINT_MIN_N else 1), "flagged": flagged, "parity": parity, "sweep": sweep,
            "config1_n32_10000": config1, "ragged": ragged, "config4_backward": config4,
            "config5_ragged_gd_graph": config5, "real_dgeev_n64": real, "eigenvectors_n64": vectors,
            "reference_gpu": reference_gpu,
        }
        print(json.dumps(out), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def run_only(args):
    """One configuration alone, for small profiling captures (prints its JSON object)."""
    import torch

    from tokura_zgeev_batched_gb300 import api, build

    build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    peak = api.probe_fp64_peak(dev)
    h = api.Handle()
    stream = torch.cuda.current_stream(dev)
    if args.only == "ragged":
        out = measure_ragged(h, dev, stream, peak, batch=args.batch or 200000)
    elif args.only == "real":
        out = measure_real(h, dev, stream, peak, n=args.n, batch=args.batch or 65536, cpu_seconds=0.5)
    elif args.only == "vectors":
        out = measure_vectors(h, dev, stream, n=args.n, batch=args.batch or 65536, cpu_seconds=0.5)
    elif args.only == "config1":
        def call(n, batch, A, eig, flag, work):
            st = api.tokura_zgeev_batched_gpu(h, n, batch, A.data_ptr(), eig.data_ptr(), work.data_ptr(),
                                              flag.data_ptr(), stream.cuda_stream)
            if st != 0:
                raise RuntimeError(f"tokura_zgeev_batched_gpu returned {st}")

        out = measure_config1(h, dev, stream, peak, call)
    elif args.only == "reference_gpu":
        out = measure_reference_gpu(h, dev, stream, peak)
    else:
        out = measure_config4(h, dev, stream, peak, batch=args.batch or 50000, orders=(args.n,))
    print(json.dumps({"only": args.only, "result": out}), flush=True)


def main():
    global CHECK_SUBSET, CHECK_FULL_FLAGS
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-sweep", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-check", action="store_true")
    ap.add_argument("--no-ragged", action="store_true")
    ap.add_argument("--no-grad", action="store_true")
    ap.add_argument("--no-real", action="store_true")
    ap.add_argument("--no-vectors", action="store_true")
    ap.add_argument("--no-reference-gpu", action="store_true")
    ap.add_argument("--only", choices=["ragged", "backward", "real", "vectors", "config1", "reference_gpu"],
                    default=None,
                    help="run one configuration alone (profiling cases); --batch sets its size")
    ap.add_argument("--n", type=int, default=N, help="matrix order of the timed workload (profiling cases)")
    ap.add_argument("--batch", type=int, default=0, help="matrices per GPU (default: 4 GiB of input)")
    ap.add_argument("--lanes", type=int, default=0, choices=[0, 1, 2, 4, 8],
                    help="lanes per matrix of the timed workload (profiling cases; 0 = the library's choice)")
    ap.add_argument("--check-subset", type=int, default=CHECK_SUBSET,
                    help="matrices per configuration whose eigenvalues are matched against LAPACK")
    ap.add_argument("--check-flags", choices=["all", "subset"], default="all",
                    help="LAPACK on every matrix of each batch for flag parity, or on the subset only")
    args = ap.parse_args()
    set_workload(args.n, args.batch)
    CHECK_SUBSET = args.check_subset
    CHECK_FULL_FLAGS = args.check_flags == "all"
    if args.impl == "reference":
        run_reference(args)
    elif args.only is not None:
        run_only(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
