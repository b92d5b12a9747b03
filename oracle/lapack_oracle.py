"""TEST INFRASTRUCTURE — parity oracle for batched eigenvalue-only ZGEEV.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg may use this module; the product never does.

Oracle = LAPACK zgeev with JOBVL = JOBVR = 'N' in FP64, the routine the
reference compares against (stream_test_with_MKL/get_eig_MKL.c:33-46 calls
MKL's LAPACKE_zgeev(LAPACK_COL_MAJOR, 'N', 'N', ...)). MKL is an un-vendored,
unpinned dependency of the reference and is absent here; the same published
LAPACK routine is taken from the OpenBLAS 0.3.34 LAPACK bundled with scipy
1.18.1 (symbols ``scipy_LAPACKE_zgeev`` / ``scipy_LAPACKE_zgeevx``), driven
from the small C harness ``oracle/cpu_zgeev.c``. That harness also serves as
the timed CPU baseline (one zgeev per matrix, threads over the batch, as
get_eig_MKL.c:26-51 does with OpenMP).

The parity metric replaces the reference's sort-based relative error
(stream_test_with_MKL/main.cu:16-181): eigenvalues are matched per matrix by
an optimal assignment (Hungarian method) and the error is
max |lambda - lambda_LAPACK| / ||A||_F, checked against 1e-11 on matrices whose
eigenvalue condition numbers (1/RCONDE from zgeevx, no balancing) are <= 1e3.
"""
from __future__ import annotations

import ctypes
import glob
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD_DIR = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD_DIR, "libcpu_zgeev.so")
SRC = os.path.join(HERE, "cpu_zgeev.c")
REF_SRC = os.path.join(HERE, "ref_algorithm.c")
MODEL_SRC = os.path.join(HERE, "model_qr.c")

TOL_REL_FRO = 1e-11
COND_MAX = 1e3

_lib = None


def find_lapack() -> str:
    """Path of the LAPACK shared library bundled with scipy (LP64 OpenBLAS)."""
    import scipy

    root = os.path.dirname(os.path.dirname(scipy.__file__))
    cands = sorted(glob.glob(os.path.join(root, "scipy.libs", "libscipy_openblas*.so*")))
    if not cands:
        raise RuntimeError("scipy's bundled OpenBLAS (scipy.libs/libscipy_openblas*.so) not found")
    return cands[0]


def build(force: bool = False) -> str:
    """Compiles the C harness with gcc (plain C, no vendored sources)."""
    newest = max(os.path.getmtime(SRC), os.path.getmtime(REF_SRC), os.path.getmtime(MODEL_SRC))
    if not force and os.path.exists(LIB_PATH) and os.path.getmtime(LIB_PATH) >= newest:
        return LIB_PATH
    os.makedirs(BUILD_DIR, exist_ok=True)
    tmp = LIB_PATH + ".tmp"
    # -ffp-contract=off: the restatement rounds each operation as written.
    cmd = ["gcc", "-O2", "-std=c11", "-ffp-contract=off", "-shared", "-fPIC", "-o", tmp, SRC, REF_SRC, MODEL_SRC,
           "-ldl", "-lpthread", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


def _load():
    global _lib
    if _lib is None:
        build()
        lib = ctypes.CDLL(LIB_PATH)
        lib.cpu_zgeev_open.argtypes = [ctypes.c_char_p]
        lib.cpu_zgeev_batched.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.cpu_zgeevx_batched.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int,
                                           ctypes.POINTER(ctypes.c_double)]
        lib.cpu_zgeev_vectors_batched.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5 + [
            ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.cpu_dgeev_batched.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4 + [
            ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.ref_zgeev_batched.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p]
        lib.ref_zgeev_batched_sweeps.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4
        lib.model_zgeev_batched.argtypes = [ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 5
        lib.model_zgeev_batched_opts.argtypes = ([ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 4
                                                 + [ctypes.c_double] + [ctypes.c_void_p] * 3 + [ctypes.c_int]
                                                 + [ctypes.c_void_p, ctypes.c_long, ctypes.c_void_p])
        lib.model_estimates_batched.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_float, ctypes.c_void_p]
        st = lib.cpu_zgeev_open(find_lapack().encode())
        if st != 0:
            raise RuntimeError(f"cannot open LAPACK ({st})")
        _lib = lib
    return _lib


def default_threads() -> int:
    return max(1, len(os.sched_getaffinity(0)))


def _as_batch(A: np.ndarray) -> np.ndarray:
    A = np.ascontiguousarray(A, dtype=np.complex128)
    if A.ndim == 2:
        A = A[None]
    return A


def zgeev(A: np.ndarray, threads: int | None = None):
    """LAPACK zgeev('N','N') per matrix.

    ``A[k]`` is read as the column-major buffer of matrix k, i.e. the
    eigenvalues returned are those of ``A[k].T`` — identical to those of
    ``A[k]``. Returns ``(w[batch, n], info[batch], seconds)``.
    """
    lib = _load()
    A = _as_batch(A)
    b, n, _ = A.shape
    w = np.empty((b, n), np.complex128)
    info = np.empty(b, np.int32)
    sec = ctypes.c_double()
    lib.cpu_zgeev_batched(n, b, A.ctypes.data, w.ctypes.data, info.ctypes.data, threads or default_threads(),
                          ctypes.byref(sec))
    return w, info, sec.value


def dgeev(A: np.ndarray, threads: int | None = None):
    """LAPACK dgeev('N','N') per real matrix (``A[k]`` read as a column-major
    buffer). Returns ``(wr[batch, n], wi[batch, n], info[batch], seconds)``."""
    lib = _load()
    A = np.ascontiguousarray(A, dtype=np.float64)
    if A.ndim == 2:
        A = A[None]
    b, n, _ = A.shape
    wr = np.empty((b, n), np.float64)
    wi = np.empty((b, n), np.float64)
    info = np.empty(b, np.int32)
    sec = ctypes.c_double()
    lib.cpu_dgeev_batched(n, b, A.ctypes.data, wr.ctypes.data, wi.ctypes.data, info.ctypes.data,
                          threads or default_threads(), ctypes.byref(sec))
    return wr, wi, info, sec.value


def check_conjugate_pairs(wr: np.ndarray, wi: np.ndarray) -> bool:
    """LAPACK's real-eigenvalue output convention: wi[k] > 0 starts a pair
    with (wr[k+1], wi[k+1]) == (wr[k], -wi[k]) exactly; any other entry has
    wi == 0."""
    n = wr.shape[-1]
    for r, im in zip(wr.reshape(-1, n), wi.reshape(-1, n)):
        k = 0
        while k < n:
            if im[k] == 0.0:
                k += 1
            elif im[k] > 0.0 and k + 1 < n and r[k + 1] == r[k] and im[k + 1] == -im[k]:
                k += 2
            else:
                return False
    return True


def zgeev_vectors(A: np.ndarray, threads: int | None = None):
    """zgeev('V','V'): ``(w, VL, VR, info)``; VL/VR ``[batch, n, n]`` with column i (``VR[k][:, i]``)
    the eigenvector of ``w[k, i]`` for the column-major reading of ``A[k]``."""
    lib = _load()
    A = _as_batch(A)
    b, n, _ = A.shape
    w = np.empty((b, n), np.complex128)
    vl = np.empty((b, n, n), np.complex128)
    vr = np.empty((b, n, n), np.complex128)
    info = np.empty(b, np.int32)
    sec = ctypes.c_double()
    lib.cpu_zgeev_vectors_batched(n, b, A.ctypes.data, w.ctypes.data, vl.ctypes.data, vr.ctypes.data,
                                  info.ctypes.data, threads or default_threads(), ctypes.byref(sec))
    # Buffers are column-major: element (r, c) of matrix k sits at [k, c, r] of the array.
    return w, vl.transpose(0, 2, 1), vr.transpose(0, 2, 1), info


def zgeevx_rconde(A: np.ndarray, threads: int | None = None):
    """zgeevx(BALANC='N', SENSE='E'): ``(w, rconde, info)`` per matrix."""
    lib = _load()
    A = _as_batch(A)
    b, n, _ = A.shape
    w = np.empty((b, n), np.complex128)
    rc = np.empty((b, n), np.float64)
    info = np.empty(b, np.int32)
    sec = ctypes.c_double()
    lib.cpu_zgeevx_batched(n, b, A.ctypes.data, w.ctypes.data, rc.ctypes.data, info.ctypes.data,
                           threads or default_threads(), ctypes.byref(sec))
    return w, rc, info


def reference_algorithm(A: np.ndarray, return_sweeps: bool = False):
    """The reference's own GPU algorithm restated serially in C (oracle/ref_algorithm.c).

    Returns ``(w[batch, n], flag[batch])``; flag 1 means its n^4 sweep cap was hit. With
    ``return_sweeps`` also the passes of its sweep loop per matrix.
    """
    lib = _load()
    A = _as_batch(A)
    b, n, _ = A.shape
    w = np.empty((b, n), np.complex128)
    flag = np.empty(b, np.int32)
    sweeps = np.empty(b, np.int64)
    lib.ref_zgeev_batched_sweeps(n, b, A.ctypes.data, w.ctypes.data, flag.ctypes.data, sweeps.ctypes.data)
    return (w, flag, sweeps) if return_sweeps else (w, flag)


def model_qr(A: np.ndarray, est: np.ndarray | None = None):
    """CPU model of this library's own iteration (oracle/model_qr.c): Householder
    Hessenberg, then single-shift QR with Ahues-Tisseur deflation, Wilkinson and ad hoc
    shifts and, given ``est`` (complex64 ``[batch, n]``), the nearest unused estimate as
    the first shift after each deflation. Returns ``(w, flag, sweeps)`` per matrix."""
    lib = _load()
    A = _as_batch(A)
    b, n, _ = A.shape
    w = np.empty((b, n), np.complex128)
    flag = np.empty(b, np.int32)
    sweeps = np.empty(b, np.int64)
    e = None
    if est is not None:
        e = np.ascontiguousarray(est, dtype=np.complex64).reshape(b, n)
    lib.model_zgeev_batched(n, b, A.ctypes.data, w.ctypes.data, None if e is None else e.ctypes.data,
                            flag.ctypes.data, sweeps.ctypes.data)
    return w, flag, sweeps


def model_qr_variant(A: np.ndarray, est: np.ndarray | None = None, start_row: bool = False,
                     estimate_twice: bool = False, lam: np.ndarray | None = None, tol: float = 2.0 ** -52,
                     trace: bool = False, scaled: bool = False, elementary: bool = False):
    """model_qr with variants: the two the library does not use (zlahqr's start-row search;
    the estimate as the shift of the second sweep too), and the gradient's Schur iteration
    (``lam``: FP64 eigenvalues as first shifts after each deflation, deflation at ``tol``).
    Returns ``(w, flag, sweeps, work)``, work = element-pair rotation updates per matrix, plus
    with ``trace`` a list of per-matrix arrays: the active window of every sweep (the first
    16n + 64 sweeps). ``scaled``: the same iteration with scaled rotations (row and column
    scale factors, two complex multiply-adds per element pair; n <= 64; not with ``lam``,
    ``start_row``, ``estimate_twice`` or ``trace``); then a fifth value, the rescales per
    matrix. ``elementary``: Hessenberg form by stabilized elementary similarity transforms
    (EISPACK comhes) instead of Householder reflectors."""
    lib = _load()
    A = _as_batch(A)
    b, n, _ = A.shape
    w = np.empty((b, n), np.complex128)
    flag = np.empty(b, np.int32)
    sweeps = np.empty(b, np.int64)
    work = np.empty(b, np.int64)
    e = None if est is None else np.ascontiguousarray(est, dtype=np.complex64).reshape(b, n)
    lm = None if lam is None else np.ascontiguousarray(lam, dtype=np.complex128).reshape(b, n)
    cap = 16 * n + 64 if trace else 0  # windows beyond 16 sweeps per eigenvalue on average are not kept
    tr = np.zeros((b, cap), np.int32) if trace else None
    if scaled and (n > 64 or lam is not None or start_row or estimate_twice or trace):
        raise ValueError("scaled rotations: n <= 64, without lam, start_row, estimate_twice or trace")
    resc = np.zeros(b, np.int64)
    lib.model_zgeev_batched_opts(n, b, A.ctypes.data, w.ctypes.data, None if e is None else e.ctypes.data,
                                 None if lm is None else lm.ctypes.data, float(tol),
                                 flag.ctypes.data, sweeps.ctypes.data, work.ctypes.data,
                                 int(start_row) | (2 if estimate_twice else 0) | (4 if scaled else 0)
                                 | (8 if elementary else 0),
                                 None if tr is None else tr.ctypes.data, cap, resc.ctypes.data)
    if scaled:
        return w, flag, sweeps, work, resc
    if trace:
        return w, flag, sweeps, work, [tr[j, :sweeps[j]] for j in range(b)]
    return w, flag, sweeps, work


def model_estimates(A: np.ndarray, tol: float = 1e-5, return_sweeps: bool = False):
    """CPU model of the FP32 estimator (oracle/model_qr.c): complex64 ``[batch, n]``
    estimates with deflation tolerance ``tol`` (the library uses 1e-5); with
    ``return_sweeps`` also the FP32 QR's sweeps per matrix."""
    lib = _load()
    A = _as_batch(A)
    b, n, _ = A.shape
    est = np.empty((b, n), np.complex64)
    sweeps = np.empty(b, np.int64)
    lib.model_estimates_batched(n, b, A.ctypes.data, est.ctypes.data, float(tol), sweeps.ctypes.data)
    return (est, sweeps) if return_sweeps else est


def _match_one(a: np.ndarray, b: np.ndarray) -> np.ndarray:
    """Per-eigenvalue |error| of one matrix (w_ref a, w_test b) after an optimal assignment."""
    from scipy.optimize import linear_sum_assignment

    d = np.abs(a[:, None] - b[None, :])
    if not np.all(np.isfinite(d)):
        return np.full(a.shape, np.inf)
    out = np.empty(a.shape, np.float64)
    r, c = linear_sum_assignment(d)
    out[r] = d[r, c]
    return out


def matched_abs_errors(w_test: np.ndarray, w_ref: np.ndarray, block: int = 1024) -> np.ndarray:
    """Per-eigenvalue |error| after optimal per-matrix matching; shape [batch, n], in w_ref's order.

    Vectorized over blocks of matrices: where every reference eigenvalue's nearest test
    eigenvalue is distinct (a permutation) and each such error is below a quarter of the
    distance to the second-nearest one, that permutation is the optimal assignment and is
    taken as is; any other matrix (or one with non-finite values) goes through the
    Hungarian method (scipy's linear_sum_assignment), matrix by matrix."""
    w_test = np.atleast_2d(np.asarray(w_test))
    w_ref = np.atleast_2d(np.asarray(w_ref))
    b, n = w_ref.shape
    out = np.empty((b, n), np.float64)
    for s0 in range(0, b, block):
        a = w_ref[s0:s0 + block]
        t = w_test[s0:s0 + block]
        m = a.shape[0]
        with np.errstate(invalid="ignore"):
            d = np.abs(a[:, :, None] - t[:, None, :])  # [m, n(ref), n(test)]
        fin = np.isfinite(d).all(axis=(1, 2))
        d = np.where(np.isfinite(d), d, np.inf)
        nn = np.argmin(d, axis=2)
        best = np.take_along_axis(d, nn[:, :, None], axis=2)[:, :, 0]
        if n > 1:
            perm = (np.diff(np.sort(nn, axis=1), axis=1) != 0).all(axis=1)
            second = np.partition(d, 1, axis=2)[:, :, 1]
            gap = (best * 4 < second).all(axis=1)
            good = fin & perm & gap
        else:
            good = fin
        out[s0:s0 + m][good] = best[good]
        for k in np.nonzero(~good)[0]:
            out[s0 + k] = _match_one(a[k], t[k]) if fin[k] else np.inf
    return out


def parity_report(A: np.ndarray, w_test: np.ndarray, flag_test: np.ndarray, threads: int | None = None,
                  with_cond: bool = True, w_ref: np.ndarray | None = None, info: np.ndarray | None = None) -> dict:
    """Compares eigenvalues/flags against LAPACK zgeev on the same inputs (``w_ref``/``info``:
    LAPACK's results when already computed for these matrices)."""
    A = _as_batch(A)
    if w_ref is None or info is None:
        w_ref, info, _ = zgeev(A, threads)
    fro = np.sqrt(np.sum(np.abs(A) ** 2, axis=(1, 2)))
    fro = np.where(fro == 0, 1.0, fro)
    ok = (info == 0) & (np.asarray(flag_test) == 0)
    err = np.full(w_ref.shape, np.nan)
    if ok.any():
        err[ok] = matched_abs_errors(np.asarray(w_test)[ok], w_ref[ok])
    rel = np.full(A.shape[0], np.nan)
    if ok.any():
        rel[ok] = np.max(err[ok], axis=1) / fro[ok]
    rep = {
        "batch": int(A.shape[0]),
        "flag_mismatch": int(np.sum((info != 0) != (np.asarray(flag_test) != 0))),
        "lapack_fail": int(np.sum(info != 0)),
        "max_rel_err": float(np.nanmax(rel)) if ok.any() else float("nan"),
        "p99_rel_err": float(np.nanpercentile(rel[ok], 99)) if ok.any() else float("nan"),
    }
    if with_cond:
        _, rc, _ = zgeevx_rconde(A, threads)
        cond = 1.0 / np.maximum(rc, 1e-300)
        well = ok & (np.max(cond, axis=1) <= COND_MAX)
        rep["well_conditioned"] = int(well.sum())
        rep["max_rel_err_well"] = float(np.nanmax(rel[well])) if well.any() else float("nan")
        rep["p99_rel_err_well"] = float(np.nanpercentile(rel[well], 99)) if well.any() else float("nan")
        rep["well"] = well
    rep["rel_err"] = rel
    return rep


def batch_parity(A: np.ndarray, w_test: np.ndarray, flag_test: np.ndarray, subset: int = 10000, seed: int = 0,
                 full_flags: bool = True, threads: int | None = None) -> dict:
    """Parity of a whole batch at its full size: LAPACK zgeev on every matrix for flag parity
    (``full_flags``; else on the subset only), and the matched eigenvalue error, with zgeevx
    condition numbers, on a seeded random subset of ``subset`` matrices (all of them when the
    batch is no larger). Returns the report of :func:`parity_report` on the subset (without
    ``rel_err``) plus ``flags_checked``, ``flag_mismatch`` / ``lapack_fail`` over those,
    ``gpu_flagged`` and ``checked``."""
    A = _as_batch(A)
    b = A.shape[0]
    flag_test = np.asarray(flag_test).reshape(b)
    w_test = np.asarray(w_test).reshape(b, -1)
    if b <= subset:
        pick = np.arange(b)
    else:
        pick = np.sort(np.random.default_rng(seed).choice(b, size=subset, replace=False))
    if full_flags:
        w_all, info_all, _ = zgeev(A, threads)
        w_ref, info = w_all[pick], info_all[pick]
        flags_checked = b
        mism = int(np.sum((info_all != 0) != (flag_test != 0)))
        fail = int(np.sum(info_all != 0))
    else:
        w_ref, info, _ = zgeev(A[pick], threads)
        flags_checked = len(pick)
        mism = int(np.sum((info != 0) != (flag_test[pick] != 0)))
        fail = int(np.sum(info != 0))
    rep = parity_report(A[pick], w_test[pick], flag_test[pick], threads, True, w_ref=w_ref, info=info)
    rep.pop("rel_err")
    rep.pop("well")
    rep.update({"checked": int(len(pick)), "flags_checked": int(flags_checked), "flag_mismatch": mism,
                "lapack_fail": fail, "gpu_flagged": int(np.count_nonzero(flag_test))})
    return rep


def ragged_batch_parity(A_flat: np.ndarray, ns: np.ndarray, offsets: np.ndarray, w_flat: np.ndarray,
                        eig_offsets: np.ndarray, flag_test: np.ndarray, subset: int = 10000, seed: int = 0,
                        full_flags: bool = True, threads: int | None = None) -> dict:
    """:func:`batch_parity` for a ragged batch: matrix j has order ``ns[j]`` and its column-major
    entries start at ``A_flat[offsets[j]]``; its eigenvalues at ``w_flat[eig_offsets[j]]``.
    LAPACK runs per order on every matrix (``full_flags``) or on the seeded subset only; the
    matched error (with zgeevx condition numbers) covers the subset."""
    A_flat = np.asarray(A_flat).reshape(-1)
    ns = np.asarray(ns).astype(np.int64)
    offsets = np.asarray(offsets).astype(np.int64)
    eig_offsets = np.asarray(eig_offsets).astype(np.int64)
    flag_test = np.asarray(flag_test).reshape(-1)
    w_flat = np.asarray(w_flat).reshape(-1)
    b = ns.shape[0]
    in_sub = np.zeros(b, bool)
    if b <= subset:
        in_sub[:] = True
    else:
        in_sub[np.random.default_rng(seed).choice(b, size=subset, replace=False)] = True
    mism = fail = flags_checked = 0
    rels, wells = [], []
    for k in np.unique(ns):
        js = np.nonzero(ns == k)[0]
        sel = js if full_flags else js[in_sub[js]]
        if sel.size == 0:
            continue
        k = int(k)
        mats = A_flat[offsets[sel][:, None] + np.arange(k * k)[None, :]].reshape(sel.size, k, k)
        w_ref, info, _ = zgeev(mats, threads)
        f = flag_test[sel]
        mism += int(np.sum((info != 0) != (f != 0)))
        fail += int(np.sum(info != 0))
        flags_checked += int(sel.size)
        sub = in_sub[sel]
        if not sub.any():
            continue
        wt = w_flat[eig_offsets[sel[sub]][:, None] + np.arange(k)[None, :]]
        rep = parity_report(mats[sub], wt, f[sub], threads, True, w_ref=w_ref[sub], info=info[sub])
        rels.append(rep["rel_err"])
        wells.append(rep["well"])
    rel = np.concatenate(rels)
    well = np.concatenate(wells)
    ok = np.isfinite(rel)
    return {"batch": int(b), "checked": int(in_sub.sum()), "flags_checked": flags_checked, "flag_mismatch": mism,
            "lapack_fail": fail, "gpu_flagged": int(np.count_nonzero(flag_test)),
            "max_rel_err": float(np.nanmax(rel)) if ok.any() else float("nan"),
            "p99_rel_err": float(np.nanpercentile(rel[ok], 99)) if ok.any() else float("nan"),
            "well_conditioned": int(well.sum()),
            "max_rel_err_well": float(np.nanmax(rel[well])) if well.any() else float("nan"),
            "p99_rel_err_well": float(np.nanpercentile(rel[well], 99)) if well.any() else float("nan")}


def real_parity_report(A: np.ndarray, wr: np.ndarray, wi: np.ndarray, flag_test: np.ndarray,
                       threads: int | None = None) -> dict:
    """Compares real-path eigenvalues/flags against LAPACK dgeev on the same
    real inputs (``A[k]`` column-major buffers), with the eigenvalue condition
    numbers of zgeevx on the same matrices selecting the well-conditioned ones."""
    A = np.ascontiguousarray(A, dtype=np.float64)
    if A.ndim == 2:
        A = A[None]
    wr_ref, wi_ref, info, _ = dgeev(A, threads)
    w_ref = wr_ref + 1j * wi_ref
    w_test = np.asarray(wr) + 1j * np.asarray(wi)
    fro = np.sqrt(np.sum(A ** 2, axis=(1, 2)))
    fro = np.where(fro == 0, 1.0, fro)
    flag_test = np.asarray(flag_test)
    ok = (info == 0) & (flag_test == 0)
    rel = np.full(A.shape[0], np.nan)
    if ok.any():
        err = matched_abs_errors(w_test[ok], w_ref[ok])
        rel[ok] = np.max(err, axis=1) / fro[ok]
    _, rc, _ = zgeevx_rconde(A.astype(np.complex128), threads)
    cond = 1.0 / np.maximum(rc, 1e-300)
    well = ok & (np.max(cond, axis=1) <= COND_MAX)
    return {
        "batch": int(A.shape[0]),
        "flag_mismatch": int(np.sum((info != 0) != (flag_test != 0))),
        "lapack_fail": int(np.sum(info != 0)),
        "pairs_ok": bool(check_conjugate_pairs(np.asarray(wr)[ok], np.asarray(wi)[ok])) if ok.any() else True,
        "max_rel_err": float(np.nanmax(rel)) if ok.any() else float("nan"),
        "well_conditioned": int(well.sum()),
        "max_rel_err_well": float(np.nanmax(rel[well])) if well.any() else float("nan"),
        "rel_err": rel,
    }
