"""CPU model of this library's own iteration (oracle/model_qr.c): its
eigenvalues agree with LAPACK, and it gives the sweep counts per eigenvalue
quoted for the FP32 shift hints (Wilkinson shifts only; hints of FP32
accuracy; hints accurate to FP32 rounding)."""
import numpy as np
import pytest

from oracle import lapack_oracle as lo
from tokura_zgeev_batched_gb300 import workloads as wl


@pytest.mark.parametrize("gen", ["gaussian", "companion", "vdv"])
@pytest.mark.parametrize("n", [1, 2, 5, 16, 64])
def test_model_agrees_with_lapack(gen, n):
    A = wl.GENERATORS[gen](12, n, seed=40 + n)
    w_ref, info, _ = lo.zgeev(A, threads=2)
    w, flag, _ = lo.model_qr(A)
    assert (flag == 0).all() and (info == 0).all()
    fro = np.maximum(np.linalg.norm(A, axis=(1, 2)), 1e-300)
    _, rc, _ = lo.zgeevx_rconde(A, threads=2)
    well = (1.0 / np.maximum(rc, 1e-300)).max(axis=1) <= lo.COND_MAX
    err = lo.matched_abs_errors(w, w_ref).max(axis=1) / fro
    assert np.all(err[well] <= lo.TOL_REL_FRO), err


def test_model_sweeps_per_eigenvalue_with_and_without_hints():
    import scipy.linalg.lapack as lapack

    n, b = 64, 16
    A = wl.gaussian(b, n, seed=7)
    w_ref = lo.zgeev(A, threads=2)[0]
    # FP32 eigenvalues of the same matrices (the library reads A[k] column-major: A[k].T).
    fp32 = np.stack([lapack.cgeev(A[k].T.astype(np.complex64), compute_vl=0, compute_vr=0)[0] for k in range(b)])
    per_eig = {}
    for tag, est in (("wilkinson", None), ("fp32", fp32), ("rounded", w_ref.astype(np.complex64))):
        w, flag, sweeps = lo.model_qr(A, est)
        assert (flag == 0).all()
        assert lo.matched_abs_errors(w, w_ref).max() <= lo.TOL_REL_FRO * np.linalg.norm(A, axis=(1, 2)).min()
        per_eig[tag] = sweeps.sum() / (b * n)
    assert 3.1 <= per_eig["wilkinson"] <= 3.6, per_eig
    assert 2.3 <= per_eig["fp32"] <= 2.9, per_eig
    assert 1.8 <= per_eig["rounded"] <= 2.3, per_eig


def test_model_estimator_accuracy_and_tolerance():
    """The FP32 estimator model at the library's 1e-5 deflation tolerance: estimates within
    ~1e-6 of LAPACK (relative, median), and the FP64 sweeps they lead to barely differ from
    those of estimates deflated at FP32's ulp."""
    n, b = 64, 16
    A = wl.gaussian(b, n, seed=11)
    w_ref = lo.zgeev(A, threads=2)[0]
    sweeps, fp32_sweeps = {}, {}
    for tol in (5.9604644775390625e-08, 1e-5):
        est, sw32 = lo.model_estimates(A, tol, return_sweeps=True)
        fp32_sweeps[tol] = sw32.sum() / (b * n)
        rel = lo.matched_abs_errors(est.astype(np.complex128), w_ref) / np.abs(w_ref)
        assert np.median(rel) < 3e-6 and rel.max() < 1e-3, (tol, np.median(rel), rel.max())
        w, flag, sw = lo.model_qr(A, est)
        assert (flag == 0).all()
        sweeps[tol] = sw.sum() / (b * n)
    assert 2.3 <= sweeps[1e-5] <= 2.9 and abs(sweeps[1e-5] - sweeps[5.9604644775390625e-08]) < 0.15, sweeps
    # the tolerance's point: the FP32 QR itself stops ~0.3 sweeps per eigenvalue earlier
    assert fp32_sweeps[1e-5] < fp32_sweeps[5.9604644775390625e-08] - 0.2, fp32_sweeps


def test_model_variants_not_adopted():
    """The two shift-strategy variants the library does not use: zlahqr's start-row search
    saves only a few percent of the rotation work; the estimate as the second sweep's shift
    costs sweeps."""
    n, b = 64, 16
    A = wl.gaussian(b, n, seed=13)
    w_ref = lo.zgeev(A, threads=2)[0]
    est = lo.model_estimates(A)
    base = lo.model_qr_variant(A, est)
    start = lo.model_qr_variant(A, est, start_row=True)
    twice = lo.model_qr_variant(A, est, estimate_twice=True)
    for w, flag, _, _ in (base, start, twice):
        assert (flag == 0).all()
        assert lo.matched_abs_errors(w, w_ref).max() <= lo.TOL_REL_FRO * np.linalg.norm(A, axis=(1, 2)).min()
    saving = 1.0 - start[3].sum() / base[3].sum()
    assert 0.0 <= saving < 0.06, saving
    assert twice[2].sum() > 1.05 * base[2].sum()
    w0, f0, s0 = lo.model_qr(A, est)
    assert np.array_equal(s0, base[2]) and np.array_equal(w0.view(np.uint64), base[0].view(np.uint64))


def test_model_gradient_schur_iteration():
    """The gradient's Schur iteration (forward eigenvalues as first shifts, deflation at
    100 ulp): about one sweep per eigenvalue, against ~1.7 at the ulp and ~3.1 with Wilkinson
    shifts, with unchanged accuracy."""
    ulp = 2.0 ** -52
    n, b = 48, 24
    A = wl.vdv(b, n, seed=5, min_sep=0.05)
    w_ref = lo.zgeev(A, threads=2)[0]
    fro = np.linalg.norm(A, axis=(1, 2))
    per_eig = {}
    for tag, lam, tol in (("wilkinson", None, ulp), ("perfect_ulp", w_ref, ulp), ("perfect_100ulp", w_ref, 100 * ulp)):
        w, flag, sweeps, _ = lo.model_qr_variant(A, lam=lam, tol=tol)
        assert (flag == 0).all()
        assert (lo.matched_abs_errors(w, w_ref).max(axis=1) / fro).max() <= 1e-13
        per_eig[tag] = sweeps.sum() / (b * n)
    assert 2.8 <= per_eig["wilkinson"] <= 3.6, per_eig
    assert 1.5 <= per_eig["perfect_ulp"] <= 2.0, per_eig
    assert 0.8 <= per_eig["perfect_100ulp"] <= 1.2, per_eig


def _lockstep_efficiency(traces, order, width=32):
    """Matrices sharing a warp run their sweeps in lockstep (one lane each): a sweep costs what
    the largest active window costs, ~ (m - 1)(m + 2) element-pair updates. Returns the useful
    fraction of lane time for the given grouping."""
    def cost(m):
        return (m - 1) * (m + 2)

    useful = lanes = 0
    for k in range(0, len(order), width):
        group = [traces[i] for i in order[k:k + width]]
        steps = max(len(t) for t in group)
        useful += sum(int(cost(t).sum()) for t in group)
        lanes += len(group) * sum(max(int(cost(t[s])) if s < len(t) else 0 for t in group) for s in range(steps))
    return useful / lanes


def test_model_lockstep_divergence_and_grouping():
    """One matrix per lane (the large-batch shape): window variation between the 32 matrices of
    a warp wastes only a few percent of lane time, and grouping matrices by the estimator's own
    sweep count (known before the FP64 QR) does not reduce it."""
    n, b = 64, 256
    A = wl.gaussian(b, n, seed=99)
    est, s32 = lo.model_estimates(A, return_sweeps=True)
    _, flag, sweeps, work, traces = lo.model_qr_variant(A, est, trace=True)
    assert (flag == 0).all() and all(len(t) == s for t, s in zip(traces, sweeps))
    rand = _lockstep_efficiency(traces, np.random.default_rng(0).permutation(b))
    by_fp32 = _lockstep_efficiency(traces, np.argsort(s32, kind="stable"))
    by_work = _lockstep_efficiency(traces, np.argsort(work, kind="stable"))
    assert 0.9 <= rand <= 0.99, rand
    assert abs(by_fp32 - rand) < 0.01, (rand, by_fp32)
    assert by_work >= rand, (rand, by_work)


@pytest.mark.parametrize("gen", ["gaussian", "vdv", "companion", "uniform"])
@pytest.mark.parametrize("n", [2, 8, 33, 64])
def test_model_scaled_rotations(gen, n):
    """Scaled rotations (two complex multiply-adds per element pair instead of the plain
    rotation's 12 FP64 operations): the same sweeps as the plain iteration, LAPACK accuracy,
    and rescaling of rows/columns only now and then (O(n) each)."""
    A = wl.GENERATORS[gen](24, n, seed=300 + n)
    w_ref = lo.zgeev(A, threads=2)[0]
    fro = np.maximum(np.linalg.norm(A, axis=(1, 2)), 1e-300)
    _, rc, _ = lo.zgeevx_rconde(A, threads=2)
    well = (1.0 / np.maximum(rc, 1e-300)).max(axis=1) <= lo.COND_MAX
    est = lo.model_estimates(A)
    for hints in (None, est):
        w0, f0, s0, _ = lo.model_qr_variant(A, hints)
        w, f, s, work, resc = lo.model_qr_variant(A, hints, scaled=True)
        assert (f == 0).all() and (f0 == 0).all()
        assert abs(int(s.sum()) - int(s0.sum())) <= max(2, s0.sum() // 100)
        err = lo.matched_abs_errors(w, w_ref).max(axis=1) / fro
        assert np.all(err[well] <= lo.TOL_REL_FRO), err
        assert resc.sum() <= 8 * s.sum()  # a few row/column rescales per sweep at most


def test_model_scaled_rescales_are_rare():
    """With the factor floor at 2^-150 a 64x64 Gaussian matrix needs a few dozen O(n)
    rescales over its ~170 sweeps (185 at a 2^-60 floor). On the GPU a rescale runs only in the
    lanes whose factor fell below the floor while the rest of the warp waits, so their number,
    not their own arithmetic, is what they cost."""
    A = wl.gaussian(64, 64, seed=5)
    est = lo.model_estimates(A)
    _, f, s, _, resc = lo.model_qr_variant(A, est, scaled=True)
    assert (f == 0).all()
    assert 20 <= resc.mean() <= 80, resc.mean()
    assert resc.mean() <= 0.5 * s.mean()  # fewer than one rescale every other sweep


@pytest.mark.parametrize("gen", ["gaussian", "vdv", "companion", "uniform"])
def test_model_elementary_hessenberg(gen):
    """Hessenberg form by stabilized elementary similarity transforms (half the multiply-adds):
    on these classes as accurate as the Householder reduction (it is not adopted: its
    stability is not guaranteed in general)."""
    n = 64
    A = wl.GENERATORS[gen](24, n, seed=700)
    w_ref = lo.zgeev(A, threads=2)[0]
    fro = np.linalg.norm(A, axis=(1, 2))
    _, rc, _ = lo.zgeevx_rconde(A, threads=2)
    well = (1.0 / np.maximum(rc, 1e-300)).max(axis=1) <= lo.COND_MAX
    w, f, _, _ = lo.model_qr_variant(A, elementary=True)
    assert (f == 0).all()
    err = lo.matched_abs_errors(w, w_ref).max(axis=1) / fro
    assert np.all(err[well] <= 1e-13), err
