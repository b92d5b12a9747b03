"""Property tests (hypothesis) for the oracle and the host-side helpers: the
LAPACK harness against trace/determinant identities on generated matrices,
the optimal-matching metric, ragged packing and the workspace size queries."""
import numpy as np
import pytest

hypothesis = pytest.importorskip("hypothesis")
from hypothesis import given, settings  # noqa: E402
from hypothesis import strategies as st  # noqa: E402

from oracle import lapack_oracle as lo  # noqa: E402
from tokura_zgeev_batched_gb300 import api  # noqa: E402
from tokura_zgeev_batched_gb300 import workloads as wl  # noqa: E402

# Derandomized: the same examples on every run, so the suite cannot fail by chance.
SETTINGS = settings(max_examples=60, deadline=None, derandomize=True, database=None)
finite = st.floats(min_value=-8.0, max_value=8.0, allow_nan=False, allow_infinity=False, width=64)


def complex_matrix(n):
    return st.lists(finite, min_size=2 * n * n, max_size=2 * n * n).map(
        lambda v: (np.array(v[: n * n]) + 1j * np.array(v[n * n:])).reshape(n, n))


@SETTINGS
@given(st.integers(1, 6).flatmap(complex_matrix))
def test_oracle_trace_and_determinant(A):
    """sum(eig) = trace, prod(eig) = det, for the column-major reading of the buffer (A^T)."""
    w, info, _ = lo.zgeev(A[None], threads=1)
    assert info[0] == 0
    fro = max(np.linalg.norm(A), 1.0)
    n = A.shape[0]
    assert abs(w[0].sum() - np.trace(A)) <= 1e-12 * n * fro
    det = np.linalg.det(A.T)
    assert abs(np.prod(w[0]) - det) <= 1e-10 * fro ** n


@SETTINGS
@given(st.integers(1, 6).flatmap(lambda n: st.lists(finite, min_size=n * n, max_size=n * n).map(
    lambda v: np.array(v).reshape(n, n))))
def test_real_oracle_pairs_and_trace(A):
    wr, wi, info, _ = lo.dgeev(A[None], threads=1)
    assert info[0] == 0
    assert lo.check_conjugate_pairs(wr, wi)
    assert abs(wr[0].sum() - np.trace(A)) <= 1e-12 * A.shape[0] * max(np.linalg.norm(A), 1.0)
    assert abs(wi[0].sum()) <= 1e-12 * max(np.linalg.norm(A), 1.0)


@SETTINGS
@given(st.integers(1, 12), st.integers(0, 2 ** 32 - 1), st.floats(0.0, 1e-3))
def test_matching_metric_properties(n, seed, eps):
    rng = np.random.default_rng(seed)
    w = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    perm = rng.permutation(n)
    assert lo.matched_abs_errors(w[perm][None], w[None]).max() == 0.0  # order does not matter
    e1 = lo.matched_abs_errors((w + eps)[None], w[None]).max()
    e2 = lo.matched_abs_errors(w[None], (w + eps)[None]).max()
    # symmetric, and bounded by the shift (plus the rounding of w + eps)
    assert e1 == pytest.approx(e2) and e1 <= eps + 1e-15 * (1.0 + np.abs(w).max())


@SETTINGS
@given(st.lists(st.integers(1, 9), min_size=1, max_size=20))
def test_pack_ragged_layout(sizes):
    mats = [np.full((k, k), float(i), np.complex128) for i, k in enumerate(sizes)]
    buf, ns, offs, eoffs = wl.pack_ragged(mats)
    assert ns.tolist() == sizes
    assert offs.tolist() == np.concatenate([[0], np.cumsum(np.array(sizes) ** 2)[:-1]]).tolist()
    assert eoffs.tolist() == np.concatenate([[0], np.cumsum(sizes)[:-1]]).tolist()
    for i, k in enumerate(sizes):
        assert (buf[offs[i]: offs[i] + k * k] == i).all()


@SETTINGS
@given(st.integers(1, 64), st.integers(1, 1 << 20))
def test_workspace_queries(n, batch):
    lib = api.lib()
    assert api.tokura_get_zgeeveigenvaluesgetworspacesize(n, batch) == 16 * n * n * batch + 16 * n * batch
    assert lib.tokura_get_dgeev_workspacesize(n, batch) == 8 * n * n * batch
    assert lib.tokura_get_zgeev_vectors_workspacesize(n, batch) == 48 * n * n * batch + 24 * n * batch + 4 * batch
    total = n * n * batch
    rag = lib.tokura_get_zgeev_ragged_workspacesize(batch, total)
    assert rag >= 16 * total + 516 * batch
    assert lib.tokura_get_zgeev_ragged_workspacesize(batch, total + 1) >= rag  # monotone in the elements
