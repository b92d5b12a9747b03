"""The reference library builds for sm_103a from its own sources plus the restated glue
(oracle/ref_gpu_glue.cu), with every helper it calls defined; its sources stay out of git."""
import os
import subprocess

import pytest

from oracle import ref_gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def built():
    if not ref_gpu.stage():
        pytest.skip("the reference's sources are neither present nor staged")
    path = ref_gpu.build()
    if path is None:
        pytest.skip("nvcc not available")
    return path


def test_links_with_every_called_helper_defined(built):
    assert ref_gpu.undefined_symbols(built) == []
    out = subprocess.run(["nm", "-D", "--defined-only", built], capture_output=True, text=True, check=True).stdout
    names = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    for sym in (ref_gpu.SYM_CREATE, ref_gpu.SYM_DESTROY, ref_gpu.SYM_WORKSPACE, ref_gpu.SYM_SOLVE,
                "_Z20tokura_zgehrd_helperP12tokurablas_t", "_Z35tokura_matrix_rearrangements_helperP12tokurablas_t",
                "_Z42tokura_eigenvaluesrearrangement_for_outputP12tokurablas_t"):
        assert sym in names, sym


def test_reference_sources_are_not_tracked():
    out = subprocess.run(["git", "ls-files", "oracle/_ref"], cwd=ROOT, capture_output=True, text=True).stdout
    assert out.strip() == ""
    chk = subprocess.run(["git", "check-ignore", "-q", "oracle/_ref/src/tokura_zgeev_batched.cu"], cwd=ROOT)
    assert chk.returncode == 0
