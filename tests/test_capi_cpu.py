"""C-ABI library: builds, loads, exports every declared symbol, validates arguments (no GPU needed)."""
import ctypes
import os
import re
import subprocess

import pytest

from tokura_zgeev_batched_gb300 import api, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in sorted(os.listdir(os.path.join(ROOT, "include")))]


def declared_symbols():
    names = []
    for h in HEADERS:
        text = open(h).read()
        names += re.findall(r"TOKURA_API\s+[\w\s\*]+?\b(\w+)\s*\(", text)
    return names


@pytest.fixture(scope="module")
def lib():
    return api.lib()


def defined_dynamic_symbols():
    out = subprocess.run(["nm", "-D", "--defined-only", build.LIB_PATH], capture_output=True, text=True, check=True)
    return {ln.split()[-1] for ln in out.stdout.splitlines() if ln.strip()}


def test_every_declared_symbol_is_exported(lib):
    decl = declared_symbols()
    assert "tokura_zgeev_batched_gpu" in decl and len(decl) >= 8
    syms = defined_dynamic_symbols()
    for name in decl:
        assert name in syms, name
        getattr(lib, name)


def test_reference_mangled_names_exported(lib):
    syms = defined_dynamic_symbols()
    for mangled in (
        "_Z12tokuraCreatePP12tokurablas_t",
        "_Z13tokuraDestroyP12tokurablas_t",
        "_Z42tokura_get_zgeeveigenvaluesgetworspacesizeii",
        "_Z24tokura_zgeev_batched_gpuP12tokurablas_tiiP7double2S2_S2_PcP11CUstream_st",
    ):
        assert mangled in syms, mangled


def test_python_signature_table_covers_header():
    assert set(declared_symbols()) <= set(api.exported_symbols())


def test_workspace_size_formula(lib):
    ws = api.tokura_get_zgeeveigenvaluesgetworspacesize
    assert ws(32, 10000) == 16 * 32 * 32 * 10000 + 16 * 32 * 10000
    assert ws(1, 1) == 32
    assert ws(64, 65536) == 16 * 64 * 64 * 65536 + 16 * 64 * 65536
    size_max = 2 ** 64 - 1
    assert ws(0, 5) == size_max and ws(65, 5) == size_max and ws(-3, 5) == size_max
    assert ws(8, 0) == size_max - 1 and ws(8, -1) == size_max - 1


def test_argument_validation_codes(lib):
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: every call below fails validation first
    p = 0x2000
    f = api.tokura_zgeev_batched_gpu
    assert f(None, 8, 4, p, p, p, p, 0) == -1
    assert f(fake, 0, 4, p, p, p, p, 0) == -2
    assert f(fake, 65, 4, p, p, p, p, 0) == -2
    assert f(fake, 8, 4, None, p, p, p, 0) == -3
    assert f(fake, 8, 4, p, None, p, p, 0) == -4
    assert f(fake, 8, 4, p, p, None, p, 0) == -5
    assert f(fake, 8, 0, p, p, p, p, 0) == -6
    assert f(fake, 8, -2, p, p, p, p, 0) == -6
    assert f(fake, 8, 4, p, p, p, None, 0) == -7
    # order of checks follows the reference (tokura_zgeev_batched.cu:237-264)
    assert f(fake, 0, 0, None, None, None, None, 0) == -2


def test_layout_entry_points_validation(lib):
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: every call below fails validation first
    p = 0x2000
    f = api.tokura_zgeev_strided_batched_gpu
    assert f(None, 8, 4, p, 8, 64, p, 8, p, p) == -1
    assert f(fake, 65, 4, p, 8, 64, p, 8, p, p) == -2
    assert f(fake, 8, 4, None, 8, 64, p, 8, p, p) == -3
    assert f(fake, 8, 4, p, 8, 64, None, 8, p, p) == -4
    assert f(fake, 8, 4, p, 8, 64, p, 8, None, p) == -5
    assert f(fake, 8, 0, p, 8, 64, p, 8, p, p) == -6
    assert f(fake, 8, 4, p, 8, 64, p, 8, p, None) == -7
    assert f(fake, 8, 4, p, 7, 64, p, 8, p, p) == -8
    assert f(fake, 8, 4, p, 8, -1, p, 8, p, p) == -9
    assert f(fake, 8, 4, p, 8, 64, p, 7, p, p) == -9
    g = api.tokura_zgeev_pointer_batched_gpu
    assert g(None, 8, 4, p, 8, p, p, p) == -1
    assert g(fake, 0, 4, p, 8, p, p, p) == -2
    assert g(fake, 8, 4, None, 8, p, p, p) == -3
    assert g(fake, 8, 4, p, 8, p, p, None) == -7
    assert g(fake, 8, 4, p, 3, p, p, p) == -8
    c = api.tokura_cgeev_batched_gpu
    assert c(None, 8, 4, p, p, p, p) == -1
    assert c(fake, 65, 4, p, p, p, p) == -2
    assert c(fake, 8, 4, p, None, p, p) == -4
    assert c(fake, 8, -1, p, p, p, p) == -6


def test_real_entry_points_validation(lib):
    fake = ctypes.c_void_p(0x1000)  # never dereferenced: every call below fails validation first
    p = 0x2000
    for f in (api.tokura_dgeev_batched_gpu, api.tokura_sgeev_batched_gpu):
        assert f(None, 8, 4, p, p, p, p, p) == -1
        assert f(fake, 0, 4, p, p, p, p, p) == -2
        assert f(fake, 65, 4, p, p, p, p, p) == -2
        assert f(fake, 8, 4, None, p, p, p, p) == -3
        assert f(fake, 8, 4, p, None, p, p, p) == -4
        assert f(fake, 8, 4, p, p, None, p, p) == -4
        assert f(fake, 8, 4, p, p, p, None, p) == -5
        assert f(fake, 8, 0, p, p, p, p, p) == -6
        assert f(fake, 8, 4, p, p, p, p, None) == -7
    ws = api.tokura_get_dgeev_workspacesize
    assert ws(64, 65536) == 8 * 64 * 64 * 65536
    assert ws(0, 5) == 2 ** 64 - 1 and ws(8, 0) == 2 ** 64 - 2
    assert lib.tokuraSetRealConfig(None, 8, 1, 128) == -1


def test_create_destroy_null(lib):
    assert lib.tokuraCreate(None) == -1
    assert lib.tokuraDestroy(None) == 0
    assert lib.tokuraSetSweepCap(None, 3) == -1
    assert lib.tokuraSetBalancing(None, 3) == -1
    assert lib.tokuraSetShiftHints(None, 1) == -1
    assert lib.tokuraSetScaledRotations(None, 24) == -1
    assert lib.tokuraSetHostLinkRate(None, 10.0) == -1
    assert lib.tokuraSetRaggedHintMinOrder(None, 48) == -1
    # Host allocator: argument checks and unknown pointers need no GPU.
    p = ctypes.c_void_p()
    assert lib.tokuraHostAlloc(None, 16) == -1
    assert lib.tokuraHostAlloc(ctypes.byref(p), 0) == -2 and p.value is None
    assert lib.tokuraHostFree(None) == 0
    assert lib.tokuraHostAlloc(ctypes.byref(p), 2 ** 64 - 1) == 2 and p.value is None
    buf = ctypes.create_string_buffer(64)
    assert lib.tokuraHostFree(ctypes.cast(buf, ctypes.c_void_p)) == -1
    assert lib.tokuraSetRaggedLanes(None, 2) == -1


def test_reference_style_caller_links(tmp_path, lib):
    """An object compiled against the reference's (C++-linkage) declarations links to this library."""
    src = tmp_path / "caller.cpp"
    src.write_text(
        "#include <cuda_runtime_api.h>\n#include <cuComplex.h>\n#include <stddef.h>\n"
        "typedef struct tokurablas_t tokurablas_t;\n"
        "int tokuraCreate(tokurablas_t** h);\nint tokuraDestroy(tokurablas_t* h);\n"
        "size_t tokura_get_zgeeveigenvaluesgetworspacesize(int, int);\n"
        "int tokura_zgeev_batched_gpu(tokurablas_t*, int, int, cuDoubleComplex*, cuDoubleComplex*, cuDoubleComplex*,"
        " char*, cudaStream_t);\n"
        "int main() { return (int)tokura_get_zgeeveigenvaluesgetworspacesize(2, 1) == 96 ? 0 : 1; }\n"
    )
    exe = tmp_path / "caller"
    cuda_inc = "/usr/local/cuda/include"
    r = subprocess.run(["g++", str(src), "-I", cuda_inc, "-o", str(exe), build.LIB_PATH,
                        "-Wl,-rpath," + os.path.dirname(build.LIB_PATH), "-Wl,--unresolved-symbols=ignore-in-shared-libs"],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", str(exe)], capture_output=True, text=True).stdout
    assert "_Z42tokura_get_zgeeveigenvaluesgetworspacesizeii" in nm
    run = subprocess.run([str(exe)], capture_output=True, text=True)
    assert run.returncode == 0


def test_c_caller_compiles_against_header(tmp_path):
    src = tmp_path / "c_caller.c"
    src.write_text('#include "tokura_blas_ext.h"\nint main(void){ tokurablas_t* h = 0; (void)h;'
                   ' return (int)(tokura_get_zgeeveigenvaluesgetworspacesize(1, 1) != 32); }\n')
    r = subprocess.run(["gcc", "-std=c99", "-c", str(src), "-I", os.path.join(ROOT, "include"), "-I",
                        "/usr/local/cuda/include", "-o", str(tmp_path / "c_caller.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


def test_reference_header_constants_and_enums(tmp_path):
    """The reference header's public macros and enums (tokura_blas.h:12-48 of the reference)
    exist with the same names and values, in C and in C++."""
    body = ("#include \"tokura_blas.h\"\n"
            "typedef char a1[TARGET_CUDA_WARP == 32 ? 1 : -1];\n"
            "typedef char a2[TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE == 64 ? 1 : -1];\n"
            "typedef char a3[TOKURA_ZGEEV_BATCHED_GEHRD_TUNING_BATCHCOUNT == 8192 ? 1 : -1];\n"
            "typedef char a4[TOKURA_ZGEEV_BATCHED_HSEQR_TUNING_BATCHCOUNT == 8192 ? 1 : -1];\n"
            "typedef char a5[TOKURA_ZGEEV_BATCHED_TUNING_COUNT == 1 ? 1 : -1];\n"
            "typedef char a6[TOKURA_BLAS_SUCCESS == 0 && TOKURA_BLAS_FAIL == 1 ? 1 : -1];\n"
            "typedef char a7[MatrixWise == 0 && ElementWise == 1 && RowWise == 2 && NotSet == 3 ? 1 : -1];\n"
            "typedef char a8[ZGEHRD_NORMAL_MWB_METHOD == 0 && ZGEHRD_SHARED_MWB_METHOD == 1 ? 1 : -1];\n"
            "typedef char a9[ZHSEQR_NORMAL_MWB == 0 ? 1 : -1];\n"
            "TOKURA_ZGEEV_BATCHED_STATUS s = TOKURA_BLAS_FAIL;\n"
            "TOKURA_ZGEEV_BATCHED_MATRIX_ARRANGEMENT m = NotSet;\n"
            "TOKURA_ZGEHRD_BATCHED_WHICHFAST g = ZGEHRD_SHARED_MWB_METHOD;\n"
            "TOKURA_ZHSEQR_BATCHED_WHICHFAST q = ZHSEQR_NORMAL_MWB;\n")
    for compiler, ext, extra in (("gcc", "c", ["-std=c99"]), ("g++", "cpp", ["-std=c++17"])):
        src = tmp_path / f"consts.{ext}"
        cpp_tail = "void f(void) { gpuErrchk(cudaSuccess); }\n" if ext == "cpp" else ""
        src.write_text(body + cpp_tail)
        r = subprocess.run([compiler] + extra + ["-Wall", "-Werror", "-Wno-unused-variable", "-c", str(src),
                            "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
                            "-o", str(tmp_path / f"consts_{ext}.o")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def _reference_driver() -> str:
    from oracle import ref_gpu

    return os.path.join(ref_gpu.reference_root(), "stream_test", "main.cu")


REFERENCE_DRIVER = _reference_driver()


@pytest.mark.skipif(not os.path.exists(REFERENCE_DRIVER), reason="the reference's sources are not mounted here")
def test_reference_driver_compiles_against_header(tmp_path):
    """The reference's own MKL-free throughput driver (stream_test/main.cu, compiled there by
    stream_test/compile.sh:1 against the reference's include/) compiles unchanged against this
    library's include/ (compile only: nothing of the reference is linked or run)."""
    r = subprocess.run(["nvcc", "-c", REFERENCE_DRIVER, "-I", os.path.join(ROOT, "include"), "-Xcompiler",
                        "-fopenmp", "-gencode", "arch=compute_103a,code=sm_103a", "-o", str(tmp_path / "driver.o")],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    nm = subprocess.run(["nm", "-u", str(tmp_path / "driver.o")], capture_output=True, text=True).stdout
    # C linkage here: the driver's object refers to the plain names this library exports.
    for sym in ("tokuraCreate", "tokura_get_zgeeveigenvaluesgetworspacesize", "tokura_zgeev_batched_gpu"):
        assert sym in nm.split(), sym


def test_ragged_workspace_size(lib):
    ws = api.tokura_get_zgeev_ragged_workspacesize
    size_max = 2 ** 64 - 1
    assert ws(0, 10) == size_max - 1 and ws(5, 0) == size_max - 2
    b, t = 200000, 200000 * 1400
    need = ws(b, t)
    hints = (8 * 64 + 4) * b  # FP32 shift hints (64 float2) and the phase state per matrix
    assert need >= 16 * t + 12 * b + hints and need % 256 == 0 and need < 16 * t + 12 * b + hints + 64 * 1024


def test_ragged_argument_validation(lib):
    fake = ctypes.c_void_p(0x1000)
    p = 0x2000
    f = api.tokura_zgeev_ragged_gpu
    assert f(None, 4, p, p, None, 100, p, p, p, p) == -1
    assert f(fake, 4, None, p, None, 100, p, p, p, p) == -2
    assert f(fake, 4, p, p, None, 100, None, p, p, p) == -3
    assert f(fake, 4, p, p, None, 100, p, None, p, p) == -4
    assert f(fake, 4, p, p, None, 100, p, p, None, p) == -5
    assert f(fake, 0, p, p, None, 100, p, p, p, p) == -6
    assert f(fake, 4, p, p, None, 100, p, p, p, None) == -7
    assert f(fake, 4, p, None, None, 100, p, p, p, p) == -8
    assert f(fake, 4, p, p, None, 0, p, p, p, p) == -9


def test_host_alloc_without_a_gpu_fails_cleanly(lib):
    """Without a CUDA driver the registration fails: status 1, no pointer, nothing leaked."""
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is present: tokuraHostAlloc succeeds there (tests/test_host_api_gpu.py)")
    p = ctypes.c_void_p()
    assert lib.tokuraHostAlloc(ctypes.byref(p), 1 << 20) == 1 and p.value is None
    with pytest.raises(RuntimeError):
        api.host_empty((4, 4), torch.complex128)


def test_more_workspace_formulas(lib):
    """Size queries of the backward, vectors and workspace-free entry points (documented in
    include/tokura_blas_ext.h)."""
    for n, b in ((1, 1), (16, 50000), (64, 65536)):
        assert lib.tokura_get_zgeev_backward_workspacesize(n, b) == 48 * n * n * b + 16 * n * b
        assert lib.tokura_get_zgeev_vectors_workspacesize(n, b) == 48 * n * n * b + 24 * n * b + 4 * b
    for f in (lib.tokura_get_zgeev_backward_workspacesize, lib.tokura_get_zgeev_vectors_workspacesize):
        assert f(0, 5) == 2 ** 64 - 1 and f(65, 5) == 2 ** 64 - 1 and f(8, 0) == 2 ** 64 - 2
    rb = lib.tokura_get_zgeev_ragged_backward_workspacesize
    assert rb(0, 100) == 2 ** 64 - 2 and rb(10, 0) == 2 ** 64 - 3
    assert rb(1000, 1000 * 64 * 64) >= 4 * 16 * 1000 * 64 * 64  # four staging regions per element
    assert lib.tokura_zgeev_noalloc_max_bytes() == 32 << 20


def test_null_handle_is_rejected_first(lib):
    """Every handle-taking entry point checks the handle before anything else (the reference's
    order), so these need no device."""
    p = ctypes.c_void_p(1)
    lanes, threads = ctypes.c_int(), ctypes.c_int()
    assert lib.tokuraAutotune(None, 1, 2, 10, None) == -1
    assert lib.tokuraAutotuneRagged(None, 10, 1, 64, None) == -1
    assert lib.tokuraSetPlainConfig(None, 8, 1, 32) == -1
    assert lib.tokuraSetPlainQrLanes(None, 8, 2) == -1
    assert lib.tokuraGetPlainConfig(None, 8, 10, ctypes.byref(lanes), ctypes.byref(threads)) == -1
    assert lib.tokuraSaveTuning(None, b"/nonexistent/t") == -1 and lib.tokuraLoadTuning(None, b"/nonexistent/t") == -1
    assert lib.tokura_zgeev_backward_gpu(None, 8, 1, p, p, p, p, p, p, None) == -1
    assert lib.tokura_zgeev_ragged_backward_gpu(None, 1, p, p, None, 64, p, p, p, p, p, p, None) == -1
    assert lib.tokura_zgeev_vectors_batched_gpu(None, 8, 1, p, p, p, p, p, p, None) == -1
    assert lib.tokura_zgeev_batched_gpu_noalloc(None, 8, 1, p, p, p, None) == -1
    assert lib.tokura_zgeev_batched_host(None, 8, 1, p, p, p, 0) == -1
    assert lib.tokura_zgeev_strided_batched_gpu(None, 8, 1, p, 8, 64, p, 8, p, p, None) == -1
    assert lib.tokura_zgeev_pointer_batched_gpu(None, 8, 1, p, 8, p, p, p, None) == -1
    assert lib.tokura_probe_fp64_peak(None, None, 0, None) == -1
