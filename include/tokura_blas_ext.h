/*
 * tokura_blas_ext.h — entry points beyond the reference's API.
 *
 * The reference (hirokitokura/tokura_zgeev_batched) has no counterpart for
 * these; each comment says what it adds. All data pointers are device
 * pointers; all calls are asynchronous on `stream` unless stated.
 *
 * Compute calls do not write the handle, so one handle serves several
 * streams and host threads at once. The tokuraSet* calls, tokuraLoadTuning
 * and the autotuners change its settings: make them before those calls
 * start, not while other threads are computing with the same handle.
 */
#ifndef TOKURA_BLAS_EXT_GB300_H
#define TOKURA_BLAS_EXT_GB300_H

#include "tokura_blas.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Per-eigenvalue QR sweep cap used by later calls on this handle
 * (0 restores LAPACK's rule 30*max(10, n)). A small cap forces flag[j] = 1,
 * which the tests use to exercise the non-convergence path.
 * Returns 0, or -1 for a NULL handle / negative cap. Configuration call:
 * do not race it with compute calls on the same handle. */
TOKURA_API int tokuraSetSweepCap(tokurablas_t* handle, int cap);

/* Balancing before the eigenvalue solves of later calls on this handle (plain,
 * ragged, host-buffer and workspace-free entry points): 0 none (default, the
 * reference's behaviour, README.md:79), 1 permutation only, 2 scaling only,
 * 3 both (LAPACK zgeev's choice, zgebal JOB='B'). Permutation isolates
 * eigenvalues exposed by zero rows/columns; scaling applies exact powers of
 * two. Eigenvalues are unchanged in exact arithmetic; badly scaled matrices
 * gain accuracy. Returns 0, -1 NULL handle, -2 bad mode. */
TOKURA_API int tokuraSetBalancing(tokurablas_t* handle, int mode);

/* FP32 shift hints for later eigenvalue calls on this handle. A separate,
 * cheap kernel (one warp per matrix in shared memory) computes
 * single-precision eigenvalue estimates, running on a second stream beside
 * the FP64 Hessenberg phase; the FP64 QR then uses the nearest unused
 * estimate as the shift of the first sweep after each deflation (about 2.1
 * sweeps per eigenvalue instead of 3.4). Modes: 1 (default) for the plain,
 * strided, pointer-array, complex64, host-buffer and workspace-free entry
 * points with n >= 12, and the ragged entry point for its matrices of order
 * >= tokuraSetRaggedHintMinOrder's value; 2 for every eigenvalue entry
 * point and order, ragged included; 0 off
 * (Wilkinson shifts only). Results keep the FP64 accuracy in every mode (the
 * estimates only steer the iteration; results are not bitwise identical
 * between modes). The estimates use 8n bytes per matrix of the workspace
 * after the staging area, inside the reference's workspace formula.
 * Returns 0, -1 NULL handle, -2 bad mode. */
TOKURA_API int tokuraSetShiftHints(tokurablas_t* handle, int mode);

/* Orders from which the eigenvalue calls (plain, strided, pointer-array,
 * complex64, host-buffer, workspace-free and ragged entry points), the
 * gradients (plain and ragged backward) and the eigenvector call run their QR
 * with scaled rotations, per lane: with L lanes per matrix (the launch shape),
 * orders n >= max(7, L * min_order). The Hessenberg matrix is kept with real
 * row and column scale factors, which makes each rotation update two complex
 * multiply-adds per element pair (8 FP64 instructions instead of 12) at the
 * same rounding-error bound; the factors live in matrix entries the QR does
 * not use, so the workspace is unchanged. min_order 1..64; 65 = never;
 * default 16 (1 lane: n = 64 -10 % call time, 32 -5 %, 16 -0.6 %; 4 lanes at
 * n = 32: +9 %, since a rotation's fixed cost is paid per lane group while its
 * savings shrink with the pairs each lane updates). Results keep the FP64
 * accuracy either way but are not bitwise identical.
 * Returns 0, -1 NULL handle, -2 min_order outside 1..65. */
TOKURA_API int tokuraSetScaledRotations(tokurablas_t* handle, int min_order);

/* Smallest order whose matrices get shift hints in ragged calls under mode 1
 * (1..64; 65 = none; default 48). The estimator costs about n^2 per matrix
 * and saves about n^3 of QR work, so on mixed orders it pays on the largest
 * (200,000 orders in U{1..64}: 676 ms without hints, 645 ms with 48).
 * Returns 0, -1 NULL handle, -2 n outside 1..65. */
TOKURA_API int tokuraSetRaggedHintMinOrder(tokurablas_t* handle, int n);

/* Launch shape of the plain kernel for order n: lanes per matrix (1, 2, 4, 8,
 * 16, 32; 0 = choose from the batch size) and threads per block (32..256, multiple
 * of 32; 0 = 32). Replaces the reference's compile-time tables
 * (include/tokura_zhseqr_parameters.h, tokura_zgeev_batched.cu:13-60).
 * Returns 0, -1 NULL handle, -2 n out of range, -3 bad lanes, -4 bad threads. */
TOKURA_API int tokuraSetPlainConfig(tokurablas_t* handle, int n, int lanes_per_matrix, int threads_per_block);

/* The launch shape the next plain call with (n, batch_count) will use. */
TOKURA_API int tokuraGetPlainConfig(const tokurablas_t* handle, int n, int batch_count, int* lanes_per_matrix,
                                    int* threads_per_block);

/* Lanes per matrix of the QR phase of plain calls of order n that use shift
 * hints (tokuraSetShiftHints), where staging + Hessenberg and the QR are two
 * launches: 1, 2, 4, 8, 16 or 32, or 0 for the library's choice (the width of the
 * first launch, except two lanes after a four-lane first launch for n <= 24).
 * Fewer lanes than the first launch means fewer instructions per matrix
 * spent on rotation generation and shifts, in fewer, fuller warps.
 * Returns 0, -1 NULL handle, -2 n out of range, -3 bad lanes. */
TOKURA_API int tokuraSetPlainQrLanes(tokurablas_t* handle, int n, int lanes_per_matrix);

/* Autotuner (replaces the reference's build-time tuner,
 * src/TOKURA_ZHSEQR_BATCHED_GEHRD_TUNING_main.cu:89-227, and its generated
 * tables). For each order n in [n_min, n_max], times every plain-kernel shape
 * (lanes per matrix 1/2/4/8/16/32 x threads per block 32/64/128/256) on batch_count
 * seeded synthetic complex Gaussian matrices and stores the fastest in the
 * handle. Allocates its own scratch (cudaMalloc), synchronizes `stream`.
 * Returns 0; -1 NULL handle, -2 bad range, -6 batch_count <= 0,
 * 2 allocation failure, 1 CUDA failure. */
TOKURA_API int tokuraAutotune(tokurablas_t* handle, int n_min, int n_max, int batch_count, cudaStream_t stream);

/* Same for the ragged solvers (lanes per matrix, 0 = automatic, 1, 2, 4, 8) on
 * batch_count matrices with orders uniform in [n_min, n_max]. */
TOKURA_API int tokuraAutotuneRagged(tokurablas_t* handle, int batch_count, int n_min, int n_max,
                                    cudaStream_t stream);

/* Writes / reads the handle's tuned shapes as a text file keyed by device name
 * and SM count. Load returns 0; 1 cannot open, 2 malformed, 3 the file was
 * tuned on another device (the handle is left unchanged unless 0).
 * tokuraCreate applies the file named by the environment variable
 * TOKURA_ZGEEV_TUNING_FILE when it matches the device. */
TOKURA_API int tokuraSaveTuning(const tokurablas_t* handle, const char* path);
TOKURA_API int tokuraLoadTuning(tokurablas_t* handle, const char* path);

/* Measures the device's FP64 FMA throughput (FLOP/s, 2 per FMA) with a
 * saturating FMA loop; synchronizes `stream`. scratch: >= 512*SMs doubles.
 * Returns 0, -1 NULL pointer, -2 scratch too small, 1 CUDA failure. */
TOKURA_API int tokura_probe_fp64_peak(double* flops_per_second, double* scratch, int scratch_doubles,
                                      cudaStream_t stream);

/* Ragged batch: matrix j has its own order n[j] (1..64) and starts at element
 * offsets[j] of A (column-major, 16*n[j]^2 bytes), A holding total_elements
 * complex entries. Its eigenvalues go to eigenvalues[eig_offsets[j] + i]; if
 * eig_offsets is NULL they follow one another (exclusive prefix sum of n).
 * One persistent launch pulls size-bucketed tiles (largest n first) from a
 * device work queue; planning runs on the device, so the call is
 * asynchronous and can be captured in a CUDA graph. flag[j] as for the plain
 * call, plus 3 when n[j] or offsets[j] is invalid (order outside 1..64, or
 * the matrix does not lie inside A) or the matrices' sizes sum to more than
 * total_elements. n, offsets, eig_offsets: device arrays of batch_count.
 * work: tokura_get_zgeev_ragged_workspacesize(batch_count, total_elements)
 * bytes. The reference has no counterpart (it takes one n per call).
 * Returns 0; -1 NULL handle, -2 n NULL, -3 A NULL, -4 eigenvalues NULL,
 * -5 work NULL, -6 batch_count <= 0, -7 flag NULL, -8 offsets NULL,
 * -9 total_elements <= 0; 1 launch failure. */
TOKURA_API int tokura_zgeev_ragged_gpu(tokurablas_t* handle, int batch_count, const int* n, const long long* offsets,
                                       const long long* eig_offsets, long long total_elements,
                                       const cuDoubleComplex* A, cuDoubleComplex* eigenvalues, void* work, char* flag,
                                       cudaStream_t stream);

/* Workspace bytes of tokura_zgeev_ragged_gpu: 16*total_elements staging plus
 * the work queue and bookkeeping and 516 bytes per matrix for the FP32 shift
 * hints and phase state (tokuraSetShiftHints); (size_t)-2 if batch_count <= 0,
 * (size_t)-3 if total_elements <= 0. */
TOKURA_API size_t tokura_get_zgeev_ragged_workspacesize(int batch_count, long long total_elements);

/* Differentiable mode (no counterpart in the reference). Given A (as passed to
 * the forward, column-major), the forward's eigenvalues and the gradients of
 * a real loss with respect to them (torch's convention for complex tensors:
 * dL/dRe + i dL/dIm), returns grad_A in A's layout:
 *     grad_A = Q X^{-H} diag(grad_eigenvalues) X^H Q^H,
 * with A = Q T Q^H recomputed (Schur form; the forward's eigenvalues serve as
 * shifts and are matched to the diagonal of T) and X the right eigenvectors of
 * T. Only A and the eigenvalues need to be kept from the forward.
 * flag[j]: 0 ok, 1 QR cap hit (grad_A NaN), 2 non-finite A (grad_A NaN),
 * 4 two eigenvalues coincide to working precision (derivative undefined;
 * denominators clamped). work: tokura_get_zgeev_backward_workspacesize bytes
 * (48*n*n*batch + 16*n*batch). Returns 0; -1 NULL handle, -2 bad n, -3 A NULL,
 * -4 eigenvalues or grad_eigenvalues NULL, -5 work NULL, -6 batch_count <= 0,
 * -7 flag NULL, -8 grad_A NULL; 1 launch failure. */
TOKURA_API int tokura_zgeev_backward_gpu(tokurablas_t* handle, int n, int batch_count, const cuDoubleComplex* A,
                                         const cuDoubleComplex* eigenvalues, const cuDoubleComplex* grad_eigenvalues,
                                         cuDoubleComplex* grad_A, void* work, char* flag, cudaStream_t stream);
TOKURA_API size_t tokura_get_zgeev_backward_workspacesize(int n, int batch_count);

/* Ragged backward: layouts as tokura_zgeev_ragged_gpu (grad_A at offsets[j],
 * eigenvalues and grad_eigenvalues at eig_offsets[j] or packed); flags as the
 * plain backward plus 3 for invalid entries. -10: grad_A NULL. */
TOKURA_API int tokura_zgeev_ragged_backward_gpu(tokurablas_t* handle, int batch_count, const int* n,
                                                const long long* offsets, const long long* eig_offsets,
                                                long long total_elements, const cuDoubleComplex* A,
                                                const cuDoubleComplex* eigenvalues,
                                                const cuDoubleComplex* grad_eigenvalues, cuDoubleComplex* grad_A,
                                                void* work, char* flag, cudaStream_t stream);
TOKURA_API size_t tokura_get_zgeev_ragged_backward_workspacesize(int batch_count, long long total_elements);

/* Eigenvalues and eigenvectors (ZGEEV with JOBVL/JOBVR = 'V'; the reference
 * computes eigenvalues only, README.md:63). VR[:, i] / VL[:, i] (column-major
 * n x n per matrix, matrices one after another) are the right / left
 * eigenvectors of eigenvalues[i] (A VR = VR diag(w), VL^H A = diag(w) VL^H),
 * each with unit 2-norm and its largest-modulus component real and positive,
 * as LAPACK zgeev returns them. VL or VR may be NULL. flag: 0 converged,
 * 1 QR cap hit, 2 non-finite input. work:
 * tokura_get_zgeev_vectors_workspacesize(n, batch_count) bytes (48*n*n*batch
 * + 24*n*batch + 4*batch; the last 8*n*batch + 4*batch hold the FP32 shift
 * hints of tokuraSetShiftHints and the per-matrix state between the two
 * kernels of a hinted call). Return codes as tokura_zgeev_batched_gpu. */
TOKURA_API int tokura_zgeev_vectors_batched_gpu(tokurablas_t* handle, int n, int batch_count, const cuDoubleComplex* A,
                                                cuDoubleComplex* eigenvalues, cuDoubleComplex* VL,
                                                cuDoubleComplex* VR, void* work, char* flag, cudaStream_t stream);
TOKURA_API size_t tokura_get_zgeev_vectors_workspacesize(int n, int batch_count);

/* Lanes per matrix of the ragged solvers (1, 2, 4, 8; 0 = chosen per launch). */
TOKURA_API int tokuraSetRaggedLanes(tokurablas_t* handle, int lanes_per_matrix);

/* Pinned host memory for host-buffer calls: anonymous memory aligned to and
 * backed by transparent huge pages where the kernel allows, registered with
 * CUDA (cudaHostRegister). Copies from it keep the host link's full rate after
 * idle periods, where copies from cudaHostAlloc memory (base pages, one IOMMU
 * translation each) slow down. Free with tokuraHostFree.
 * Returns 0; -1 ptr NULL, -2 bytes == 0; 2 mapping failed, 1 registration failed. */
TOKURA_API int tokuraHostAlloc(void** ptr, size_t bytes);
/* Frees memory from tokuraHostAlloc (NULL: no-op). Returns 0; -1 not from
 * tokuraHostAlloc (or already freed); 1 CUDA unregistration failed. */
TOKURA_API int tokuraHostFree(void* ptr);

/* Host-to-device rate (GB/s) that tokura_zgeev_batched_host plans its chunks
 * for; 0 (the default) uses the rate its previous call on the handle measured.
 * Returns 0; -1 NULL handle, -2 gbs negative or not finite. */
TOKURA_API int tokuraSetHostLinkRate(tokurablas_t* handle, double gbs);

/* Host-buffer variant of tokura_zgeev_batched_gpu: A, eigenvalues and flag are
 * HOST pointers (layouts as the device call). The batch is cut into chunks of
 * chunk_matrices (0 = automatic: 2 equal chunks, or growing chunks from 1/16
 * of the batch when the previous call on the handle saw a host-to-device rate
 * below 100 GB/s) issued round-robin on the handle's own streams, copies in
 * chunk order, so host-device copies overlap the solves; returns when the results
 * are in host memory. Replaces the reference's multi-stream example driver
 * (stream_test_with_MKL/main.cu:236-288). Host memory should be pinned for the
 * copies to overlap. Device buffers are cached in the handle (freed by
 * tokuraDestroy); host-buffer calls on one handle are serialized.
 * Returns 0; -1 NULL handle, -2 bad n, -3 A NULL, -4 eigenvalues NULL,
 * -6 batch_count <= 0, -7 flag NULL, -8 chunk_matrices < 0; 2 device
 * allocation failure, 1 CUDA failure. */
TOKURA_API int tokura_zgeev_batched_host(tokurablas_t* handle, int n, int batch_count, const cuDoubleComplex* A,
                                         cuDoubleComplex* eigenvalues, char* flag, int chunk_matrices);

/* Other input layouts and precisions (no reference counterpart: the
 * reference takes contiguous n x n FP64 column-major matrices only,
 * tokura_zgeev_batched.cu:212-285). All three use the plain solver and the
 * workspace of tokura_get_zgeeveigenvaluesgetworspacesize(n, batch_count);
 * results are bitwise equal to tokura_zgeev_batched_gpu on the same matrix
 * entries. A is read only. Return codes are those of
 * tokura_zgeev_batched_gpu plus the ones listed.
 *
 * Strided: matrix j is column-major at A + j*strideA with leading dimension
 * lda (element (r,c) at A[j*strideA + r + c*lda]); its eigenvalues go to
 * eigenvalues[j*strideW + i]. strideA may be 0 (one matrix, many copies) or
 * smaller than lda*n (overlapping read-only views). -8 lda < n,
 * -9 strideA < 0 or strideW < n. */
TOKURA_API int tokura_zgeev_strided_batched_gpu(tokurablas_t* handle, int n, int batch_count, const cuDoubleComplex* A,
                                                int lda, long long strideA, cuDoubleComplex* eigenvalues,
                                                long long strideW, cuDoubleComplex* work, char* flag,
                                                cudaStream_t cudastream);

/* Pointer array (cuBLAS batched style): Aarray is a DEVICE array of
 * batch_count device pointers, matrix j column-major at Aarray[j] with
 * leading dimension lda; eigenvalues contiguous as in tokura_zgeev_batched_gpu.
 * A NULL entry gives NaN eigenvalues and flag[j] = 3. -8 lda < n. */
TOKURA_API int tokura_zgeev_pointer_batched_gpu(tokurablas_t* handle, int n, int batch_count,
                                                const cuDoubleComplex* const* Aarray, int lda,
                                                cuDoubleComplex* eigenvalues, cuDoubleComplex* work, char* flag,
                                                cudaStream_t cudastream);

/* Single-precision complex in and out (LAPACK cgeev's types), computed in
 * FP64: entries are widened exactly on load and the eigenvalues rounded to
 * nearest on store, so they are the FP64 eigenvalues of the given FP32
 * matrix, correctly rounded from the FP64 result. Layout as
 * tokura_zgeev_batched_gpu. */
TOKURA_API int tokura_cgeev_batched_gpu(tokurablas_t* handle, int n, int batch_count, const cuComplex* A,
                                        cuComplex* eigenvalues, cuDoubleComplex* work, char* flag,
                                        cudaStream_t cudastream);

/* Real matrices (LAPACK dgeev / sgeev with JOBVL = JOBVR = 'N'; no reference
 * counterpart, the reference takes complex input only). Matrix j is n x n
 * column-major at A + j*n*n; eigenvalue i of matrix j is
 * wr[i + j*n] + i*wi[i + j*n], in LAPACK's convention: complex conjugate
 * pairs are adjacent with the positive imaginary part first and are exact
 * conjugates; real eigenvalues have wi exactly 0. Computed by a real
 * Householder Hessenberg reduction and the Francis double-shift QR in FP64
 * (about a quarter of the complex path's arithmetic). flag[j] as for
 * tokura_zgeev_batched_gpu (balancing per tokuraSetBalancing, sweep cap per
 * tokuraSetSweepCap). work: tokura_get_dgeev_workspacesize(n, batch_count)
 * bytes. A is read only. Returns 0; -1 NULL handle, -2 bad n, -3 A NULL,
 * -4 wr or wi NULL, -5 work NULL, -6 batch_count <= 0, -7 flag NULL,
 * 1 launch failure. The sgeev variant takes FP32 A and writes FP32 wr/wi
 * (entries widened exactly, results rounded to nearest from FP64). */
TOKURA_API size_t tokura_get_dgeev_workspacesize(int n, int batch_count);
TOKURA_API int tokura_dgeev_batched_gpu(tokurablas_t* handle, int n, int batch_count, const double* A, double* wr,
                                        double* wi, double* work, char* flag, cudaStream_t cudastream);
TOKURA_API int tokura_sgeev_batched_gpu(tokurablas_t* handle, int n, int batch_count, const float* A, float* wr,
                                        float* wi, double* work, char* flag, cudaStream_t cudastream);

/* Launch shape of the real kernel for order n (as tokuraSetPlainConfig). */
TOKURA_API int tokuraSetRealConfig(tokurablas_t* handle, int n, int lanes_per_matrix, int threads_per_block);

/* Same computation and outputs as tokura_zgeev_batched_gpu, but it allocates
 * nothing and takes no workspace: it has no counterpart in the reference.
 * It is for callers that cannot allocate device memory when they need the
 * eigenvalues — e.g. plugins whose host application owns all device
 * memory. The staging area is a 32 MiB static device array in the library
 * (held by every GPU that loads it until exit), so 16*n*n*batch_count must be
 * <= tokura_zgeev_noalloc_max_bytes(): at most 512 matrices of order 64,
 * 2048 of order 32 (the shift hints of tokuraSetShiftHints are used when
 * their (8*n + 4)*batch_count bytes of estimates and phase state also fit:
 * up to 508 matrices of order 64, 2016 of order 32). The first call on a
 * device looks up that array's device address (a host-side query); the
 * address is kept for the life of the process, so calls
 * after a cudaDeviceReset of that device are not supported. The handle's
 * device must be the current device (else 1). All calls share the
 * array: calls that overlap on the GPU race and must be ordered by the
 * caller (e.g. one stream). A is not modified.
 * Returns the codes of tokura_zgeev_batched_gpu (no -5: there is no work),
 * -8 if the batch exceeds the static array, 1 if the current device is not
 * the handle's or the address lookup or the launch fails. */
TOKURA_API int tokura_zgeev_batched_gpu_noalloc(tokurablas_t* handle, int n, int batch_count, cuDoubleComplex* A,
                                                cuDoubleComplex* eigenvalues, char* flag, cudaStream_t cudastream);

/* Bounds-checked build only (the library compiled with -DTOKURA_DEBUG_BOUNDS,
 * the stand-in for a memory checker): attaches a device record of six 64-bit
 * words {violations, first row, first column, first order, int* sweeps,
 * sweeps length} that the kernels then fill: every matrix-element access is
 * checked against its matrix and, when outside, counted, recorded and
 * redirected in bounds (no trap, no wait); the plain kernels write each
 * matrix's QR sweep count to sweeps[j]. NULL detaches. Returns 0, 1 on a CUDA
 * failure, -2 in the release build (which checks nothing). */
TOKURA_API int tokuraDebugAttach(void* record);

/* Size in bytes of the static array behind tokura_zgeev_batched_gpu_noalloc (32 MiB). */
TOKURA_API size_t tokura_zgeev_noalloc_max_bytes(void);

#ifdef __cplusplus
}
#endif

#endif /* TOKURA_BLAS_EXT_GB300_H */
