/*
 * tokura_blas.h — C ABI of the GB300-native batched eigenvalue-only ZGEEV.
 *
 * Drop-in for the public API of hirokitokura/tokura_zgeev_batched
 * (tokura_zgeev_batched_library/include/tokura_blas.h:129-151, documented in
 * README.md:26-74). Same names, argument order, argument meaning, return
 * codes and data layouts. Differences a caller may notice:
 *   - every symbol here has C linkage (the reference exports C++-mangled
 *     names; the library also exports those mangled names as forwarding
 *     shims, so objects built against the reference header still link);
 *   - tokurablas_t is opaque (the reference exposes its fields, which no
 *     reference caller reads);
 *   - A is read but not modified (the reference clobbers it; callers must
 *     still assume nothing about A after the call, as README.md:69 says);
 *   - the handle is never written by a call, so one handle may be used from
 *     several host threads at once.
 *
 * All data pointers are device pointers owned by the caller. All calls are
 * asynchronous on the given stream (NULL = legacy default stream).
 */
#ifndef TOKURA_BLAS_GB300_H
#define TOKURA_BLAS_GB300_H

#include <stddef.h>
#include <cuda_runtime_api.h>
#include <cuComplex.h>

/* Public constants and enums of the reference header
 * (tokura_zgeev_batched_library/include/tokura_blas.h:12-48), same names and
 * values, so that caller source naming them compiles unchanged. This library
 * reads none of them: the tuning batch counts describe the reference's
 * build-time tuner (replaced by tokuraAutotune), and the layout/method enums
 * name internal stages the reference keeps in its (here opaque) handle. */
#define TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE 64
#define TARGET_CUDA_WARP 32
#define TOKURA_ZGEEV_BATCHED_GEHRD_TUNING_BATCHCOUNT (1024 * 8)
#define TOKURA_ZGEEV_BATCHED_HSEQR_TUNING_BATCHCOUNT (1024 * 8)
#define TOKURA_ZGEEV_BATCHED_TUNING_COUNT 1

typedef enum { TOKURA_BLAS_SUCCESS = 0, TOKURA_BLAS_FAIL } TOKURA_ZGEEV_BATCHED_STATUS;

typedef enum { MatrixWise = 0, ElementWise, RowWise, NotSet } TOKURA_ZGEEV_BATCHED_MATRIX_ARRANGEMENT;

typedef enum { ZGEHRD_NORMAL_MWB_METHOD = 0, ZGEHRD_SHARED_MWB_METHOD } TOKURA_ZGEHRD_BATCHED_WHICHFAST;

typedef enum { ZHSEQR_NORMAL_MWB = 0 } TOKURA_ZHSEQR_BATCHED_WHICHFAST;

#if defined(__GNUC__)
#define TOKURA_API __attribute__((visibility("default")))
#else
#define TOKURA_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tokurablas_t tokurablas_t;

/* Allocates a handle bound to the current CUDA device.
 * Returns 0 on success, -1 if handle is NULL or host allocation fails,
 * 1 if the device cannot be queried.
 * Replaces tokuraCreate (tokura_zgeev_batched.cu:64-160). */
TOKURA_API int tokuraCreate(tokurablas_t** handle);

/* Frees a handle (NULL is accepted). Returns 0.
 * Replaces tokuraDestroy (tokura_zgeev_batched.cu:161-190). */
TOKURA_API int tokuraDestroy(tokurablas_t* handle);

/* Workspace bytes for tokura_zgeev_batched_gpu: 16*n*n*batch + 16*n*batch,
 * the reference's formula; (size_t)-1 if n is not in [1,64],
 * (size_t)-2 if batch_count <= 0.
 * Replaces tokura_get_zgeeveigenvaluesgetworspacesize (tokura_zgeev_batched.cu:192-210). */
TOKURA_API size_t tokura_get_zgeeveigenvaluesgetworspacesize(int n, int batch_count);

/* All eigenvalues of batch_count n-by-n complex matrices (1 <= n <= 64).
 * A: batch_count matrices, column-major, one after another (16*n*n bytes each).
 * eigenvalues[i + j*n]: i-th eigenvalue of matrix j (Schur-diagonal order).
 * work: at least tokura_get_zgeeveigenvaluesgetworspacesize(n, batch_count) bytes.
 * flag[j]: 0 if all eigenvalues of matrix j converged, 1 if the QR iteration
 * cap was hit, 2 if matrix j holds Inf or NaN (its eigenvalues are NaN).
 * Returns 0 on success; -1 NULL handle, -2 n out of range, -3 A NULL,
 * -4 eigenvalues NULL, -5 work NULL, -6 batch_count <= 0, -7 flag NULL;
 * 1 if the kernel could not be launched.
 * Replaces tokura_zgeev_batched_gpu (tokura_zgeev_batched.cu:212-285). */
TOKURA_API int tokura_zgeev_batched_gpu(tokurablas_t* handle, int n, int batch_count, cuDoubleComplex* A,
                             cuDoubleComplex* eigenvalues, cuDoubleComplex* work, char* flag,
                             cudaStream_t cudastream);

#ifdef __cplusplus
}
#endif

#ifdef __cplusplus
#include <stdio.h>
/* The reference header's error-print helper (tokura_blas.h:152-160): prints
 * a failed CUDA status with file and line and carries on (it never aborts).
 * C++ only, as in the reference (default argument). */
#ifndef gpuErrchk
#define gpuErrchk(ans) \
  { gpuAssert((ans), __FILE__, __LINE__); }
#endif
inline void gpuAssert(cudaError_t code, const char* file, int line, bool abort = true) {
  (void)abort;
  if (code != cudaSuccess) fprintf(stderr, "GPUassert: %s %s %d\n", cudaGetErrorString(code), file, line);
}
#endif

#endif /* TOKURA_BLAS_GB300_H */
