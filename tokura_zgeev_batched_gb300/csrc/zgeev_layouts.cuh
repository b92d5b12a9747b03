// Eigenvalue entry points for other input layouts and precisions:
//   tokura_zgeev_strided_batched_gpu  — column-major with leading dimension
//                                       lda, matrices strideA elements apart,
//                                       eigenvalue vectors strideW apart
//   tokura_zgeev_pointer_batched_gpu  — cuBLAS-style device array of matrix
//                                       pointers (leading dimension lda)
//   tokura_cgeev_batched_gpu          — single-precision complex matrices in
//                                       and eigenvalues out, FP64 inside
// The reference takes only contiguous n x n FP64 matrices
// (tokura_zgeev_batched.cu:212-285). Each path runs the plain solver
// (zgeev_plain.cuh) with its own batch type, so results are bitwise equal to
// the contiguous entry point on the same matrix entries: only the addresses
// (and the FP32->FP64 widening / FP64->FP32 rounding) differ.
#pragma once

#include "../../include/tokura_blas_ext.h"
#include "tokura_handle.h"
#include "zgeev_plain.cuh"

namespace tzg {

// Checks shared by the three entry points, in the reference's order
// (tokura_zgeev_batched.cu:237-264).
inline int check_common(const tokurablas_t* handle, int n, const void* A, const void* eigenvalues, const void* work,
                        int batch_count, const char* flag) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (A == nullptr) return -3;
  if (eigenvalues == nullptr) return -4;
  if (work == nullptr) return -5;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  return 0;
}

inline int itmax_of(const tokurablas_t* handle, int n) {
  return handle->itmax_override > 0 ? handle->itmax_override : default_itmax(n);
}

}  // namespace tzg
