// TEST INFRASTRUCTURE — host glue that lets the reference library
// (hirokitokura/tokura_zgeev_batched, tokura_zgeev_batched_library/) be built
// and run unmodified for a GPU comparison. Never linked into the product.
//
// The reference's header declares three host functions that its sources call
// but never define (include/tokura_blas.h:142-148; called at
// src/tokura_zgeev_batched.cu:266 and :278 and src/tokura_zhseqr_helper.cu:41),
// so its library cannot link as shipped. This file restates them from what the
// reference's kernels and orchestration require:
//   * tokura_matrix_rearrangements_helper: the caller's "MatrixWise" layout
//     (matrix k column-major at A + k*n*n) becomes the kernels' "ElementWise"
//     layout (element (r, c) of matrix k at ((c*n + r)*batch + k),
//     src/tokura_zgehrd_MWB_kernel.cuh:170-174,220; src/tokura_zhseqr_MWB_kernel.cuh:620-625)
//     in the caller's A, with work[0 : n*n*batch] as scratch
//     (src/tokura_zgeev_batched.cu:226-228);
//   * tokura_zgehrd_helper: that rearrangement, then the Hessenberg kernel
//     tokura_zgehrd_normal_MWB_kernel<32> in place with block (32, T_n), T_n
//     the handle's tuned table, and the shared memory its indexing uses:
//     (n-1)*32 Householder entries plus 32*T_n reduction doubles
//     (src/tokura_zgehrd_MWB_kernel.cuh:176-178, 72, 18);
//   * tokura_eigenvaluesrearrangement_for_output: eigenvalues from the QR
//     kernel's interleaved work[n*n*batch + i*batch + k]
//     (src/tokura_zhseqr_MWB_kernel.cuh:110, 625) to the caller's
//     eigenvalues[i + k*n] (README.md:70).
// The transposes are plain grid-stride copies written for this glue.
#include <climits>
#include <cstddef>
#include <cstdio>  // the reference header calls fprintf without including it

#include <tokura_blas.h>

#include "tokura_zgehrd_MWB_kernel.cuh"

namespace {

__global__ void glue_matrixwise_to_elementwise(const cuDoubleComplex* __restrict__ src,
                                               cuDoubleComplex* __restrict__ dst, int n, int batch) {
  const long long total = (long long)n * n * batch;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long k = e % batch;   // matrix
    const long long rc = e / batch;  // c*n + r
    dst[e] = src[k * n * n + rc];
  }
}

__global__ void glue_eigenvalues_to_output(const cuDoubleComplex* __restrict__ src, cuDoubleComplex* __restrict__ dst,
                                           int n, int batch) {
  const long long total = (long long)n * batch;
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
       e += (long long)gridDim.x * blockDim.x) {
    const long long k = e / n;  // matrix
    const long long i = e % n;  // eigenvalue
    dst[e] = src[i * batch + k];
  }
}

unsigned grid_for(long long total) {
  long long g = (total + 255) / 256;
  return (unsigned)(g < 4096 ? (g > 0 ? g : 1) : 4096);
}

}  // namespace

void tokura_matrix_rearrangements_helper(tokurablas_t* handle) {
  if (handle->currentmatrixarrange == handle->nexttmatrixarrange) {  // already arranged
    handle->execstatus = TOKURA_BLAS_SUCCESS;
    return;
  }
  if (!(handle->currentmatrixarrange == MatrixWise && handle->nexttmatrixarrange == ElementWise)) {
    handle->execstatus = TOKURA_BLAS_FAIL;  // the only conversion the reference's kernels need
    return;
  }
  const int n = handle->zgeev_n, batch = handle->zgeev_batchcount;
  const long long total = (long long)n * n * batch;
  glue_matrixwise_to_elementwise<<<grid_for(total), 256, 0, handle->stream>>>(handle->zgeev_srcmatrices,
                                                                               handle->zgeev_wrkmatrices, n, batch);
  cudaError_t err = cudaGetLastError();
  if (err == cudaSuccess)
    err = cudaMemcpyAsync(handle->zgeev_srcmatrices, handle->zgeev_wrkmatrices, sizeof(cuDoubleComplex) * total,
                          cudaMemcpyDeviceToDevice, handle->stream);
  handle->currentmatrixarrange = ElementWise;
  handle->execstatus = err == cudaSuccess ? TOKURA_BLAS_SUCCESS : TOKURA_BLAS_FAIL;
}

void tokura_zgehrd_helper(tokurablas_t* handle) {
  handle->nexttmatrixarrange = ElementWise;
  tokura_matrix_rearrangements_helper(handle);
  if (handle->execstatus != TOKURA_BLAS_SUCCESS) return;
  const int n = handle->zgeev_n, batch = handle->zgeev_batchcount;
  const int t = handle->zgehrd_normal_MWB[n];
  const dim3 block(TARGET_CUDA_WARP, t);
  const dim3 grid((batch + TARGET_CUDA_WARP - 1) / TARGET_CUDA_WARP);
  const size_t smem = sizeof(cuDoubleComplex) * (size_t)(n - 1) * TARGET_CUDA_WARP +
                      sizeof(double) * (size_t)TARGET_CUDA_WARP * t;
  tokura_zgehrd_normal_MWB_kernel<TARGET_CUDA_WARP><<<grid, block, smem, handle->stream>>>(
      n, batch, handle->zgeev_srcmatrices);
  handle->execstatus = cudaGetLastError() == cudaSuccess ? TOKURA_BLAS_SUCCESS : TOKURA_BLAS_FAIL;
}

void tokura_eigenvaluesrearrangement_for_output(tokurablas_t* handle) {
  const int n = handle->zgeev_n, batch = handle->zgeev_batchcount;
  const long long total = (long long)n * batch;
  glue_eigenvalues_to_output<<<grid_for(total), 256, 0, handle->stream>>>(handle->zgeev_srceigenvalues,
                                                                           handle->zgeev_wrkeigenvalues, n, batch);
  handle->execstatus = cudaGetLastError() == cudaSuccess ? TOKURA_BLAS_SUCCESS : TOKURA_BLAS_FAIL;
}
