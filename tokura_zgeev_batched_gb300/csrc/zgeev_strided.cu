// tokura_zgeev_strided_batched_gpu: column-major matrices with leading dimension lda,
// strideA elements apart; eigenvalue vectors strideW apart (see zgeev_layouts.cuh).
#include "zgeev_layouts.cuh"

extern "C" TOKURA_API int tokura_zgeev_strided_batched_gpu(tokurablas_t* handle, int n, int batch_count,
                                                            const cuDoubleComplex* A, int lda, long long strideA,
                                                            cuDoubleComplex* eigenvalues, long long strideW,
                                                            cuDoubleComplex* work, char* flag,
                                                            cudaStream_t cudastream) {
  const int bad = tzg::check_common(handle, n, A, eigenvalues, work, batch_count, flag);
  if (bad != 0) return bad;
  if (lda < n) return -8;
  if (strideA < 0 || strideW < n) return -9;
  const tzg::StridedBatch B{reinterpret_cast<const double2*>(A), lda, strideA, strideW,
                            reinterpret_cast<double2*>(eigenvalues)};
  const cudaError_t err = tzg::launch_batch(tzg::plain_config_for(handle, n, batch_count), n, batch_count, B,
                                             reinterpret_cast<double2*>(work), flag, tzg::itmax_of(handle, n),
                                             cudastream, handle->balance_mode, tzg::use_shift_hints(handle, n),
                                            &handle->fj);
  return err == cudaSuccess ? 0 : 1;
}
