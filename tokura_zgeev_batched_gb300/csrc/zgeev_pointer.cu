// tokura_zgeev_pointer_batched_gpu: cuBLAS-style device array of matrix pointers
// (see zgeev_layouts.cuh).
#include "zgeev_layouts.cuh"

extern "C" TOKURA_API int tokura_zgeev_pointer_batched_gpu(tokurablas_t* handle, int n, int batch_count,
                                                            const cuDoubleComplex* const* Aarray, int lda,
                                                            cuDoubleComplex* eigenvalues, cuDoubleComplex* work,
                                                            char* flag, cudaStream_t cudastream) {
  const int bad = tzg::check_common(handle, n, Aarray, eigenvalues, work, batch_count, flag);
  if (bad != 0) return bad;
  if (lda < n) return -8;
  const tzg::PointerBatch B{reinterpret_cast<const double2* const*>(Aarray), lda,
                            reinterpret_cast<double2*>(eigenvalues)};
  const cudaError_t err = tzg::launch_batch(tzg::plain_config_for(handle, n, batch_count), n, batch_count, B,
                                             reinterpret_cast<double2*>(work), flag, tzg::itmax_of(handle, n),
                                             cudastream, handle->balance_mode, tzg::use_shift_hints(handle, n),
                                            &handle->fj);
  return err == cudaSuccess ? 0 : 1;
}
