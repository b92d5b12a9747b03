// tokura_cgeev_batched_gpu: single-precision complex matrices in and eigenvalues
// out, FP64 inside (see zgeev_layouts.cuh).
#include "zgeev_layouts.cuh"

extern "C" TOKURA_API int tokura_cgeev_batched_gpu(tokurablas_t* handle, int n, int batch_count, const cuComplex* A,
                                                    cuComplex* eigenvalues, cuDoubleComplex* work, char* flag,
                                                    cudaStream_t cudastream) {
  const int bad = tzg::check_common(handle, n, A, eigenvalues, work, batch_count, flag);
  if (bad != 0) return bad;
  const tzg::Complex64Batch B{reinterpret_cast<const float2*>(A), reinterpret_cast<float2*>(eigenvalues), n};
  const cudaError_t err = tzg::launch_batch(tzg::plain_config_for(handle, n, batch_count), n, batch_count, B,
                                             reinterpret_cast<double2*>(work), flag, tzg::itmax_of(handle, n),
                                             cudastream, handle->balance_mode, tzg::use_shift_hints(handle, n),
                                            &handle->fj);
  return err == cudaSuccess ? 0 : 1;
}
