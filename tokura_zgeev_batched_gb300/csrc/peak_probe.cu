// FP64 peak probe: the denominator of the roofline fraction.
//
// The path is bound by the FP64 CUDA-core rate (no step is a dense
// contraction), which the device's published figures do not pin down for a
// given clock. This kernel measures it: every thread runs 8 independent
// dependent-FMA chains in 256-thread blocks, two blocks per SM (16 warps per
// SM, 4 per sub-partition), so the FP64 pipe of every SM sub-partition is
// saturated. Reported as FP64 FLOP/s (2 flops per FMA).
#include <cuda_runtime.h>

#include "../../include/tokura_blas_ext.h"

namespace tzg {

__global__ void __launch_bounds__(256) fp64_fma_probe_kernel(double* out, int iters, double b, double c) {
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = threadIdx.x * 1e-3 + k;
  for (int it = 0; it < iters; ++it) {
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
  }
  double s = 0.0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

}  // namespace tzg

extern "C" TOKURA_API int tokura_probe_fp64_peak(double* flops_per_second, double* scratch, int scratch_doubles,
                                                  cudaStream_t stream) {
  if (flops_per_second == nullptr || scratch == nullptr) return -1;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return 1;
  const int threads = 256, blocks = sms * 2;
  if (scratch_doubles < threads * blocks) return -2;
  const int iters = 4000;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  tzg::fp64_fma_probe_kernel<<<blocks, threads, 0, stream>>>(scratch, iters / 8, 0.999, 1e-3);  // warm-up
  cudaEventRecord(e0, stream);
  tzg::fp64_fma_probe_kernel<<<blocks, threads, 0, stream>>>(scratch, iters, 0.999, 1e-3);
  cudaEventRecord(e1, stream);
  const cudaError_t err = cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess || ms <= 0.f) return 1;
  *flops_per_second = 2.0 * 8.0 * (double)iters * threads * blocks / (ms * 1e-3);
  return 0;
}
