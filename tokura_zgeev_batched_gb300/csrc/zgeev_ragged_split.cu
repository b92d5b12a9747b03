// Ragged forward with FP32 shift hints, in two persistent launches:
//   caller's stream: [planning] [kPrepare: stage + Hessenberg of every tile] --join--> [kQR]
//   second stream:   [FP32 estimator over the batch] ----------------------------^
// As for uniform batches (zgeev_plain.cuh), the estimator (shared memory,
// FP32) runs beside the FP64 Hessenberg phase, and the QR phase uses the
// nearest unused estimate as the first shift after each deflation.
#include "zgeev_ragged.cuh"

namespace tzg {

// One warp per matrix in index order (shared memory sized for n = 64);
// invalid entries (the planner flags them) and orders below min_n are skipped.
__global__ void __launch_bounds__(32) ragged_estimate_kernel(int batch, const int* __restrict__ n,
                                                             const long long* __restrict__ offsets, long long total,
                                                             const double2* __restrict__ A, float2* __restrict__ est,
                                                             int min_n) {
  extern __shared__ float2 ragged_estimate_smem[];
  for (long long j = blockIdx.x; j < batch; j += gridDim.x) {
    const int nj = n[j];
    const long long off = offsets[j];
    if (nj < min_n || !ragged_valid(nj, off, total)) continue;
    estimate_matrix(SrcContig{A + off}, nj, ragged_estimate_smem, est + j * kMaxN);
  }
}

cudaError_t launch_ragged_estimates(int sms, int batch, const int* n, const long long* offsets, long long total,
                                    const double2* A, float2* est, int min_n, cudaStream_t stream) {
  const size_t smem = sizeof(float2) * kMaxN * (kMaxN + 1);
  int per_sm = 0;
  const cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ragged_estimate_kernel, 32, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) per_sm = 1;
  long long blocks = (long long)(sms > 0 ? sms : 1) * per_sm;
  if (blocks > batch) blocks = batch;
  ragged_estimate_kernel<<<(unsigned)blocks, 32, smem, stream>>>(batch, n, offsets, total, A, est, min_n);
  return cudaGetLastError();
}

cudaError_t ragged_fork_estimates(int sms, int batch, const int* n, const long long* offsets, long long total,
                                  const double2* A, float2* est, int min_n, cudaStream_t stream,
                                  const ForkJoin& fj) {
  cudaError_t err;
  if ((err = cudaEventRecord(fj.fork, stream)) != cudaSuccess) return err;
  if ((err = cudaStreamWaitEvent(fj.aux, fj.fork, 0)) != cudaSuccess) return err;
  if ((err = launch_ragged_estimates(sms, batch, n, offsets, total, A, est, min_n, fj.aux)) != cudaSuccess)
    return err;
  return cudaEventRecord(fj.join, fj.aux);
}

cudaError_t ragged_launch_phases(int lanes, int sms, RaggedPlan* plan, const RaggedArgs& args, bool balance,
                                 cudaStream_t stream, const ForkJoin& fj) {
  cudaError_t err = balance ? launch_ragged_kernel<false, true, kPhasePrepare>(lanes, sms, plan, args, stream)
                            : launch_ragged_kernel<false, false, kPhasePrepare>(lanes, sms, plan, args, stream);
  if (err != cudaSuccess) return err;
  if ((err = cudaStreamWaitEvent(stream, fj.join, 0)) != cudaSuccess) return err;
  return launch_ragged_kernel<false, false, kPhaseQR>(lanes, sms, plan, args, stream);
}

}  // namespace tzg
