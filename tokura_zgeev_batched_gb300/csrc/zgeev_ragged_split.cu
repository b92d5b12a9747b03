// Ragged forward with FP32 shift hints, in two persistent launches:
//   caller's stream: [planning] [kPrepare: stage + Hessenberg of every tile] --join--> [kQR]
//   second stream:   [FP32 estimator over the batch] ----------------------------^
// As for uniform batches (zgeev_plain.cuh), the estimator (shared memory,
// FP32) runs beside the FP64 Hessenberg phase, and the QR phase uses the
// nearest unused estimate as the first shift after each deflation.
#include "zgeev_ragged.cuh"

namespace tzg {

// One warp per matrix of order min_n .. max_n, in index order, with shared
// memory for order max_n; invalid entries (the planner flags them) and other
// orders are skipped.
__global__ void __launch_bounds__(32) ragged_estimate_kernel(int batch, const int* __restrict__ n,
                                                             const long long* __restrict__ offsets, long long total,
                                                             const double2* __restrict__ A, float2* __restrict__ est,
                                                             int min_n, int max_n) {
  extern __shared__ float2 ragged_estimate_smem[];
  for (long long j = blockIdx.x; j < batch; j += gridDim.x) {
    const int nj = n[j];
    const long long off = offsets[j];
    if (nj < min_n || nj > max_n || !ragged_valid(nj, off, total)) continue;
    estimate_matrix(SrcContig{A + off}, nj, ragged_estimate_smem, est + j * kMaxN);
  }
}

// The estimator is bound by the latency of its rotation rounds, so its speed
// is the number of matrices in flight, which shared memory limits: one band
// of orders per launch, each with shared memory for its largest order (n = 64:
// 33 KB, 6 warps per SM; n = 47: 18 KB, 12; n = 31: 8 KB, as many as the
// registers allow), largest orders first.
cudaError_t launch_ragged_estimates(int sms, int batch, const int* n, const long long* offsets, long long total,
                                    const double2* A, float2* est, int min_n, cudaStream_t stream) {
  static const int kBandTop[3] = {kMaxN, 47, 31};
  for (int b = 0; b < 3; ++b) {
    const int hi = kBandTop[b], lo = b + 1 < 3 ? kBandTop[b + 1] + 1 : 1;
    const int from = min_n > lo ? min_n : lo;
    if (from > hi) continue;
    const size_t smem = sizeof(float2) * hi * (hi + 1);
    int per_sm = 0;
    const cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, ragged_estimate_kernel, 32, smem);
    if (err != cudaSuccess) return err;
    if (per_sm < 1) per_sm = 1;
    long long blocks = (long long)(sms > 0 ? sms : 1) * per_sm;
    if (blocks > batch) blocks = batch;
    ragged_estimate_kernel<<<(unsigned)blocks, 32, smem, stream>>>(batch, n, offsets, total, A, est, from, hi);
    const cudaError_t le = cudaGetLastError();
    if (le != cudaSuccess) return le;
  }
  return cudaSuccess;
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
