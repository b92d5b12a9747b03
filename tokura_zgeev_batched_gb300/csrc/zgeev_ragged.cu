// Ragged batched eigenvalue-only ZGEEV: matrices of individual orders 1..64,
// packed one after another, in one persistent launch.
//
// The reference supports one n per call only (README.md:5); this entry point
// has no counterpart there. Device-side planning (no host round trip, so the
// whole call can be captured in a CUDA graph):
//   1. count:   validate n[j] / offsets[j], histogram of n;
//   2. plan:    one block orders the size bins from n = 64 down to 1 and cuts
//               each bin into tiles of 32/L matrices (largest work first);
//   3. scatter: each matrix gets its slot inside its bin;
//   4. scan:    eigenvalue offsets = exclusive prefix sum of n (if the caller
//               passed none);
//   5. solve:   a persistent grid whose warps take tiles from per-SM shares
//               of the tile list through atomic counters (no spin-waits, see
//               ragged_next_tile) and run the same per-matrix solver as the
//               plain kernel. Tiles hold matrices of one n, so lanes of a warp
//               do identical amounts of Hessenberg work, and long tiles are
//               issued first so uneven QR iteration counts and sizes do not
//               leave SMs idle at the end.
#include <cmath>
#include <mutex>

#include "zgeev_ragged.cuh"

namespace tzg {

size_t ragged_workspace_bytes(int batch, long long total_elements) {
  return ragged_layout(batch, total_elements).total;
}

size_t ragged_backward_workspace_bytes(int batch, long long total_elements) {
  return ragged_layout(batch, total_elements, 4).total;
}

__global__ void ragged_count_kernel(int batch, const int* __restrict__ n, const long long* __restrict__ offsets,
                                    long long total, RaggedPlan* plan, char* __restrict__ flag) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < batch; j += gridDim.x * blockDim.x) {
    const int nj = n[j];
    if (ragged_valid(nj, offsets[j], total))
      atomicAdd(&plan->hist[nj], 1);
    else
      flag[j] = (char)kInvalidInput;
  }
}

// FP64 instructions per matrix of order n, per lane group (Hessenberg ~6.7 n^3,
// QR ~16 n^3, shifts/rotations/deflation ~O(n^2)); only ratios matter here.
__device__ __forceinline__ double ragged_work(int n) { return 25.0 * n * n * n + 400.0 * n * n; }

// Orders the bins from n = 64 down to 1 (largest work first) and cuts each
// into tiles of 32/L matrices. With fixed_lanes = 0 the lane width is chosen
// per bin (smallest L in {1, 2, 4, 8} keeping a tile below a third of the
// average load of an SM sub-partition); the solvers launched here pass the
// launch's lane width, since one kernel instantiation serves one width.
__global__ void ragged_plan_kernel(RaggedPlan* plan, int sms, int fixed_lanes, long long total) {
  if (threadIdx.x != 0) return;
  double W = 0.0;
  for (int nb = 1; nb <= kMaxN; ++nb) W += plan->hist[nb] * ragged_work(nb);
  const double cap = W / (32.0 * 4.0 * (double)(sms > 0 ? sms : 1)) / 3.0;
  int first = 0, tiles = 0;
  long long stage = 0;
  for (int b = 0; b < kMaxN; ++b) {
    const int nb = kMaxN - b;
    RaggedBin& bin = plan->bins[b];
    int lanes = fixed_lanes;
    if (lanes <= 0) {
      lanes = 1;
      while (lanes < 8 && ragged_work(nb) / lanes > cap) lanes *= 2;
    }
    const int tile_width = 32 / lanes;
    bin.n = nb;
    bin.count = plan->hist[nb];
    bin.first = first;
    bin.tile_start = tiles;
    bin.tiles = (bin.count + tile_width - 1) / tile_width;
    bin.lanes = lanes;
    bin.stage = stage;
    first += bin.count;
    tiles += bin.tiles;
    stage += (long long)bin.count * nb * nb;
    plan->cursor[nb] = 0;
  }
  // Matrices may overlap in A; the staging area holds total elements only.
  plan->overflow = stage > total;
  plan->num_tiles = plan->overflow ? 0 : tiles;
}

__global__ void ragged_scatter_kernel(int batch, const int* __restrict__ n, const long long* __restrict__ offsets,
                                      long long total, RaggedPlan* plan, int* __restrict__ sorted,
                                      char* __restrict__ flag) {
  for (int j = blockIdx.x * blockDim.x + threadIdx.x; j < batch; j += gridDim.x * blockDim.x) {
    const int nj = n[j];
    if (!ragged_valid(nj, offsets[j], total)) continue;
    if (plan->overflow) {
      flag[j] = (char)kInvalidInput;
      continue;
    }
    const int pos = atomicAdd(&plan->cursor[nj], 1);
    sorted[plan->bins[kMaxN - nj].first + pos] = j;
  }
}

// Exclusive prefix sum of n (invalid orders count as 0), one block.
__global__ void __launch_bounds__(1024) ragged_scan_kernel(int batch, const int* __restrict__ n,
                                                           long long* __restrict__ eoff) {
  __shared__ long long part[1024];
  const int t = threadIdx.x;
  const long long per = ((long long)batch + blockDim.x - 1) / blockDim.x;
  const long long lo = min((long long)batch, t * per), hi = min((long long)batch, lo + per);
  long long s = 0;
  for (long long j = lo; j < hi; ++j) {
    const int nj = n[j];
    s += (nj >= 1 && nj <= kMaxN) ? nj : 0;
  }
  part[t] = s;
  __syncthreads();
  for (int o = 1; o < blockDim.x; o <<= 1) {
    const long long v = t >= o ? part[t - o] : 0;
    __syncthreads();
    part[t] += v;
    __syncthreads();
  }
  long long run = part[t] - s;
  for (long long j = lo; j < hi; ++j) {
    eoff[j] = run;
    const int nj = n[j];
    run += (nj >= 1 && nj <= kMaxN) ? nj : 0;
  }
}

// Device-side planning shared by the forward and backward ragged solvers.
cudaError_t ragged_prepare(int lanes, int sms, int batch, const int* n, const long long* offsets,
                           const long long* eig_offsets, long long total_elements, const RaggedLayout& lay,
                           void* work, char* flag, cudaStream_t stream, RaggedPlan** plan_out, int** sorted_out,
                           const long long** eoff_out) {
  char* w = static_cast<char*>(work);
  RaggedPlan* plan = reinterpret_cast<RaggedPlan*>(w + lay.plan_off);
  int* sorted = reinterpret_cast<int*>(w + lay.sorted_off);
  long long* eoff = reinterpret_cast<long long*>(w + lay.eoff_off);
  cudaError_t err = cudaMemsetAsync(plan, 0, sizeof(RaggedPlan), stream);
  if (err != cudaSuccess) return err;
  const int threads = 256;
  const int blocks = (int)min((long long)sms * 8, ((long long)batch + threads - 1) / threads);
  ragged_count_kernel<<<blocks, threads, 0, stream>>>(batch, n, offsets, total_elements, plan, flag);
  ragged_plan_kernel<<<1, 32, 0, stream>>>(plan, sms, lanes, total_elements);
  ragged_scatter_kernel<<<blocks, threads, 0, stream>>>(batch, n, offsets, total_elements, plan, sorted, flag);
  const long long* eo = eig_offsets;
  if (eo == nullptr) {
    ragged_scan_kernel<<<1, 1024, 0, stream>>>(batch, n, eoff);
    eo = eoff;
  }
  *plan_out = plan;
  *sorted_out = sorted;
  *eoff_out = eo;
  return cudaGetLastError();
}

cudaError_t launch_ragged(int lanes, int sms, int batch, const int* n, const long long* offsets,
                          const long long* eig_offsets, long long total_elements, const double2* A, double2* eig,
                          void* work, char* flag, int itmax_override, cudaStream_t stream, int balance,
                          int hint_min_n, const ForkJoin* fj, int scaled_min_n) {
  // Shift hints for the matrices of order >= hint_min_n (0: none).
  const bool hints = hint_min_n > 0 && hint_min_n <= kMaxN;
  // lanes == 0: each size bin gets its own lane width from the planner (ragged_plan_kernel).
  if (!(lanes == 0 || lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8)) return cudaErrorInvalidValue;
  const RaggedLayout lay = ragged_layout(batch, total_elements);
  char* w = static_cast<char*>(work);
  double2* stage = reinterpret_cast<double2*>(w + lay.stage_off);
  float2* est = hints ? reinterpret_cast<float2*>(w + lay.est_off) : nullptr;
  int* state = reinterpret_cast<int*>(w + lay.state_off);
  const bool split = hints && fj != nullptr && fj->aux != nullptr;
  std::unique_lock<std::mutex> lock;
  cudaError_t err = cudaSuccess;
  if (split) {  // the estimator starts first, beside the planning and the prepare phase
    lock = std::unique_lock<std::mutex>(*fj->mu);
    err = ragged_fork_estimates(sms, batch, n, offsets, total_elements, A, est, hint_min_n, stream, *fj);
  } else if (hints) {
    err = launch_ragged_estimates(sms, batch, n, offsets, total_elements, A, est, hint_min_n, stream);
  }
  if (err != cudaSuccess) return err;
  RaggedPlan* plan;
  int* sorted;
  const long long* eo;
  err = ragged_prepare(lanes, sms, batch, n, offsets, eig_offsets, total_elements, lay, work, flag, stream, &plan,
                       &sorted, &eo);
  if (err != cudaSuccess) return err;
  const RaggedArgs args{offsets, eo, A, eig, nullptr, nullptr, nullptr, stage, total_elements, flag, sorted,
                        itmax_override, balance, est, state, hint_min_n, scaled_min_n};
  if (split) return ragged_launch_phases(lanes, sms, plan, args, balance != 0, stream, *fj);
  if (balance != 0) return launch_ragged_kernel<false, true, kPhaseAll>(lanes, sms, plan, args, stream);
  return launch_ragged_kernel<false, false, kPhaseAll>(lanes, sms, plan, args, stream);
}


}  // namespace tzg
