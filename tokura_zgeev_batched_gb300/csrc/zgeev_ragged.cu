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
//   5. solve:   a persistent grid whose warps take tiles from an atomic ticket
//               counter (no spin-waits) and run the same per-matrix solver as
//               the plain kernel. Tiles hold matrices of one n, so lanes of a
//               warp do identical amounts of Hessenberg work, and long tiles
//               are issued first so uneven QR iteration counts and sizes do
//               not leave SMs idle at the end.
#include "zgeev_backward.cuh"
#include "zgeev_internal.h"
#include "zgeev_lane.cuh"

namespace tzg {

struct RaggedBin {
  int n;
  int count;
  int first;          // first position of this bin in sorted[]
  int tile_start;     // first ticket of this bin
  int tiles;
  int pad;
  long long stage;    // first staging element of this bin
};

struct RaggedPlan {
  int hist[kMaxN + 1];
  int cursor[kMaxN + 1];
  RaggedBin bins[kMaxN];  // bins[b] holds n = 64 - b
  int num_tiles;
  int ticket;
  int overflow;
  int pad;
};

// Workspace layout (all sections 256-byte aligned).
struct RaggedLayout {
  size_t stage_off, plan_off, sorted_off, eoff_off, total;
};

static inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// `regions` staging areas of total_elements entries: 1 for the forward, 4 for
// the backward (T, Q, XY and the per-matrix vectors).
static RaggedLayout ragged_layout(int batch, long long total_elements, int regions = 1) {
  RaggedLayout l;
  l.stage_off = 0;
  l.plan_off = align256(l.stage_off + sizeof(double2) * (size_t)total_elements * (size_t)regions);
  l.sorted_off = align256(l.plan_off + sizeof(RaggedPlan));
  l.eoff_off = align256(l.sorted_off + sizeof(int) * (size_t)batch);
  l.total = align256(l.eoff_off + sizeof(long long) * (size_t)batch);
  return l;
}

size_t ragged_workspace_bytes(int batch, long long total_elements) {
  return ragged_layout(batch, total_elements).total;
}

size_t ragged_backward_workspace_bytes(int batch, long long total_elements) {
  return ragged_layout(batch, total_elements, 4).total;
}

__device__ __forceinline__ bool ragged_valid(int nj, long long off, long long total) {
  return nj >= 1 && nj <= kMaxN && off >= 0 && off <= total - (long long)nj * nj;
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

__global__ void ragged_plan_kernel(RaggedPlan* plan, int tile_width, long long total) {
  if (threadIdx.x != 0) return;
  int first = 0, tiles = 0;
  long long stage = 0;
  for (int b = 0; b < kMaxN; ++b) {
    const int nb = kMaxN - b;
    RaggedBin& bin = plan->bins[b];
    bin.n = nb;
    bin.count = plan->hist[nb];
    bin.first = first;
    bin.tile_start = tiles;
    bin.tiles = (bin.count + tile_width - 1) / tile_width;
    bin.stage = stage;
    first += bin.count;
    tiles += bin.tiles;
    stage += (long long)bin.count * nb * nb;
    plan->cursor[nb] = 0;
  }
  // Matrices may overlap in A; the staging area holds total elements only.
  plan->overflow = stage > total;
  plan->num_tiles = plan->overflow ? 0 : tiles;
  plan->ticket = 0;
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

// Resident blocks per SM the compiler is asked to allow (register budget).
#ifndef TZG_RAGGED_MIN_BLOCKS
#define TZG_RAGGED_MIN_BLOCKS 1
#endif

template <int L>
__global__ void __launch_bounds__(128, TZG_RAGGED_MIN_BLOCKS) zgeev_ragged_kernel(const int* __restrict__ n,
                                                           const long long* __restrict__ offsets,
                                                           const long long* __restrict__ eoff,
                                                           const double2* __restrict__ A, double2* __restrict__ eig,
                                                           double2* __restrict__ stage, char* __restrict__ flag,
                                                           RaggedPlan* plan, const int* __restrict__ sorted,
                                                           int itmax_override) {
  constexpr int TW = 32 / L;
  const int lane = threadIdx.x & 31;
  const int slot = lane / L;
  const int num_tiles = plan->num_tiles;
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(&plan->ticket, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= num_tiles) break;
    // Bin of ticket t: largest b with bins[b].tile_start <= t (bins are in ticket order).
    int lo = 0, hi = kMaxN - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (plan->bins[mid].tile_start <= t) lo = mid; else hi = mid - 1;
    }
    const RaggedBin& bin = plan->bins[lo];
    const int nb = bin.n;
    const int u = t - bin.tile_start;
    const int tw = min(TW, bin.count - u * TW);
    if (slot < tw) {
      const Group<L> G;
      const int j = sorted[bin.first + u * TW + slot];
      const long long nn = (long long)nb * nb;
      MatView M{stage + bin.stage + (long long)u * TW * nn + slot, nb, tw};
      const int itmax = itmax_override > 0 ? itmax_override : default_itmax(nb);
      const int status = solve_matrix<L>(A + offsets[j], M, G, eig + eoff[j], itmax);
      if (G.rank == 0) flag[j] = (char)status;
    }
    __syncwarp();
  }
}

// Backward over a ragged batch: same tiles and queue as the forward solver;
// each matrix's T/Q/XY/vector views sit at the same offset in four regions.
template <int L>
__global__ void __launch_bounds__(128) zgeev_ragged_backward_kernel(
    const int* __restrict__ n, const long long* __restrict__ offsets, const long long* __restrict__ eoff,
    const double2* __restrict__ A, const double2* __restrict__ lam, const double2* __restrict__ gbar,
    double2* __restrict__ gA, double2* __restrict__ stage, long long region, char* __restrict__ flag,
    RaggedPlan* plan, const int* __restrict__ sorted, int itmax_override) {
  constexpr int TW = 32 / L;
  const int lane = threadIdx.x & 31;
  const int slot = lane / L;
  const int num_tiles = plan->num_tiles;
  for (;;) {
    int t = 0;
    if (lane == 0) t = atomicAdd(&plan->ticket, 1);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t >= num_tiles) break;
    int lo = 0, hi = kMaxN - 1;
    while (lo < hi) {
      const int mid = (lo + hi + 1) >> 1;
      if (plan->bins[mid].tile_start <= t) lo = mid; else hi = mid - 1;
    }
    const RaggedBin& bin = plan->bins[lo];
    const int nb = bin.n;
    const int u = t - bin.tile_start;
    const int tw = min(TW, bin.count - u * TW);
    if (slot < tw) {
      const Group<L> G;
      const int j = sorted[bin.first + u * TW + slot];
      const long long nn = (long long)nb * nb;
      double2* base = stage + bin.stage + (long long)u * TW * nn + slot;
      BwdViews V{MatView{base, nb, tw}, MatView{base + region, nb, tw}, MatView{base + 2 * region, nb, tw},
                 base + 3 * region, tw};
      const int itmax = itmax_override > 0 ? itmax_override : default_itmax(nb);
      const int status =
          backward_matrix<L>(A + offsets[j], lam + eoff[j], gbar + eoff[j], gA + offsets[j], V, G, itmax);
      if (G.rank == 0) flag[j] = (char)status;
    }
    __syncwarp();
  }
}

template <int L>
static cudaError_t launch_ragged_solver(int sms, const int* n, const long long* offsets, const long long* eoff,
                                        const double2* A, double2* eig, double2* stage, char* flag, RaggedPlan* plan,
                                        const int* sorted, int itmax_override, cudaStream_t stream) {
  int per_sm = 0;
  cudaError_t err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zgeev_ragged_kernel<L>, 128, 0);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) per_sm = 1;
  zgeev_ragged_kernel<L><<<sms * per_sm, 128, 0, stream>>>(n, offsets, eoff, A, eig, stage, flag, plan, sorted,
                                                          itmax_override);
  return cudaGetLastError();
}

// Device-side planning shared by the forward and backward ragged solvers.
static cudaError_t ragged_prepare(int lanes, int sms, int batch, const int* n, const long long* offsets,
                                  const long long* eig_offsets, long long total_elements, const RaggedLayout& lay,
                                  void* work, char* flag, cudaStream_t stream, RaggedPlan** plan_out,
                                  int** sorted_out, const long long** eoff_out) {
  char* w = static_cast<char*>(work);
  RaggedPlan* plan = reinterpret_cast<RaggedPlan*>(w + lay.plan_off);
  int* sorted = reinterpret_cast<int*>(w + lay.sorted_off);
  long long* eoff = reinterpret_cast<long long*>(w + lay.eoff_off);
  const int tile_width = 32 / lanes;
  cudaError_t err = cudaMemsetAsync(plan, 0, sizeof(RaggedPlan), stream);
  if (err != cudaSuccess) return err;
  const int threads = 256;
  const int blocks = (int)min((long long)sms * 8, ((long long)batch + threads - 1) / threads);
  ragged_count_kernel<<<blocks, threads, 0, stream>>>(batch, n, offsets, total_elements, plan, flag);
  ragged_plan_kernel<<<1, 32, 0, stream>>>(plan, tile_width, total_elements);
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

template <typename Kernel>
static int persistent_blocks(Kernel k, int sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

cudaError_t launch_ragged(int lanes, int sms, int batch, const int* n, const long long* offsets,
                          const long long* eig_offsets, long long total_elements, const double2* A, double2* eig,
                          void* work, char* flag, int itmax_override, cudaStream_t stream) {
  const RaggedLayout lay = ragged_layout(batch, total_elements);
  double2* stage = reinterpret_cast<double2*>(static_cast<char*>(work) + lay.stage_off);
  RaggedPlan* plan;
  int* sorted;
  const long long* eo;
  cudaError_t err = ragged_prepare(lanes, sms, batch, n, offsets, eig_offsets, total_elements, lay, work, flag,
                                   stream, &plan, &sorted, &eo);
  if (err != cudaSuccess) return err;
  switch (lanes) {
    case 1:
      return launch_ragged_solver<1>(sms, n, offsets, eo, A, eig, stage, flag, plan, sorted, itmax_override, stream);
    case 2:
      return launch_ragged_solver<2>(sms, n, offsets, eo, A, eig, stage, flag, plan, sorted, itmax_override, stream);
    case 4:
      return launch_ragged_solver<4>(sms, n, offsets, eo, A, eig, stage, flag, plan, sorted, itmax_override, stream);
    default:
      return cudaErrorInvalidValue;
  }
}

cudaError_t launch_ragged_backward(int lanes, int sms, int batch, const int* n, const long long* offsets,
                                   const long long* eig_offsets, long long total_elements, const double2* A,
                                   const double2* lam, const double2* gbar, double2* gA, void* work, char* flag,
                                   int itmax_override, cudaStream_t stream) {
  const RaggedLayout lay = ragged_layout(batch, total_elements, 4);
  double2* stage = reinterpret_cast<double2*>(static_cast<char*>(work) + lay.stage_off);
  RaggedPlan* plan;
  int* sorted;
  const long long* eo;
  cudaError_t err = ragged_prepare(lanes, sms, batch, n, offsets, eig_offsets, total_elements, lay, work, flag,
                                   stream, &plan, &sorted, &eo);
  if (err != cudaSuccess) return err;
  switch (lanes) {
    case 1:
      zgeev_ragged_backward_kernel<1><<<persistent_blocks(zgeev_ragged_backward_kernel<1>, sms), 128, 0, stream>>>(
          n, offsets, eo, A, lam, gbar, gA, stage, total_elements, flag, plan, sorted, itmax_override);
      break;
    case 2:
      zgeev_ragged_backward_kernel<2><<<persistent_blocks(zgeev_ragged_backward_kernel<2>, sms), 128, 0, stream>>>(
          n, offsets, eo, A, lam, gbar, gA, stage, total_elements, flag, plan, sorted, itmax_override);
      break;
    case 4:
      zgeev_ragged_backward_kernel<4><<<persistent_blocks(zgeev_ragged_backward_kernel<4>, sms), 128, 0, stream>>>(
          n, offsets, eo, A, lam, gbar, gA, stage, total_elements, flag, plan, sorted, itmax_override);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tzg
