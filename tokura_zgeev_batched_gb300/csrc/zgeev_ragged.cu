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
  int lanes;          // lanes per matrix for this bin's tiles (1, 2, 4 or 8); a tile holds 32/lanes matrices
  long long stage;    // first staging element of this bin
};

constexpr int kMaxQueues = 256;  // per-SM work queues (SM count of the device, at most this)

struct RaggedPlan {
  int hist[kMaxN + 1];
  int cursor[kMaxN + 1];
  RaggedBin bins[kMaxN];  // bins[b] holds n = 64 - b
  int num_tiles;
  int ticket;             // unused by the solvers; kept zero
  int overflow;
  int pad;
  int queue[kMaxQueues];  // next position in each SM's share of the tiles
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

// Ticket -> bin: largest b with bins[b].tile_start <= t (bins are in ticket order).
__device__ __forceinline__ const RaggedBin& ragged_bin_of(const RaggedPlan* plan, int t) {
  int lo = 0, hi = kMaxN - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (plan->bins[mid].tile_start <= t) lo = mid; else hi = mid - 1;
  }
  return plan->bins[lo];
}

// Arguments of the ragged solvers.
struct RaggedArgs {
  const long long* offsets;
  const long long* eoff;
  const double2* A;
  double2* eig;          // forward: eigenvalues out
  const double2* lam;    // backward: forward eigenvalues
  const double2* gbar;   // backward: their gradients
  double2* gA;           // backward: gradient out
  double2* stage;
  long long region;      // backward: elements per staging region
  char* flag;
  const int* sorted;
  int itmax_override;
  int balance;           // forward: balancing mode
};

// Tile scheduling. Tiles are numbered in descending-work order; SM s owns
// tiles s, s+Q, s+2Q, ... (Q queues, one per SM), i.e. an equal share of every
// size class, and its warps take them in order through an atomic counter.
// When its share is used up a warp takes tiles from the other SMs' shares.
// Every atomicAdd returns a distinct position and a warp gives up after one
// pass over all queues, so nothing waits on anything. Unlike a single global
// ticket counter, the balance does not depend on the order in which blocks
// reach the SMs.
__device__ __forceinline__ unsigned sm_id() {
  unsigned id;
  asm volatile("mov.u32 %0, %%smid;" : "=r"(id));
  return id;
}

__device__ __forceinline__ int ragged_next_tile(RaggedPlan* plan, int queues, int num_tiles, int& q) {
  for (int tries = 0; tries < queues; ++tries) {
    const int pos = atomicAdd(&plan->queue[q], 1);
    const long long t = (long long)q + (long long)queues * pos;
    if (t < num_tiles) return (int)t;
    q = (q + 1 == queues) ? 0 : q + 1;  // this share is used up: move on to the next SM's share
  }
  return -1;
}

// Persistent solver with L lanes per matrix: takes tiles until all shares are
// used up and solves (kBackward = false) or differentiates (true) each one;
// kBalance (forward only) balances each matrix first with a.balance.
// One instantiation per lane width, so each has its own register budget.
template <int L, bool kBackward, bool kBalance = false>
__global__ void __launch_bounds__(128) zgeev_ragged_kernel(RaggedPlan* plan, RaggedArgs a, int queues) {
  constexpr int TW = 32 / L;
  const int lane = threadIdx.x & 31;
  const int slot = lane / L;
  const int num_tiles = plan->num_tiles;
  int q = (int)(sm_id() % (unsigned)queues);
  for (;;) {
    int t = 0;
    if (lane == 0) t = ragged_next_tile(plan, queues, num_tiles, q);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t < 0) break;
    const RaggedBin& bin = ragged_bin_of(plan, t);
    const int u = t - bin.tile_start;
    const int tw = min(TW, bin.count - u * TW);
    if (slot < tw) {
      const Group<L> G;
      const int nb = bin.n;
      const int j = a.sorted[bin.first + u * TW + slot];
      const long long nn = (long long)nb * nb;
      double2* base = a.stage + bin.stage + (long long)u * TW * nn + slot;
      const int itmax = a.itmax_override > 0 ? a.itmax_override : default_itmax(nb);
      int status;
      if (kBackward) {
        BwdViews V{MatView{base, nb, tw}, MatView{base + a.region, nb, tw}, MatView{base + 2 * a.region, nb, tw},
                   base + 3 * a.region, tw};
        status = backward_matrix<L>(a.A + a.offsets[j], a.lam + a.eoff[j], a.gbar + a.eoff[j],
                                    a.gA + a.offsets[j], V, G, itmax);
      } else {
        status = solve_matrix<L, kBalance>(a.A + a.offsets[j], MatView{base, nb, tw}, G, a.eig + a.eoff[j], itmax,
                                           a.balance);
      }
      if (G.rank == 0) a.flag[j] = (char)status;
    }
    __syncwarp();
  }
}

template <typename Kernel>
static int persistent_blocks(Kernel k, int sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

template <bool kBackward, bool kBalance = false>
static cudaError_t launch_ragged_kernel(int lanes, int sms, RaggedPlan* plan, const RaggedArgs& args,
                                        cudaStream_t stream) {
  const int queues = sms < 1 ? 1 : (sms > kMaxQueues ? kMaxQueues : sms);
  switch (lanes) {
    case 1:
      zgeev_ragged_kernel<1, kBackward, kBalance><<<persistent_blocks(zgeev_ragged_kernel<1, kBackward, kBalance>, sms),
                                                    128, 0, stream>>>(plan, args, queues);
      break;
    case 2:
      zgeev_ragged_kernel<2, kBackward, kBalance><<<persistent_blocks(zgeev_ragged_kernel<2, kBackward, kBalance>, sms),
                                                    128, 0, stream>>>(plan, args, queues);
      break;
    case 4:
      zgeev_ragged_kernel<4, kBackward, kBalance><<<persistent_blocks(zgeev_ragged_kernel<4, kBackward, kBalance>, sms),
                                                    128, 0, stream>>>(plan, args, queues);
      break;
    case 8:
      zgeev_ragged_kernel<8, kBackward, kBalance><<<persistent_blocks(zgeev_ragged_kernel<8, kBackward, kBalance>, sms),
                                                    128, 0, stream>>>(plan, args, queues);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Lane width of a ragged launch when the caller did not fix one: the smallest
// L such that a tile of 32/L order-64 matrices (the worst case the host can
// assume) stays below a third of the average work of an SM sub-partition,
// estimated from batch_count and the mean order sqrt(total_elements/batch).
int ragged_auto_lanes(int sms, int batch, long long total_elements) {
  const double mean_n = std::sqrt((double)total_elements / (double)batch);
  const auto work = [](double n) { return 25.0 * n * n * n + 400.0 * n * n; };
  const double per_smsp = (double)batch * work(mean_n) / (32.0 * 4.0 * (double)(sms > 0 ? sms : 1));
  int lanes = 1;
  while (lanes < 8 && work(64.0) / lanes > per_smsp / 3.0) lanes *= 2;
  return lanes;
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
                          void* work, char* flag, int itmax_override, cudaStream_t stream, int balance) {
  if (lanes == 0) lanes = ragged_auto_lanes(sms, batch, total_elements);
  if (!(lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8)) return cudaErrorInvalidValue;
  const RaggedLayout lay = ragged_layout(batch, total_elements);
  double2* stage = reinterpret_cast<double2*>(static_cast<char*>(work) + lay.stage_off);
  RaggedPlan* plan;
  int* sorted;
  const long long* eo;
  cudaError_t err = ragged_prepare(lanes, sms, batch, n, offsets, eig_offsets, total_elements, lay, work, flag,
                                   stream, &plan, &sorted, &eo);
  if (err != cudaSuccess) return err;
  const RaggedArgs args{offsets, eo, A, eig, nullptr, nullptr, nullptr, stage, total_elements, flag, sorted,
                        itmax_override, balance};
  if (balance != 0) return launch_ragged_kernel<false, true>(lanes, sms, plan, args, stream);
  return launch_ragged_kernel<false>(lanes, sms, plan, args, stream);
}

cudaError_t launch_ragged_backward(int lanes, int sms, int batch, const int* n, const long long* offsets,
                                   const long long* eig_offsets, long long total_elements, const double2* A,
                                   const double2* lam, const double2* gbar, double2* gA, void* work, char* flag,
                                   int itmax_override, cudaStream_t stream) {
  if (lanes == 0) lanes = ragged_auto_lanes(sms, batch, total_elements);
  if (!(lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8)) return cudaErrorInvalidValue;
  const RaggedLayout lay = ragged_layout(batch, total_elements, 4);
  double2* stage = reinterpret_cast<double2*>(static_cast<char*>(work) + lay.stage_off);
  RaggedPlan* plan;
  int* sorted;
  const long long* eo;
  cudaError_t err = ragged_prepare(lanes, sms, batch, n, offsets, eig_offsets, total_elements, lay, work, flag,
                                   stream, &plan, &sorted, &eo);
  if (err != cudaSuccess) return err;
  const RaggedArgs args{offsets, eo, A, nullptr, lam, gbar, gA, stage, total_elements, flag, sorted, itmax_override,
                        0};
  return launch_ragged_kernel<true>(lanes, sms, plan, args, stream);
}

}  // namespace tzg
