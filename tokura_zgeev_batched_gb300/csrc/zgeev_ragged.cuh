// Ragged batches: shared definitions of the planner, the work queues and the
// persistent solver (planning and the single-phase launches are in
// zgeev_ragged.cu, the two-phase forward with FP32 shift hints in
// zgeev_ragged_split.cu).
#pragma once

#include "zgeev_backward.cuh"
#include "zgeev_estimate.cuh"
#include "zgeev_internal.h"
#include "zgeev_lane.cuh"
#include "zgeev_scaled_qr.cuh"

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
  int overflow;
  int queue[kMaxQueues];     // next position in each SM's share of the tiles
  int queue_qr[kMaxQueues];  // the same for the QR phase of a split solve
};

// Workspace layout (all sections 256-byte aligned). The forward also holds the
// FP32 shift hints (kMaxN float2 per matrix) and the per-matrix phase state.
struct RaggedLayout {
  size_t stage_off, plan_off, sorted_off, eoff_off, est_off, state_off, total;
};

inline size_t align256(size_t x) { return (x + 255) & ~size_t(255); }

// `regions` staging areas of total_elements entries: 1 for the forward, 4 for
// the backward (T, Q, XY and the per-matrix vectors).
inline RaggedLayout ragged_layout(int batch, long long total_elements, int regions = 1) {
  RaggedLayout l;
  l.stage_off = 0;
  l.plan_off = align256(l.stage_off + sizeof(double2) * (size_t)total_elements * (size_t)regions);
  l.sorted_off = align256(l.plan_off + sizeof(RaggedPlan));
  l.eoff_off = align256(l.sorted_off + sizeof(int) * (size_t)batch);
  const bool fwd = regions == 1;
  l.est_off = align256(l.eoff_off + sizeof(long long) * (size_t)batch);
  l.state_off = align256(l.est_off + (fwd ? sizeof(float2) * kMaxN * (size_t)batch : 0));
  l.total = align256(l.state_off + (fwd ? sizeof(int) * (size_t)batch : 0));
  return l;
}

__device__ __forceinline__ bool ragged_valid(int nj, long long off, long long total) {
  return nj >= 1 && nj <= kMaxN && off >= 0 && off <= total - (long long)nj * nj;
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
  const float2* est;     // forward: FP32 shift hints, kMaxN per matrix (or null)
  int* state;            // forward, split solve: pre-scaling exponent or kStateDone per matrix
  int est_min_n;         // forward: orders from which est holds hints
  int scaled_min_n = 65;  // QR with scaled rotations from order max(7, lanes * scaled_min_n); > 64: never
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

__device__ __forceinline__ int ragged_next_tile(int* queue, int queues, int num_tiles, int& q) {
  for (int tries = 0; tries < queues; ++tries) {
    const int pos = atomicAdd(&queue[q], 1);
    const long long t = (long long)q + (long long)queues * pos;
    if (t < num_tiles) return (int)t;
    q = (q + 1 == queues) ? 0 : q + 1;  // this share is used up: move on to the next SM's share
  }
  return -1;
}

// Solves (kBackward = false) or differentiates (true) the matrices of tile t
// of `bin` with L lanes per matrix; kBalance (forward only) balances each
// matrix first with a.balance. The forward runs whole (kPhaseAll) or split:
// kPhasePrepare stages and reduces every matrix and records its state,
// kPhaseQR finishes it with the hints.
template <int L, bool kBackward, bool kBalance, int kPhase>
__device__ __forceinline__ void ragged_tile(const RaggedBin& bin, int t, const RaggedArgs& a, int lane) {
  constexpr int TW = 32 / L;
  const int slot = lane / L;
  const int u = t - bin.tile_start;
  const int tw = min(TW, bin.count - u * TW);
  if (slot >= tw) return;  // whole lane groups leave together
  const Group<L> G;
  const int nb = bin.n;
  const int j = a.sorted[bin.first + u * TW + slot];
  const long long nn = (long long)nb * nb;
  double2* base = a.stage + bin.stage + (long long)u * TW * nn + slot;
  const int itmax = a.itmax_override > 0 ? a.itmax_override : default_itmax(nb);
  const float2* est = a.est != nullptr && nb >= a.est_min_n ? a.est + (long long)j * kMaxN : nullptr;
  // scaled rotations from order max(7, L * scaled_min_n) (a.scaled_min_n > 64: never)
  const bool scaled = a.scaled_min_n <= kMaxN && nb >= kScaledMinN && nb >= L * a.scaled_min_n;
  int status = kPrepared;  // kPrepared: no flag to write yet
  if (kBackward) {
    BwdViews V{MatView{base, nb, tw}, MatView{base + a.region, nb, tw}, MatView{base + 2 * a.region, nb, tw},
               base + 3 * a.region, tw};
    status = backward_matrix<L>(a.A + a.offsets[j], a.lam + a.eoff[j], a.gbar + a.eoff[j], a.gA + a.offsets[j], V,
                                G, itmax, scaled ? nb : kMaxN + 1);
  } else if (kPhase == kPhaseAll) {
    int shift;
    const MatView M{base, nb, tw};
    status = prepare_matrix<L, kBalance>(SrcContig{a.A + a.offsets[j]}, M, G, a.eig + a.eoff[j], a.balance, shift);
    if (status == kPrepared)
      status = scaled ? qr_eigenvalues_scaled<L>(M, G, a.eig + a.eoff[j], shift, itmax, est)
                      : qr_eigenvalues<L>(M, G, a.eig + a.eoff[j], shift, itmax, est);
  } else if (kPhase == kPhasePrepare) {
    int shift;
    status = prepare_matrix<L, kBalance>(SrcContig{a.A + a.offsets[j]}, MatView{base, nb, tw}, G, a.eig + a.eoff[j],
                                         a.balance, shift);
    if (G.rank == 0) a.state[j] = status != kPrepared ? kStateDone : shift;
  } else {
    const int s = a.state[j];
    if (s != kStateDone)
      status = scaled ? qr_eigenvalues_scaled<L>(MatView{base, nb, tw}, G, a.eig + a.eoff[j], s, itmax, est)
                      : qr_eigenvalues<L>(MatView{base, nb, tw}, G, a.eig + a.eoff[j], s, itmax, est);
  }
  if (G.rank == 0 && status != kPrepared) a.flag[j] = (char)status;
}

// Persistent solver: takes tiles until all shares are used up. kL = 1, 2, 4 or
// 8 fixes the lanes per matrix for every tile (one instantiation per width, so
// each has its own register budget); kL = 0 takes each tile's width from its
// bin (the planner's per-bin choice; one kernel holds all four variants).
template <int kL, bool kBackward, bool kBalance, int kPhase>
__global__ void __launch_bounds__(128) zgeev_ragged_kernel(RaggedPlan* plan, RaggedArgs a, int queues) {
  const int lane = threadIdx.x & 31;
  const int num_tiles = plan->num_tiles;
  int* queue = kPhase == kPhaseQR ? plan->queue_qr : plan->queue;
  int q = (int)(sm_id() % (unsigned)queues);
  for (;;) {
    int t = 0;
    if (lane == 0) t = ragged_next_tile(queue, queues, num_tiles, q);
    t = __shfl_sync(0xffffffffu, t, 0);
    if (t < 0) break;
    const RaggedBin& bin = ragged_bin_of(plan, t);
    if (kL != 0) {
      ragged_tile<kL == 0 ? 1 : kL, kBackward, kBalance, kPhase>(bin, t, a, lane);
    } else {
      switch (bin.lanes) {  // warp-uniform
        case 1: ragged_tile<1, kBackward, kBalance, kPhase>(bin, t, a, lane); break;
        case 2: ragged_tile<2, kBackward, kBalance, kPhase>(bin, t, a, lane); break;
        case 4: ragged_tile<4, kBackward, kBalance, kPhase>(bin, t, a, lane); break;
        default: ragged_tile<8, kBackward, kBalance, kPhase>(bin, t, a, lane); break;
      }
    }
    __syncwarp();
  }
}

template <typename Kernel>
inline int persistent_blocks(Kernel k, int sms) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 128, 0) != cudaSuccess || per_sm < 1) per_sm = 1;
  return sms * per_sm;
}

template <int L, bool kBackward, bool kBalance, int kPhase>
inline cudaError_t launch_ragged_l(int sms, RaggedPlan* plan, const RaggedArgs& args, cudaStream_t stream) {
  const auto k = zgeev_ragged_kernel<L, kBackward, kBalance, kPhase>;
  if (kPhase != kPhaseAll) {  // shared memory for the FP32 estimator running beside it
    const cudaError_t err =
        cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (err != cudaSuccess) return err;
  }
  const int queues = sms < 1 ? 1 : (sms > kMaxQueues ? kMaxQueues : sms);
  k<<<persistent_blocks(k, sms), 128, 0, stream>>>(plan, args, queues);
  return cudaGetLastError();
}

template <bool kBackward, bool kBalance, int kPhase>
inline cudaError_t launch_ragged_kernel(int lanes, int sms, RaggedPlan* plan, const RaggedArgs& args,
                                        cudaStream_t stream) {
  switch (lanes) {
    case 0: return launch_ragged_l<0, kBackward, kBalance, kPhase>(sms, plan, args, stream);
    case 1: return launch_ragged_l<1, kBackward, kBalance, kPhase>(sms, plan, args, stream);
    case 2: return launch_ragged_l<2, kBackward, kBalance, kPhase>(sms, plan, args, stream);
    case 4: return launch_ragged_l<4, kBackward, kBalance, kPhase>(sms, plan, args, stream);
    case 8: return launch_ragged_l<8, kBackward, kBalance, kPhase>(sms, plan, args, stream);
    default: return cudaErrorInvalidValue;
  }
}

// Device-side planning shared by the forward and backward solvers (zgeev_ragged.cu).
cudaError_t ragged_prepare(int lanes, int sms, int batch, const int* n, const long long* offsets,
                           const long long* eig_offsets, long long total_elements, const RaggedLayout& lay,
                           void* work, char* flag, cudaStream_t stream, RaggedPlan** plan_out, int** sorted_out,
                           const long long** eoff_out);

// Defined in zgeev_ragged_split.cu (the hinted, two-phase forward).
// Estimator for every valid matrix of order >= min_n, on `stream`.
cudaError_t launch_ragged_estimates(int sms, int batch, const int* n, const long long* offsets, long long total,
                                    const double2* A, float2* est, int min_n, cudaStream_t stream);
// Fork from `stream` to fj.aux, estimator there (call with *fj.mu held).
cudaError_t ragged_fork_estimates(int sms, int batch, const int* n, const long long* offsets, long long total,
                                  const double2* A, float2* est, int min_n, cudaStream_t stream,
                                  const ForkJoin& fj);
// Prepare phase on `stream`, join with the estimator, QR phase (*fj.mu held).
cudaError_t ragged_launch_phases(int lanes, int sms, RaggedPlan* plan, const RaggedArgs& args, bool balance,
                                 cudaStream_t stream, const ForkJoin& fj);

}  // namespace tzg
