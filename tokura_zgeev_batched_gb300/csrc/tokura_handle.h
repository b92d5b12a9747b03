// Contents of the opaque tokurablas_t handle and the launch-shape policy.
#pragma once

#include <mutex>

#include "zgeev_internal.h"

namespace tzg {

// Device buffers and streams of the host-buffer entry point, cached per handle.
struct HostPipeline {
  static constexpr int kStreams = 16;  // at most one stream per chunk in flight
  void* d_a[kStreams] = {};
  void* d_eig[kStreams] = {};
  void* d_work[kStreams] = {};
  char* d_flag[kStreams] = {};
  cudaStream_t stream[kStreams] = {};
  cudaEvent_t copied[kStreams] = {};  // end of the host-to-device copy last issued on each stream
  cudaEvent_t copy_begin = nullptr, copy_end = nullptr;  // timing of one call's host-to-device copies
  double link_gbs = 0.0;  // host-to-device rate seen by the last call (GB/s; 0 = not measured yet)
  double link_gbs_fixed = 0.0;  // rate set by tokuraSetHostLinkRate (> 0 replaces the measured one)
  size_t cap_a[kStreams] = {}, cap_eig[kStreams] = {}, cap_work[kStreams] = {}, cap_flag[kStreams] = {};
  void release();
};

}  // namespace tzg

namespace tzg {
// Default smallest order of the plain QR with scaled rotations.
constexpr int kScaledRotationDefaultMinN = 16;
}  // namespace tzg
using tzg::kScaledRotationDefaultMinN;

struct tokurablas_t {
  int device = 0;
  int sm_count = 0;
  int itmax_override = 0;  // >0 replaces the per-eigenvalue sweep cap 30*max(10,n)
  // Tuned plain-kernel shape per n (index 1..64); lanes == 0 means "heuristic".
  tzg::PlainConfig plain[65] = {};
  int plain_qr_lanes[65] = {};     // lanes per matrix of the hinted QR phase per n; 0 = chosen per call
  tzg::PlainConfig real[65] = {};  // the same for the real (dgeev/sgeev) kernel
  int ragged_lanes = 0;  // lanes per matrix of the ragged solvers; 0 = chosen per launch
  int balance_mode = 0;  // balancing before the eigenvalue solves: 0 none (the reference's behaviour) .. 3 both
  int ragged_hint_min_n = 48;  // mode 1: ragged matrices of this order and above get hints (65: none)
  int scaled_min_n = kScaledRotationDefaultMinN;  // plain QR with scaled rotations from this order (65: never)
  int shift_hints = 1;   // FP32 eigenvalue estimates as first shifts: 0 off, 1 uniform batches with
                         // n >= kShiftHintMinN, 2 every eigenvalue entry point and order (ragged too)
  tzg::HostPipeline pipe;  // host-buffer entry point state (guarded by pipe_mutex)
  std::mutex pipe_mutex;
  tzg::ForkJoin fj;        // second stream + events for the FP32 estimator (created with the handle)
  std::mutex fj_mutex;
};

namespace tzg {

inline void init_default_tuning(tokurablas_t* h) {
  for (int n = 0; n <= 64; ++n) h->plain[n] = PlainConfig{0, 0};
  for (int n = 0; n <= 64; ++n) h->real[n] = PlainConfig{0, 0};
}

// Lanes per matrix: enough lane groups to give every SM sub-partition at
// least two warps (FP64 saturates at one warp per sub-partition; the second
// hides memory latency); otherwise spread each matrix over more lanes.
// One-warp blocks: when the whole batch is resident at once, the block is
// the unit the hardware spreads over the SMs, so small blocks even out the
// per-SM load (at n = 64, 65536 matrices: 2048 warps over 152 SMs run about
// 11 % faster in 32- or 64-thread blocks than in 128-thread blocks; with
// shift hints, 32-thread blocks are 5-9 % faster than 64 at batches of
// 8,000-20,000 and equal at 65,536).
// Smallest order that takes the QR with scaled rotations at `lanes` lanes per
// matrix: lanes * min_order, at least 7 (65: never). The rotation's fixed cost
// is paid per lane group while its savings scale with the pairs each lane
// updates (about n / lanes): 10,000 matrices at n = 32 on 4 lanes ran 9 %
// slower with scaled rotations, 262,144 on 1 lane 5 % faster.
inline int scaled_threshold(const tokurablas_t* h, int lanes) {
  if (h->scaled_min_n > 64) return 65;
  const int t = h->scaled_min_n * (lanes > 0 ? lanes : 1);
  return t < 7 ? 7 : (t > 65 ? 65 : t);
}

// Lane widths of the complex plain kernel (0 = chosen per call where allowed).
inline bool plain_lanes_valid(int lanes, bool allow_zero) {
  return (allow_zero && lanes == 0) || lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8 || lanes == 16 ||
         lanes == 32;
}

inline PlainConfig plain_config_for(const tokurablas_t* h, int n, int batch) {
  PlainConfig c = h->plain[n];
  if (c.lanes == 0) {
    // Batches below a quarter of the lanes that fill the GPU spread each matrix
    // over more lanes, up to n/2 (two elements of a row or column per lane) and 32:
    // 304 matrices at n = 64 (two per SM) took 73.4 ms at 4 lanes and 21.7 ms at
    // 32, 2,432 at n = 64 53.9 ms at 8 and 50.5 at 16, 1,216 at n = 32 8.1 ms at
    // 8 and 6.4 at 16 (8.4 at 32); at 65,536 matrices 32 lanes were 3.1x slower
    // than one, every lane of a warp then computing each rotation and shift.
    const long long want_lanes = (long long)h->sm_count * 4 * 2 * 32;
    if ((long long)batch >= want_lanes)
      c.lanes = 1;
    else if ((long long)batch * 2 >= want_lanes)
      c.lanes = 2;
    else if ((long long)batch * 4 >= want_lanes)
      c.lanes = 4;
    else {
      int cap = 32;
      while (cap > 4 && cap > n / 2) cap >>= 1;
      c.lanes = 4;
      while (c.lanes < cap && (long long)batch * c.lanes < want_lanes) c.lanes <<= 1;
    }
    if (n <= 2) c.lanes = 1;
  }
  if (c.threads == 0) c.threads = 32;
  c.scaled = n >= scaled_threshold(h, c.lanes) ? 1 : 0;
  // The hinted QR phase of four-lane launches runs at two lanes from n = 12 (the
  // hints' threshold) to 24: 10,000 matrices at n = 12 / 16 / 24 took 2.08 / 3.99
  // / 10.42 ms, 1.89 / 3.70 / 9.66 ms so; at n = 32 20.69 against 20.78 ms, at
  // n = 48 and 64 two lanes were 11-23 % slower.
  c.qr_lanes = h->plain_qr_lanes[n] > 0 ? h->plain_qr_lanes[n] : (c.lanes == 4 && n <= 24 ? 2 : c.lanes);
  c.scaled_qr = n >= scaled_threshold(h, c.qr_lanes) ? 1 : 0;
  return c;
}

// Lanes per matrix of the gradient and eigenvector kernels (instantiated for
// 1, 2, 4 and 8 lanes): the plain call's choice, at most 8.
inline int group_lanes_for(const tokurablas_t* h, int n, int batch) {
  const int l = plain_config_for(h, n, batch).lanes;
  return l > 8 ? 8 : l;
}

// Launch shape of the real kernel: a tuned entry, else the lane heuristic of
// the complex kernel (it depends on the batch size, not on the arithmetic),
// up to the real kernel's 8 lanes per matrix.
inline PlainConfig real_config_for(const tokurablas_t* h, int n, int batch) {
  PlainConfig c = h->real[n];
  if (c.lanes == 0) {
    const long long want_lanes = (long long)h->sm_count * 4 * 2 * 32;
    c.lanes = (long long)batch >= want_lanes ? 1 : ((long long)batch * 2 >= want_lanes ? 2 : 4);
    if (c.lanes == 4 && (long long)batch * 4 < want_lanes && n >= 16) c.lanes = 8;
    if (n <= 2) c.lanes = 1;
  }
  if (c.threads == 0) c.threads = 32;
  return c;
}

// Orders from which the FP32 estimator pays for itself (below it the FP64
// QR needs few sweeps and the extra launch dominates).
constexpr int kShiftHintMinN = 12;

inline bool use_shift_hints(const tokurablas_t* h, int n) {
  return h->shift_hints == 2 || (h->shift_hints == 1 && n >= kShiftHintMinN);
}

// Smallest order the ragged solver computes hints for (0: none). Mode 2:
// every order. Mode 1: orders >= ragged_hint_min_n (65: none). The
// estimator's cost grows like n^2 per matrix (rotation rounds) and the QR work
// it saves like n^3, so for mixed orders it pays on the large ones. On
// 200,000 orders in U{1..64}: no hints 676 ms; hints for every order 662 ms
// (the estimator, 225 ms, outlasts the Hessenberg phase it runs beside,
// 157 ms); orders >= 56: 650, >= 48: 645, >= 40: 652, >= 32: 657 ms.
inline int ragged_hint_min_order(const tokurablas_t* h) {
  if (h->shift_hints == 2) return 1;
  if (h->shift_hints == 1 && h->ragged_hint_min_n <= 64) return h->ragged_hint_min_n;
  return 0;
}


}  // namespace tzg
