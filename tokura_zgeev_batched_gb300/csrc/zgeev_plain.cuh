// The plain (uniform-n) eigenvalue solver over any batch layout.
//
// Replaces the reference's three stages (layout transpose,
// tokura_zgehrd_normal_MWB_kernel at tokura_zgehrd_MWB_kernel.cuh:159-287 and
// tokura_zhseqr_normal_MWB_kernel at tokura_zhseqr_MWB_kernel.cuh:611-791):
// each warp stages its tile of 32/L matrices into the workspace, reduces
// them to Hessenberg form and runs single-shift QR, then writes each
// matrix's eigenvalues and flag.
//
// A batch type says where matrix j is read (src), where its eigenvalues go
// (out) and whether it exists (valid): the reference's contiguous layout,
// strided, pointer-array and single-precision batches all run this code, so
// their results are bitwise equal on the same matrix entries.
//
// Without shift hints the solve is one kernel (phase kAll). With hints it is
// two kernels with the FP32 estimator beside the first:
//   caller's stream: [kPrepare: stage + Hessenberg] --join--> [kQR: QR with hints]
//   second stream:   [FP32 estimator] -----------------^
// The estimator (shared memory, FP32, latency bound) and the Hessenberg phase
// (FP64 pipe) use different resources and run side by side; the prepare
// kernel asks for the largest shared-memory carveout so the estimator's
// blocks fit on the same SMs (with the default, L1-heavy split they did not,
// and the two ran one after the other: 790 -> 680 ms at n = 64 with the
// largest carveout; smaller carveouts or an estimator grid capped to leave
// registers for the prepare grid measured slower). The QR phase starts once both are
// done. The QR kernel asks for the same carveout (it measured indifferent to
// it), so that when several calls run side by side (the host-buffer
// pipeline's chunks) one call's QR blocks do not lock another call's
// estimator out of an SM. Between the phases each matrix's pre-scaling exponent (or a finished
// status) is kept in the workspace after the hints. The arithmetic does not
// depend on the split, so a given set of hints gives bitwise the same results.
#pragma once

#include "zgeev_estimate.cuh"
#include "zgeev_internal.h"
#include "zgeev_lane.cuh"
#include "zgeev_scaled_qr.cuh"

namespace tzg {

// The reference's layout: n x n column-major matrices one after another,
// eigenvalues[i + j*n].
struct ContigBatch {
  const double2* A;
  double2* W;
  int n;
  __device__ __forceinline__ bool valid(long long) const { return true; }
  __device__ __forceinline__ SrcContig src(long long j) const { return SrcContig{A + j * n * n}; }
  __device__ __forceinline__ double2* out(long long j, int) const { return W + j * n; }
};

// Column-major with leading dimension lda, matrices strideA elements apart,
// eigenvalue vectors strideW apart.
struct StridedBatch {
  const double2* A;
  long long lda, strideA, strideW;
  double2* W;
  __device__ __forceinline__ bool valid(long long) const { return true; }
  __device__ __forceinline__ SrcStrided src(long long j) const { return SrcStrided{A + j * strideA, lda}; }
  __device__ __forceinline__ double2* out(long long j, int) const { return W + j * strideW; }
};

// Device array of matrix pointers (NULL entries are flagged, not solved).
struct PointerBatch {
  const double2* const* Aarray;
  long long lda;
  double2* W;
  __device__ __forceinline__ bool valid(long long j) const { return Aarray[j] != nullptr; }
  __device__ __forceinline__ SrcStrided src(long long j) const { return SrcStrided{Aarray[j], lda}; }
  __device__ __forceinline__ double2* out(long long j, int n) const { return W + j * n; }
};

// Single-precision complex in and out (FP64 inside).
struct Complex64Batch {
  const float2* A;
  float2* W;
  int n;
  __device__ __forceinline__ bool valid(long long) const { return true; }
  __device__ __forceinline__ SrcComplex64 src(long long j) const { return SrcComplex64{A + j * n * n}; }
  __device__ __forceinline__ float2* out(long long j, int) const { return W + j * n; }
};

// `scaled` (nonzero, n >= kScaledMinN) selects the QR with scaled rotations
// (zgeev_scaled_qr.cuh) for the QR part; the prepare part does not depend on it.
// Warp w solves matrices w*32/L .. w*32/L + 32/L - 1 with L lanes each. The
// staging area holds the batch in tiles of `stage_tw` matrices (32/L of the
// launch that staged it): the QR phase may run at fewer lanes per matrix than
// the prepare phase, a warp then spanning several staging tiles.
template <int L, bool kBalance, int kPhase, class Batch>
__global__ void __launch_bounds__(256) zgeev_plain_kernel(int n, int batch, Batch B, double2* __restrict__ work,
                                                           char* __restrict__ flag, int itmax, int balance,
                                                           const float2* __restrict__ est, int* __restrict__ state,
                                                           int scaled, int stage_tw) {
  constexpr int TW = 32 / L;  // matrices per warp (1 at 32 lanes)
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long j = warp * TW + lane / L;
  if (j >= batch) return;  // whole lane groups leave together; no warp-wide barriers follow
  const Group<L> G;
  const long long nn = (long long)n * n;
  const long long t0 = j / stage_tw * stage_tw;  // first matrix of j's staging tile
  MatView M{work + t0 * nn + (j - t0), n, (int)min((long long)stage_tw, (long long)batch - t0)};

  if (kPhase != kPhaseQR && !B.valid(j)) {  // NULL matrix pointer: NaN eigenvalues, flag 3 (group-uniform)
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int i = G.rank; i < n; i += L) put_ev(B.out(j, n) + i, make_double2(nan, nan));
    if (G.rank == 0) {
      flag[j] = (char)kInvalidInput;
      if (kPhase == kPhasePrepare) state[j] = kStateDone;
    }
    return;
  }
#ifdef TOKURA_DEBUG_BOUNDS
  int sweeps = -1;
  int* const sw = &sweeps;
  TZG_DBG_INDEX(j, batch);
#else
  int* const sw = nullptr;
#endif
  if (kPhase == kPhaseAll) {
    int shift;
    int status = prepare_matrix<L, kBalance>(B.src(j), M, G, B.out(j, n), balance, shift);
    if (status == kPrepared) {
      const float2* e = est != nullptr ? est + j * n : nullptr;
      status = (scaled != 0 && n >= kScaledMinN) ? qr_eigenvalues_scaled<L>(M, G, B.out(j, n), shift, itmax, e, sw)
                                                 : qr_eigenvalues<L>(M, G, B.out(j, n), shift, itmax, e, sw);
    }
    if (G.rank == 0) flag[j] = (char)status;
  } else if (kPhase == kPhasePrepare) {
    int shift;
    const int status = prepare_matrix<L, kBalance>(B.src(j), M, G, B.out(j, n), balance, shift);
    if (G.rank == 0) {
      if (status != kPrepared) flag[j] = (char)status;
      state[j] = status != kPrepared ? kStateDone : shift;
    }
  } else {
    const int s = state[j];
    if (s == kStateDone) return;  // group-uniform
    const int status = (scaled != 0 && n >= kScaledMinN)
                           ? qr_eigenvalues_scaled<L>(M, G, B.out(j, n), s, itmax, est + j * n, sw)
                           : qr_eigenvalues<L>(M, G, B.out(j, n), s, itmax, est + j * n, sw);
    if (G.rank == 0) flag[j] = (char)status;
  }
#ifdef TOKURA_DEBUG_BOUNDS
  if (kPhase != kPhasePrepare && G.rank == 0 && sweeps >= 0) dbg_record_sweeps(j, sweeps);
#endif
}

template <int L, bool kBalance, int kPhase, class Batch>
inline cudaError_t launch_plain_l(unsigned blocks, int threads, cudaStream_t stream, int n, int batch,
                                  const Batch& B, double2* work, char* flag, int itmax, int balance,
                                  const float2* est, int* state, int carveout, int scaled, int stage_tw) {
  if (kPhase != kPhaseAll) {  // shared memory for estimators running beside (this or another call's)
    const cudaError_t err = cudaFuncSetAttribute(zgeev_plain_kernel<L, kBalance, kPhase, Batch>,
                                                 cudaFuncAttributePreferredSharedMemoryCarveout, carveout);
    if (err != cudaSuccess) return err;
  }
  zgeev_plain_kernel<L, kBalance, kPhase, Batch>
      <<<blocks, threads, 0, stream>>>(n, batch, B, work, flag, itmax, balance, est, state, scaled, stage_tw);
  return cudaGetLastError();
}

// One instantiation per lane width and balancing choice; the QR phase does
// not depend on balancing.
template <int kPhase, class Batch>
inline cudaError_t launch_plain_phase(int L, bool bal, unsigned blocks, int threads, cudaStream_t stream, int n,
                                      int batch, const Batch& B, double2* work, char* flag, int itmax, int balance,
                                      const float2* est, int* state, int carveout, int scaled, int stage_tw) {
  constexpr bool kB = kPhase != kPhaseQR;  // balanced instantiation exists
  const bool b = bal && kB;
  const int bv = b ? balance : 0;
  switch (L) {
    case 1:
      return b ? launch_plain_l<1, kB, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, bv, est, state,
                                                        carveout, scaled, stage_tw)
               : launch_plain_l<1, false, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, 0, est, state,
                                                           carveout, scaled, stage_tw);
    case 2:
      return b ? launch_plain_l<2, kB, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, bv, est, state,
                                                        carveout, scaled, stage_tw)
               : launch_plain_l<2, false, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, 0, est, state,
                                                           carveout, scaled, stage_tw);
    case 4:
      return b ? launch_plain_l<4, kB, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, bv, est, state,
                                                        carveout, scaled, stage_tw)
               : launch_plain_l<4, false, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, 0, est, state,
                                                           carveout, scaled, stage_tw);
    case 8:
      return b ? launch_plain_l<8, kB, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, bv, est, state,
                                                        carveout, scaled, stage_tw)
               : launch_plain_l<8, false, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, 0, est, state,
                                                           carveout, scaled, stage_tw);
    case 16:
      return b ? launch_plain_l<16, kB, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, bv, est, state,
                                                        carveout, scaled, stage_tw)
               : launch_plain_l<16, false, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, 0, est, state,
                                                           carveout, scaled, stage_tw);
    case 32:
      return b ? launch_plain_l<32, kB, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, bv, est, state,
                                                        carveout, scaled, stage_tw)
               : launch_plain_l<32, false, kPhase>(blocks, threads, stream, n, batch, B, work, flag, itmax, 0, est, state,
                                                           carveout, scaled, stage_tw);
    default:
      return cudaErrorInvalidValue;
  }
}

// The whole solve of one batch on `stream` (see the file comment). With
// hints, work holds the staging area, then 8n bytes of hints and 4 bytes of
// phase state per matrix (inside the reference's 16n^2 + 16n per matrix).
template <class Batch>
cudaError_t launch_batch(const PlainConfig& cfg, int n, int batch, const Batch& B, double2* work, char* flag,
                         int itmax, cudaStream_t stream, int balance, bool hints, const ForkJoin* fj) {
  const int L = cfg.lanes;
  // Lanes per matrix of the QR phase when it runs as its own launch (with hints).
  const int Lq = cfg.qr_lanes > 0 ? cfg.qr_lanes : L;
  auto valid_lanes = [](int l) { return l == 1 || l == 2 || l == 4 || l == 8 || l == 16 || l == 32; };
  if (!valid_lanes(L) || !valid_lanes(Lq)) return cudaErrorInvalidValue;
  const int tw = 32 / L;
  const int threads = cfg.threads;
  if (threads < 32 || threads > 256 || threads % 32 != 0) return cudaErrorInvalidValue;
  auto blocks_for = [&](int lanes) {
    const long long warps = ((long long)batch + 32 / lanes - 1) / (32 / lanes);
    return (warps * 32 + threads - 1) / threads;
  };
  const long long blocks = blocks_for(L), blocks_q = blocks_for(Lq);
  if (blocks > 0x7fffffffLL || blocks_q > 0x7fffffffLL) return cudaErrorInvalidValue;
  const bool bal = balance != 0;
  const int scaled = cfg.scaled;
  constexpr int kDef = cudaSharedmemCarveoutDefault;
  if (!hints)
    return launch_plain_phase<kPhaseAll>(L, bal, (unsigned)blocks, threads, stream, n, batch, B, work, flag, itmax,
                                         balance, nullptr, nullptr, kDef, scaled, tw);
  float2* est = reinterpret_cast<float2*>(work + (size_t)n * n * batch);
  int* state = reinterpret_cast<int*>(est + (size_t)n * batch);
  cudaError_t err;
  if (fj == nullptr || fj->aux == nullptr) {  // no second stream: estimator first, then one kernel
    if ((err = launch_estimates(n, batch, B, est, stream)) != cudaSuccess) return err;
    return launch_plain_phase<kPhaseAll>(L, bal, (unsigned)blocks, threads, stream, n, batch, B, work, flag, itmax,
                                         balance, est, nullptr, kDef, scaled, tw);
  }
  std::lock_guard<std::mutex> lock(*fj->mu);
  if ((err = cudaEventRecord(fj->fork, stream)) != cudaSuccess) return err;
  if ((err = cudaStreamWaitEvent(fj->aux, fj->fork, 0)) != cudaSuccess) return err;
  if ((err = launch_estimates(n, batch, B, est, fj->aux)) != cudaSuccess) return err;
  if ((err = cudaEventRecord(fj->join, fj->aux)) != cudaSuccess) return err;
  if ((err = launch_plain_phase<kPhasePrepare>(L, bal, (unsigned)blocks, threads, stream, n, batch, B, work, flag,
                                               itmax, balance, nullptr, state, cudaSharedmemCarveoutMaxShared,
                                               scaled, tw)) !=
      cudaSuccess)
    return err;
  if ((err = cudaStreamWaitEvent(stream, fj->join, 0)) != cudaSuccess) return err;
  return launch_plain_phase<kPhaseQR>(Lq, false, (unsigned)blocks_q, threads, stream, n, batch, B, work, flag, itmax,
                                      0, est, state, cudaSharedmemCarveoutMaxShared, cfg.scaled_qr, tw);
}

}  // namespace tzg
