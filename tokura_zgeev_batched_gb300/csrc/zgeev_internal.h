// Host-side internals shared by the C-ABI layer and the kernel launchers.
#pragma once

#include <mutex>

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

namespace tzg {

// Launch shape of the plain (uniform-n) forward kernel for one n.
struct PlainConfig {
  int lanes;            // lanes per matrix: 1, 2, 4 or 8
  int threads;          // threads per block (multiple of 32)
  int scaled = 0;       // QR with scaled rotations (orders >= 7; zgeev_scaled_qr.cuh)
  int qr_lanes = 0;     // lanes per matrix of the QR phase when it is its own launch (shift hints); 0: `lanes`
  int scaled_qr = 0;    // `scaled` for the QR phase at qr_lanes
};

// Iteration cap per eigenvalue: LAPACK's rule 30*max(10, n) unless overridden.
__host__ __device__ inline int default_itmax(int n) { return 30 * (n > 10 ? n : 10); }

// Launches the fused stage + Hessenberg + QR kernel on `stream`.
// `work` must hold 16*n*n*batch bytes (tile-interleaved copy of A).
// A second stream and two events for running the FP32 estimator beside the
// FP64 Hessenberg phase (fork from the caller's stream, join before the QR
// phase). The mutex serializes the enqueue sequences of concurrent callers
// so each join waits on its own fork.
struct ForkJoin {
  cudaStream_t aux = nullptr;
  cudaEvent_t fork = nullptr, join = nullptr;
  std::mutex* mu = nullptr;
};

// hints: FP32 eigenvalue estimates steer the QR's first shifts; work must then
// hold 16n^2*batch + 8n*batch + 4*batch bytes (inside the reference's
// 16n^2*batch + 16n*batch). With fj, the estimator runs on fj->aux while the
// Hessenberg phase runs on `stream`; without, it runs first on `stream`.
cudaError_t launch_plain(const PlainConfig& cfg, int n, int batch, const double2* A, double2* eig,
                         double2* work, char* flag, int itmax, cudaStream_t stream, int balance = 0,
                         bool hints = false, const ForkJoin* fj = nullptr);

// Ragged (per-matrix n) path: workspace bytes and launcher (device-side planning + persistent solve).
size_t ragged_workspace_bytes(int batch, long long total_elements);
cudaError_t launch_ragged(int lanes, int sms, int batch, const int* n, const long long* offsets,
                          const long long* eig_offsets, long long total_elements, const double2* A, double2* eig,
                          void* work, char* flag, int itmax_override, cudaStream_t stream, int balance = 0,
                          int hint_min_n = 0, const ForkJoin* fj = nullptr, int scaled_min_n = 65);  // per lane

// Backward (Abar from A, eigenvalues and their gradients).
size_t backward_workspace_bytes(int n, int batch);
cudaError_t launch_backward(int lanes, int n, int batch, const double2* A, const double2* lam, const double2* gbar,
                            double2* gA, double2* work, char* flag, int itmax, cudaStream_t stream,
                            int scaled_min_n = 65);
size_t ragged_backward_workspace_bytes(int batch, long long total_elements);
cudaError_t launch_ragged_backward(int lanes, int sms, int batch, const int* n, const long long* offsets,
                                   const long long* eig_offsets, long long total_elements, const double2* A,
                                   const double2* lam, const double2* gbar, double2* gA, void* work, char* flag,
                                   int itmax_override, cudaStream_t stream, int scaled_min_n = 65);

// Eigenvalues with eigenvectors (workspace: backward_workspace_bytes).
cudaError_t launch_vectors(int lanes, int n, int batch, const double2* A, double2* w, double2* VL, double2* VR,
                           double2* work, char* flag, int itmax, cudaStream_t stream, bool hints = false,
                           const ForkJoin* fj = nullptr, int scaled_min_n = 65);
size_t vectors_workspace_bytes(int n, int batch);

}  // namespace tzg
