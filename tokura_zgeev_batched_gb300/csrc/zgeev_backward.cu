// Plain (uniform n) backward kernel: Abar for every matrix of a batch.
// Same tiling as the forward: a warp owns a tile of 32/L matrices, staged
// tile-interleaved into three n x n workspace regions (T, Q, XY) plus an
// n-vector region.
#include "zgeev_backward.cuh"
#include "zgeev_internal.h"

namespace tzg {

template <int L>
__global__ void __launch_bounds__(128) zgeev_backward_kernel(int n, int batch, const double2* __restrict__ A,
                                                             const double2* __restrict__ lam,
                                                             const double2* __restrict__ gbar,
                                                             double2* __restrict__ gA, double2* __restrict__ work,
                                                             char* __restrict__ flag, int itmax, int scaled_min_n) {
  constexpr int TW = 32 / L;
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long g0 = warp * TW;
  if (g0 >= batch) return;
  const int tw = (int)min((long long)TW, (long long)batch - g0);
  const int slot = lane / L;
  if (slot >= tw) return;
  const Group<L> G;
  const long long nn = (long long)n * n;
  const long long region = nn * batch;
  const long long j = g0 + slot;
  double2* base = work + g0 * nn + slot;
  BwdViews V{MatView{base, n, tw}, MatView{base + region, n, tw}, MatView{base + 2 * region, n, tw},
             work + 3 * region + g0 * n + slot, tw};
  const int status =
      backward_matrix<L>(A + j * nn, lam + j * n, gbar + j * n, gA + j * nn, V, G, itmax, scaled_min_n);
  if (G.rank == 0) flag[j] = (char)status;
}

size_t backward_workspace_bytes(int n, int batch) {
  return sizeof(double2) * ((size_t)3 * n * n + n) * (size_t)batch;
}

cudaError_t launch_backward(int lanes, int n, int batch, const double2* A, const double2* lam, const double2* gbar,
                            double2* gA, double2* work, char* flag, int itmax, cudaStream_t stream,
                            int scaled_min_n) {
  const int tw = 32 / lanes;
  const long long warps = ((long long)batch + tw - 1) / tw;
  const int threads = 64;  // small blocks spread a resident batch evenly over the SMs
  const long long blocks = (warps * 32 + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  switch (lanes) {
    case 1:
      zgeev_backward_kernel<1><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, lam, gbar, gA, work, flag, itmax,
                                                                                       scaled_min_n);
      break;
    case 2:
      zgeev_backward_kernel<2><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, lam, gbar, gA, work, flag, itmax,
                                                                                       scaled_min_n);
      break;
    case 4:
      zgeev_backward_kernel<4><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, lam, gbar, gA, work, flag, itmax,
                                                                                       scaled_min_n);
      break;
    case 8:
      zgeev_backward_kernel<8><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, lam, gbar, gA, work, flag, itmax,
                                                                                       scaled_min_n);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tzg
