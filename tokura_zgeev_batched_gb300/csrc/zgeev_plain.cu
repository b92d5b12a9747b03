// Plain batched eigenvalue-only ZGEEV for a uniform matrix order n (1..64).
//
// One kernel replaces the reference's three stages (layout transpose,
// tokura_zgehrd_normal_MWB_kernel at tokura_zgehrd_MWB_kernel.cuh:159-287 and
// tokura_zhseqr_normal_MWB_kernel at tokura_zhseqr_MWB_kernel.cuh:611-791):
// each warp stages its tile of 32/L matrices into the workspace, reduces
// them to Hessenberg form and runs single-shift QR, then writes the
// eigenvalues straight to eigenvalues[i + j*n] and flag[j].
#include "zgeev_internal.h"
#include "zgeev_lane.cuh"

namespace tzg {

template <int L, bool kBalance>
__global__ void __launch_bounds__(256) zgeev_plain_kernel(int n, int batch, const double2* __restrict__ A,
                                                           double2* __restrict__ eig, double2* __restrict__ work,
                                                           char* __restrict__ flag, int itmax, int balance) {
  constexpr int TW = 32 / L;
  const int lane = threadIdx.x & 31;
  const long long warp = ((long long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const long long g0 = warp * TW;
  if (g0 >= batch) return;  // warp-uniform
  const int tw = (int)min((long long)TW, (long long)batch - g0);
  const int slot = lane / L;
  if (slot >= tw) return;  // whole lane groups leave together; no warp-wide barriers follow
  const Group<L> G;
  const long long nn = (long long)n * n;
  const long long j = g0 + slot;
  MatView M{work + g0 * nn + slot, n, tw};

  const int status = solve_matrix<L, kBalance>(A + j * nn, M, G, eig + j * n, itmax, balance);
  if (G.rank == 0) flag[j] = (char)status;
}

cudaError_t launch_plain(const PlainConfig& cfg, int n, int batch, const double2* A, double2* eig, double2* work,
                         char* flag, int itmax, cudaStream_t stream, int balance) {
  const int L = cfg.lanes;
  const int tw = 32 / L;
  const long long warps = ((long long)batch + tw - 1) / tw;
  const int threads = cfg.threads;
  const long long blocks = (warps * 32 + threads - 1) / threads;
  if (blocks > 0x7fffffffLL || threads < 32 || threads > 256 || threads % 32 != 0) return cudaErrorInvalidValue;
  switch (L) {
    case 1:
      if (balance != 0)
        zgeev_plain_kernel<1, true><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, eig, work, flag, itmax,
                                                                                balance);
      else
        zgeev_plain_kernel<1, false><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, eig, work, flag, itmax, 0);
      break;
    case 2:
      if (balance != 0)
        zgeev_plain_kernel<2, true><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, eig, work, flag, itmax,
                                                                                balance);
      else
        zgeev_plain_kernel<2, false><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, eig, work, flag, itmax, 0);
      break;
    case 4:
      if (balance != 0)
        zgeev_plain_kernel<4, true><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, eig, work, flag, itmax,
                                                                                balance);
      else
        zgeev_plain_kernel<4, false><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, eig, work, flag, itmax, 0);
      break;
    case 8:
      if (balance != 0)
        zgeev_plain_kernel<8, true><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, eig, work, flag, itmax,
                                                                                balance);
      else
        zgeev_plain_kernel<8, false><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, eig, work, flag, itmax, 0);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tzg
