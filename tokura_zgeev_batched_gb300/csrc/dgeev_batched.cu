// Batched real eigenvalue-only entry points (LAPACK dgeev / sgeev with
// JOBVL = JOBVR = 'N'): tokura_dgeev_batched_gpu (FP64) and
// tokura_sgeev_batched_gpu (FP32 in and out, FP64 inside). Matrix j is
// column-major at A + j*n*n; its eigenvalues go to wr/wi[i + j*n] in LAPACK's
// convention (complex pairs adjacent, positive imaginary part first, exact
// conjugates). Same tiling as the complex plain kernel: a warp holds 32/L
// matrices of the batch, each on L lanes, staged tile-interleaved in work.
#include <type_traits>

#include "../../include/tokura_blas_ext.h"
#include "dgeev_real.cuh"
#include "tokura_handle.h"

namespace tzg {

template <int L, bool kBalance, class T>
__global__ void __launch_bounds__(256) dgeev_plain_kernel(int n, int batch, const T* __restrict__ A,
                                                           T* __restrict__ wr, T* __restrict__ wi,
                                                           double* __restrict__ work, char* __restrict__ flag,
                                                           int itmax, int balance) {
  using Src = typename std::conditional<std::is_same<T, float>::value, SrcReal32, SrcReal64>::type;
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
  const long long j = g0 + slot;
  const RMatView M{work + g0 * nn + slot, n, tw};
  const int status = solve_real_matrix<L, kBalance>(Src{A + j * nn}, M, G, wr + j * n, wi + j * n, itmax, balance);
  if (G.rank == 0) flag[j] = (char)status;
}

template <int L, class T>
static void launch_real_l(unsigned blocks, int threads, cudaStream_t stream, int n, int batch, const T* A, T* wr,
                          T* wi, double* work, char* flag, int itmax, int balance) {
  if (balance != 0)
    dgeev_plain_kernel<L, true, T><<<blocks, threads, 0, stream>>>(n, batch, A, wr, wi, work, flag, itmax, balance);
  else
    dgeev_plain_kernel<L, false, T><<<blocks, threads, 0, stream>>>(n, batch, A, wr, wi, work, flag, itmax, 0);
}

template <class T>
static cudaError_t launch_real(const tokurablas_t* h, int n, int batch, const T* A, T* wr, T* wi, double* work,
                               char* flag, cudaStream_t stream) {
  const PlainConfig cfg = real_config_for(h, n, batch);
  const int L = cfg.lanes;
  const int tw = 32 / L;
  const long long warps = ((long long)batch + tw - 1) / tw;
  const int threads = cfg.threads;
  const long long blocks = (warps * 32 + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  const int itmax = h->itmax_override > 0 ? h->itmax_override : default_itmax(n);
  const int bal = h->balance_mode;
  switch (L) {
    case 1: launch_real_l<1>((unsigned)blocks, threads, stream, n, batch, A, wr, wi, work, flag, itmax, bal); break;
    case 2: launch_real_l<2>((unsigned)blocks, threads, stream, n, batch, A, wr, wi, work, flag, itmax, bal); break;
    case 4: launch_real_l<4>((unsigned)blocks, threads, stream, n, batch, A, wr, wi, work, flag, itmax, bal); break;
    case 8: launch_real_l<8>((unsigned)blocks, threads, stream, n, batch, A, wr, wi, work, flag, itmax, bal); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

template <class T>
static int real_entry(tokurablas_t* handle, int n, int batch_count, const T* A, T* wr, T* wi, double* work,
                      char* flag, cudaStream_t stream) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (A == nullptr) return -3;
  if (wr == nullptr || wi == nullptr) return -4;
  if (work == nullptr) return -5;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  return launch_real(handle, n, batch_count, A, wr, wi, work, flag, stream) == cudaSuccess ? 0 : 1;
}

}  // namespace tzg

extern "C" TOKURA_API size_t tokura_get_dgeev_workspacesize(int n, int batch_count) {
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return (size_t)-1;
  if (!(batch_count > 0)) return (size_t)-2;
  return sizeof(double) * (size_t)n * (size_t)n * (size_t)batch_count;
}

extern "C" TOKURA_API int tokura_dgeev_batched_gpu(tokurablas_t* handle, int n, int batch_count, const double* A,
                                                    double* wr, double* wi, double* work, char* flag,
                                                    cudaStream_t cudastream) {
  return tzg::real_entry(handle, n, batch_count, A, wr, wi, work, flag, cudastream);
}

extern "C" TOKURA_API int tokura_sgeev_batched_gpu(tokurablas_t* handle, int n, int batch_count, const float* A,
                                                    float* wr, float* wi, double* work, char* flag,
                                                    cudaStream_t cudastream) {
  return tzg::real_entry(handle, n, batch_count, A, wr, wi, work, flag, cudastream);
}
