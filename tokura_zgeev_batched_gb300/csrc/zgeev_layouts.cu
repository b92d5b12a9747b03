// Eigenvalue entry points for other input layouts and precisions:
//   tokura_zgeev_strided_batched_gpu  — column-major with leading dimension
//                                       lda, matrices strideA elements apart,
//                                       eigenvalue vectors strideW apart
//   tokura_zgeev_pointer_batched_gpu  — cuBLAS-style device array of matrix
//                                       pointers (leading dimension lda)
//   tokura_cgeev_batched_gpu          — single-precision complex matrices in
//                                       and eigenvalues out, FP64 inside
// The reference takes only contiguous n x n FP64 matrices
// (tokura_zgeev_batched.cu:212-285). Each path runs the plain solver
// (zgeev_lane.cuh) with its own loader/storer, so results are bitwise equal to
// the contiguous entry point on the same matrix entries: only the addresses
// (and the FP32->FP64 widening / FP64->FP32 rounding) differ.
#include "../../include/tokura_blas_ext.h"
#include "tokura_handle.h"
#include "zgeev_internal.h"
#include "zgeev_lane.cuh"

namespace tzg {

struct StridedBatch {
  const double2* A;
  long long lda, strideA, strideW;
  double2* W;
  __device__ __forceinline__ bool valid(long long) const { return true; }
  __device__ __forceinline__ SrcStrided src(long long j) const { return SrcStrided{A + j * strideA, lda}; }
  __device__ __forceinline__ double2* out(long long j, int) const { return W + j * strideW; }
};

struct PointerBatch {
  const double2* const* Aarray;
  long long lda;
  double2* W;
  __device__ __forceinline__ bool valid(long long j) const { return Aarray[j] != nullptr; }
  __device__ __forceinline__ SrcStrided src(long long j) const { return SrcStrided{Aarray[j], lda}; }
  __device__ __forceinline__ double2* out(long long j, int n) const { return W + j * n; }
};

struct Complex64Batch {
  const float2* A;
  float2* W;
  int n;
  __device__ __forceinline__ bool valid(long long) const { return true; }
  __device__ __forceinline__ SrcComplex64 src(long long j) const { return SrcComplex64{A + j * n * n}; }
  __device__ __forceinline__ float2* out(long long j, int) const { return W + j * n; }
};

// Same tiling as zgeev_plain_kernel: a warp holds 32/L matrices, L lanes each.
template <int L, bool kBalance, class Batch>
__global__ void __launch_bounds__(256) zgeev_layout_kernel(int n, int batch, Batch B, double2* __restrict__ work,
                                                            char* __restrict__ flag, int itmax, int balance) {
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
  MatView M{work + g0 * nn + slot, n, tw};
  int status;
  if (!B.valid(j)) {  // NULL matrix pointer: NaN eigenvalues, flag 3 (group-uniform)
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int i = G.rank; i < n; i += L) put_ev(B.out(j, n) + i, make_double2(nan, nan));
    status = kInvalidInput;
  } else {
    status = solve_matrix<L, kBalance>(B.src(j), M, G, B.out(j, n), itmax, balance);
  }
  if (G.rank == 0) flag[j] = (char)status;
}

template <int L, class Batch>
static void launch_layout_l(unsigned blocks, int threads, cudaStream_t stream, int n, int batch, const Batch& B,
                            double2* work, char* flag, int itmax, int balance) {
  if (balance != 0)
    zgeev_layout_kernel<L, true, Batch><<<blocks, threads, 0, stream>>>(n, batch, B, work, flag, itmax, balance);
  else
    zgeev_layout_kernel<L, false, Batch><<<blocks, threads, 0, stream>>>(n, batch, B, work, flag, itmax, 0);
}

template <class Batch>
static cudaError_t launch_layout(const PlainConfig& cfg, int n, int batch, const Batch& B, double2* work, char* flag,
                                 int itmax, cudaStream_t stream, int balance) {
  const int L = cfg.lanes;
  const int tw = 32 / L;
  const long long warps = ((long long)batch + tw - 1) / tw;
  const int threads = cfg.threads;
  if (threads < 32 || threads > 256 || threads % 32 != 0) return cudaErrorInvalidValue;
  const long long blocks = (warps * 32 + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  switch (L) {
    case 1: launch_layout_l<1>((unsigned)blocks, threads, stream, n, batch, B, work, flag, itmax, balance); break;
    case 2: launch_layout_l<2>((unsigned)blocks, threads, stream, n, batch, B, work, flag, itmax, balance); break;
    case 4: launch_layout_l<4>((unsigned)blocks, threads, stream, n, batch, B, work, flag, itmax, balance); break;
    case 8: launch_layout_l<8>((unsigned)blocks, threads, stream, n, batch, B, work, flag, itmax, balance); break;
    default: return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

// Checks shared by the three entry points, in the reference's order
// (tokura_zgeev_batched.cu:237-264).
static int check_common(const tokurablas_t* handle, int n, const void* A, const void* eigenvalues, const void* work,
                        int batch_count, const char* flag) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (A == nullptr) return -3;
  if (eigenvalues == nullptr) return -4;
  if (work == nullptr) return -5;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  return 0;
}

static int itmax_of(const tokurablas_t* handle, int n) {
  return handle->itmax_override > 0 ? handle->itmax_override : default_itmax(n);
}

}  // namespace tzg

extern "C" TOKURA_API int tokura_zgeev_strided_batched_gpu(tokurablas_t* handle, int n, int batch_count,
                                                            const cuDoubleComplex* A, int lda, long long strideA,
                                                            cuDoubleComplex* eigenvalues, long long strideW,
                                                            cuDoubleComplex* work, char* flag,
                                                            cudaStream_t cudastream) {
  const int bad = tzg::check_common(handle, n, A, eigenvalues, work, batch_count, flag);
  if (bad != 0) return bad;
  if (lda < n) return -8;
  if (strideA < 0 || strideW < n) return -9;
  const tzg::StridedBatch B{reinterpret_cast<const double2*>(A), lda, strideA, strideW,
                            reinterpret_cast<double2*>(eigenvalues)};
  const cudaError_t err = tzg::launch_layout(tzg::plain_config_for(handle, n, batch_count), n, batch_count, B,
                                             reinterpret_cast<double2*>(work), flag, tzg::itmax_of(handle, n),
                                             cudastream, handle->balance_mode);
  return err == cudaSuccess ? 0 : 1;
}

extern "C" TOKURA_API int tokura_zgeev_pointer_batched_gpu(tokurablas_t* handle, int n, int batch_count,
                                                            const cuDoubleComplex* const* Aarray, int lda,
                                                            cuDoubleComplex* eigenvalues, cuDoubleComplex* work,
                                                            char* flag, cudaStream_t cudastream) {
  const int bad = tzg::check_common(handle, n, Aarray, eigenvalues, work, batch_count, flag);
  if (bad != 0) return bad;
  if (lda < n) return -8;
  const tzg::PointerBatch B{reinterpret_cast<const double2* const*>(Aarray), lda,
                            reinterpret_cast<double2*>(eigenvalues)};
  const cudaError_t err = tzg::launch_layout(tzg::plain_config_for(handle, n, batch_count), n, batch_count, B,
                                             reinterpret_cast<double2*>(work), flag, tzg::itmax_of(handle, n),
                                             cudastream, handle->balance_mode);
  return err == cudaSuccess ? 0 : 1;
}

extern "C" TOKURA_API int tokura_cgeev_batched_gpu(tokurablas_t* handle, int n, int batch_count, const cuComplex* A,
                                                    cuComplex* eigenvalues, cuDoubleComplex* work, char* flag,
                                                    cudaStream_t cudastream) {
  const int bad = tzg::check_common(handle, n, A, eigenvalues, work, batch_count, flag);
  if (bad != 0) return bad;
  const tzg::Complex64Batch B{reinterpret_cast<const float2*>(A), reinterpret_cast<float2*>(eigenvalues), n};
  const cudaError_t err = tzg::launch_layout(tzg::plain_config_for(handle, n, batch_count), n, batch_count, B,
                                             reinterpret_cast<double2*>(work), flag, tzg::itmax_of(handle, n),
                                             cudastream, handle->balance_mode);
  return err == cudaSuccess ? 0 : 1;
}
