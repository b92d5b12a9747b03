// tokura_zgeev_batched_gpu_noalloc: the plain eigenvalue path without a
// caller-provided workspace.
//
// Who needs it: callers that cannot allocate device memory at the moment they
// need eigenvalues — for example a plugin living inside a host application
// that owns the whole device-memory budget and forbids out-of-band
// allocations. They still pass A, eigenvalues and flag.
//
// The kernel's staging area (the tile-interleaved copy of A) lives in a
// file-scope __device__ array of kNoAllocScratchBytes (32 MiB), which every GPU
// that loads this library keeps until the process exits. Calls with
// 16*n*n*batch_count > 32 MiB are rejected with -8 (e.g. at most 512 matrices
// of order 64, 2048 of order 32, 8192 of order 16). The FP32 shift hints
// and the phase state (8n + 4 bytes per matrix) go behind the staging area
// when they fit there; otherwise the call runs with Wilkinson shifts only.
//
// Host code must not hand the array's name to a kernel: on the host it is only
// a stand-in symbol. The device address is obtained once per device, with that
// device current, by cudaGetSymbolAddress on the first call made on that device
// (a host-side query); the address is
// cached for the life of the process, so a cudaDeviceReset of that device
// invalidates it and later calls are unsupported. All calls share
// the array and it keeps the previous call's contents; the kernel overwrites
// every staging element before reading it, so nothing needs clearing. Calls
// whose executions overlap on the GPU (different streams, or different host
// threads without ordering) race on the array and must be serialized by the
// caller, e.g. by issuing them on one stream.
#include <mutex>

#include "../../include/tokura_blas_ext.h"
#include "tokura_handle.h"
#include "zgeev_internal.h"

namespace tzg {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;
constexpr size_t kNoAllocScratchElems = kNoAllocScratchBytes / sizeof(double2);
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double2 g_noalloc_scratch[kNoAllocScratchElems];

static std::mutex g_noalloc_mutex;
static double2* g_noalloc_ptr[kNoAllocMaxDevices] = {};

// Device address of g_noalloc_scratch on the current device (looked up once per device).
static cudaError_t noalloc_scratch_ptr(double2** out) {
  int dev = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err != cudaSuccess) return err;
  if (dev < 0 || dev >= kNoAllocMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_noalloc_mutex);
  if (g_noalloc_ptr[dev] == nullptr) {
    void* p = nullptr;
    err = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (err != cudaSuccess) return err;
    g_noalloc_ptr[dev] = static_cast<double2*>(p);
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

}  // namespace tzg

extern "C" TOKURA_API size_t tokura_zgeev_noalloc_max_bytes(void) { return tzg::kNoAllocScratchBytes; }

extern "C" TOKURA_API int tokura_zgeev_batched_gpu_noalloc(tokurablas_t* handle, int n, int batch_count,
                                                            cuDoubleComplex* A, cuDoubleComplex* eigenvalues,
                                                            char* flag, cudaStream_t cudastream) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (A == nullptr) return -3;
  if (eigenvalues == nullptr) return -4;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  const size_t need = sizeof(double2) * (size_t)n * (size_t)n * (size_t)batch_count;
  if (need > tzg::kNoAllocScratchBytes) return -8;
  // Shift hints only when they fit behind the staging area.
  const bool hints = tzg::use_shift_hints(handle, n) &&
                     need + (sizeof(float2) * (size_t)n + sizeof(int)) * (size_t)batch_count <=
                         tzg::kNoAllocScratchBytes;
  // The estimator runs on the handle's second stream, which belongs to the
  // handle's device: the scratch array must be that device's too.
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev != handle->device) return 1;
  double2* scratch = nullptr;
  if (tzg::noalloc_scratch_ptr(&scratch) != cudaSuccess) return 1;
  const tzg::PlainConfig cfg = tzg::plain_config_for(handle, n, batch_count);
  const int itmax = handle->itmax_override > 0 ? handle->itmax_override : tzg::default_itmax(n);
  const cudaError_t err =
      tzg::launch_plain(cfg, n, batch_count, reinterpret_cast<const double2*>(A),
                        reinterpret_cast<double2*>(eigenvalues), scratch, flag, itmax, cudastream,
                        handle->balance_mode, hints, &handle->fj);
  return err == cudaSuccess ? 0 : 1;
}
