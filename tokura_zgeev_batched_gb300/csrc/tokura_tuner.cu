// Runtime autotuner for the launch shapes of the plain and ragged kernels.
//
// Replaces the reference's build-time tuner (src/TOKURA_ZHSEQR_BATCHED_GEHRD_
// TUNING_main.cu:89-227, which timed threads-per-matrix for each n once on
// 8192 random matrices and wrote #define tables that were compiled into the
// library, include/tokura_zhseqr_parameters.h). Here the candidates — lanes
// per matrix (1 to 32) x threads per block (32, 64, 128, 256) — are timed with
// CUDA events on seeded synthetic complex Gaussian matrices at the caller's
// batch size, the fastest shape is stored in the handle, and the table can be
// saved to / loaded from a text file keyed by device name and SM count.
#include <cstdio>
#include <cstring>
#include <functional>
#include <string>

#include "../../include/tokura_blas_ext.h"
#include "tokura_handle.h"
#include "zgeev_internal.h"

namespace tzg {

// Counter-based uniform in (0, 1]: 53 random bits from a 64-bit mix.
__device__ __forceinline__ double hash_uniform(unsigned long long x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return ((double)(x >> 11) + 1.0) * (1.0 / 9007199254740992.0);
}

// Complex Gaussian entries (Box-Muller on hashed counters).
__global__ void fill_cgauss_kernel(double2* a, long long count, unsigned long long seed) {
  for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < count; e += (long long)gridDim.x * blockDim.x) {
    const double u1 = hash_uniform(seed ^ (2ULL * e));
    const double u2 = hash_uniform(seed ^ (2ULL * e + 1ULL) ^ 0x9e3779b97f4a7c15ULL);
    const double r = sqrt(-2.0 * log(u1));
    double sn, cn;
    sincospi(2.0 * u2, &sn, &cn);
    a[e] = make_double2(r * cn, r * sn);
  }
}

__global__ void fill_sizes_kernel(int* n, long long* off, int batch, int nmin, int nmax, unsigned long long seed) {
  // One thread: sizes and packed offsets (tuning batches are modest).
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  long long o = 0;
  for (int j = 0; j < batch; ++j) {
    const int k = nmin + (int)(hash_uniform(seed + j) * (nmax - nmin + 1) - 1e-12);
    n[j] = k < nmin ? nmin : (k > nmax ? nmax : k);
    off[j] = o;
    o += (long long)n[j] * n[j];
  }
}

struct DeviceBuffers {
  void* p[6] = {};
  ~DeviceBuffers() {
    for (void* q : p)
      if (q) cudaFree(q);
  }
};

static float time_launches(cudaStream_t s, int reps, const std::function<cudaError_t()>& fn, cudaError_t* err) {
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  *err = fn();  // warm-up
  cudaEventRecord(e0, s);
  for (int r = 0; r < reps && *err == cudaSuccess; ++r) *err = fn();
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0.f;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return ms / (float)reps;
}

}  // namespace tzg

using namespace tzg;

extern "C" TOKURA_API int tokuraAutotune(tokurablas_t* handle, int n_min, int n_max, int batch_count,
                                         cudaStream_t stream) {
  if (handle == nullptr) return -1;
  if (!(1 <= n_min && n_min <= n_max && n_max <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (!(batch_count > 0)) return -6;
  const size_t nn = (size_t)n_max * n_max;
  DeviceBuffers b;
  if (cudaMalloc(&b.p[0], sizeof(double2) * nn * batch_count) != cudaSuccess ||
      cudaMalloc(&b.p[1], sizeof(double2) * (size_t)n_max * batch_count) != cudaSuccess ||
      cudaMalloc(&b.p[2], sizeof(double2) * (nn + (size_t)n_max) * batch_count) != cudaSuccess ||
      cudaMalloc(&b.p[3], (size_t)batch_count) != cudaSuccess)
    return 2;
  double2* A = static_cast<double2*>(b.p[0]);
  double2* eig = static_cast<double2*>(b.p[1]);
  double2* work = static_cast<double2*>(b.p[2]);
  char* flag = static_cast<char*>(b.p[3]);
  static const int kLanes[6] = {1, 2, 4, 8, 16, 32};
  static const int kThreads[4] = {32, 64, 128, 256};
  for (int n = n_min; n <= n_max; ++n) {
    const long long count = (long long)n * n * batch_count;
    fill_cgauss_kernel<<<handle->sm_count * 4, 256, 0, stream>>>(A, count, 0x5eed0000ULL + n);
    float best = 1e30f;
    PlainConfig best_cfg{1, 64};
    for (int li = 0; li < 6; ++li) {
      if (n <= 2 && kLanes[li] > 1) continue;
      for (int ti = 0; ti < 4; ++ti) {
        PlainConfig cfg{kLanes[li], kThreads[ti]};
        cfg.scaled = n >= scaled_threshold(handle, cfg.lanes) ? 1 : 0;
        cfg.qr_lanes = cfg.lanes;
        cfg.scaled_qr = cfg.scaled;
        cudaError_t err;
        const float ms = time_launches(stream, 2, [&]() {
          return launch_plain(cfg, n, batch_count, A, eig, work, flag, default_itmax(n), stream, 0,
                              use_shift_hints(handle, n), &handle->fj);
        }, &err);
        if (err != cudaSuccess) return 1;
        if (ms < best) {
          best = ms;
          best_cfg = cfg;
        }
      }
    }
    handle->plain[n] = best_cfg;
  }
  return cudaStreamSynchronize(stream) == cudaSuccess ? 0 : 1;
}

extern "C" TOKURA_API int tokuraAutotuneRagged(tokurablas_t* handle, int batch_count, int n_min, int n_max,
                                               cudaStream_t stream) {
  if (handle == nullptr) return -1;
  if (!(1 <= n_min && n_min <= n_max && n_max <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (!(batch_count > 0)) return -6;
  // Upper bound of the packed size; sizes are drawn uniformly in [n_min, n_max].
  const long long total = (long long)n_max * n_max * batch_count;
  const size_t wbytes = ragged_workspace_bytes(batch_count, total);
  DeviceBuffers b;
  if (cudaMalloc(&b.p[0], sizeof(double2) * (size_t)total) != cudaSuccess ||
      cudaMalloc(&b.p[1], sizeof(double2) * (size_t)n_max * batch_count) != cudaSuccess ||
      cudaMalloc(&b.p[2], wbytes) != cudaSuccess || cudaMalloc(&b.p[3], (size_t)batch_count) != cudaSuccess ||
      cudaMalloc(&b.p[4], sizeof(int) * (size_t)batch_count) != cudaSuccess ||
      cudaMalloc(&b.p[5], sizeof(long long) * (size_t)batch_count) != cudaSuccess)
    return 2;
  double2* A = static_cast<double2*>(b.p[0]);
  int* n = static_cast<int*>(b.p[4]);
  long long* off = static_cast<long long*>(b.p[5]);
  fill_cgauss_kernel<<<handle->sm_count * 4, 256, 0, stream>>>(A, total, 0x5eed7777ULL);
  fill_sizes_kernel<<<1, 1, 0, stream>>>(n, off, batch_count, n_min, n_max, 0x5eed1234ULL);
  float best = 1e30f;
  int best_lanes = 0;
  for (int lanes : {0, 1, 2, 4, 8}) {  // 0: lane width chosen per size bin
    cudaError_t err;
    const float ms = time_launches(stream, 2, [&]() {
      return launch_ragged(lanes, handle->sm_count, batch_count, n, off, nullptr, total, A,
                           static_cast<double2*>(b.p[1]), b.p[2], static_cast<char*>(b.p[3]), 0, stream, 0,
                           ragged_hint_min_order(handle), &handle->fj, handle->scaled_min_n);
    }, &err);
    if (err != cudaSuccess) return 1;
    if (ms < best) {
      best = ms;
      best_lanes = lanes;
    }
  }
  handle->ragged_lanes = best_lanes;
  return cudaStreamSynchronize(stream) == cudaSuccess ? 0 : 1;
}

static std::string device_key(const tokurablas_t* h) {
  cudaDeviceProp p;
  std::string name = "unknown";
  if (cudaGetDeviceProperties(&p, h->device) == cudaSuccess) name = p.name;
  for (char& c : name)
    if (c == ' ' || c == '\n' || c == '\t') c = '_';
  return name;
}

extern "C" TOKURA_API int tokuraSaveTuning(const tokurablas_t* handle, const char* path) {
  if (handle == nullptr || path == nullptr) return -1;
  FILE* f = std::fopen(path, "w");
  if (!f) return 1;
  std::fprintf(f, "tokura_zgeev_gb300_tuning 1\ndevice %s\nsms %d\n", device_key(handle).c_str(), handle->sm_count);
  for (int n = 1; n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE; ++n)
    if (handle->plain[n].lanes > 0)
      std::fprintf(f, "plain %d %d %d\n", n, handle->plain[n].lanes, handle->plain[n].threads);
  std::fprintf(f, "ragged %d\n", handle->ragged_lanes);
  return std::fclose(f) == 0 ? 0 : 1;
}

extern "C" TOKURA_API int tokuraLoadTuning(tokurablas_t* handle, const char* path) {
  if (handle == nullptr || path == nullptr) return -1;
  FILE* f = std::fopen(path, "r");
  if (!f) return 1;
  char word[64], dev[256];
  int version = 0, sms = 0;
  int status = 0;
  if (std::fscanf(f, "%63s %d", word, &version) != 2 || std::strcmp(word, "tokura_zgeev_gb300_tuning") != 0 ||
      version != 1 || std::fscanf(f, "%63s %255s", word, dev) != 2 || std::strcmp(word, "device") != 0 ||
      std::fscanf(f, "%63s %d", word, &sms) != 2 || std::strcmp(word, "sms") != 0) {
    std::fclose(f);
    return 2;  // malformed
  }
  if (device_key(handle) != dev || sms != handle->sm_count) {
    std::fclose(f);
    return 3;  // tuned for another device
  }
  tzg::PlainConfig table[65];
  for (int n = 0; n <= 64; ++n) table[n] = handle->plain[n];
  int ragged = handle->ragged_lanes;
  while (std::fscanf(f, "%63s", word) == 1) {
    if (std::strcmp(word, "plain") == 0) {
      int n, lanes, threads;
      if (std::fscanf(f, "%d %d %d", &n, &lanes, &threads) != 3 || n < 1 || n > 64 ||
          !plain_lanes_valid(lanes, false) || threads < 32 || threads > 256 || threads % 32) {
        status = 2;
        break;
      }
      table[n] = tzg::PlainConfig{lanes, threads};
    } else if (std::strcmp(word, "ragged") == 0) {
      if (std::fscanf(f, "%d", &ragged) != 1 || !(ragged >= 0 && ragged <= 8 && (ragged & (ragged - 1)) == 0)) {
        status = 2;
        break;
      }
    } else {
      status = 2;
      break;
    }
  }
  std::fclose(f);
  if (status != 0) return status;
  for (int n = 0; n <= 64; ++n) handle->plain[n] = table[n];
  handle->ragged_lanes = ragged;
  return 0;
}
