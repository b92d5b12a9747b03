// Host-buffer entry point: eigenvalues of matrices that live in host memory.
//
// Replaces the reference's multi-stream example driver
// (stream_test_with_MKL/main.cu:236-288: 8 streams x 8192-matrix chunks of
// H2D copy, tokura_zgeev_batched_gpu, D2H copy) with a library call. The
// batch is cut into chunks that are issued round-robin on the handle's own
// streams, so the copies of one chunk overlap the solves of others and
// several chunk kernels run side by side on the GPU. Device buffers are
// cached in the handle (grown on demand, freed by tokuraDestroy); a mutex in
// the handle serializes host-buffer calls on the same handle. Host memory
// should be pinned (cudaHostAlloc / cudaHostRegister) for the copies to
// overlap; pageable memory works but the driver then stages each copy.
#include <mutex>
#include <vector>

#include "../../include/tokura_blas_ext.h"
#include "tokura_handle.h"
#include "zgeev_internal.h"

namespace tzg {

void HostPipeline::release() {
  for (int s = 0; s < kStreams; ++s) {
    if (d_a[s]) cudaFree(d_a[s]);
    if (d_eig[s]) cudaFree(d_eig[s]);
    if (d_work[s]) cudaFree(d_work[s]);
    if (d_flag[s]) cudaFree(d_flag[s]);
    if (stream[s]) cudaStreamDestroy(stream[s]);
    if (copied[s]) cudaEventDestroy(copied[s]);
    d_a[s] = d_eig[s] = d_work[s] = nullptr;
    d_flag[s] = nullptr;
    stream[s] = nullptr;
    copied[s] = nullptr;
  }
  if (copy_begin) cudaEventDestroy(copy_begin);
  if (copy_end) cudaEventDestroy(copy_end);
  copy_begin = copy_end = nullptr;
  link_gbs = 0.0;
  for (int s = 0; s < kStreams; ++s) cap_a[s] = cap_eig[s] = cap_work[s] = cap_flag[s] = 0;
}

static cudaError_t grow(void** p, size_t* cap, size_t need) {
  if (need <= *cap) return cudaSuccess;
  if (*p) cudaFree(*p);
  *p = nullptr;
  *cap = 0;
  cudaError_t err = cudaMalloc(p, need);
  if (err == cudaSuccess) *cap = need;
  return err;
}

// Streams 0..streams-1 with device buffers for chunk[s] matrices each.
static cudaError_t ensure(HostPipeline& P, int n, const std::vector<int>& chunk, int streams) {
  cudaError_t err;
  if (!P.copy_begin && (err = cudaEventCreate(&P.copy_begin)) != cudaSuccess) return err;
  if (!P.copy_end && (err = cudaEventCreate(&P.copy_end)) != cudaSuccess) return err;
  for (int s = 0; s < streams; ++s) {
    if (!P.stream[s] && (err = cudaStreamCreateWithFlags(&P.stream[s], cudaStreamNonBlocking)) != cudaSuccess)
      return err;
    if (!P.copied[s] && (err = cudaEventCreateWithFlags(&P.copied[s], cudaEventDisableTiming)) != cudaSuccess)
      return err;
    const size_t a = sizeof(double2) * (size_t)n * n * chunk[s];
    const size_t e = sizeof(double2) * (size_t)n * chunk[s];
    const size_t w = a + e;  // staging plus the shift hints (the device call's workspace formula)
    if ((err = grow(&P.d_a[s], &P.cap_a[s], a)) != cudaSuccess) return err;
    if ((err = grow(&P.d_eig[s], &P.cap_eig[s], e)) != cudaSuccess) return err;
    if ((err = grow(&P.d_work[s], &P.cap_work[s], w)) != cudaSuccess) return err;
    if ((err = grow(reinterpret_cast<void**>(&P.d_flag[s]), &P.cap_flag[s], (size_t)chunk[s])) != cudaSuccess)
      return err;
  }
  return cudaSuccess;
}

}  // namespace tzg

extern "C" TOKURA_API int tokura_zgeev_batched_host(tokurablas_t* handle, int n, int batch_count,
                                                    const cuDoubleComplex* A, cuDoubleComplex* eigenvalues,
                                                    char* flag, int chunk_matrices) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (A == nullptr) return -3;
  if (eigenvalues == nullptr) return -4;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  if (chunk_matrices < 0) return -8;
  using tzg::HostPipeline;
  std::lock_guard<std::mutex> lock(handle->pipe_mutex);
  HostPipeline& P = handle->pipe;
  // Chunk plan, one stream and buffer set per chunk. With chunk_matrices > 0:
  // equal chunks of that size, round-robin over up to 16 streams. Otherwise
  // by the host-to-device rate the previous call saw (or the caller set with
  // tokuraSetHostLinkRate):
  //  * fast link (>= kFastLinkGBs; or the first call): 2 equal chunks (at
  //    least 1,024 matrices each). All copies land within a few percent of the
  //    solve time, and fewer, larger chunks leave the shortest tail: 65,536
  //    64x64 matrices over a 211 GB/s link took 597-599 ms with 2 chunks,
  //    615 ms with 1, 625-642 ms with 4, 699 ms with 8, against 592 ms for the
  //    solve alone (the second chunk's copy overlaps the first chunk's solve,
  //    and the two solves together fill the GPU).
  //  * slow link: growing chunks of 1/16, 1/16, 1/8, 1/4, 1/2 of the batch (at
  //    least 1,024 matrices each): the first solve starts after a small copy,
  //    and while the largest chunk is still arriving the earlier ones keep the
  //    GPU busy.
  constexpr double kFastLinkGBs = 100.0;
  std::vector<int> sizes;
  if (chunk_matrices > 0) {
    for (long long first = 0; first < batch_count; first += chunk_matrices)
      sizes.push_back((int)(batch_count - first < chunk_matrices ? batch_count - first : chunk_matrices));
  } else if (const double rate = P.link_gbs_fixed > 0.0 ? P.link_gbs_fixed : P.link_gbs;
             rate == 0.0 || rate >= kFastLinkGBs) {
    int parts = (batch_count + 1023) / 1024;
    if (parts > 2) parts = 2;
    const int c = (int)(((long long)batch_count + parts - 1) / parts);
    for (long long first = 0; first < batch_count; first += c)
      sizes.push_back((int)(batch_count - first < c ? batch_count - first : c));
  } else {
    int c = (batch_count + 15) / 16;
    if (c < 1024) c = 1024;
    long long left = batch_count;
    for (int k = 0; left > 0; ++k) {
      const int want = k <= 1 ? c : (int)(sizes.back() * 2LL < left ? sizes.back() * 2LL : left);
      const int m = (int)(want < left ? want : left);
      sizes.push_back(m);
      left -= m;
    }
  }
  const int nchunks = (int)sizes.size();
  const int streams = nchunks < HostPipeline::kStreams ? nchunks : HostPipeline::kStreams;
  std::vector<int> cap(streams, 0);  // largest chunk each stream carries
  for (int k = 0; k < nchunks; ++k) cap[k % streams] = sizes[k] > cap[k % streams] ? sizes[k] : cap[k % streams];
  if (tzg::ensure(P, n, cap, streams) != cudaSuccess) return 2;
  const int itmax = handle->itmax_override > 0 ? handle->itmax_override : tzg::default_itmax(n);
  const size_t nn = (size_t)n * n;
  // One launch shape for all chunks: they run side by side like one batch.
  const tzg::PlainConfig cfg = tzg::plain_config_for(handle, n, batch_count);
  long long first = 0;
  for (int k = 0; k < nchunks; first += sizes[k], ++k) {
    const int s = k % streams;
    const int m = sizes[k];
    cudaStream_t st = P.stream[s];
    // Copies go one after another, in chunk order: issued on separate streams
    // they could share the host link and delay the first, small chunk.
    if (k > 0 && cudaStreamWaitEvent(st, P.copied[(k - 1) % streams], 0) != cudaSuccess) return 1;
    if (k == 0 && cudaEventRecord(P.copy_begin, st) != cudaSuccess) return 1;
    if (cudaMemcpyAsync(P.d_a[s], A + first * nn, sizeof(double2) * nn * m, cudaMemcpyHostToDevice, st) !=
            cudaSuccess ||
        cudaEventRecord(P.copied[s], st) != cudaSuccess)
      return 1;
    if (k == nchunks - 1 && cudaEventRecord(P.copy_end, st) != cudaSuccess) return 1;
    if (tzg::launch_plain(cfg, n, m, static_cast<const double2*>(P.d_a[s]), static_cast<double2*>(P.d_eig[s]),
                          static_cast<double2*>(P.d_work[s]), P.d_flag[s], itmax, st, handle->balance_mode,
                          tzg::use_shift_hints(handle, n), &handle->fj) != cudaSuccess)
      return 1;
    if (cudaMemcpyAsync(eigenvalues + first * n, P.d_eig[s], sizeof(double2) * (size_t)n * m,
                        cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaMemcpyAsync(flag + first, P.d_flag[s], (size_t)m, cudaMemcpyDeviceToHost, st) != cudaSuccess)
      return 1;
  }
  for (int s = 0; s < streams; ++s)
    if (cudaStreamSynchronize(P.stream[s]) != cudaSuccess) return 1;
  // Without stream reuse the copies ran back to back, so the events bracket
  // the transfer alone (calls too small to time leave the previous rate).
  float ms = 0.0f;
  if (nchunks <= streams && cudaEventElapsedTime(&ms, P.copy_begin, P.copy_end) == cudaSuccess && ms > 0.05f)
    P.link_gbs = (double)sizeof(double2) * (double)nn * (double)batch_count / ((double)ms * 1e6);
  return 0;
}
