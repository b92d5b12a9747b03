// C-ABI layer: handle lifecycle, argument validation with the reference's
// return codes, workspace query and dispatch to the sm_103a kernels.
//
// Reference interface replaced: tokura_zgeev_batched_library/src/
// tokura_zgeev_batched.cu:64-285 (tokuraCreate, tokuraDestroy,
// tokura_get_zgeeveigenvaluesgetworspacesize, tokura_zgeev_batched_gpu).
// Unlike the reference, the handle is not written by calls (the reference
// stores every call's arguments in it, tokura_zgeev_batched.cu:224-235), and
// the NULL-handle check happens before any dereference.
#include <cstdlib>
#include <new>

#include "../../include/tokura_blas_ext.h"
#include "tokura_handle.h"
#include "zgeev_internal.h"

using tzg::PlainConfig;

extern "C" int tokuraCreate(tokurablas_t** handle) {
  if (handle == nullptr) return -1;
  tokurablas_t* h = new (std::nothrow) tokurablas_t();
  if (h == nullptr) return -1;
  if (cudaGetDevice(&h->device) != cudaSuccess ||
      cudaDeviceGetAttribute(&h->sm_count, cudaDevAttrMultiProcessorCount, h->device) != cudaSuccess) {
    delete h;
    return 1;
  }
  tzg::init_default_tuning(h);
  // The estimator's second stream; without it calls run the estimator first on the caller's stream.
  h->fj.mu = &h->fj_mutex;
  if (cudaStreamCreateWithFlags(&h->fj.aux, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->fj.fork, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventCreateWithFlags(&h->fj.join, cudaEventDisableTiming) != cudaSuccess) {
    cudaGetLastError();
    if (h->fj.aux) cudaStreamDestroy(h->fj.aux);
    if (h->fj.fork) cudaEventDestroy(h->fj.fork);
    if (h->fj.join) cudaEventDestroy(h->fj.join);
    h->fj.aux = nullptr;
    h->fj.fork = h->fj.join = nullptr;
  }
  // A tuning file written by tokuraSaveTuning for this device is applied if named in the environment.
  if (const char* path = std::getenv("TOKURA_ZGEEV_TUNING_FILE")) tokuraLoadTuning(h, path);
  *handle = h;
  return 0;
}

extern "C" int tokuraDestroy(tokurablas_t* handle) {
  if (handle != nullptr) {
    int prev = 0;
    const bool switch_dev = cudaGetDevice(&prev) == cudaSuccess && prev != handle->device;
    if (switch_dev) cudaSetDevice(handle->device);
    handle->pipe.release();
    if (handle->fj.aux) cudaStreamDestroy(handle->fj.aux);
    if (handle->fj.fork) cudaEventDestroy(handle->fj.fork);
    if (handle->fj.join) cudaEventDestroy(handle->fj.join);
    if (switch_dev) cudaSetDevice(prev);
  }
  delete handle;
  return 0;
}

extern "C" size_t tokura_get_zgeeveigenvaluesgetworspacesize(int n, int batch_count) {
  if (!(0 < n && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return (size_t)-1;
  if (!(0 < batch_count)) return (size_t)-2;
  const size_t nn = (size_t)n * (size_t)n;
  return sizeof(cuDoubleComplex) * nn * (size_t)batch_count + sizeof(cuDoubleComplex) * (size_t)n * (size_t)batch_count;
}

extern "C" int tokura_zgeev_batched_gpu(tokurablas_t* handle, int n, int batch_count, cuDoubleComplex* A,
                                        cuDoubleComplex* eigenvalues, cuDoubleComplex* work, char* flag,
                                        cudaStream_t cudastream) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (A == nullptr) return -3;
  if (eigenvalues == nullptr) return -4;
  if (work == nullptr) return -5;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  const PlainConfig cfg = tzg::plain_config_for(handle, n, batch_count);
  const int itmax = handle->itmax_override > 0 ? handle->itmax_override : tzg::default_itmax(n);
  const cudaError_t err = tzg::launch_plain(cfg, n, batch_count, reinterpret_cast<const double2*>(A),
                                            reinterpret_cast<double2*>(eigenvalues),
                                            reinterpret_cast<double2*>(work), flag, itmax, cudastream,
                                            handle->balance_mode, tzg::use_shift_hints(handle, n), &handle->fj);
  return err == cudaSuccess ? 0 : 1;
}

extern "C" int tokuraSetSweepCap(tokurablas_t* handle, int cap) {
  if (handle == nullptr || cap < 0) return -1;
  handle->itmax_override = cap;
  return 0;
}

extern "C" int tokuraSetPlainConfig(tokurablas_t* handle, int n, int lanes_per_matrix, int threads_per_block) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (!tzg::plain_lanes_valid(lanes_per_matrix, true)) return -3;
  if (!(threads_per_block == 0 || (threads_per_block >= 32 && threads_per_block <= 256 && threads_per_block % 32 == 0)))
    return -4;
  handle->plain[n] = PlainConfig{lanes_per_matrix, threads_per_block};
  return 0;
}

extern "C" int tokuraSetPlainQrLanes(tokurablas_t* handle, int n, int lanes_per_matrix) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (!tzg::plain_lanes_valid(lanes_per_matrix, true)) return -3;
  handle->plain_qr_lanes[n] = lanes_per_matrix;
  return 0;
}

extern "C" int tokuraSetRealConfig(tokurablas_t* handle, int n, int lanes_per_matrix, int threads_per_block) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (!(lanes_per_matrix == 0 || lanes_per_matrix == 1 || lanes_per_matrix == 2 || lanes_per_matrix == 4 ||
        lanes_per_matrix == 8))
    return -3;
  if (!(threads_per_block == 0 || (threads_per_block >= 32 && threads_per_block <= 256 && threads_per_block % 32 == 0)))
    return -4;
  handle->real[n] = PlainConfig{lanes_per_matrix, threads_per_block};
  return 0;
}

extern "C" int tokuraGetPlainConfig(const tokurablas_t* handle, int n, int batch_count, int* lanes_per_matrix,
                                    int* threads_per_block) {
  if (handle == nullptr || lanes_per_matrix == nullptr || threads_per_block == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (!(batch_count > 0)) return -6;
  const PlainConfig c = tzg::plain_config_for(handle, n, batch_count);
  *lanes_per_matrix = c.lanes;
  *threads_per_block = c.threads;
  return 0;
}

extern "C" size_t tokura_get_zgeev_ragged_workspacesize(int batch_count, long long total_elements) {
  if (!(batch_count > 0)) return (size_t)-2;
  if (!(total_elements > 0)) return (size_t)-3;
  return tzg::ragged_workspace_bytes(batch_count, total_elements);
}

extern "C" int tokura_zgeev_ragged_gpu(tokurablas_t* handle, int batch_count, const int* n, const long long* offsets,
                                       const long long* eig_offsets, long long total_elements,
                                       const cuDoubleComplex* A, cuDoubleComplex* eigenvalues, void* work, char* flag,
                                       cudaStream_t stream) {
  if (handle == nullptr) return -1;
  if (n == nullptr) return -2;
  if (A == nullptr) return -3;
  if (eigenvalues == nullptr) return -4;
  if (work == nullptr) return -5;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  if (offsets == nullptr) return -8;
  if (!(total_elements > 0)) return -9;
  const cudaError_t err = tzg::launch_ragged(handle->ragged_lanes, handle->sm_count, batch_count, n, offsets, eig_offsets,
                                             total_elements, reinterpret_cast<const double2*>(A),
                                             reinterpret_cast<double2*>(eigenvalues), work, flag,
                                             handle->itmax_override, stream, handle->balance_mode,
                                             tzg::ragged_hint_min_order(handle), &handle->fj, handle->scaled_min_n);
  return err == cudaSuccess ? 0 : 1;
}

extern "C" int tokuraSetHostLinkRate(tokurablas_t* handle, double gbs) {
  if (handle == nullptr) return -1;
  if (!(gbs >= 0.0 && gbs < 1e9)) return -2;  // also rejects NaN
  std::lock_guard<std::mutex> lock(handle->pipe_mutex);
  handle->pipe.link_gbs_fixed = gbs;
  return 0;
}

extern "C" int tokuraSetRaggedHintMinOrder(tokurablas_t* handle, int n) {
  if (handle == nullptr) return -1;
  if (!(n >= 1 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE + 1)) return -2;
  handle->ragged_hint_min_n = n;
  return 0;
}

extern "C" int tokuraSetRaggedLanes(tokurablas_t* handle, int lanes_per_matrix) {
  if (handle == nullptr) return -1;
  if (!(lanes_per_matrix == 0 || lanes_per_matrix == 1 || lanes_per_matrix == 2 || lanes_per_matrix == 4 ||
        lanes_per_matrix == 8))
    return -3;
  handle->ragged_lanes = lanes_per_matrix;
  return 0;
}

extern "C" size_t tokura_get_zgeev_backward_workspacesize(int n, int batch_count) {
  if (!(0 < n && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return (size_t)-1;
  if (!(0 < batch_count)) return (size_t)-2;
  return tzg::backward_workspace_bytes(n, batch_count);
}

extern "C" int tokura_zgeev_backward_gpu(tokurablas_t* handle, int n, int batch_count, const cuDoubleComplex* A,
                                         const cuDoubleComplex* eigenvalues, const cuDoubleComplex* grad_eigenvalues,
                                         cuDoubleComplex* grad_A, void* work, char* flag, cudaStream_t stream) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (A == nullptr) return -3;
  if (eigenvalues == nullptr || grad_eigenvalues == nullptr) return -4;
  if (work == nullptr) return -5;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  if (grad_A == nullptr) return -8;
  const int lanes = tzg::group_lanes_for(handle, n, batch_count);
  const int itmax = handle->itmax_override > 0 ? handle->itmax_override : tzg::default_itmax(n);
  const cudaError_t err = tzg::launch_backward(
      lanes, n, batch_count, reinterpret_cast<const double2*>(A), reinterpret_cast<const double2*>(eigenvalues),
      reinterpret_cast<const double2*>(grad_eigenvalues), reinterpret_cast<double2*>(grad_A),
      static_cast<double2*>(work), flag, itmax, stream, tzg::scaled_threshold(handle, lanes));
  return err == cudaSuccess ? 0 : 1;
}

extern "C" size_t tokura_get_zgeev_ragged_backward_workspacesize(int batch_count, long long total_elements) {
  if (!(batch_count > 0)) return (size_t)-2;
  if (!(total_elements > 0)) return (size_t)-3;
  return tzg::ragged_backward_workspace_bytes(batch_count, total_elements);
}

extern "C" int tokura_zgeev_ragged_backward_gpu(tokurablas_t* handle, int batch_count, const int* n,
                                                const long long* offsets, const long long* eig_offsets,
                                                long long total_elements, const cuDoubleComplex* A,
                                                const cuDoubleComplex* eigenvalues,
                                                const cuDoubleComplex* grad_eigenvalues, cuDoubleComplex* grad_A,
                                                void* work, char* flag, cudaStream_t stream) {
  if (handle == nullptr) return -1;
  if (n == nullptr) return -2;
  if (A == nullptr) return -3;
  if (eigenvalues == nullptr || grad_eigenvalues == nullptr) return -4;
  if (work == nullptr) return -5;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  if (offsets == nullptr) return -8;
  if (!(total_elements > 0)) return -9;
  if (grad_A == nullptr) return -10;
  const cudaError_t err = tzg::launch_ragged_backward(
      handle->ragged_lanes, handle->sm_count, batch_count, n, offsets, eig_offsets, total_elements,
      reinterpret_cast<const double2*>(A), reinterpret_cast<const double2*>(eigenvalues),
      reinterpret_cast<const double2*>(grad_eigenvalues), reinterpret_cast<double2*>(grad_A), work, flag,
      handle->itmax_override, stream, handle->scaled_min_n);
  return err == cudaSuccess ? 0 : 1;
}

extern "C" size_t tokura_get_zgeev_vectors_workspacesize(int n, int batch_count) {
  if (!(0 < n && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return (size_t)-1;
  if (!(0 < batch_count)) return (size_t)-2;
  return tzg::vectors_workspace_bytes(n, batch_count);
}

extern "C" int tokura_zgeev_vectors_batched_gpu(tokurablas_t* handle, int n, int batch_count,
                                                const cuDoubleComplex* A, cuDoubleComplex* eigenvalues,
                                                cuDoubleComplex* VL, cuDoubleComplex* VR, void* work, char* flag,
                                                cudaStream_t stream) {
  if (handle == nullptr) return -1;
  if (!(n > 0 && n <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE)) return -2;
  if (A == nullptr) return -3;
  if (eigenvalues == nullptr) return -4;
  if (work == nullptr) return -5;
  if (!(batch_count > 0)) return -6;
  if (flag == nullptr) return -7;
  const int lanes = tzg::group_lanes_for(handle, n, batch_count);
  const int itmax = handle->itmax_override > 0 ? handle->itmax_override : tzg::default_itmax(n);
  const cudaError_t err = tzg::launch_vectors(
      lanes, n, batch_count, reinterpret_cast<const double2*>(A), reinterpret_cast<double2*>(eigenvalues),
      reinterpret_cast<double2*>(VL), reinterpret_cast<double2*>(VR), static_cast<double2*>(work), flag, itmax, stream,
      tzg::use_shift_hints(handle, n), &handle->fj, tzg::scaled_threshold(handle, lanes));
  return err == cudaSuccess ? 0 : 1;
}

extern "C" int tokuraSetBalancing(tokurablas_t* handle, int mode) {
  if (handle == nullptr) return -1;
  if (mode < 0 || mode > 3) return -2;
  handle->balance_mode = mode;
  return 0;
}

extern "C" int tokuraSetScaledRotations(tokurablas_t* handle, int min_order) {
  if (handle == nullptr) return -1;
  if (!(min_order >= 1 && min_order <= TOKURA_ZGEEV_BATCHED_MAX_MATRIX_SIZE + 1)) return -2;
  handle->scaled_min_n = min_order;
  return 0;
}

extern "C" int tokuraSetShiftHints(tokurablas_t* handle, int mode) {
  if (handle == nullptr) return -1;
  if (mode < 0 || mode > 2) return -2;
  handle->shift_hints = mode;
  return 0;
}
