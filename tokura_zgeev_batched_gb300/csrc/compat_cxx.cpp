// C++-linkage forwarding shims carrying the reference's mangled symbol names.
//
// The reference header declares its API without extern "C"
// (tokura_zgeev_batched_library/include/tokura_blas.h:129-151), so objects
// compiled against it reference names such as
// _Z24tokura_zgeev_batched_gpuP12tokurablas_tiiP7double2S2_S2_PcP11CUstream_st.
// This file defines those C++ functions and forwards them to the C-ABI entry
// points, so such objects link against this library unchanged. It does not
// include tokura_blas.h: the C symbols are reached through asm labels.
#include <cuda_runtime_api.h>
#include <vector_types.h>
#include <stddef.h>

struct tokurablas_t;

extern "C" {
int tzg_c_tokuraCreate(tokurablas_t** h) __asm__("tokuraCreate");
int tzg_c_tokuraDestroy(tokurablas_t* h) __asm__("tokuraDestroy");
size_t tzg_c_workspace(int n, int batch) __asm__("tokura_get_zgeeveigenvaluesgetworspacesize");
int tzg_c_zgeev(tokurablas_t* h, int n, int batch, double2* A, double2* eig, double2* work, char* flag,
                cudaStream_t s) __asm__("tokura_zgeev_batched_gpu");
}

__attribute__((visibility("default"))) int tokuraCreate(tokurablas_t** h) { return tzg_c_tokuraCreate(h); }
__attribute__((visibility("default"))) int tokuraDestroy(tokurablas_t* h) { return tzg_c_tokuraDestroy(h); }
__attribute__((visibility("default"))) size_t tokura_get_zgeeveigenvaluesgetworspacesize(int n, int batch) {
  return tzg_c_workspace(n, batch);
}
__attribute__((visibility("default"))) int tokura_zgeev_batched_gpu(tokurablas_t* h, int n, int batch, double2* A,
                                                                    double2* eig, double2* work, char* flag,
                                                                    cudaStream_t s) {
  return tzg_c_zgeev(h, n, batch, A, eig, work, flag, s);
}
