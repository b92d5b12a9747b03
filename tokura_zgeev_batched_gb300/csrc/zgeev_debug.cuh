// Bounds-checked build (-DTOKURA_DEBUG_BOUNDS): the stand-in for a memory
// checker. Every element access through a matrix view (MatView, RMatView and
// the estimator's shared-memory SMat) checks its (row, column) against the
// matrix order; strided runs of element pairs check their last element the
// same way (TZG_DBG_TOUCH at the call sites). A violation increments a device
// counter, records the first offending index and redirects the access to
// element (0, 0) of the same matrix, which is in bounds: nothing traps and
// nothing waits. The plain kernels also write each matrix's QR sweep count.
// The release build compiles none of this (the macros expand to nothing).
//
// The record is attached with tokuraDebugAttach (the debug library's only
// extra behaviour): a device struct of six 64-bit words, see DebugRecord.
#pragma once

#include <cuda_runtime.h>

namespace tzg {

// Device record (six 64-bit words, filled by the caller before attaching).
struct DebugRecord {
  unsigned long long violations;  // accesses outside their matrix
  long long first_r, first_c, first_n;  // the first of them (row, column, order)
  int* sweeps;                    // per-matrix QR sweeps of the plain kernels (may be null)
  long long sweeps_len;           // entries of sweeps
};

#ifdef TOKURA_DEBUG_BOUNDS

// One copy per translation unit (each kernel reads its own unit's copy);
// tokuraDebugAttach sets them all through the registry below.
static __device__ DebugRecord* g_tzg_dbg = nullptr;

__device__ __forceinline__ void dbg_violation(int r, int c, int n) {
  DebugRecord* d = g_tzg_dbg;
  if (d == nullptr) return;
  if (atomicAdd(&d->violations, 1ull) == 0ull) {
    d->first_r = r;
    d->first_c = c;
    d->first_n = n;
  }
}

// True (and counted) when (r, c) is outside an n x n matrix.
__device__ __forceinline__ bool dbg_out(int r, int c, int n) {
  if ((unsigned)r < (unsigned)n && (unsigned)c < (unsigned)n) return false;
  dbg_violation(r, c, n);
  return true;
}

__device__ __forceinline__ void dbg_record_sweeps(long long j, int sweeps) {
  DebugRecord* d = g_tzg_dbg;
  if (d != nullptr && d->sweeps != nullptr && j >= 0 && j < d->sweeps_len) d->sweeps[j] = sweeps;
}

// Checks an index against a bound (outputs, workspace entries).
__device__ __forceinline__ void dbg_index(long long i, long long bound) {
  if (i < 0 || i >= bound) dbg_violation((int)i, -1, (int)(bound > 0x7fffffffLL ? 0x7fffffff : bound));
}

using DebugAttachFn = cudaError_t (*)(DebugRecord*);
void debug_register(DebugAttachFn fn);  // tokura_capi.cpp

namespace {
cudaError_t debug_attach_unit(DebugRecord* rec) { return cudaMemcpyToSymbol(g_tzg_dbg, &rec, sizeof(rec)); }
struct DebugUnitRegistration {
  DebugUnitRegistration() { debug_register(&debug_attach_unit); }
};
DebugUnitRegistration g_debug_unit_registration;
}  // namespace

#define TZG_DBG_TOUCH(view, r, c) ((void)(view).at((r), (c)))
#define TZG_DBG_INDEX(i, bound) ::tzg::dbg_index((long long)(i), (long long)(bound))
// First and last elements (each with its pair partner at offset pr, pc) of a
// run of `count` elements from (r0, c0) in steps (dr, dc); nothing when empty.
#define TZG_DBG_RUN(view, r0, c0, dr, dc, count, pr, pc)                                                  \
  do {                                                                                                    \
    if ((count) > 0) {                                                                                    \
      TZG_DBG_TOUCH(view, (r0), (c0));                                                                    \
      TZG_DBG_TOUCH(view, (r0) + ((count)-1) * (dr) + (pr), (c0) + ((count)-1) * (dc) + (pc));            \
    }                                                                                                     \
  } while (0)

#else

#define TZG_DBG_TOUCH(view, r, c) ((void)0)
#define TZG_DBG_INDEX(i, bound) ((void)0)
#define TZG_DBG_RUN(view, r0, c0, dr, dc, count, pr, pc) ((void)0)

#endif

}  // namespace tzg
