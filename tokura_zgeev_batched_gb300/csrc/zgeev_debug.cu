// tokuraDebugAttach: attaches a device DebugRecord (zgeev_debug.cuh) to every
// translation unit's kernels in the bounds-checked build; the release build
// exports the same entry point and returns -2.
#include <vector>

#include "../../include/tokura_blas_ext.h"
#include "zgeev_debug.cuh"

namespace tzg {
#ifdef TOKURA_DEBUG_BOUNDS
static std::vector<DebugAttachFn>& debug_registry() {
  static std::vector<DebugAttachFn> fns;
  return fns;
}
void debug_register(DebugAttachFn fn) { debug_registry().push_back(fn); }
#endif
}  // namespace tzg

extern "C" TOKURA_API int tokuraDebugAttach(void* record) {
#ifdef TOKURA_DEBUG_BOUNDS
  for (tzg::DebugAttachFn fn : tzg::debug_registry())
    if (fn(static_cast<tzg::DebugRecord*>(record)) != cudaSuccess) return 1;
  return 0;
#else
  (void)record;
  return -2;
#endif
}
