// Plain batched eigenvalue-only ZGEEV in the reference's layout (contiguous
// n x n column-major matrices, eigenvalues[i + j*n]); the solver itself is
// in zgeev_plain.cuh.
#include "zgeev_plain.cuh"

namespace tzg {

cudaError_t launch_plain(const PlainConfig& cfg, int n, int batch, const double2* A, double2* eig, double2* work,
                         char* flag, int itmax, cudaStream_t stream, int balance, bool hints, const ForkJoin* fj) {
  return launch_batch(cfg, n, batch, ContigBatch{A, eig, n}, work, flag, itmax, stream, balance, hints, fj);
}

}  // namespace tzg
