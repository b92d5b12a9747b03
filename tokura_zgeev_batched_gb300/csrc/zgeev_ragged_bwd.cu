// Ragged backward (Abar for a batch of mixed orders): the planning of
// zgeev_ragged.cu, then the persistent solver in backward mode. A translation
// unit of its own so that it compiles in parallel with the forward's.
#include "zgeev_ragged.cuh"

namespace tzg {

cudaError_t launch_ragged_backward(int lanes, int sms, int batch, const int* n, const long long* offsets,
                                   const long long* eig_offsets, long long total_elements, const double2* A,
                                   const double2* lam, const double2* gbar, double2* gA, void* work, char* flag,
                                   int itmax_override, cudaStream_t stream, int scaled_min_n) {
  if (!(lanes == 0 || lanes == 1 || lanes == 2 || lanes == 4 || lanes == 8)) return cudaErrorInvalidValue;
  const RaggedLayout lay = ragged_layout(batch, total_elements, 4);
  double2* stage = reinterpret_cast<double2*>(static_cast<char*>(work) + lay.stage_off);
  RaggedPlan* plan;
  int* sorted;
  const long long* eo;
  cudaError_t err = ragged_prepare(lanes, sms, batch, n, offsets, eig_offsets, total_elements, lay, work, flag,
                                   stream, &plan, &sorted, &eo);
  if (err != cudaSuccess) return err;
  const RaggedArgs args{offsets, eo, A, nullptr, lam, gbar, gA, stage, total_elements, flag, sorted, itmax_override,
                        0, nullptr, nullptr, 0, scaled_min_n};
  return launch_ragged_kernel<true, false, kPhaseAll>(lanes, sms, plan, args, stream);
}

}  // namespace tzg
