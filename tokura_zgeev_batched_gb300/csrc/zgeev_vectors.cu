// Eigenvalues with left and/or right eigenvectors (ZGEEV, JOBVL/JOBVR = 'V').
//
// The reference computes eigenvalues only (README.md:63: "No eigenvectors are
// computed"). Per matrix (one lane group), reusing the gradient path's pieces:
// Hessenberg with tau kept, Q from the reflectors, single-shift QR to Schur
// form T with Q accumulated (Wilkinson shifts, ulp-level deflation as the
// eigenvalue path), eigenvectors X (T X = X diag T) and Y (Y^H T = diag T Y^H)
// of the triangular T, then VR = Q X and VL = Q Y, each column scaled like
// LAPACK zgeev: unit 2-norm, component of largest modulus real and positive.
#include "zgeev_backward.cuh"
#include "zgeev_internal.h"
#include "zgeev_plain.cuh"

namespace tzg {

// out[:, k] = Q C[:, k] for the columns k owned by this lane, C unit-diagonal
// triangular stored in XY (kUpper: C_jk for j < k; else C_jk for j > k),
// then LAPACK's normalization. out is the caller's column-major n x n matrix.
template <int L, bool kUpper>
__device__ void schur_vectors(const BwdViews& V, const Group<L>& G, double2* __restrict__ out) {
  const MatView& Q = V.Q;
  const MatView& XY = V.XY;
  const int n = Q.n;
  for (int k = G.rank; k < n; k += L) {
    const int j0 = kUpper ? 0 : k, j1 = kUpper ? k : n - 1;
    double nrm2 = 0.0, best = -1.0;
    int rbest = 0;
    for (int r = 0; r < n; ++r) {
      double2 acc = *Q.at(r, k);  // C_kk = 1
      for (int j = j0; j <= j1; ++j) {
        if (j == k) continue;
        const double2 q = *Q.at(r, j), c = *XY.at(j, k);
        acc.x = fma(q.x, c.x, fma(-q.y, c.y, acc.x));
        acc.y = fma(q.x, c.y, fma(q.y, c.x, acc.y));
      }
      out[r + k * n] = acc;
      const double m2 = fma(acc.x, acc.x, acc.y * acc.y);
      nrm2 += m2;
      if (m2 > best) {
        best = m2;
        rbest = r;
      }
    }
    // Scale by conj(v_r*) / (|v_r*| * ||v||): unit norm, v_r* real positive.
    const double2 vb = out[rbest + k * n];
    const double s = (best > 0.0 && nrm2 > 0.0) ? 1.0 / sqrt(best * nrm2) : 0.0;
    const double2 f = make_double2(vb.x * s, -vb.y * s);
    for (int r = 0; r < n; ++r) out[r + k * n] = cmul(out[r + k * n], f);
    out[rbest + k * n].y = 0.0;
  }
}

// First half: stage, Hessenberg (tau kept), Q. Returns kPrepared with the
// pre-scaling exponent in `shift`, or the flag of a non-finite matrix (whose
// outputs are then written).
template <int L>
__device__ int vectors_prepare(const double2* __restrict__ src, double2* __restrict__ w_out, double2* __restrict__ VL,
                               double2* __restrict__ VR, const BwdViews& V, const Group<L>& G, int& shift) {
  const int n = V.T.n;
  bool nonfinite, zero;
  shift = stage_and_scale<L>(src, V.T, G, nonfinite, zero);
  if (nonfinite) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int i = G.rank; i < n; i += L) w_out[i] = make_double2(nan, nan);
    for (int e = G.rank; e < n * n; e += L) {
      if (VL) VL[e] = make_double2(nan, nan);
      if (VR) VR[e] = make_double2(nan, nan);
    }
    return kNonFinite;
  }
  hessenberg<L>(V.T, G, V.vec, V.vs);
  G.sync();
  form_q<L>(V, G);
  return kPrepared;
}

// Second half: Schur form with Q, eigenvalues, eigenvectors.
template <int L>
__device__ int vectors_finish(double2* __restrict__ w_out, double2* __restrict__ VL, double2* __restrict__ VR,
                              const BwdViews& V, const Group<L>& G, int itmax, int shift,
                              const float2* __restrict__ est, int scaled_min_n) {
  const int n = V.T.n;
  const int status = (n >= scaled_min_n && n >= kScaledMinN) ? schur_qr_scaled<L>(V, G, nullptr, nullptr, 1.0, itmax, est)
                                                            : schur_qr<L>(V, G, nullptr, nullptr, 1.0, itmax, est);
  const double unscale = shift != 0 ? pow2(shift) : 1.0;
  for (int i = G.rank; i < n; i += L) {
    const double2 d = *V.T.at(i, i);
    w_out[i] = make_double2(d.x * unscale, d.y * unscale);
  }
  if (status != kConverged) return status;
  G.sync();
  eigenvectors_of_t<L>(V, G);
  if (VR) schur_vectors<L, true>(V, G, VR);
  if (VL) schur_vectors<L, false>(V, G, VL);
  return kConverged;
}

// kPhaseAll: the whole computation; kPhasePrepare / kPhaseQR: the two halves
// in separate launches (state[j]: pre-scaling exponent or kStateDone), so the
// FP32 estimator can run beside the first.
template <int L, int kPhase>
__global__ void __launch_bounds__(128) zgeev_vectors_kernel(int n, int batch, const double2* __restrict__ A,
                                                            double2* __restrict__ w, double2* __restrict__ VL,
                                                            double2* __restrict__ VR, double2* __restrict__ work,
                                                            char* __restrict__ flag, int itmax,
                                                            const float2* __restrict__ est, int* __restrict__ state,
                                                            int scaled_min_n) {
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
  const long long region = nn * batch;
  const long long j = g0 + slot;
  double2* base = work + g0 * nn + slot;
  BwdViews V{MatView{base, n, tw}, MatView{base + region, n, tw}, MatView{base + 2 * region, n, tw},
             work + 3 * region + g0 * n + slot, tw};
  double2* vl = VL ? VL + j * nn : nullptr;
  double2* vr = VR ? VR + j * nn : nullptr;
  const float2* e = est != nullptr ? est + j * n : nullptr;
  int status;
  if (kPhase == kPhaseQR) {
    const int s = state[j];
    if (s == kStateDone) return;  // group-uniform
    status = vectors_finish<L>(w + j * n, vl, vr, V, G, itmax, s, e, scaled_min_n);
  } else {
    int shift;
    status = vectors_prepare<L>(A + j * nn, w + j * n, vl, vr, V, G, shift);
    if (kPhase == kPhasePrepare) {
      if (G.rank == 0) state[j] = status == kPrepared ? shift : kStateDone;
      if (status == kPrepared) return;
    } else if (status == kPrepared) {
      status = vectors_finish<L>(w + j * n, vl, vr, V, G, itmax, shift, e, scaled_min_n);
    }
  }
  if (G.rank == 0) flag[j] = (char)status;
}

size_t vectors_workspace_bytes(int n, int batch) {
  return backward_workspace_bytes(n, batch) + (sizeof(float2) * (size_t)n + sizeof(int)) * (size_t)batch;
}

template <int kPhase>
static cudaError_t launch_vectors_phase(int lanes, unsigned blocks, int threads, cudaStream_t stream, int n,
                                        int batch, const double2* A, double2* w, double2* VL, double2* VR,
                                        double2* work, char* flag, int itmax, const float2* est, int* state,
                                        int scaled_min_n) {
  const auto launch = [&](auto k) -> cudaError_t {
    if (kPhase != kPhaseAll) {  // shared memory for the estimator running beside
      const cudaError_t err =
          cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
      if (err != cudaSuccess) return err;
    }
    k<<<blocks, threads, 0, stream>>>(n, batch, A, w, VL, VR, work, flag, itmax, est, state, scaled_min_n);
    return cudaGetLastError();
  };
  switch (lanes) {
    case 1: return launch(zgeev_vectors_kernel<1, kPhase>);
    case 2: return launch(zgeev_vectors_kernel<2, kPhase>);
    case 4: return launch(zgeev_vectors_kernel<4, kPhase>);
    case 8: return launch(zgeev_vectors_kernel<8, kPhase>);
    default: return cudaErrorInvalidValue;
  }
}

// hints: FP32 estimates steer the first shift after each deflation of the
// Schur iteration, as in the eigenvalue path; they and the phase state go
// after the backward-sized workspace. With fj the estimator runs on fj->aux
// beside the first half (stage, Hessenberg, Q); without, first on `stream`.
cudaError_t launch_vectors(int lanes, int n, int batch, const double2* A, double2* w, double2* VL, double2* VR,
                           double2* work, char* flag, int itmax, cudaStream_t stream, bool hints, const ForkJoin* fj,
                           int scaled_min_n) {
  const int tw = 32 / lanes;
  const long long warps = ((long long)batch + tw - 1) / tw;
  const int threads = 32;  // one-warp blocks spread a resident batch evenly over the SMs
  const long long blocks = (warps * 32 + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  if (!hints)
    return launch_vectors_phase<kPhaseAll>(lanes, (unsigned)blocks, threads, stream, n, batch, A, w, VL, VR, work,
                                           flag, itmax, nullptr, nullptr, scaled_min_n);
  float2* est = reinterpret_cast<float2*>(reinterpret_cast<char*>(work) + backward_workspace_bytes(n, batch));
  int* state = reinterpret_cast<int*>(est + (size_t)n * batch);
  const ContigBatch src{A, nullptr, n};
  cudaError_t err;
  if (fj == nullptr || fj->aux == nullptr) {
    if ((err = launch_estimates(n, batch, src, est, stream)) != cudaSuccess) return err;
    return launch_vectors_phase<kPhaseAll>(lanes, (unsigned)blocks, threads, stream, n, batch, A, w, VL, VR, work,
                                           flag, itmax, est, nullptr, scaled_min_n);
  }
  std::lock_guard<std::mutex> lock(*fj->mu);
  if ((err = cudaEventRecord(fj->fork, stream)) != cudaSuccess) return err;
  if ((err = cudaStreamWaitEvent(fj->aux, fj->fork, 0)) != cudaSuccess) return err;
  if ((err = launch_estimates(n, batch, src, est, fj->aux)) != cudaSuccess) return err;
  if ((err = cudaEventRecord(fj->join, fj->aux)) != cudaSuccess) return err;
  if ((err = launch_vectors_phase<kPhasePrepare>(lanes, (unsigned)blocks, threads, stream, n, batch, A, w, VL, VR,
                                                 work, flag, itmax, nullptr, state, scaled_min_n)) != cudaSuccess)
    return err;
  if ((err = cudaStreamWaitEvent(stream, fj->join, 0)) != cudaSuccess) return err;
  return launch_vectors_phase<kPhaseQR>(lanes, (unsigned)blocks, threads, stream, n, batch, A, w, VL, VR, work, flag,
                                        itmax, est, state, scaled_min_n);
}

}  // namespace tzg
