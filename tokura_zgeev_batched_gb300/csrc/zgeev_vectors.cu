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

template <int L>
__device__ int vectors_matrix(const double2* __restrict__ src, double2* __restrict__ w_out, double2* __restrict__ VL,
                              double2* __restrict__ VR, const BwdViews& V, const Group<L>& G, int itmax,
                              const float2* __restrict__ est) {
  const int n = V.T.n;
  bool nonfinite, zero;
  const int shift = stage_and_scale<L>(src, V.T, G, nonfinite, zero);
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
  const int status = schur_qr<L>(V, G, nullptr, nullptr, 1.0, itmax, est);
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

template <int L>
__global__ void __launch_bounds__(128) zgeev_vectors_kernel(int n, int batch, const double2* __restrict__ A,
                                                            double2* __restrict__ w, double2* __restrict__ VL,
                                                            double2* __restrict__ VR, double2* __restrict__ work,
                                                            char* __restrict__ flag, int itmax,
                                                            const float2* __restrict__ est) {
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
  const int status = vectors_matrix<L>(A + j * nn, w + j * n, VL ? VL + j * nn : nullptr, VR ? VR + j * nn : nullptr,
                                       V, G, itmax, est != nullptr ? est + j * n : nullptr);
  if (G.rank == 0) flag[j] = (char)status;
}

size_t vectors_workspace_bytes(int n, int batch) {
  return backward_workspace_bytes(n, batch) + sizeof(float2) * (size_t)n * (size_t)batch;
}

// hints: the FP32 estimator runs first on `stream` (its eigenvalues steer the
// first shift after each deflation of the Schur iteration, as in the
// eigenvalue path); they go after the backward-sized workspace.
cudaError_t launch_vectors(int lanes, int n, int batch, const double2* A, double2* w, double2* VL, double2* VR,
                           double2* work, char* flag, int itmax, cudaStream_t stream, bool hints) {
  float2* est = nullptr;
  if (hints) {
    est = reinterpret_cast<float2*>(reinterpret_cast<char*>(work) + backward_workspace_bytes(n, batch));
    const cudaError_t err = launch_estimates(n, batch, ContigBatch{A, nullptr, n}, est, stream);
    if (err != cudaSuccess) return err;
  }
  const int tw = 32 / lanes;
  const long long warps = ((long long)batch + tw - 1) / tw;
  const int threads = 64;  // small blocks spread a resident batch evenly over the SMs
  const long long blocks = (warps * 32 + threads - 1) / threads;
  if (blocks > 0x7fffffffLL) return cudaErrorInvalidValue;
  switch (lanes) {
    case 1:
      zgeev_vectors_kernel<1><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, w, VL, VR, work, flag, itmax, est);
      break;
    case 2:
      zgeev_vectors_kernel<2><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, w, VL, VR, work, flag, itmax, est);
      break;
    case 4:
      zgeev_vectors_kernel<4><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, w, VL, VR, work, flag, itmax, est);
      break;
    case 8:
      zgeev_vectors_kernel<8><<<(unsigned)blocks, threads, 0, stream>>>(n, batch, A, w, VL, VR, work, flag, itmax, est);
      break;
    default:
      return cudaErrorInvalidValue;
  }
  return cudaGetLastError();
}

}  // namespace tzg
