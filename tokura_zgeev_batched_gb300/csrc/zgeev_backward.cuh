// Backward of the eigenvalue map: Abar from (A, lambda, gbar), one lane group per matrix.
//
// The reference computes eigenvalues only and has no derivative. Here the
// forward stores nothing but A and its eigenvalues; the backward recomputes
// the Schur form A = Q T Q^H and returns, in torch's convention for complex
// gradients,
//     Abar = W diag(gbar) V^H,  V = Q X (right eigenvectors), W = Q X^{-H},
// where T X = X diag(T) with X unit upper triangular. X^{-1} = Y^H with Y^H the
// unit upper triangular matrix of left eigenvectors of T, so
//     Abar = Q (Y diag(gbar) X^H) Q^H,
// and the middle factor M = Y diag(gbar) X^H is lower triangular.
//
// Steps (FP64 instructions at n = 48 in parentheses, forward ~ 2.7 M):
//   1. stage + exact pre-scaling, Householder Hessenberg keeping tau (0.74 M);
//   2. Q from the reflectors by backward accumulation (0.3 M);
//   3. single-shift QR with full-row/column updates and Q accumulation, with
//      the forward's eigenvalues as shifts ("perfect shifts"; Wilkinson/ad hoc
//      shifts if one misses). A perfect-shift sweep leaves the bottom
//      subdiagonal near, but often just above, ulp * |diagonal|; deflating
//      at kGradDeflationTol = 100 ulp instead (a backward error of ~2e-14 in
//      T, i.e. ~1e-13 relative in the gradient for separated spectra) brings
//      the cost to ~1.0 sweep per eigenvalue instead of ~1.75 (~3.4 with
//      Wilkinson shifts alone);
//      each deflated T_ii is matched to the nearest unused forward eigenvalue,
//      whose gradient it takes (~1.8 M);
//   4. X and Y by triangular back-substitution (0.2 M);
//   5. Z = diag(gbar) X^H, M = Y Z in place, P = Q M, Abar = P Q^H (0.8 M).
#pragma once

#include "zgeev_lane.cuh"
#include "zgeev_scaled_qr.cuh"

namespace tzg {

// Flag: two eigenvalues of T coincide to working precision, so the derivative
// does not exist; Abar is still returned with the denominators clamped.
constexpr int kCloseEigenvalues = 4;

// Relative deflation threshold of the gradient's Schur recomputation.
constexpr double kGradDeflationTol = 100.0 * kUlp;

struct BwdViews {
  MatView T, Q, XY;  // tile-interleaved n x n views (same layout as the forward's staging)
  double2* vec;      // n entries at vec[i * vs]: tau during step 2, gradient per T_ii after step 3
  int vs;
};

// Q <- P_0 P_1 ... P_{n-3} (backward accumulation; P_r only touches rows and
// columns r+1..n-1 of the partial product).
template <int L>
__device__ void form_q(const BwdViews& V, const Group<L>& G) {
  const MatView& T = V.T;
  const MatView& Q = V.Q;
  const int n = T.n, rs = T.rs;
  for (int c = G.rank; c < n; c += L)
    for (int r = 0; r < n; ++r) *Q.at(r, c) = make_double2(r == c ? 1.0 : 0.0, 0.0);
  G.sync();
  for (int r = n - 3; r >= 0; --r) {
    const double tau = V.vec[r * V.vs].x;
    if (tau == 0.0) continue;  // same value for the whole group
    const int m = n - r - 1;
    const double2* x = T.at(r + 1, r);
    int c = r + 1 + G.rank;
    for (; c + L < n; c += 2 * L) {
      double2* p[2] = {Q.at(r + 1, c), Q.at(r + 1, c + L)};
      TZG_DBG_TOUCH(Q, r + m, c + L);
      TZG_DBG_TOUCH(T, r + m, r);
      reflect_vectors<2, false>(p, x, m, rs, rs, tau);
    }
    if (c < n) {
      double2* p[1] = {Q.at(r + 1, c)};
      TZG_DBG_TOUCH(Q, r + m, c);
      reflect_vectors<1, false>(p, x, m, rs, rs, tau);
    }
    G.sync();
  }
}

// Index of the forward eigenvalue (times `scale`) nearest to z among those not in `used`.
__device__ __forceinline__ int nearest_unused(const double2* __restrict__ lam, int n, unsigned long long used,
                                              double2 z, double scale) {
  int best = -1;
  double bd = 0.0;
  for (int k = 0; k < n; ++k) {
    if ((used >> k) & 1ull) continue;
    const double2 l = lam[k];
    const double dx = fma(l.x, scale, -z.x), dy = fma(l.y, scale, -z.y);
    const double d = fma(dx, dx, dy * dy);
    if (best < 0 || d < bd) {
      best = k;
      bd = d;
    }
  }
  if (best < 0) best = 0;
  return best;
}

// Single-shift QR to Schur form with Q accumulated; full-width updates.
// Gradient mode (lam != nullptr): the forward's eigenvalues are the shifts,
// deflation uses kGradDeflationTol, and gbar of the matched forward eigenvalue
// is written to vec[i] for every diagonal position i. Eigenvector mode
// (lam == nullptr): Wilkinson/ad hoc shifts and the forward's ulp-level test.
template <int L>
__device__ int schur_qr(const BwdViews& V, const Group<L>& G, const double2* __restrict__ lam,
                        const double2* __restrict__ gbar, double lam_scale, int itmax,
                        const float2* __restrict__ est = nullptr) {
  const double tol = lam != nullptr ? kGradDeflationTol : kUlp;
  const MatView& T = V.T;
  const MatView& Q = V.Q;
  const int n = T.n, rs = T.rs, cs = n * rs;
  const double smlnum = kSafeMin * ((double)n / kUlp);
  unsigned long long used = 0ull;
  int status = kConverged;
  int i = n - 1, lo = 0, its = 0, kdefl = 0;
  while (true) {
    for (;;) {
      int hit = lo;
      for (int k = i - G.rank; k > lo; k -= L) {
        if (negligible_subdiag(T, k, lo, i, smlnum, tol)) {
          hit = k;
          break;
        }
      }
      lo = G.imax(hit);
      if (lo < i) break;
      if (lam != nullptr) {
        const int kb = nearest_unused(lam, n, used, *T.at(i, i), lam_scale);
        used |= 1ull << kb;
        if (G.rank == 0) V.vec[i * V.vs] = gbar[kb];
      } else if (est != nullptr) {
        const int kb = nearest_estimate(est, n, used, *T.at(i, i));
        if (kb >= 0) used |= 1ull << kb;
      }
      i -= 1;
      lo = 0;
      its = 0;
      kdefl = 0;
      if (i < 0) break;
    }
    if (i < 0) break;
    if (its > itmax) {
      status = kNotConverged;
      break;
    }
    double2 sigma;
    const double2 wk = wilkinson_shift(*T.at(i - 1, i - 1), *T.at(i - 1, i), *T.at(i, i - 1), *T.at(i, i));
    int kb_est;
    if (its == 0 && lam != nullptr) {
      const double2 l = lam[nearest_unused(lam, n, used, wk, lam_scale)];
      sigma = make_double2(l.x * lam_scale, l.y * lam_scale);
      if (!(isfinite(sigma.x) && isfinite(sigma.y))) sigma = wk;
    } else if (its == 0 && est != nullptr && (kb_est = nearest_estimate(est, n, used, wk)) >= 0) {
      const float2 e = est[kb_est];  // FP32 shift hint (see zgeev_estimate.cuh)
      sigma = make_double2((double)e.x, (double)e.y);
    } else if ((kdefl + 1) % (2 * kExceptionalPeriod) == 0) {
      const double2 d = *T.at(i, i);
      sigma = make_double2(d.x + kExceptionalWeight * cabs1(*T.at(i, i - 1)), d.y);
    } else if ((kdefl + 1) % kExceptionalPeriod == 0) {
      const double2 d = *T.at(lo, lo);
      sigma = make_double2(d.x + kExceptionalWeight * cabs1(*T.at(lo + 1, lo)), d.y);
    } else {
      sigma = wk;
    }
    ++its;
    ++kdefl;
    for (int j = lo; j < i; ++j) {
      double2 x, y, rr;
      if (j == lo) {
        x = csub(*T.at(lo, lo), sigma);
        y = *T.at(lo + 1, lo);
      } else {
        x = *T.at(j, j - 1);
        y = *T.at(j + 1, j - 1);
      }
      const Rot g = make_rot(x, y, rr);
      G.sync();
      if (j > lo && G.rank == 0) *T.at(j, j - 1) = rr;
      // Left: rows (j, j+1), columns j .. n-1.
      TZG_DBG_RUN(T, j, j + G.rank, 0, L, strided_count(j + G.rank, n - 1, L), 1, 0);
      rotate_pairs<false>(g, T.ptr(j, j + G.rank), strided_count(j + G.rank, n - 1, L), L * cs, rs);
      G.sync();
      // Right: columns (j, j+1), rows 0 .. min(j+1, i); bulge row j+2; and Q's rows 0 .. n-1.
      const int qend = min(j + 1, i);
      TZG_DBG_RUN(T, G.rank, j, L, 0, strided_count(G.rank, qend, L), 0, 1);
      rotate_pairs<true>(g, T.ptr(G.rank, j), strided_count(G.rank, qend, L), L * rs, cs);
      if (j + 2 <= i && G.rank == ((j + 2) & (L - 1))) {
        double2* pb = T.at(j + 2, j);
        TZG_DBG_TOUCH(T, j + 2, j + 1);
        const double2 b = pb[cs];
        pb[0] = make_double2(fma(g.s.x, b.x, g.s.y * b.y), fma(g.s.x, b.y, -g.s.y * b.x));
        pb[cs] = make_double2(g.c * b.x, g.c * b.y);
      }
      TZG_DBG_RUN(Q, G.rank, j, L, 0, strided_count(G.rank, n - 1, L), 0, 1);
      rotate_pairs<true>(g, Q.ptr(G.rank, j), strided_count(G.rank, n - 1, L), L * rs, cs);
      G.sync();
    }
  }
  return status;
}

// schur_qr with scaled rotations (zgeev_scaled_qr.cuh): T = K * u_r * v_c and
// Q = KQ * v_c (Q's columns rotate with T's, so they share the column factors).
// Full-width updates as schur_qr: left over columns j .. n-1, right over rows
// 0 .. min(j+1, i) of T and all rows of Q; rescales cover those live ranges.
// On return T's upper triangle and Q hold true values again (also when the
// sweep cap is hit), so the eigenvector and gradient steps are unchanged.
template <int L>
__device__ int schur_qr_scaled(const BwdViews& V, const Group<L>& G, const double2* __restrict__ lam,
                               const double2* __restrict__ gbar, double lam_scale, int itmax,
                               const float2* __restrict__ est = nullptr) {
  const double tol = lam != nullptr ? kGradDeflationTol : kUlp;
  const MatView& T = V.T;
  const MatView& Q = V.Q;
  const int n = T.n, rs = T.rs, cs = n * rs;
  const double smlnum = kSafeMin * ((double)n / kUlp);
  for (int k = G.rank; k < n; k += L) *scale_slot(T, k) = make_double2(1.0, 1.0);
  G.sync();
  unsigned long long used = 0ull;
  int status = kConverged;
  int i = n - 1, lo = 0, its = 0, kdefl = 0;
  while (true) {
    for (;;) {
      int hit = lo;
      for (int k = i - G.rank; k > lo; k -= L) {
        if (negligible_subdiag_scaled(T, k, lo, i, smlnum, tol)) {
          hit = k;
          break;
        }
      }
      lo = G.imax(hit);
      if (lo < i) {
        // the split entry lies outside the rows the left rotations update (see qr_eigenvalues_scaled)
        if (lo > 0 && G.rank == 0) *T.at(lo, lo - 1) = make_double2(0.0, 0.0);
        break;
      }
      if (lam != nullptr) {
        const int kb = nearest_unused(lam, n, used, true_entry(T, i, i), lam_scale);
        used |= 1ull << kb;
        if (G.rank == 0) V.vec[i * V.vs] = gbar[kb];
      } else if (est != nullptr) {
        const int kb = nearest_estimate(est, n, used, true_entry(T, i, i));
        if (kb >= 0) used |= 1ull << kb;
      }
      i -= 1;
      lo = 0;
      its = 0;
      kdefl = 0;
      if (i < 0) break;
    }
    if (i < 0) break;
    if (its > itmax) {
      status = kNotConverged;
      break;
    }
    double2 sigma;
    const double2 wk = wilkinson_shift(true_entry(T, i - 1, i - 1), true_entry(T, i - 1, i), true_entry(T, i, i - 1),
                                       true_entry(T, i, i));
    int kb_est;
    if (its == 0 && lam != nullptr) {
      const double2 l = lam[nearest_unused(lam, n, used, wk, lam_scale)];
      sigma = make_double2(l.x * lam_scale, l.y * lam_scale);
      if (!(isfinite(sigma.x) && isfinite(sigma.y))) sigma = wk;
    } else if (its == 0 && est != nullptr && (kb_est = nearest_estimate(est, n, used, wk)) >= 0) {
      const float2 e = est[kb_est];
      sigma = make_double2((double)e.x, (double)e.y);
    } else if ((kdefl + 1) % (2 * kExceptionalPeriod) == 0) {
      const double2 d = true_entry(T, i, i);
      sigma = make_double2(d.x + kExceptionalWeight * cabs1(true_entry(T, i, i - 1)), d.y);
    } else if ((kdefl + 1) % kExceptionalPeriod == 0) {
      const double2 d = true_entry(T, lo, lo);
      sigma = make_double2(d.x + kExceptionalWeight * cabs1(true_entry(T, lo + 1, lo)), d.y);
    } else {
      sigma = wk;
    }
    ++its;
    ++kdefl;
    const double2 f0 = *scale_slot(T, lo);
    double u0 = f0.x, v0 = f0.y, vp = 1.0;
    for (int j = lo; j < i; ++j) {
      const double2 f1 = *scale_slot(T, j + 1);
      double u1 = f1.x, v1 = f1.y;
      double2 x, y, rr;
      if (j == lo) {
        x = csub(cscale(*T.at(lo, lo), u0 * v0), sigma);
        y = cscale(*T.at(lo + 1, lo), u1 * v0);
      } else {
        x = cscale(*T.at(j, j - 1), u0 * vp);
        y = cscale(*T.at(j + 1, j - 1), u1 * vp);
      }
      const Rot g = make_rot(x, y, rr);
      G.sync();
      const int c0 = j + G.rank;
      const int ccount = strided_count(c0, n - 1, L);
      const int qend = min(j + 1, i);
      const int tcount = strided_count(G.rank, qend, L);
      const int qcount = strided_count(G.rank, n - 1, L);
      if (!is_zero(g.c)) {
        double rl, rr2;
        rotation_reciprocals(g.c, u0, u1, v0, v1, rl, rr2);
        const double2 alpha = cscale(g.s, u1 * u1 * rl);
        const double2 beta = make_double2(-g.s.x * (u0 * u0 * rl), g.s.y * (u0 * u0 * rl));
        if (j > lo && G.rank == 0) {
          double2* pk = T.at(j, j - 1);
          TZG_DBG_TOUCH(T, j + 1, j - 1);
          *pk = cmadd(*pk, alpha, pk[rs]);
        }
        TZG_DBG_RUN(T, j, c0, 0, L, ccount, 1, 0);
        scaled_pairs(alpha, beta, T.ptr(j, c0), ccount, L * cs, rs);
        u0 *= g.c;
        u1 *= g.c;
        G.sync();
        const double2 gamma = make_double2(g.s.x * (v1 * v1 * rr2), -g.s.y * (v1 * v1 * rr2));
        const double2 delta = cscale(g.s, -(v0 * v0 * rr2));
        TZG_DBG_RUN(T, G.rank, j, L, 0, tcount, 0, 1);
        scaled_pairs(gamma, delta, T.ptr(G.rank, j), tcount, L * rs, cs);
        if (j + 2 <= i && G.rank == ((j + 2) & (L - 1))) {
          double2* pb = T.at(j + 2, j);
          TZG_DBG_TOUCH(T, j + 2, j + 1);
          pb[0] = cmul(gamma, pb[cs]);
        }
        TZG_DBG_RUN(Q, G.rank, j, L, 0, qcount, 0, 1);
        scaled_pairs(gamma, delta, Q.ptr(G.rank, j), qcount, L * rs, cs);
        v0 *= g.c;
        v1 *= g.c;
      } else {
        const double2 sc = make_double2(g.s.x, -g.s.y), msc = make_double2(-g.s.x, g.s.y);
        const double2 ms = make_double2(-g.s.x, -g.s.y);
        if (j > lo && G.rank == 0) {
          double2* pk = T.at(j, j - 1);
          TZG_DBG_TOUCH(T, j + 1, j - 1);
          *pk = cmul(g.s, pk[rs]);
        }
        TZG_DBG_RUN(T, j, c0, 0, L, ccount, 1, 0);
        swap_pairs(g.s, msc, T.ptr(j, c0), ccount, L * cs, rs);
        { const double t = u0; u0 = u1; u1 = t; }
        G.sync();
        TZG_DBG_RUN(T, G.rank, j, L, 0, tcount, 0, 1);
        swap_pairs(sc, ms, T.ptr(G.rank, j), tcount, L * rs, cs);
        if (j + 2 <= i && G.rank == ((j + 2) & (L - 1))) {
          double2* pb = T.at(j + 2, j);
          TZG_DBG_TOUCH(T, j + 2, j + 1);
          pb[0] = cmul(sc, pb[cs]);
          pb[cs] = make_double2(0.0, 0.0);
        }
        TZG_DBG_RUN(Q, G.rank, j, L, 0, qcount, 0, 1);
        swap_pairs(sc, ms, Q.ptr(G.rank, j), qcount, L * rs, cs);
        { const double t = v0; v0 = v1; v1 = t; }
      }
      G.sync();
      if (nonneg_lt(u0, kScaleFloor) || nonneg_lt(u1, kScaleFloor) || nonneg_lt(v0, kScaleFloor) ||
          nonneg_lt(v1, kScaleFloor)) {
        // live ranges: row r at columns max(0, r-2) .. n-1; column c of T at rows 0 .. min(c+2, i)
        // (the bulge at c+2) and of Q at every row.
        if (u0 < kScaleFloor) {
          for (int c = max(0, j - 2) + G.rank; c < n; c += L) *T.at(j, c) = cscale(*T.at(j, c), u0);
          u0 = 1.0;
        }
        if (u1 < kScaleFloor) {
          for (int c = max(0, j - 1) + G.rank; c < n; c += L) *T.at(j + 1, c) = cscale(*T.at(j + 1, c), u1);
          u1 = 1.0;
        }
        G.sync();
        if (v0 < kScaleFloor) {
          for (int r = G.rank; r <= min(j + 2, i); r += L) *T.at(r, j) = cscale(*T.at(r, j), v0);
          for (int r = G.rank; r < n; r += L) *Q.at(r, j) = cscale(*Q.at(r, j), v0);
          v0 = 1.0;
        }
        if (v1 < kScaleFloor) {
          for (int r = G.rank; r <= min(j + 3, i); r += L) *T.at(r, j + 1) = cscale(*T.at(r, j + 1), v1);
          for (int r = G.rank; r < n; r += L) *Q.at(r, j + 1) = cscale(*Q.at(r, j + 1), v1);
          v1 = 1.0;
        }
        G.sync();
      }
      if (G.rank == 0) *scale_slot(T, j) = make_double2(u0, v0);
      vp = v0;
      u0 = u1;
      v0 = v1;
    }
    if (G.rank == 0) *scale_slot(T, i) = make_double2(u0, v0);
    G.sync();
  }
  // True values back into T's upper triangle and Q (column c owned by rank c mod L).
  G.sync();
  for (int c = G.rank; c < n; c += L) {
    const double2 fc = *scale_slot(T, c);
    for (int r = 0; r <= c; ++r) *T.at(r, c) = cscale(*T.at(r, c), scale_slot(T, r)->x * fc.y);
    for (int r = 0; r < n; ++r) *Q.at(r, c) = cscale(*Q.at(r, c), fc.y);
  }
  G.sync();
  return status;
}

// Divides s by d with |d| clamped from below by smin (marks `close`).
__device__ __forceinline__ double2 div_clamped(double2 s, double2 d, double smin, bool& close) {
  if (cabs1(d) < smin) {
    d = make_double2(smin, 0.0);
    close = true;
  }
  const double r = 1.0 / fma(d.x, d.x, d.y * d.y);
  return make_double2(fma(s.x, d.x, s.y * d.y) * r, fma(s.y, d.x, -s.x * d.y) * r);
}

// X (strict upper part of XY, unit diagonal implied): T X = X diag(T).
// Y (strict lower part of XY): Y^H T = diag(T) Y^H, Y = (Y^H)^H, unit diagonal implied.
template <int L>
__device__ bool eigenvectors_of_t(const BwdViews& V, const Group<L>& G) {
  const MatView& T = V.T;
  const MatView& XY = V.XY;
  const int n = T.n;
  double tmax = 0.0;
  for (int k = 0; k < n; ++k) tmax = fmax(tmax, cabs1(*T.at(k, k)));
  const double smin = fmax(kUlp * tmax, kSafeMin * ((double)n / kUlp));
  bool close = false;
  for (int k = 1 + G.rank; k < n; k += L) {
    const double2 tkk = *T.at(k, k);
    for (int i = k - 1; i >= 0; --i) {
      double2 s = *T.at(i, k);
      for (int j = i + 1; j < k; ++j) {
        const double2 t = *T.at(i, j), x = *XY.at(j, k);
        s.x = fma(t.x, x.x, fma(-t.y, x.y, s.x));
        s.y = fma(t.x, x.y, fma(t.y, x.x, s.y));
      }
      const double2 q = div_clamped(s, csub(*T.at(i, i), tkk), smin, close);
      *XY.at(i, k) = make_double2(-q.x, -q.y);
    }
  }
  for (int k = G.rank; k + 1 < n; k += L) {
    const double2 tkk = *T.at(k, k);
    // Row k of Y^H: y_j for j > k (y_k = 1); stored conjugated at XY(j, k).
    for (int j = k + 1; j < n; ++j) {
      double2 s = *T.at(k, j);
      for (int i = k + 1; i < j; ++i) {
        const double2 yc = *XY.at(i, k);  // conj(y_i)
        const double2 t = *T.at(i, j);
        // s += y_i t = conj(yc) t
        s.x = fma(yc.x, t.x, fma(yc.y, t.y, s.x));
        s.y = fma(yc.x, t.y, fma(-yc.y, t.x, s.y));
      }
      const double2 q = div_clamped(s, csub(*T.at(j, j), tkk), smin, close);
      *XY.at(j, k) = make_double2(-q.x, q.y);  // conj(-q)
    }
  }
  G.sync();
  return G.ior(close ? 1 : 0) != 0;
}

// Abar = Q M Q^H with M = Y diag(g) X^H (lower triangular), written to the
// caller's column-major gA. Uses T's lower part for Z/M and XY for P.
template <int L>
__device__ void assemble_gradient(const BwdViews& V, const Group<L>& G, double2* __restrict__ gA) {
  const MatView& T = V.T;
  const MatView& Q = V.Q;
  const MatView& XY = V.XY;
  const int n = T.n;
  // Z_kj = g_k conj(X_jk) for k >= j (X_kk = 1) into T(k, j).
  for (int j = G.rank; j < n; j += L) {
    for (int k = j; k < n; ++k) {
      const double2 gk = V.vec[k * V.vs];
      if (k == j) {
        *T.at(k, j) = gk;
      } else {
        const double2 x = *XY.at(j, k);
        *T.at(k, j) = make_double2(fma(gk.x, x.x, gk.y * x.y), fma(gk.y, x.x, -gk.x * x.y));
      }
    }
  }
  G.sync();
  // M = Y Z in place, bottom-up per column: M_ij = Z_ij + sum_{k=j}^{i-1} Y_ik Z_kj.
  for (int j = G.rank; j < n; j += L) {
    for (int i = n - 1; i > j; --i) {
      double2 s = *T.at(i, j);
      for (int k = j; k < i; ++k) {
        const double2 y = *XY.at(i, k), z = *T.at(k, j);
        s.x = fma(y.x, z.x, fma(-y.y, z.y, s.x));
        s.y = fma(y.x, z.y, fma(y.y, z.x, s.y));
      }
      *T.at(i, j) = s;
    }
  }
  G.sync();
  // P = Q M into XY: P_ij = sum_{k >= j} Q_ik M_kj (four rows at a time).
  for (int j = G.rank; j < n; j += L) {
    for (int i0 = 0; i0 < n; i0 += 4) {
      double2 acc[4] = {};
      for (int k = j; k < n; ++k) {
        const double2 mk = *T.at(k, j);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (i0 + u < n) {
            const double2 q = *Q.at(i0 + u, k);
            acc[u].x = fma(q.x, mk.x, fma(-q.y, mk.y, acc[u].x));
            acc[u].y = fma(q.x, mk.y, fma(q.y, mk.x, acc[u].y));
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u < n) *XY.at(i0 + u, j) = acc[u];
    }
  }
  G.sync();
  // Abar = P Q^H: Abar_ij = sum_k P_ik conj(Q_jk), column j written contiguously.
  for (int j = G.rank; j < n; j += L) {
    for (int i0 = 0; i0 < n; i0 += 4) {
      double2 acc[4] = {};
      for (int k = 0; k < n; ++k) {
        const double2 q = *Q.at(j, k);
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          if (i0 + u < n) {
            const double2 p = *XY.at(i0 + u, k);
            // acc += p conj(q)
            acc[u].x = fma(p.x, q.x, fma(p.y, q.y, acc[u].x));
            acc[u].y = fma(p.y, q.x, fma(-p.x, q.y, acc[u].y));
          }
        }
      }
#pragma unroll
      for (int u = 0; u < 4; ++u)
        if (i0 + u < n) gA[i0 + u + j * n] = acc[u];
    }
  }
}

// Full backward of one matrix. lam: the forward's n eigenvalues of this matrix,
// gbar: their gradients, gA: output (column-major n x n, same layout as A).
template <int L>
__device__ int backward_matrix(const double2* __restrict__ src, const double2* __restrict__ lam,
                               const double2* __restrict__ gbar, double2* __restrict__ gA, const BwdViews& V,
                               const Group<L>& G, int itmax, int scaled_min_n = kMaxN + 1) {
  const int n = V.T.n;
  bool nonfinite, zero;
  const int shift = stage_and_scale<L>(src, V.T, G, nonfinite, zero);
  if (nonfinite || zero) {
    const double v = nonfinite ? __longlong_as_double(0x7ff8000000000000LL) : 0.0;
    for (int e = G.rank; e < n * n; e += L) gA[e] = make_double2(v, v);
    return nonfinite ? kNonFinite : (n > 1 ? kCloseEigenvalues : kConverged);
  }
  hessenberg<L>(V.T, G, V.vec, V.vs);
  G.sync();
  form_q<L>(V, G);
  const double lam_scale = shift == 0 ? 1.0 : (shift > 1022 ? 0.5 * pow2(-1022) : pow2(-shift));
  const int status = (n >= scaled_min_n && n >= kScaledMinN) ? schur_qr_scaled<L>(V, G, lam, gbar, lam_scale, itmax)
                                                            : schur_qr<L>(V, G, lam, gbar, lam_scale, itmax);
  if (status != kConverged) {
    const double nan = __longlong_as_double(0x7ff8000000000000LL);
    for (int e = G.rank; e < n * n; e += L) gA[e] = make_double2(nan, nan);
    return status;
  }
  G.sync();
  const bool close = eigenvectors_of_t<L>(V, G);
  assemble_gradient<L>(V, G, gA);
  return close ? kCloseEigenvalues : kConverged;
}

}  // namespace tzg
