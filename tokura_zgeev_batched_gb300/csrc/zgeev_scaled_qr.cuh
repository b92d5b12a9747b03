// Single-shift complex QR with scaled rotations (eigenvalues only).
//
// The same iteration as qr_eigenvalues (zgeev_lane.cuh: Ahues-Tisseur
// deflation, Wilkinson / FP32-hint / ad hoc shifts, one sweep per loop
// iteration, LAPACK's per-eigenvalue cap), with a cheaper rotation update.
// The Hessenberg matrix is kept as K with real row and column factors,
//     H(r, c) = K(r, c) * u[r] * v[c].
// A rotation G = [c s; -conj(s) c] (c real) of rows j, j+1 is then
//     K(j, :) += alpha K(j+1, :),  K(j+1, :) += beta K(j, :)   (old K(j, :)),
//     alpha = s u[j+1] / (c u[j]),  beta = -conj(s) u[j] / (c u[j+1]),
// with u[j], u[j+1] multiplied by c; of columns j, j+1 (G^H from the right)
//     K(:, j) += gamma K(:, j+1),  K(:, j+1) += delta K(:, j)  (old K(:, j)),
//     gamma = conj(s) v[j+1] / (c v[j]),  delta = -s v[j] / (c v[j+1]),
// with v[j], v[j+1] multiplied by c. Each element pair costs two complex
// multiply-adds, 8 FP64 instructions, instead of the 12 of the plain rotation
// (rot_left / rot_right). The rounding error of an update, scaled back to H,
// is eps * (c |H(j, :)| + |s| |H(j+1, :)|): the same bound as the plain
// rotation's. Factors only shrink (c <= 1); a row or column whose factor
// falls below 2^-150 is multiplied into K over its live entries and reset to 1
// (an O(n) rescale, 46 per 64 x 64 Gaussian matrix with hints). The floor is
// low because a rescale runs in the lanes that need it while the rest of the
// warp waits: at 2^-60 (185 rescales per matrix) a rescale somewhere in the
// warp came with most rotations and cost the QR phase about a tenth of its
// FP64 lane slots. It is high enough for every product to stay finite: the
// pre-scaled matrix has entries below 2^61 and Frobenius norm below 2^68,
// make_rot's c is at least 2^-482 / ||H||_F^2 > 2^-618 (below, the rotation
// is a swap), so K stays below 2^368 and the largest intermediate (the
// updated K(j, :) of a rotation with the smallest c, before its rescale)
// below 2^990. An exact swap (c = 0)
// exchanges the two factors and applies s directly. Entries outside the
// active block keep stale factors; the only one read again, the negligible
// subdiagonal entry where the block splits from the rows above, is stored as
// an exact zero when the split is found.
//
// The factors (u[k], v[k]) of position k live as one double2 in an element of
// the matrix that the QR never reads or writes: below the second subdiagonal
// (rows k+3 of column 0 for k <= n-4, rows 4..6 of column 1 for the last
// three), so the workspace holds nothing extra. Needs n >= kScaledMinN.
//
// Shifts, rotation generation, deflation tests and eigenvalues read true
// entries K * u * v. Lanes of a group compute every factor identically (same
// inputs, same operations), keep the current pair in registers, and rank 0
// stores a position's factors once the sweep has passed it.
#pragma once

#include "zgeev_lane.cuh"

namespace tzg {

// Smallest order the scaled iteration supports (slots of the factors need rows
// 3..n-1 of column 0 and 4..6 of column 1).
constexpr int kScaledMinN = 7;
// Rescale threshold of a row or column factor.
constexpr double kScaleFloor = 0x1p-150;

__device__ __forceinline__ double2* scale_slot(const MatView& M, int k) {
  return k <= M.n - 4 ? M.at(k + 3, 0) : M.at(k - M.n + 7, 1);
}

// 1/(c u0 u1) and 1/(c v0 v1) from one reciprocal of their product when it
// stays normal (c and the factors can each be as small as ~2^-618 and 2^-150),
// else from two.
__device__ __forceinline__ void rotation_reciprocals(double c, double u0, double u1, double v0, double v1, double& rl,
                                                     double& rr) {
  const double pl = c * u0 * u1, pr = c * v0 * v1;
  const double prod = pl * pr;
  if (nonneg_lt(1e-290, prod)) {
    const double inv = 1.0 / prod;
    rl = inv * pr;
    rr = inv * pl;
  } else {
    rl = 1.0 / pl;
    rr = 1.0 / pr;
  }
}

// a + f * b (complex multiply-add, 4 FP64 instructions).
__device__ __forceinline__ double2 cmadd(double2 a, double2 f, double2 b) {
  return make_double2(fma(f.x, b.x, fma(-f.y, b.y, a.x)), fma(f.x, b.y, fma(f.y, b.x, a.y)));
}

// k_a += fa * k_b, k_b += fb * k_a(old) on `count` element pairs p[t*step],
// p[t*step + pair]; pair t+1 is loaded before pair t is stored.
__device__ __forceinline__ void scaled_pairs(double2 fa, double2 fb, double2* p, int count, int step, int pair) {
  if (count <= 0) return;
  double2 a = p[0], b = p[pair];
  for (int t = 1; t < count; ++t) {
    double2* pn = p + step;
    const double2 an = pn[0], bn = pn[pair];
    p[0] = cmadd(a, fa, b);
    p[pair] = cmadd(b, fb, a);
    a = an;
    b = bn;
    p = pn;
  }
  p[0] = cmadd(a, fa, b);
  p[pair] = cmadd(b, fb, a);
}

// The exact swap-like rotation (c = 0): k_a <- fa * k_b, k_b <- fb * k_a.
__device__ __forceinline__ void swap_pairs(double2 fa, double2 fb, double2* p, int count, int step, int pair) {
  for (int t = 0; t < count; ++t, p += step) {
    const double2 a = p[0], b = p[pair];
    p[0] = cmul(fa, b);
    p[pair] = cmul(fb, a);
  }
}

// Deflation test of negligible_subdiag on the true entries K * u * v (tol:
// relative threshold, as negligible_subdiag's).
__device__ __forceinline__ bool negligible_subdiag_scaled(const MatView& M, int k, int lo, int hi, double smlnum,
                                                          double tol = kUlp) {
  const double2 sk = *scale_slot(M, k), sk1 = *scale_slot(M, k - 1);
  const double h1 = cabs1(*M.at(k, k - 1)) * (sk.x * sk1.y);
  if (nonneg_le(h1, smlnum)) return true;
  const double2 dkk = cscale(*M.at(k, k), sk.x * sk.y);
  const double2 dk1 = cscale(*M.at(k - 1, k - 1), sk1.x * sk1.y);
  double tst = cabs1(dk1) + cabs1(dkk);
  if (is_zero(tst)) {
    if (k - 2 >= lo) tst += cabs1(*M.at(k - 1, k - 2)) * (sk1.x * scale_slot(M, k - 2)->y);
    if (k + 1 <= hi) tst += cabs1(*M.at(k + 1, k)) * (scale_slot(M, k + 1)->x * sk.y);
  }
  if (nonneg_lt(tol * tst, h1)) return false;
  const double hu = cabs1(*M.at(k - 1, k)) * (sk1.x * sk.y);
  const double ab = fmax(h1, hu), ba = fmin(h1, hu);
  const double dd = cabs1(csub(dk1, dkk));
  const double d1 = cabs1(dkk);
  const double aa = fmax(d1, dd), bb = fmin(d1, dd);
  const double s = aa + ab;
  return ba * (ab / s) <= fmax(smlnum, tol * (bb * (aa / s)));
}

// True entry H(r, c).
__device__ __forceinline__ double2 true_entry(const MatView& M, int r, int c) {
  return cscale(*M.at(r, c), scale_slot(M, r)->x * scale_slot(M, c)->y);
}

template <int L, class Out = double2>
__device__ int qr_eigenvalues_scaled(const MatView& M, const Group<L>& G, Out* __restrict__ eig_out, int shift,
                                     int itmax, const float2* __restrict__ est = nullptr,
                                     int* sweeps_out = nullptr) {
  const int n = M.n;
  const int rs = M.rs;
  const int cs = n * rs;
  const double smlnum = kSafeMin * ((double)n / kUlp);
  const double unscale = (shift != 0) ? pow2(shift) : 1.0;
  for (int k = G.rank; k < n; k += L) *scale_slot(M, k) = make_double2(1.0, 1.0);
  G.sync();
  int status = kConverged;
  int i = n - 1, lo = 0, its = 0, kdefl = 0, sweeps = 0;
  unsigned long long used = 0;
  while (true) {
    for (;;) {
      int hit = lo;
      for (int k = i - G.rank; k > lo; k -= L) {
        if (negligible_subdiag_scaled(M, k, lo, i, smlnum)) {
          hit = k;
          break;
        }
      }
      lo = G.imax(hit);
      if (lo < i) {
        // A split inside the matrix: store the negligible entry as an exact zero (as
        // LAPACK does). It lies outside the block the sweeps update, so a later rescale
        // or swap of row lo's factor would otherwise change its true value.
        if (lo > 0 && G.rank == 0) *M.at(lo, lo - 1) = make_double2(0.0, 0.0);
        break;
      }
      {
        const double2 d = true_entry(M, i, i);
        if (G.rank == 0) put_ev(eig_out + i, make_double2(d.x * unscale, d.y * unscale));
        if (est != nullptr) {
          const int k = nearest_estimate(est, n, used, d);
          if (k >= 0) used |= 1ull << k;
        }
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
    ++its;
    ++kdefl;
    ++sweeps;
    double2 sigma;
    if (kdefl % (2 * kExceptionalPeriod) == 0) {
      const double2 d = true_entry(M, i, i);
      sigma = make_double2(d.x + kExceptionalWeight * cabs1(true_entry(M, i, i - 1)), d.y);
    } else if (kdefl % kExceptionalPeriod == 0) {
      const double2 d = true_entry(M, lo, lo);
      sigma = make_double2(d.x + kExceptionalWeight * cabs1(true_entry(M, lo + 1, lo)), d.y);
    } else {
      sigma = wilkinson_shift(true_entry(M, i - 1, i - 1), true_entry(M, i - 1, i), true_entry(M, i, i - 1),
                              true_entry(M, i, i));
      if (est != nullptr && its == 1) {
        const int k = nearest_estimate(est, n, used, sigma);
        if (k >= 0) {
          const float2 e = est[k];
          sigma = make_double2((double)e.x, (double)e.y);
        }
      }
    }
    // Factors of the current pair (u0, v0) = position j, (u1, v1) = position j+1,
    // and vp = v[j-1] (final for this sweep), carried in registers across the sweep.
    double2 f0 = *scale_slot(M, lo);
    double u0 = f0.x, v0 = f0.y, vp = 1.0;
    for (int j = lo; j < i; ++j) {
      const double2 f1 = *scale_slot(M, j + 1);
      double u1 = f1.x, v1 = f1.y;
      double2 x, y, rr;
      if (j == lo) {
        x = csub(cscale(*M.at(lo, lo), u0 * v0), sigma);
        y = cscale(*M.at(lo + 1, lo), u1 * v0);
      } else {
        x = cscale(*M.at(j, j - 1), u0 * vp);
        y = cscale(*M.at(j + 1, j - 1), u1 * vp);
      }
      const Rot g = make_rot(x, y, rr);
      G.sync();  // all lanes have read the bulge before it is overwritten
      const int c0 = j + G.rank;
      const int qend = min(j + 1, i);
      const int q0 = lo + G.rank;
      if (!is_zero(g.c)) {
        // Left: rows (j, j+1) over columns j .. i (and j-1, whose row j+1 entry is annihilated).
        double rl, rr2;
        rotation_reciprocals(g.c, u0, u1, v0, v1, rl, rr2);
        const double2 alpha = cscale(g.s, u1 * u1 * rl);
        const double2 beta = make_double2(-g.s.x * (u0 * u0 * rl), g.s.y * (u0 * u0 * rl));
        if (j > lo && G.rank == 0) {
          double2* pk = M.at(j, j - 1);
          TZG_DBG_TOUCH(M, j + 1, j - 1);
          *pk = cmadd(*pk, alpha, pk[rs]);
        }
        TZG_DBG_RUN(M, j, c0, 0, L, strided_count(c0, i, L), 1, 0);
        scaled_pairs(alpha, beta, M.ptr(j, c0), strided_count(c0, i, L), L * cs, rs);
        u0 *= g.c;
        u1 *= g.c;
        G.sync();
        // Right: columns (j, j+1) over rows lo .. min(j+1, i); row j+2 gets the new bulge
        // K(j+2, j) = gamma K(j+2, j+1) (its column-j entry is zero), K(j+2, j+1) unchanged.
        const double2 gamma = make_double2(g.s.x * (v1 * v1 * rr2), -g.s.y * (v1 * v1 * rr2));
        const double2 delta = cscale(g.s, -(v0 * v0 * rr2));
        TZG_DBG_RUN(M, q0, j, L, 0, strided_count(q0, qend, L), 0, 1);
        scaled_pairs(gamma, delta, M.ptr(q0, j), strided_count(q0, qend, L), L * rs, cs);
        if (j + 2 <= i && G.rank == ((j + 2 - lo) & (L - 1))) {
          double2* pb = M.at(j + 2, j);
          TZG_DBG_TOUCH(M, j + 2, j + 1);
          pb[0] = cmul(gamma, pb[cs]);
        }
        v0 *= g.c;
        v1 *= g.c;
      } else {
        // Exact swap: rows j <-> j+1 times (s, -conj(s)); factors exchanged.
        const double2 sc = make_double2(g.s.x, -g.s.y), msc = make_double2(-g.s.x, g.s.y);
        if (j > lo && G.rank == 0) {
          double2* pk = M.at(j, j - 1);
          TZG_DBG_TOUCH(M, j + 1, j - 1);
          *pk = cmul(g.s, pk[rs]);
        }
        TZG_DBG_RUN(M, j, c0, 0, L, strided_count(c0, i, L), 1, 0);
        swap_pairs(g.s, msc, M.ptr(j, c0), strided_count(c0, i, L), L * cs, rs);
        { const double t = u0; u0 = u1; u1 = t; }
        G.sync();
        TZG_DBG_RUN(M, q0, j, L, 0, strided_count(q0, qend, L), 0, 1);
        swap_pairs(sc, make_double2(-g.s.x, -g.s.y), M.ptr(q0, j), strided_count(q0, qend, L), L * rs, cs);
        if (j + 2 <= i && G.rank == ((j + 2 - lo) & (L - 1))) {
          double2* pb = M.at(j + 2, j);
          TZG_DBG_TOUCH(M, j + 2, j + 1);
          pb[0] = cmul(sc, pb[cs]);
          pb[cs] = make_double2(0.0, 0.0);
        }
        { const double t = v0; v0 = v1; v1 = t; }
      }
      G.sync();
      // Rescale factors that fell below 2^-150 (group-uniform decision) over the live
      // entries: row r at columns max(lo, r-2) .. i, column c at rows lo .. min(c+2, i).
      if (nonneg_lt(u0, kScaleFloor) || nonneg_lt(u1, kScaleFloor) || nonneg_lt(v0, kScaleFloor) ||
          nonneg_lt(v1, kScaleFloor)) {
        if (u0 < kScaleFloor) {
          for (int c = max(lo, j - 2) + G.rank; c <= i; c += L) *M.at(j, c) = cscale(*M.at(j, c), u0);
          u0 = 1.0;
        }
        if (u1 < kScaleFloor) {
          for (int c = max(lo, j - 1) + G.rank; c <= i; c += L) *M.at(j + 1, c) = cscale(*M.at(j + 1, c), u1);
          u1 = 1.0;
        }
        G.sync();
        if (v0 < kScaleFloor) {
          for (int r = lo + G.rank; r <= min(j + 2, i); r += L) *M.at(r, j) = cscale(*M.at(r, j), v0);
          v0 = 1.0;
        }
        if (v1 < kScaleFloor) {
          for (int r = lo + G.rank; r <= min(j + 3, i); r += L) *M.at(r, j + 1) = cscale(*M.at(r, j + 1), v1);
          v1 = 1.0;
        }
        G.sync();
      }
      if (G.rank == 0) *scale_slot(M, j) = make_double2(u0, v0);  // final for this sweep
      vp = v0;
      u0 = u1;
      v0 = v1;
    }
    if (G.rank == 0) *scale_slot(M, i) = make_double2(u0, v0);
    G.sync();
  }
  if (status != kConverged && G.rank == 0) {
    for (int k = 0; k <= i; ++k) {
      const double2 d = true_entry(M, k, k);
      put_ev(eig_out + k, make_double2(d.x * unscale, d.y * unscale));
    }
  }
  if (sweeps_out != nullptr) *sweeps_out = sweeps;
  return status;
}

}  // namespace tzg
