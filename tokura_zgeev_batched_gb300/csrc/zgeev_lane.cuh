// Per-matrix algorithm executed by one lane group (L lanes of a warp).
//
// The functions here are the hot path: stage + scale, Householder
// Hessenberg reduction, single-shift complex QR to Schur diagonal, and the
// eigenvalue/flag write-out. Every lane of a group runs the same control
// flow (all decisions come from bitwise-identical group reductions), so the
// only divergence inside a warp is between different matrices.
#pragma once

#include "zgeev_device.cuh"

namespace tzg {

// Result codes of the per-matrix solve, stored in flag[] (0 = converged,
// which is the reference's contract, tokura_zhseqr_MWB_kernel.cuh:768-776).
enum : int { kConverged = 0, kNotConverged = 1, kNonFinite = 2, kInvalidInput = 3 };

// Sources of the matrix entries, addressed by the column-major linear index
// e = r + c*n of an n x n matrix (all loads are read-only, no alignment
// demands beyond the element type's).
struct SrcContig {  // n x n column-major, contiguous (the reference's layout)
  const double2* p;
  __device__ __forceinline__ double2 load(int e, int) const { return p[e]; }
};
struct SrcStrided {  // column-major with leading dimension ld >= n
  const double2* p;
  long long ld;
  __device__ __forceinline__ double2 load(int e, int n) const {
    const int c = e / n;
    return p[(e - c * n) + c * ld];
  }
};
struct SrcComplex64 {  // contiguous single-precision complex, widened on load
  const float2* p;
  __device__ __forceinline__ double2 load(int e, int) const {
    const float2 z = p[e];
    return make_double2((double)z.x, (double)z.y);
  }
};

// Eigenvalue stores: full precision, or rounded to single precision.
__device__ __forceinline__ void put_ev(double2* p, double2 v) { *p = v; }
__device__ __forceinline__ void put_ev(float2* p, double2 v) { *p = make_float2((float)v.x, (float)v.y); }

// Stage matrix `slot` of a tile from `src` into the tile-interleaved view,
// scaling by an exact power of two when the largest |Re|,|Im| lies outside
// [2^-60, 2^60] (zgeev's pre-scaling, done exactly). Returns the applied
// exponent shift (eigenvalues are multiplied by 2^shift on output), or sets
// `nonfinite`.
template <int L, class Src>
__device__ __forceinline__ int stage_and_scale(const Src& src, const MatView& M, const Group<L>& G, bool& nonfinite,
                                               bool& zero) {
  const int n = M.n;
  const int nn = n * n;
  int emax = 0;
  for (int e = G.rank; e < nn; e += L) {
    const double2 z = src.load(e, n);
    emax = max(emax, max(dexp_field(z.x), dexp_field(z.y)));
  }
  emax = G.imax(emax);
  nonfinite = (emax == 0x7ff);
  zero = (emax == 0);
  int shift = 0;
  if (!nonfinite && !zero) {
    const int top = emax - 1023;  // |largest| in [2^top, 2^(top+1))
    if (top > 60 || top < -60) shift = top;
  }
  if (shift == 0) {
    for (int e = G.rank; e < nn; e += L) M.p[e * M.rs] = src.load(e, n);
  } else {
    const double sc = shift > 1022 ? 0.5 * pow2(-1022) : pow2(-shift);  // 2^-1023 is subnormal
    for (int e = G.rank; e < nn; e += L) {
      const double2 z = src.load(e, n);
      M.p[e * M.rs] = make_double2(z.x * sc, z.y * sc);
    }
  }
  G.sync();
  return shift;
}

// Column-major contiguous source (the reference's layout).
template <int L>
__device__ __forceinline__ int stage_and_scale(const double2* __restrict__ src, const MatView& M,
                                               const Group<L>& G, bool& nonfinite, bool& zero) {
  return stage_and_scale<L>(SrcContig{src}, M, G, nonfinite, zero);
}

// Applies P = I - tau v v^H (v[0] = 1, v[i] at x[i*xs]) to NV vectors of
// length m at p[k][i*es]: a <- a - tau v (v^H a). With kConjV the reflector
// acts from the right on rows instead: a <- a - tau (a v) v^H, which is the
// same formula with v conjugated. The NV dot products share the loads of v
// and run as independent FMA chains; the update loop loads element i+1
// before storing element i so memory latency overlaps the arithmetic.
template <int NV, bool kConjV>
__device__ __forceinline__ void reflect_vectors(double2* const (&p)[NV], const double2* x, int m, int es, int xs,
                                                double tau) {
  double2 w[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) w[k] = p[k][0];
  for (int i = 1; i < m; ++i) {
    const double2 v = x[i * xs];
    const double vy = kConjV ? -v.y : v.y;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      const double2 a = p[k][i * es];
      w[k].x = fma(v.x, a.x, fma(vy, a.y, w[k].x));
      w[k].y = fma(v.x, a.y, fma(-vy, a.x, w[k].y));
    }
  }
  double2 t[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    t[k] = make_double2(w[k].x * tau, w[k].y * tau);
    p[k][0] = csub(p[k][0], t[k]);
  }
  if (m < 2) return;
  double2 v = x[xs];
  double2 a[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) a[k] = p[k][es];
  for (int i = 1; i < m; ++i) {
    double2 vn = v, an[NV];
    if (i + 1 < m) {
      vn = x[(i + 1) * xs];
#pragma unroll
      for (int k = 0; k < NV; ++k) an[k] = p[k][(i + 1) * es];
    }
    const double vy = kConjV ? -v.y : v.y;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
      // a -= v' t, v' = (v.x, vy)
      a[k].x = fma(-v.x, t[k].x, fma(vy, t[k].y, a[k].x));
      a[k].y = fma(-v.x, t[k].y, fma(-vy, t[k].x, a[k].y));
      p[k][i * es] = a[k];
    }
    v = vn;
#pragma unroll
    for (int k = 0; k < NV; ++k) a[k] = an[k];
  }
}

// Balancing modes (LAPACK zgebal's JOB): none, permute only, scale only, both.
enum : int { kBalanceNone = 0, kBalancePermute = 1, kBalanceScale = 2, kBalanceBoth = 3 };

// Element helpers shared by the complex (double2) and real (double) views.
__device__ __forceinline__ double acc_abs2(double acc, double2 a) { return fma(a.x, a.x, fma(a.y, a.y, acc)); }
__device__ __forceinline__ double acc_abs2(double acc, double a) { return fma(a, a, acc); }
__device__ __forceinline__ double2 scaled(double2 a, double f) { return make_double2(a.x * f, a.y * f); }
__device__ __forceinline__ double scaled(double a, double f) { return a * f; }

// True if every entry of row (kRow) / column j inside [lo, hi], other than
// the diagonal, is exactly zero (bit test, no FP64 work).
template <bool kRow, class View>
__device__ __forceinline__ bool offdiag_zero(const View& M, int j, int lo, int hi) {
  for (int k = lo; k <= hi; ++k) {
    if (k == j) continue;
    if (!is_zero(kRow ? *M.at(j, k) : *M.at(k, j))) return false;
  }
  return true;
}

// Swaps rows and columns a and b (a similarity by a permutation).
template <class View>
__device__ __forceinline__ void swap_rc(const View& M, int a, int b) {
  if (a == b) return;
  for (int k = 0; k < M.n; ++k) {
    const auto t = *M.at(k, a);
    *M.at(k, a) = *M.at(k, b);
    *M.at(k, b) = t;
  }
  for (int k = 0; k < M.n; ++k) {
    const auto t = *M.at(a, k);
    *M.at(a, k) = *M.at(b, k);
    *M.at(b, k) = t;
  }
}

// Balancing before the Hessenberg reduction (the procedure of Parlett and
// Reinsch that LAPACK's zgeev applies through zgebal; the reference does not
// balance, README.md:79). Permutation moves rows/columns that isolate an
// eigenvalue to the bottom/top; scaling then applies exact powers of two
// D^{-1} A D to the remaining block [lo, hi], accepting a factor for index i
// only when it lowers ||column i|| + ||row i|| (2-norms over [lo, hi]) by at
// least 5 %. Eigenvalues are unchanged; the isolated ones deflate at once in
// the QR. The permutation search (bit tests only) runs on rank 0; the norms
// and the row/column scaling of each index are split across the group.
template <int L, class View>
__device__ void balance(const View& M, const Group<L>& G, int mode) {
  const int n = M.n;
  int lo = 0, hi = n - 1;
  if (mode & kBalancePermute) {
    if (G.rank == 0) {
      for (bool found = true; found && hi > lo;) {  // rows isolating an eigenvalue -> bottom
        found = false;
        for (int j = hi; j >= lo; --j) {
          if (offdiag_zero<true>(M, j, lo, hi)) {
            swap_rc(M, j, hi);
            --hi;
            found = true;
            break;
          }
        }
      }
      for (bool found = true; found && hi > lo;) {  // columns isolating an eigenvalue -> top
        found = false;
        for (int j = lo; j <= hi; ++j) {
          if (offdiag_zero<false>(M, j, lo, hi)) {
            swap_rc(M, j, lo);
            ++lo;
            found = true;
            break;
          }
        }
      }
    }
    lo = G.imax(G.rank == 0 ? lo : 0);
    hi = G.imax(G.rank == 0 ? hi : 0);
    G.sync();
  }
  if (!(mode & kBalanceScale) || hi <= lo) return;
  int total[kMaxN];  // accumulated exponent of each index, kept within +-200
  for (int i = 0; i < n; ++i) total[i] = 0;
  bool noconv = true;
  for (int pass = 0; noconv && pass < 64; ++pass) {  // group-uniform control flow throughout
    noconv = false;
    for (int i = lo; i <= hi; ++i) {
      double c = 0.0, r = 0.0;
      for (int k = lo + G.rank; k <= hi; k += L) {
        c = acc_abs2(c, *M.at(k, i));
        r = acc_abs2(r, *M.at(i, k));
      }
      c = G.sum(c);
      r = G.sum(r);
      if (c == 0.0 || r == 0.0) continue;
      c = sqrt(c);
      r = sqrt(r);
      // Power of two f = 2^e with c*f and r/f within a factor 2 of each other.
      int e = 0;
      double cf = c, rf = r;
      while (cf < rf * 0.5 && e < 60) { cf *= 2.0; rf *= 0.5; ++e; }
      while (cf >= rf * 2.0 && e > -60) { cf *= 0.5; rf *= 2.0; --e; }
      if (e == 0 || cf + rf >= 0.95 * (c + r)) continue;
      if (total[i] + e > 200 || total[i] + e < -200) continue;
      total[i] += e;
      noconv = true;
      const double f = pow2(e), g = pow2(-e);
      for (int k = G.rank; k < n; k += L) {  // column i times f, row i times 1/f
        auto* a = M.at(k, i);
        *a = scaled(*a, f);
        auto* b = M.at(i, k);
        *b = scaled(*b, g);
      }
      G.sync();
    }
  }
}

// Householder reduction to upper Hessenberg form, in place. The reflector for
// column r is P = I - tau v v^H with v[0] = 1, tau real, stored below the
// subdiagonal of column r (v[1..]). Algorithmic FP64 work ~ (20/3) n^3 ops.
// If tau_out is given, tau of column r is written to tau_out[r * tau_stride].x
// (0 for columns that needed no reflector), for forming Q later.
template <int L>
__device__ void hessenberg(const MatView& M, const Group<L>& G, double2* tau_out = nullptr, int tau_stride = 0) {
  const int n = M.n;
  const int rs = M.rs;
  const int cs = n * rs;  // column stride
  for (int r = 0; r + 2 < n; ++r) {
    const int m = n - r - 1;  // x = H[r+1 .. n-1, r]
    double2* x = M.at(r + 1, r);
    double s2 = 0.0;
    for (int i = 1 + G.rank; i < m; i += L) {
      const double2 z = x[i * rs];
      s2 = fma(z.x, z.x, fma(z.y, z.y, s2));
    }
    s2 = G.sum(s2);
    if (s2 == 0.0) {  // column already in Hessenberg form (group-uniform)
      if (tau_out != nullptr && G.rank == 0) tau_out[r * tau_stride] = make_double2(0.0, 0.0);
      continue;
    }
    const double2 x0 = x[0];
    const double a0sq = fma(x0.x, x0.x, x0.y * x0.y);
    const double tot = a0sq + s2;
    const double rxn = rsqrt(tot);  // 1/||x||
    const double xn = tot * rxn;    // ||x||
    double tau;
    double2 cg;     // v[i] = x[i] * cg
    double2 alpha;  // new subdiagonal entry
    if (a0sq > 0.0) {
      const double ra0 = rsqrt(a0sq);
      const double a0 = a0sq * ra0;        // |x0|
      const double d = a0 + xn;            // |u0|
      const double ig = ra0 / d;           // 1/(|x0| (|x0| + ||x||))
      cg = make_double2(x0.x * ig, -x0.y * ig);
      const double f = -xn * ra0;          // alpha = -x0 ||x|| / |x0|
      alpha = make_double2(x0.x * f, x0.y * f);
      tau = d * rxn;                       // (|x0| + ||x||)/||x||
    } else {
      cg = make_double2(rxn, 0.0);
      alpha = make_double2(-xn, 0.0);
      tau = 1.0;
    }
    TZG_DBG_TOUCH(M, r + m, r);  // last entry of the reflector vector
    for (int i = 1 + G.rank; i < m; i += L) x[i * rs] = cmul(x[i * rs], cg);
    G.sync();
    if (G.rank == 0) {
      x[0] = alpha;
      if (tau_out != nullptr) tau_out[r * tau_stride] = make_double2(tau, 0.0);
    }
    // Left update: H[r+1:, c] -= tau v (v^H H[r+1:, c]) for c = r+1 .. n-1, two columns at a time.
    {
      int c = r + 1 + G.rank;
      for (; c + L < n; c += 2 * L) {
        double2* p[2] = {M.at(r + 1, c), M.at(r + 1, c + L)};
        TZG_DBG_TOUCH(M, r + m, c + L);
        reflect_vectors<2, false>(p, x, m, rs, rs, tau);
      }
      if (c < n) {
        double2* p[1] = {M.at(r + 1, c)};
        TZG_DBG_TOUCH(M, r + m, c);
        reflect_vectors<1, false>(p, x, m, rs, rs, tau);
      }
    }
    G.sync();
    // Right update: H[q, r+1:] -= tau (H[q, r+1:] v) v^H for every row q, two rows at a time.
    {
      int q = G.rank;
      for (; q + L < n; q += 2 * L) {
        double2* p[2] = {M.at(q, r + 1), M.at(q + L, r + 1)};
        TZG_DBG_TOUCH(M, q + L, r + m);
        reflect_vectors<2, true>(p, x, m, cs, rs, tau);
      }
      if (q < n) {
        double2* p[1] = {M.at(q, r + 1)};
        TZG_DBG_TOUCH(M, q, r + m);
        reflect_vectors<1, true>(p, x, m, cs, rs, tau);
      }
    }
    G.sync();
  }
}

// Index of the unused estimate nearest to t (bit k of `used` marks estimate k
// as used), or -1 if none is finite. The scan is FP32 and identical in every
// lane of a group, so all lanes agree.
__device__ __forceinline__ int nearest_estimate(const float2* __restrict__ est, int n, unsigned long long used,
                                                double2 t) {
  const float tx = (float)t.x, ty = (float)t.y;
  float best = 3.0e38f;
  int k_best = -1;
  for (int k = 0; k < n; ++k) {
    if ((used >> k) & 1ull) continue;
    const float2 e = est[k];
    const float dx = e.x - tx, dy = e.y - ty;
    const float d2 = fmaf(dx, dx, dy * dy);
    if (d2 < best) {
      best = d2;
      k_best = k;
    }
  }
  return k_best;
}

// Deflation test for subdiagonal entry k (k >= 1) of the active block [lo, hi]:
// negligible by the Ahues-Tisseur criterion (LAPACK Working Note 122), with
// smlnum guarding underflow. `tol` is the relative threshold (ulp for the
// eigenvalue path; the gradient path relaxes it, see zgeev_backward.cuh).
__device__ __forceinline__ bool negligible_subdiag(const MatView& M, int k, int lo, int hi, double smlnum,
                                                   double tol = kUlp) {
  const double2 hk = *M.at(k, k - 1);
  const double h1 = cabs1(hk);
  if (nonneg_le(h1, smlnum)) return true;
  const double2 dkk = *M.at(k, k);
  const double2 dk1 = *M.at(k - 1, k - 1);
  double tst = cabs1(dk1) + cabs1(dkk);
  if (is_zero(tst)) {
    if (k - 2 >= lo) tst += cabs1(*M.at(k - 1, k - 2));
    if (k + 1 <= hi) tst += cabs1(*M.at(k + 1, k));
  }
  if (nonneg_lt(tol * tst, h1)) return false;
  const double2 up = *M.at(k - 1, k);
  const double hu = cabs1(up);
  const double ab = fmax(h1, hu), ba = fmin(h1, hu);
  const double dd = cabs1(csub(dk1, dkk));
  const double d1 = cabs1(dkk);
  const double aa = fmax(d1, dd), bb = fmin(d1, dd);
  const double s = aa + ab;
  return ba * (ab / s) <= fmax(smlnum, tol * (bb * (aa / s)));
}

// Single-shift complex QR on the Hessenberg matrix (eigenvalues only), from
// the bottom up. On return eig_out[i] holds the i-th Schur diagonal entry
// (times 2^shift). Returns kConverged or kNotConverged. The per-eigenvalue
// sweep cap defaults to LAPACK's 30*max(10, n).
template <int L, class Out = double2>
__device__ int qr_eigenvalues(const MatView& M, const Group<L>& G, Out* __restrict__ eig_out, int shift, int itmax,
                              const float2* __restrict__ est = nullptr, int* sweeps_out = nullptr) {
  const int n = M.n;
  const int rs = M.rs;
  const int cs = n * rs;
  const double smlnum = kSafeMin * ((double)n / kUlp);
  const double unscale = (shift != 0) ? pow2(shift) : 1.0;
  int status = kConverged;
  int i = n - 1;   // last unconverged row
  int lo = 0;      // top of the active block [lo, i]
  int its = 0;     // sweeps since the last deflation (LAPACK's per-eigenvalue cap)
  int kdefl = 0;   // sweeps since the last deflation, for ad hoc shifts
  unsigned long long used = 0;  // estimates already matched to a deflated eigenvalue
  int sweeps = 0;               // sweeps of this matrix (reported when sweeps_out is given)
  // One loop iteration = (deflations, then) one sweep. Lanes of a warp hold
  // different matrices; keeping them in lockstep per sweep rather than per
  // eigenvalue means a lane whose eigenvalue converged early goes straight
  // on to its next sweep instead of idling until every lane has converged.
  while (true) {
    // Deflation: peel converged entries off the bottom (usually 0 or 1 per sweep).
    for (;;) {
      // Lowest negligible subdiagonal in (lo, i]; lanes scan interleaved k's
      // from the bottom and the group keeps the largest hit.
      int hit = lo;
      for (int k = i - G.rank; k > lo; k -= L) {
        if (negligible_subdiag(M, k, lo, i, smlnum)) {
          hit = k;
          break;
        }
      }
      lo = G.imax(hit);
      if (lo < i) break;
      {
        const double2 d = *M.at(i, i);
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
    {
      // Shift selection.
      double2 sigma;
      if (kdefl % (2 * kExceptionalPeriod) == 0) {
        const double2 d = *M.at(i, i);
        sigma = make_double2(d.x + kExceptionalWeight * cabs1(*M.at(i, i - 1)), d.y);
      } else if (kdefl % kExceptionalPeriod == 0) {
        const double2 d = *M.at(lo, lo);
        sigma = make_double2(d.x + kExceptionalWeight * cabs1(*M.at(lo + 1, lo)), d.y);
      } else {
        sigma = wilkinson_shift(*M.at(i - 1, i - 1), *M.at(i - 1, i), *M.at(i, i - 1), *M.at(i, i));
        if (est != nullptr && its == 1) {  // first sweep for this position: the nearest FP32 estimate
          const int k = nearest_estimate(est, n, used, sigma);
          if (k >= 0) {
            const float2 e = est[k];
            sigma = make_double2((double)e.x, (double)e.y);
          }
        }
      }
      // One implicit single-shift sweep over the active block [lo, i].
      for (int j = lo; j < i; ++j) {
        double2 x, y, rr;
        if (j == lo) {
          x = csub(*M.at(lo, lo), sigma);
          y = *M.at(lo + 1, lo);
        } else {
          x = *M.at(j, j - 1);
          y = *M.at(j + 1, j - 1);
        }
        const Rot g = make_rot(x, y, rr);
        G.sync();  // all lanes have read the bulge before it is overwritten
        if (j > lo && G.rank == 0) *M.at(j, j - 1) = rr;
        // Left: rows (j, j+1), columns j .. i.
        {
          const int c0 = j + G.rank;
          TZG_DBG_RUN(M, j, c0, 0, L, strided_count(c0, i, L), 1, 0);
          rotate_pairs<false>(g, M.ptr(j, c0), strided_count(c0, i, L), L * cs, rs);
        }
        G.sync();
        // Right: columns (j, j+1), rows lo .. min(j+2, i); row j+2 holds the
        // new bulge (its column-j entry is zero before the rotation).
        {
          const int qend = min(j + 1, i);
          const int q0 = lo + G.rank;
          TZG_DBG_RUN(M, q0, j, L, 0, strided_count(q0, qend, L), 0, 1);
          rotate_pairs<true>(g, M.ptr(q0, j), strided_count(q0, qend, L), L * rs, cs);
          if (j + 2 <= i && G.rank == ((j + 2 - lo) & (L - 1))) {
            double2* pb = M.at(j + 2, j);
            TZG_DBG_TOUCH(M, j + 2, j + 1);
            const double2 b = pb[cs];
            // a' = conj(s) b ; b' = c b
            pb[0] = make_double2(fma(g.s.x, b.x, g.s.y * b.y), fma(g.s.x, b.y, -g.s.y * b.x));
            pb[cs] = make_double2(g.c * b.x, g.c * b.y);
          }
        }
        G.sync();
      }
    }
  }
  if (status != kConverged && G.rank == 0) {
    // Unconverged positions 0..i carry their current diagonal entries.
    for (int k = 0; k <= i; ++k) {
      const double2 d = *M.at(k, k);
      put_ev(eig_out + k, make_double2(d.x * unscale, d.y * unscale));
    }
  }
  if (sweeps_out != nullptr) *sweeps_out = sweeps;
  return status;
}

// Full solve of one matrix by its lane group: stage (with exact pre-scaling),
// Hessenberg reduction, QR, eigenvalue write-out. Returns the flag value.
// kBalance selects the instantiation that runs balance() with balance_mode;
// without it the balancing code is not compiled into the kernel at all.
// Phases of a solve split in two launches (stage + Hessenberg, then QR), and
// the per-matrix state value meaning "eigenvalues and flag already written".
enum : int { kPhaseAll = 0, kPhasePrepare = 1, kPhaseQR = 2 };
constexpr int kStateDone = -2147483647 - 1;

// First half of solve_matrix: staging, balancing, Hessenberg reduction.
// Returns kPrepared with the pre-scaling exponent in `shift` when the QR is
// still to run, or the final flag value (eigenvalues already written) for
// non-finite and zero matrices.
constexpr int kPrepared = -1;

template <int L, bool kBalance = false, class Src = SrcContig, class Out = double2>
__device__ __forceinline__ int prepare_matrix(const Src& src, const MatView& M, const Group<L>& G,
                                              Out* __restrict__ ev, int balance_mode, int& shift) {
  bool nonfinite, zero;
  shift = stage_and_scale<L>(src, M, G, nonfinite, zero);
  if (nonfinite || zero) {
    const double v = nonfinite ? __longlong_as_double(0x7ff8000000000000LL) : 0.0;
    for (int i = G.rank; i < M.n; i += L) put_ev(ev + i, make_double2(v, v));
    return nonfinite ? kNonFinite : kConverged;
  }
  if (kBalance) balance<L>(M, G, balance_mode);
  hessenberg<L>(M, G);
  return kPrepared;
}

template <int L, bool kBalance = false, class Src = SrcContig, class Out = double2>
__device__ __forceinline__ int solve_matrix(const Src& src, const MatView& M, const Group<L>& G,
                                            Out* __restrict__ ev, int itmax, int balance_mode = kBalanceNone,
                                            const float2* __restrict__ est = nullptr) {
  int shift;
  const int status = prepare_matrix<L, kBalance>(src, M, G, ev, balance_mode, shift);
  if (status != kPrepared) return status;
  return qr_eigenvalues<L>(M, G, ev, shift, itmax, est);
}

// Contiguous column-major double-complex source (the reference's layout).
template <int L, bool kBalance = false>
__device__ __forceinline__ int solve_matrix(const double2* __restrict__ src, const MatView& M, const Group<L>& G,
                                            double2* __restrict__ ev, int itmax, int balance_mode = kBalanceNone,
                                            const float2* __restrict__ est = nullptr) {
  return solve_matrix<L, kBalance, SrcContig, double2>(SrcContig{src}, M, G, ev, itmax, balance_mode, est);
}

}  // namespace tzg
