// Real nonsymmetric eigenvalues (LAPACK dgeev with JOBVL = JOBVR = 'N') for
// one matrix per lane group: exact power-of-two pre-scaling, optional
// balancing, Householder Hessenberg reduction in real arithmetic, and the
// Francis double-shift QR iteration with real 2x2 blocks (the algorithm of
// LAPACK's dlahqr: Ahues-Tisseur deflation, two-consecutive-small-
// subdiagonal start, ad hoc shifts every 10 sweeps without deflation),
// finished by the standardization of each 2x2 block (dlanv2) so complex
// eigenvalues come out as exact conjugate pairs, positive imaginary part
// first — LAPACK's output convention. The reference has no real-input path
// (it takes cuDoubleComplex only, include/tokura_blas.h:129-151); a real
// matrix costs about a quarter of the complex FP64 work this way.
#pragma once

#include "zgeev_lane.cuh"

namespace tzg {

// View of one real matrix inside an interleaved tile: (r, c) at p[(c*n + r)*rs].
struct RMatView {
  double* p;
  int n;
  int rs;
  __device__ __forceinline__ double* at(int r, int c) const {
#ifdef TOKURA_DEBUG_BOUNDS
    if (dbg_out(r, c, n)) return p;
#endif
    return p + (c * n + r) * rs;
  }
  __device__ __forceinline__ double* ptr(int r, int c) const { return p + (c * n + r) * rs; }
};

struct SrcReal64 {
  const double* p;
  __device__ __forceinline__ double load(int e) const { return p[e]; }
};
struct SrcReal32 {  // single precision, widened exactly on load
  const float* p;
  __device__ __forceinline__ double load(int e) const { return (double)p[e]; }
};

__device__ __forceinline__ void put_real(double* p, double v) { *p = v; }
__device__ __forceinline__ void put_real(float* p, double v) { *p = (float)v; }

// Stage + exact pre-scaling, as stage_and_scale for complex input.
template <int L, class Src>
__device__ __forceinline__ int stage_and_scale_real(const Src& src, const RMatView& M, const Group<L>& G,
                                                    bool& nonfinite, bool& zero) {
  const int nn = M.n * M.n;
  int emax = 0;
  for (int e = G.rank; e < nn; e += L) emax = max(emax, dexp_field(src.load(e)));
  emax = G.imax(emax);
  nonfinite = (emax == 0x7ff);
  zero = (emax == 0);
  int shift = 0;
  if (!nonfinite && !zero) {
    const int top = emax - 1023;
    if (top > 60 || top < -60) shift = top;
  }
  const double sc = shift == 0 ? 1.0 : (shift > 1022 ? 0.5 * pow2(-1022) : pow2(-shift));
  for (int e = G.rank; e < nn; e += L) M.p[e * M.rs] = src.load(e) * sc;
  G.sync();
  return shift;
}

// a <- a - tau v (v^T a) for NV vectors of length m at p[k][i*es], with
// v[0] = 1 and v[i] = x[i*xs]. Real counterpart of reflect_vectors.
template <int NV>
__device__ __forceinline__ void reflect_real(double* const (&p)[NV], const double* x, int m, int es, int xs,
                                             double tau) {
  double w[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) w[k] = p[k][0];
  for (int i = 1; i < m; ++i) {
    const double v = x[i * xs];
#pragma unroll
    for (int k = 0; k < NV; ++k) w[k] = fma(v, p[k][i * es], w[k]);
  }
  double t[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) {
    t[k] = w[k] * tau;
    p[k][0] -= t[k];
  }
  if (m < 2) return;
  double v = x[xs];
  double a[NV];
#pragma unroll
  for (int k = 0; k < NV; ++k) a[k] = p[k][es];
  for (int i = 1; i < m; ++i) {
    double vn = v, an[NV];
    if (i + 1 < m) {
      vn = x[(i + 1) * xs];
#pragma unroll
      for (int k = 0; k < NV; ++k) an[k] = p[k][(i + 1) * es];
    }
#pragma unroll
    for (int k = 0; k < NV; ++k) p[k][i * es] = fma(-v, t[k], a[k]);
    v = vn;
#pragma unroll
    for (int k = 0; k < NV; ++k) a[k] = an[k];
  }
}

// Householder reduction to upper Hessenberg form (dgehd2's reflectors:
// beta = -sign(alpha) ||x||, tau = (beta - alpha)/beta, v = x/(alpha - beta)).
// Entries below the third subdiagonal keep reflector data; the QR below
// never reads them.
template <int L>
__device__ void hessenberg_real(const RMatView& M, const Group<L>& G) {
  const int n = M.n;
  const int rs = M.rs;
  const int cs = n * rs;
  for (int r = 0; r + 2 < n; ++r) {
    const int m = n - r - 1;
    double* x = M.at(r + 1, r);
    double s2 = 0.0;
    for (int i = 1 + G.rank; i < m; i += L) s2 = fma(x[i * rs], x[i * rs], s2);
    s2 = G.sum(s2);
    if (s2 == 0.0) continue;  // tau = 0 (group-uniform)
    const double alpha = x[0];
    const double xn = sqrt(fma(alpha, alpha, s2));
    const double beta = alpha >= 0.0 ? -xn : xn;
    const double tau = (beta - alpha) / beta;
    const double scal = 1.0 / (alpha - beta);
    for (int i = 1 + G.rank; i < m; i += L) x[i * rs] *= scal;
    G.sync();
    if (G.rank == 0) x[0] = beta;
    {
      int c = r + 1 + G.rank;
      for (; c + L < n; c += 2 * L) {
        double* p[2] = {M.at(r + 1, c), M.at(r + 1, c + L)};
        reflect_real<2>(p, x, m, rs, rs, tau);
      }
      if (c < n) {
        double* p[1] = {M.at(r + 1, c)};
        reflect_real<1>(p, x, m, rs, rs, tau);
      }
    }
    G.sync();
    {
      int q = G.rank;
      for (; q + L < n; q += 2 * L) {
        double* p[2] = {M.at(q, r + 1), M.at(q + L, r + 1)};
        reflect_real<2>(p, x, m, cs, rs, tau);
      }
      if (q < n) {
        double* p[1] = {M.at(q, r + 1)};
        reflect_real<1>(p, x, m, cs, rs, tau);
      }
    }
    G.sync();
    // The double-shift bulge lives on the second and third subdiagonals:
    // clear the reflector entries stored there (deeper ones are never read).
    if (G.rank == 0) {
      x[rs] = 0.0;
      if (m > 2) x[2 * rs] = 0.0;
    }
  }
  G.sync();
}

// Applies the 3-element (NR = 3) or 2-element reflector of a double-shift
// step, I - t1 [1 v2 v3]^T [1 v2 v3] (with t2 = t1 v2, t3 = t1 v3), to
// `count` element triples p[t*step + {0, es, 2 es}]. Triple t+1 is loaded
// before triple t is stored, so L1 latency overlaps the arithmetic.
template <int NR>
__device__ __forceinline__ void reflect_triples(double* p, int count, int step, int es, double v2, double v3,
                                                double t1, double t2, double t3) {
  if (count <= 0) return;
  double a0 = p[0], a1 = p[es], a2 = NR == 3 ? p[2 * es] : 0.0;
  for (int t = 1; t < count; ++t) {
    double* pn = p + step;
    const double b0 = pn[0], b1 = pn[es], b2 = NR == 3 ? pn[2 * es] : 0.0;
    const double sum = NR == 3 ? fma(v3, a2, fma(v2, a1, a0)) : fma(v2, a1, a0);
    p[0] = fma(-sum, t1, a0);
    p[es] = fma(-sum, t2, a1);
    if (NR == 3) p[2 * es] = fma(-sum, t3, a2);
    a0 = b0;
    a1 = b1;
    a2 = b2;
    p = pn;
  }
  const double sum = NR == 3 ? fma(v3, a2, fma(v2, a1, a0)) : fma(v2, a1, a0);
  p[0] = fma(-sum, t1, a0);
  p[es] = fma(-sum, t2, a1);
  if (NR == 3) p[2 * es] = fma(-sum, t3, a2);
}

// Ahues-Tisseur test for subdiagonal k of the active block (dlahqr's).
__device__ __forceinline__ bool negligible_real(const RMatView& M, int k, int n, double smlnum) {
  const double h = fabs(*M.at(k, k - 1));
  if (nonneg_le(h, smlnum)) return true;
  const double dkk = *M.at(k, k), dk1 = *M.at(k - 1, k - 1);
  double tst = fabs(dk1) + fabs(dkk);
  if (is_zero(tst)) {
    if (k - 2 >= 0) tst += fabs(*M.at(k - 1, k - 2));
    if (k + 1 <= n - 1) tst += fabs(*M.at(k + 1, k));
  }
  if (nonneg_lt(kUlp * tst, h)) return false;
  const double hu = fabs(*M.at(k - 1, k));
  const double ab = fmax(h, hu), ba = fmin(h, hu);
  const double dd = fabs(dk1 - dkk);
  const double aa = fmax(fabs(dkk), dd), bb = fmin(fabs(dkk), dd);
  const double s = aa + ab;
  return ba * (ab / s) <= fmax(smlnum, kUlp * (bb * (aa / s)));
}

// Eigenvalues of the real 2x2 block [a b; c d] via its standardized Schur
// form (the procedure of LAPACK's dlanv2): a complex pair comes out as
// (p + i q, p - i q) with q > 0 and equal real parts; a real pair as two
// real numbers.
__device__ __forceinline__ void standardize_2x2(double a, double b, double c, double d, double& rt1r, double& rt1i,
                                                double& rt2r, double& rt2i) {
  if (c == 0.0) {
  } else if (b == 0.0) {
    const double t = d;  // swap rows and columns
    d = a;
    a = t;
    b = -c;
    c = 0.0;
  } else if (a - d == 0.0 && (b > 0.0) != (c > 0.0)) {
  } else {
    double temp = a - d;
    double p = 0.5 * temp;
    const double bcmax = fmax(fabs(b), fabs(c));
    const double bcmis = fmin(fabs(b), fabs(c)) * copysign(1.0, b) * copysign(1.0, c);
    const double scale = fmax(fabs(p), bcmax);
    double z = (p / scale) * p + (bcmax / scale) * bcmis;
    if (z >= 4.0 * kUlp) {  // real eigenvalues
      z = p + copysign(sqrt(scale) * sqrt(z), p);
      a = d + z;
      d = d - (bcmax / z) * bcmis;
      c = 0.0;
    } else {  // complex or nearly equal real eigenvalues: equalize the diagonal
      const double sigma = b + c;
      const double tau = hypot(sigma, temp);
      const double cs = sqrt(0.5 * (1.0 + fabs(sigma) / tau));
      const double sn = -(p / (tau * cs)) * copysign(1.0, sigma);
      const double aa = a * cs + b * sn, bb = -a * sn + b * cs;
      const double cc = c * cs + d * sn, dd = -c * sn + d * cs;
      a = aa * cs + cc * sn;
      b = bb * cs + dd * sn;
      c = -aa * sn + cc * cs;
      d = -bb * sn + dd * cs;
      temp = 0.5 * (a + d);
      a = temp;
      d = temp;
      if (c != 0.0) {
        if (b != 0.0) {
          if ((b > 0.0) == (c > 0.0)) {  // real eigenvalues after all
            const double sab = sqrt(fabs(b)), sac = sqrt(fabs(c));
            p = copysign(sab * sac, c);
            a = temp + p;
            d = temp - p;
            c = 0.0;
          }
        } else {
          b = -c;
          c = 0.0;
        }
      }
    }
  }
  rt1r = a;
  rt2r = d;
  if (c == 0.0) {
    rt1i = 0.0;
    rt2i = 0.0;
  } else {
    rt1i = sqrt(fabs(b)) * sqrt(fabs(c));
    rt2i = -rt1i;
  }
}

// First column of (H - s1)(H - s2) at row m, scaled (dlahqr's v).
__device__ __forceinline__ void double_shift_vector(const RMatView& M, int m, double rt1r, double rt1i, double rt2r,
                                                    double rt2i, double& v1, double& v2, double& v3) {
  const double hmm = *M.at(m, m);
  double h21s = *M.at(m + 1, m);
  const double s = fabs(hmm - rt2r) + fabs(rt2i) + fabs(h21s);
  h21s = h21s / s;
  v1 = h21s * *M.at(m, m + 1) + (hmm - rt1r) * ((hmm - rt2r) / s) - rt1i * (rt2i / s);
  v2 = h21s * (hmm + *M.at(m + 1, m + 1) - rt1r - rt2r);
  v3 = h21s * *M.at(m + 2, m + 1);
  const double t = fabs(v1) + fabs(v2) + fabs(v3);
  v1 /= t;
  v2 /= t;
  v3 /= t;
}

// Double-shift QR on the Hessenberg matrix, eigenvalues only, from the
// bottom up; wr/wi receive the eigenvalues times 2^shift. One loop iteration
// = deflation checks, then one sweep, so the matrices of a warp stay in
// lockstep per sweep. Returns kConverged or kNotConverged (per-block sweep
// cap itmax, LAPACK's 30*max(10, n) by default).
template <int L, class Out>
__device__ int real_qr_eigenvalues(const RMatView& M, const Group<L>& G, Out* __restrict__ wr, Out* __restrict__ wi,
                                   int shift, int itmax) {
  const int n = M.n;
  const int rs = M.rs;
  const int cs = n * rs;
  const double smlnum = kSafeMin * ((double)n / kUlp);
  const double unscale = shift != 0 ? pow2(shift) : 1.0;
  int status = kConverged;
  int i = n - 1;
  int l = 0;
  int its = 0;
  int kdefl = 0;
  while (true) {
    for (;;) {
      int hit = l;
      for (int k = i - G.rank; k > l; k -= L) {
        if (negligible_real(M, k, n, smlnum)) {
          hit = k;
          break;
        }
      }
      l = G.imax(hit);
      if (l > 0 && G.rank == 0) *M.at(l, l - 1) = 0.0;
      G.sync();
      if (l < i - 1) break;
      if (G.rank == 0) {  // a 1x1 or 2x2 block has split off at the bottom
        if (l == i) {
          put_real(wr + i, *M.at(i, i) * unscale);
          put_real(wi + i, 0.0);
        } else {
          double r1, i1, r2, i2;
          standardize_2x2(*M.at(i - 1, i - 1), *M.at(i - 1, i), *M.at(i, i - 1), *M.at(i, i), r1, i1, r2, i2);
          put_real(wr + i - 1, r1 * unscale);
          put_real(wi + i - 1, i1 * unscale);
          put_real(wr + i, r2 * unscale);
          put_real(wi + i, i2 * unscale);
        }
      }
      i = l - 1;
      l = 0;
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
    // Shifts: the eigenvalues of the trailing 2x2 (both set to the real one
    // nearer H(i,i) when they are real), or an ad hoc pair.
    double h11, h12, h21, h22;
    if (kdefl % (2 * kExceptionalPeriod) == 0) {
      const double s = fabs(*M.at(i, i - 1)) + fabs(*M.at(i - 1, i - 2));
      h11 = kExceptionalWeight * s + *M.at(i, i);
      h12 = -0.4375 * s;
      h21 = s;
      h22 = h11;
    } else if (kdefl % kExceptionalPeriod == 0) {
      const double s = fabs(*M.at(l + 1, l)) + fabs(*M.at(l + 2, l + 1));
      h11 = kExceptionalWeight * s + *M.at(l, l);
      h12 = -0.4375 * s;
      h21 = s;
      h22 = h11;
    } else {
      h11 = *M.at(i - 1, i - 1);
      h21 = *M.at(i, i - 1);
      h12 = *M.at(i - 1, i);
      h22 = *M.at(i, i);
    }
    double rt1r, rt1i, rt2r, rt2i;
    {
      const double s = fabs(h11) + fabs(h12) + fabs(h21) + fabs(h22);
      if (s == 0.0) {
        rt1r = rt1i = rt2r = rt2i = 0.0;
      } else {
        h11 /= s;
        h21 /= s;
        h12 /= s;
        h22 /= s;
        const double tr = 0.5 * (h11 + h22);
        const double det = (h11 - tr) * (h22 - tr) - h12 * h21;
        const double rtdisc = sqrt(fabs(det));
        if (det >= 0.0) {
          rt1r = tr * s;
          rt2r = rt1r;
          rt1i = rtdisc * s;
          rt2i = -rt1i;
        } else {
          rt1r = tr + rtdisc;
          rt2r = tr - rtdisc;
          if (fabs(rt1r - h22) <= fabs(rt2r - h22)) {
            rt1r *= s;
            rt2r = rt1r;
          } else {
            rt2r *= s;
            rt1r = rt2r;
          }
          rt1i = rt2i = 0.0;
        }
      }
    }
    // Start row m: the largest m in [l, i-2] where two consecutive small
    // subdiagonals let the sweep begin (lanes test interleaved candidates).
    int m;
    {
      int hit = l;
      for (int c = i - 2 - G.rank; c > l; c -= L) {
        // The test is invariant under scaling of v, so the unnormalized
        // s*v (no divisions) serves; entries of the pre-scaled matrix keep
        // the products far from overflow.
        const double hcc = *M.at(c, c), h21 = *M.at(c + 1, c), h22 = *M.at(c + 1, c + 1);
        const double u1 = fma(h21, *M.at(c, c + 1), fma(hcc - rt1r, hcc - rt2r, -rt1i * rt2i));
        const double u2 = h21 * (hcc + h22 - rt1r - rt2r);
        const double u3 = h21 * *M.at(c + 2, c + 1);
        const double h00 = fabs(*M.at(c, c - 1)) * (fabs(u2) + fabs(u3));
        const double h01 = fabs(u1) * (fabs(*M.at(c - 1, c - 1)) + fabs(hcc) + fabs(h22));
        if (nonneg_le(h00, kUlp * h01)) {
          hit = c;
          break;
        }
      }
      m = G.imax(hit);
    }
    double v1, v2, v3;
    double_shift_vector(M, m, rt1r, rt1i, rt2r, rt2i, v1, v2, v3);
    // The sweep: 3-element reflectors chase the bulge from row m to i.
    for (int k = m; k < i; ++k) {
      const int nr = min(3, i - k + 1);
      if (k > m) {
        v1 = *M.at(k, k - 1);
        v2 = *M.at(k + 1, k - 1);
        v3 = nr == 3 ? *M.at(k + 2, k - 1) : 0.0;
      } else if (nr == 2) {
        v3 = 0.0;
      }
      // Reflector (dlarfg's): beta = -sign(v1) ||v||, t1 = (beta - v1)/beta
      // = 1 + |v1|/||v||, v(2:3) /= (v1 - beta). One rsqrt and one
      // reciprocal; tiny or huge norms take the hypot route.
      double t1 = 0.0;
      const double ss = fma(v2, v2, v3 * v3);
      if (!is_zero(ss)) {
        const double nn = fma(v1, v1, ss);
        double xn, rxn;
        if (nonneg_lt(1e-280, nn) && nonneg_lt(nn, 1e280)) {
          rxn = rsqrt(nn);
          xn = nn * rxn;
        } else {
          xn = hypot(v1, hypot(v2, v3));
          rxn = 1.0 / xn;
        }
        const double a1 = fabs(v1);
        t1 = fma(a1, rxn, 1.0);
        const double scal = copysign(1.0 / (a1 + xn), v1);
        v2 *= scal;
        v3 *= scal;
        v1 = -copysign(xn, v1);
      }
      G.sync();  // every lane has read column k-1 before it changes
      if (G.rank == 0) {
        if (k > m) {
          *M.at(k, k - 1) = v1;
          *M.at(k + 1, k - 1) = 0.0;
          if (k < i - 1) *M.at(k + 2, k - 1) = 0.0;
        } else if (m > l) {
          *M.at(k, k - 1) *= (1.0 - t1);
        }
      }
      const double t2 = t1 * v2, t3 = t1 * v3;
      if (nr == 3) {
        // rows k..k+2 of columns k..i, then columns k..k+2 of rows l..min(k+3, i)
        TZG_DBG_RUN(M, k, k + G.rank, 0, L, strided_count(k + G.rank, i, L), 2, 0);
        reflect_triples<3>(M.ptr(k, k + G.rank), strided_count(k + G.rank, i, L), L * cs, rs, v2, v3, t1, t2, t3);
        G.sync();
        TZG_DBG_RUN(M, l + G.rank, k, L, 0, strided_count(l + G.rank, min(k + 3, i), L), 0, 2);
        reflect_triples<3>(M.ptr(l + G.rank, k), strided_count(l + G.rank, min(k + 3, i), L), L * rs, cs, v2, v3, t1,
                           t2, t3);
      } else {
        TZG_DBG_RUN(M, k, k + G.rank, 0, L, strided_count(k + G.rank, i, L), 1, 0);
        reflect_triples<2>(M.ptr(k, k + G.rank), strided_count(k + G.rank, i, L), L * cs, rs, v2, 0.0, t1, t2, 0.0);
        G.sync();
        TZG_DBG_RUN(M, l + G.rank, k, L, 0, strided_count(l + G.rank, i, L), 0, 1);
        reflect_triples<2>(M.ptr(l + G.rank, k), strided_count(l + G.rank, i, L), L * rs, cs, v2, 0.0, t1, t2, 0.0);
      }
      G.sync();
    }
  }
  if (status != kConverged && G.rank == 0) {
    for (int k = 0; k <= i; ++k) {
      put_real(wr + k, *M.at(k, k) * unscale);
      put_real(wi + k, 0.0);
    }
  }
  return status;
}

template <int L, bool kBalance, class Src, class Out>
__device__ __forceinline__ int solve_real_matrix(const Src& src, const RMatView& M, const Group<L>& G,
                                                 Out* __restrict__ wr, Out* __restrict__ wi, int itmax,
                                                 int balance_mode) {
  bool nonfinite, zero;
  const int shift = stage_and_scale_real<L>(src, M, G, nonfinite, zero);
  if (nonfinite || zero) {
    const double v = nonfinite ? __longlong_as_double(0x7ff8000000000000LL) : 0.0;
    for (int i = G.rank; i < M.n; i += L) {
      put_real(wr + i, v);
      put_real(wi + i, v);
    }
    return nonfinite ? kNonFinite : kConverged;
  }
  if (kBalance) balance<L>(M, G, balance_mode);
  hessenberg_real<L>(M, G);
  return real_qr_eigenvalues<L>(M, G, wr, wi, shift, itmax);
}

}  // namespace tzg
