/*
 * TEST INFRASTRUCTURE — CPU model of this library's eigenvalue iteration.
 * Never linked into or called by the product library.
 *
 * Serial, one matrix at a time, column-major storage a[c*n + r], no
 * pre-scaling in the FP64 part (inputs of moderate size). It restates the
 * mathematics of the GPU path without its lane layout:
 *   - the FP64 eigenvalue iteration (tokura_zgeev_batched_gb300/csrc/
 *     zgeev_lane.cuh: hessenberg, negligible_subdiag, nearest_estimate,
 *     qr_eigenvalues; zgeev_device.cuh: make_rot, wilkinson_shift);
 *   - the FP32 estimator (zgeev_estimate.cuh: hessenberg_f, qr_estimates);
 *   - the eigenvalue part of the gradient's Schur iteration
 *     (zgeev_backward.cuh: schur_qr, without Q or the vectors);
 * so that tests can count sweeps per eigenvalue under each shift strategy and
 * compare eigenvalues and flags with LAPACK. The reference's own algorithm is
 * restated separately (ref_algorithm.c).
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double re, im; } zc;

static zc z(double r, double i) { zc v = {r, i}; return v; }
static zc zadd(zc a, zc b) { return z(a.re + b.re, a.im + b.im); }
static zc zsub(zc a, zc b) { return z(a.re - b.re, a.im - b.im); }
static zc zmul(zc a, zc b) { return z(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static zc zconj(zc a) { return z(a.re, -a.im); }
static zc zscale(zc a, double s) { return z(a.re * s, a.im * s); }
static double zabs1(zc a) { return fabs(a.re) + fabs(a.im); }
static double zabs2(zc a) { return a.re * a.re + a.im * a.im; }
static zc zdiv(zc a, zc b) {
  double d = zabs2(b);
  return z((a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d);
}
/* Unbiased exponent field of |v| (-1023 for zero and subnormals), as the GPU's
 * dexp_field - 1023. */
static int expo(double v) {
  unsigned long long u;
  memcpy(&u, &v, sizeof u);
  return (int)((u >> 52) & 0x7ff) - 1023;
}
static int floor_half(int e) { return e >= 0 ? e / 2 : -((1 - e) / 2); }

#define H(r, c) a[(size_t)(c) * n + (r)]

static const double kUlp = 2.220446049250313080847e-16;
static const double kSafeMin = 2.225073858507201383090e-308;
static const int kPeriod = 10;        /* ad hoc shifts after 10 / 20 sweeps without deflation */
static const double kWeight = 0.75;

/* Householder reduction to upper Hessenberg form: P = I - tau v v^H with
 * v0 = 1 and tau = 1 + |x0| / ||x||, new subdiagonal -x0 ||x|| / |x0|. */
static void hessenberg(int n, zc* a, zc* v) {
  for (int r = 0; r + 2 < n; ++r) {
    int m = n - r - 1;
    double s2 = 0.0;
    for (int i = 1; i < m; ++i) s2 += zabs2(H(r + 1 + i, r));
    if (s2 == 0.0) continue;
    zc x0 = H(r + 1, r);
    double a0 = sqrt(zabs2(x0)), xn = sqrt(zabs2(x0) + s2), tau;
    zc alpha;
    v[0] = z(1.0, 0.0);
    if (a0 > 0.0) {
      zc u0 = zscale(x0, (a0 + xn) / a0); /* x0 - alpha */
      for (int i = 1; i < m; ++i) v[i] = zdiv(H(r + 1 + i, r), u0);
      alpha = zscale(x0, -xn / a0);
      tau = (a0 + xn) / xn;
    } else {
      for (int i = 1; i < m; ++i) v[i] = zscale(H(r + 1 + i, r), 1.0 / xn);
      alpha = z(-xn, 0.0);
      tau = 1.0;
    }
    H(r + 1, r) = alpha;
    for (int i = 1; i < m; ++i) H(r + 1 + i, r) = z(0.0, 0.0);
    for (int c = r + 1; c < n; ++c) { /* left: rows r+1.., w = v^H h */
      zc w = z(0.0, 0.0);
      for (int i = 0; i < m; ++i) w = zadd(w, zmul(zconj(v[i]), H(r + 1 + i, c)));
      w = zscale(w, tau);
      for (int i = 0; i < m; ++i) H(r + 1 + i, c) = zsub(H(r + 1 + i, c), zmul(v[i], w));
    }
    for (int q = 0; q < n; ++q) { /* right: columns r+1.., w = h v */
      zc w = z(0.0, 0.0);
      for (int i = 0; i < m; ++i) w = zadd(w, zmul(H(q, r + 1 + i), v[i]));
      w = zscale(w, tau);
      for (int i = 0; i < m; ++i) H(q, r + 1 + i) = zsub(H(q, r + 1 + i), zmul(w, zconj(v[i])));
    }
  }
}

/* Hessenberg form by stabilized elementary similarity transforms (EISPACK's
 * comhes: partial pivoting, multipliers of modulus <= 1 by the 1-norm, then
 * row_i -= m row_{k+1} and col_{k+1} += m col_i): half the multiply-adds of the
 * Householder reduction, without its unconditional backward stability.
 * Options bit 3; not used by the library. */
static void hessenberg_elementary(int n, zc* a) {
  for (int k = 0; k + 2 < n; ++k) {
    int p = k + 1;
    double best = zabs1(H(k + 1, k));
    for (int i = k + 2; i < n; ++i)
      if (zabs1(H(i, k)) > best) { best = zabs1(H(i, k)); p = i; }
    if (best == 0.0) continue;
    if (p != k + 1) {
      for (int c = k; c < n; ++c) { zc t = H(p, c); H(p, c) = H(k + 1, c); H(k + 1, c) = t; }
      for (int r = 0; r < n; ++r) { zc t = H(r, p); H(r, p) = H(r, k + 1); H(r, k + 1) = t; }
    }
    zc piv = H(k + 1, k);
    for (int i = k + 2; i < n; ++i) {
      zc m = zdiv(H(i, k), piv);
      if (m.re == 0.0 && m.im == 0.0) continue;
      H(i, k) = z(0.0, 0.0);
      for (int c = k + 1; c < n; ++c) H(i, c) = zsub(H(i, c), zmul(m, H(k + 1, c)));
      for (int r = 0; r < n; ++r) H(r, k + 1) = zadd(H(r, k + 1), zmul(m, H(r, i)));
    }
  }
}

/* Ahues-Tisseur deflation test of subdiagonal entry k of the block [lo, hi],
 * relative to tol (the ulp for eigenvalues; 100 ulp in the gradient's QR). */
static int negligible(int n, const zc* a, int k, int lo, int hi, double smlnum, double tol) {
  zc hk = H(k, k - 1);
  double h1 = zabs1(hk);
  if (h1 <= smlnum) return 1;
  zc dkk = H(k, k), dk1 = H(k - 1, k - 1);
  double tst = zabs1(dk1) + zabs1(dkk);
  if (tst == 0.0) {
    if (k - 2 >= lo) tst += zabs1(H(k - 1, k - 2));
    if (k + 1 <= hi) tst += zabs1(H(k + 1, k));
  }
  if (h1 > tol * tst) return 0;
  double hu = zabs1(H(k - 1, k));
  double ab = fmax(h1, hu), ba = fmin(h1, hu);
  double dd = zabs1(zsub(dk1, dkk)), d1 = zabs1(dkk);
  double aa = fmax(d1, dd), bb = fmin(d1, dd), s = aa + ab;
  return ba * (ab / s) <= fmax(smlnum, tol * (bb * (aa / s)));
}

/* Eigenvalue of [[a, b], [c, d]] nearer to d: d - bc / (x + sqrt(x^2 + bc)),
 * x = (a - d)/2, root sign with Re(conj(x) y) >= 0, after scaling x and bc by
 * the exact power of two 2^-k, k = max(exponent of |x|_1, floor(exponent of
 * |bc|_1 / 2)); the principal root from u = (|z| + |Re z|)/2 (zgeev_device.cuh:
 * wilkinson_shift, same operations). */
static zc wilkinson(zc a, zc b, zc c, zc d) {
  zc bc = zmul(b, c);
  if (bc.re == 0.0 && bc.im == 0.0) return d;
  zc x = zscale(zsub(a, d), 0.5);
  int ex = expo(zabs1(x)), eb = floor_half(expo(zabs1(bc)));
  int k = ex > eb ? ex : eb;
  double is = ldexp(1.0, -k);
  zc xs = zscale(x, is), bcs = zscale(zscale(bc, is), is);
  zc zz = zadd(zmul(xs, xs), bcs);
  double u = 0.5 * (sqrt(zabs2(zz)) + fabs(zz.re));
  zc y = z(0.0, 0.0);
  if (u > 0.0) {
    double r = 1.0 / sqrt(u), t = u * r, h = 0.5 * zz.im * r;
    y = zz.re >= 0.0 ? z(t, h) : z(fabs(h), copysign(t, zz.im));
  }
  if (xs.re * y.re + xs.im * y.im < 0.0) y = z(-y.re, -y.im);
  zc den = zadd(xs, y);
  double f = ldexp(1.0, k) / zabs2(den);
  zc num = zmul(bcs, zconj(den));
  return z(d.re - num.re * f, d.im - num.im * f);
}

/* Rotation [c s; -conj(s) c] (c real) taking (x, y) to (r, 0). */
static void make_rot(zc x, zc y, double* c, zc* s, zc* r) {
  double p = zabs2(x), q = zabs2(y), nn = p + q;
  if (q == 0.0) {
    *c = 1.0; *s = z(0.0, 0.0); *r = x;
  } else if (p * nn < 1e-290) {
    double iq = 1.0 / sqrt(q);
    *c = 0.0; *s = zscale(zconj(y), iq); *r = z(q * iq, 0.0);
  } else {
    double R = 1.0 / sqrt(p * nn);
    *c = p * R; *s = zscale(zmul(x, zconj(y)), R); *r = zscale(x, nn * R);
  }
}

/* Index of the unused FP64 value nearest to t, or -1 (the gradient's QR). */
static int nearest64(const double* lam, int n, const unsigned char* used, zc t) {
  double best = INFINITY;
  int kb = -1;
  for (int k = 0; k < n; ++k) {
    if (used[k]) continue;
    double dx = lam[2 * k] - t.re, dy = lam[2 * k + 1] - t.im, d2 = dx * dx + dy * dy;
    if (d2 < best) { best = d2; kb = k; }
  }
  return kb;
}

/* Index of the unused estimate nearest to t (FP32 distances), or -1. */
static int nearest(const float* est, int n, const unsigned char* used, zc t) {
  float tx = (float)t.re, ty = (float)t.im, best = 3.0e38f;
  int kb = -1;
  for (int k = 0; k < n; ++k) {
    if (used[k]) continue;
    float dx = est[2 * k] - tx, dy = est[2 * k + 1] - ty;
    float d2 = dx * dx + dy * dy;
    if (d2 < best) { best = d2; kb = k; }
  }
  return kb;
}

/* Single-shift QR, bottom up, one sweep per loop iteration, updates restricted
 * to the active block. est (2n floats or NULL): the nearest unused estimate
 * is the shift of the first sweep after each deflation. options (variants
 * the library does not use, kept to measure them): bit 0 begins each sweep
 * below two consecutive small subdiagonals when allowed (the published
 * zlahqr start-row test); bit 1 takes the estimate for the second sweep too.
 * lam (2n doubles or NULL) and tol model the gradient's Schur iteration
 * (zgeev_backward.cuh: schur_qr): the nearest unused forward eigenvalue is
 * the first shift after each deflation, deflating at tol instead of the ulp.
 * trace (NULL or trace_cap ints per matrix): the active window of each sweep,
 * for simulating matrices that share a warp.
 * Returns the flag (0 converged, 1 sweep cap hit) and adds the sweeps made to
 * *sweeps and the element-pair rotation updates to *work. */
static int qr(int n, zc* a, zc* w, const float* est, const double* lam, double tol, unsigned char* used,
              long* sweeps, long long* work, int options, int* trace, long trace_cap) {
  double smlnum = kSafeMin * ((double)n / kUlp);
  int itmax = 30 * (n > 10 ? n : 10);
  int i = n - 1, lo = 0, its = 0, kdefl = 0;
  for (int k = 0; k < n; ++k) used[k] = 0;
  for (;;) {
    for (;;) {
      int hit = lo;
      for (int k = i; k > lo; --k)
        if (negligible(n, a, k, lo, i, smlnum, tol)) { hit = k; break; }
      lo = hit;
      if (lo < i) break;
      w[i] = H(i, i);
      if (lam) {
        int k = nearest64(lam, n, used, w[i]);
        if (k >= 0) used[k] = 1;
      } else if (est) {
        int k = nearest(est, n, used, w[i]);
        if (k >= 0) used[k] = 1;
      }
      i -= 1; lo = 0; its = 0; kdefl = 0;
      if (i < 0) break;
    }
    if (i < 0) return 0;
    if (its > itmax) {
      for (int k = 0; k <= i; ++k) w[k] = H(k, k);
      return 1;
    }
    if (trace && *sweeps < trace_cap) trace[*sweeps] = i - lo + 1; /* active window of this sweep */
    ++its; ++kdefl; ++*sweeps;
    zc sigma;
    if (kdefl % (2 * kPeriod) == 0) {
      sigma = z(H(i, i).re + kWeight * zabs1(H(i, i - 1)), H(i, i).im);
    } else if (kdefl % kPeriod == 0) {
      sigma = z(H(lo, lo).re + kWeight * zabs1(H(lo + 1, lo)), H(lo, lo).im);
    } else {
      sigma = wilkinson(H(i - 1, i - 1), H(i - 1, i), H(i, i - 1), H(i, i));
      if (lam && its == 1) {
        int k = nearest64(lam, n, used, sigma);
        if (k >= 0) sigma = z(lam[2 * k], lam[2 * k + 1]);
      } else if (est && (its == 1 || ((options & 2) && its == 2))) {
        int k = nearest(est, n, used, sigma);
        if (k >= 0) sigma = z(est[2 * k], est[2 * k + 1]);
      }
    }
    int start = lo;
    if (options & 1) {
      for (int m = i - 1; m > lo; --m) {
        zc h11 = H(m, m), h22 = H(m + 1, m + 1), h11s = zsub(h11, sigma), h21 = H(m + 1, m);
        double sc = zabs1(h11s) + zabs1(h21);
        if (!(sc > 0.0)) continue;
        if (zabs1(H(m, m - 1)) * (zabs1(h21) / sc) <= kUlp * (zabs1(zscale(h11s, 1.0 / sc)) * (zabs1(h11) + zabs1(h22)))) {
          start = m;
          break;
        }
      }
    }
    for (int j = start; j < i; ++j) {
      zc x, y, r, s;
      double c;
      if (j == start) { x = zsub(H(start, start), sigma); y = H(start + 1, start); }
      else { x = H(j, j - 1); y = H(j + 1, j - 1); }
      make_rot(x, y, &c, &s, &r);
      if (j > start) { H(j, j - 1) = r; H(j + 1, j - 1) = z(0.0, 0.0); }
      else if (start > lo) H(start, start - 1) = zscale(H(start, start - 1), c); /* the fill-in below is negligible */
      *work += (i - j + 1) + ((j + 2 < i ? j + 2 : i) - lo + 1);
      for (int col = j; col <= i; ++col) { /* rows j, j+1 */
        zc p = H(j, col), q = H(j + 1, col);
        H(j, col) = zadd(zscale(p, c), zmul(s, q));
        H(j + 1, col) = zsub(zscale(q, c), zmul(zconj(s), p));
      }
      int qend = j + 2 < i ? j + 2 : i;
      for (int row = lo; row <= qend; ++row) { /* columns j, j+1 */
        zc p = H(row, j), q = H(row, j + 1);
        H(row, j) = zadd(zscale(p, c), zmul(zconj(s), q));
        H(row, j + 1) = zsub(zscale(q, c), zmul(s, p));
      }
    }
  }
}

/* ---- FP32 estimator (csrc/zgeev_estimate.cuh: hessenberg_f, qr_estimates,
 * estimate_matrix): the same reduction and iteration in single precision on
 * the matrix scaled by a power of two to entries below 2 in magnitude, with
 * deflation relative to `tol` instead of the ulp and a cap of 30 sweeps per
 * eigenvalue (the diagonal then serves as estimates). */

typedef struct { float re, im; } fc;

static fc f2(float r, float i) { fc v = {r, i}; return v; }
static fc fadd(fc a, fc b) { return f2(a.re + b.re, a.im + b.im); }
static fc fsub(fc a, fc b) { return f2(a.re - b.re, a.im - b.im); }
static fc fmul(fc a, fc b) { return f2(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static fc fconj(fc a) { return f2(a.re, -a.im); }
static fc fscl(fc a, float s) { return f2(a.re * s, a.im * s); }
static float fabs1(fc a) { return fabsf(a.re) + fabsf(a.im); }
static float fabs2(fc a) { return a.re * a.re + a.im * a.im; }

#define S(r, c) h[(size_t)(c) * n + (r)]

static void hessenberg_f(int n, fc* h, fc* v) {
  for (int r = 0; r + 2 < n; ++r) {
    int m = n - r - 1;
    float s2 = 0.0f;
    for (int i = 1; i < m; ++i) s2 += fabs2(S(r + 1 + i, r));
    if (s2 == 0.0f) continue;
    fc x0 = S(r + 1, r);
    float a0sq = fabs2(x0), tot = a0sq + s2, xn = sqrtf(tot), tau;
    fc alpha, cg;
    if (a0sq > 0.0f) {
      float a0 = sqrtf(a0sq), d = a0 + xn, ig = 1.0f / (a0 * d);
      cg = f2(x0.re * ig, -x0.im * ig);
      alpha = fscl(x0, -xn / a0);
      tau = d / xn;
    } else {
      cg = f2(1.0f / xn, 0.0f);
      alpha = f2(-xn, 0.0f);
      tau = 1.0f;
    }
    v[0] = f2(1.0f, 0.0f);
    for (int i = 1; i < m; ++i) v[i] = fmul(S(r + 1 + i, r), cg);
    S(r + 1, r) = alpha;
    for (int i = 1; i < m; ++i) S(r + 1 + i, r) = f2(0.0f, 0.0f);
    for (int c = r + 1; c < n; ++c) {
      fc w = f2(0.0f, 0.0f);
      for (int i = 0; i < m; ++i) w = fadd(w, fmul(fconj(v[i]), S(r + 1 + i, c)));
      w = fscl(w, tau);
      for (int i = 0; i < m; ++i) S(r + 1 + i, c) = fsub(S(r + 1 + i, c), fmul(v[i], w));
    }
    for (int q = 0; q < n; ++q) {
      fc w = f2(0.0f, 0.0f);
      for (int i = 0; i < m; ++i) w = fadd(w, fmul(S(q, r + 1 + i), v[i]));
      w = fscl(w, tau);
      for (int i = 0; i < m; ++i) S(q, r + 1 + i) = fsub(S(q, r + 1 + i), fmul(w, fconj(v[i])));
    }
  }
}

static int negligible_f(int n, const fc* h, int k, int lo, int hi, float smlnum, float tol) {
  float h1 = fabs1(S(k, k - 1));
  if (h1 <= smlnum) return 1;
  fc dkk = S(k, k), dk1 = S(k - 1, k - 1);
  float tst = fabs1(dk1) + fabs1(dkk);
  if (tst == 0.0f) {
    if (k - 2 >= lo) tst += fabs1(S(k - 1, k - 2));
    if (k + 1 <= hi) tst += fabs1(S(k + 1, k));
  }
  if (h1 > tol * tst) return 0;
  float hu = fabs1(S(k - 1, k));
  float ab = fmaxf(h1, hu), ba = fminf(h1, hu);
  float dd = fabs1(fsub(dk1, dkk)), d1 = fabs1(dkk);
  float aa = fmaxf(d1, dd), bb = fminf(d1, dd), sum = aa + ab;
  return ba * (ab / sum) <= fmaxf(smlnum, tol * (bb * (aa / sum)));
}

static fc wilkinson_f(fc a, fc b, fc c, fc d) {
  fc bc = fmul(b, c);
  if (bc.re == 0.0f && bc.im == 0.0f) return d;
  fc x = fscl(fsub(a, d), 0.5f);
  float sc = fmaxf(fabs1(x), sqrtf(fabs1(bc)));
  if (!(sc > 0.0f) || !(sc < 3.0e38f)) return d;
  fc xs = fscl(x, 1.0f / sc), bcs = fscl(bc, 1.0f / (sc * sc));
  fc zz = fadd(fmul(xs, xs), bcs);
  float m = hypotf(zz.re, zz.im);
  fc y = f2(0.0f, 0.0f);
  if (m > 0.0f) {
    float t = sqrtf(0.5f * (m + fabsf(zz.re))), hh = zz.im / (2.0f * t);
    y = zz.re >= 0.0f ? f2(t, hh) : f2(fabsf(hh), copysignf(t, zz.im));
  }
  if (xs.re * y.re + xs.im * y.im < 0.0f) y = f2(-y.re, -y.im);
  fc den = fadd(xs, y);
  float dd = fabs2(den);
  if (!(dd > 0.0f)) return d;
  fc corr = f2((bcs.re * den.re + bcs.im * den.im) / dd, (bcs.im * den.re - bcs.re * den.im) / dd);
  return fsub(d, fscl(corr, sc));
}

static void rot_f(fc x, fc y, float* c, fc* s, fc* r) {
  float p = fabs2(x), q = fabs2(y), nn = p + q;
  if (q == 0.0f) {
    *c = 1.0f; *s = f2(0.0f, 0.0f); *r = x;
  } else if (p * nn < 1e-30f) {
    float iq = 1.0f / sqrtf(q);
    *c = 0.0f; *s = fscl(fconj(y), iq); *r = f2(q * iq, 0.0f);
  } else {
    float R = 1.0f / sqrtf(p * nn);
    *c = p * R; *s = fscl(fmul(x, fconj(y)), R); *r = fscl(x, nn * R);
  }
}

static void qr_f(int n, fc* h, float* est, float f, float tol, long* sweeps) {
  const float smlnum = 1.1754943508222875e-38f * ((float)n / 5.9604644775390625e-08f);
  int i = n - 1, lo = 0, its = 0, kdefl = 0;
  for (;;) {
    for (;;) {
      int hit = lo;
      for (int k = i; k > lo; --k)
        if (negligible_f(n, h, k, lo, i, smlnum, tol)) { hit = k; break; }
      lo = hit;
      if (lo < i) break;
      est[2 * i] = S(i, i).re * f;
      est[2 * i + 1] = S(i, i).im * f;
      i -= 1; lo = 0; its = 0; kdefl = 0;
      if (i < 0) return;
    }
    if (its >= 30) {
      for (int k = 0; k <= i; ++k) { est[2 * k] = S(k, k).re * f; est[2 * k + 1] = S(k, k).im * f; }
      return;
    }
    ++its; ++kdefl; ++*sweeps;
    fc sigma;
    if (kdefl % (2 * kPeriod) == 0) sigma = f2(S(i, i).re + 0.75f * fabs1(S(i, i - 1)), S(i, i).im);
    else if (kdefl % kPeriod == 0) sigma = f2(S(lo, lo).re + 0.75f * fabs1(S(lo + 1, lo)), S(lo, lo).im);
    else sigma = wilkinson_f(S(i - 1, i - 1), S(i - 1, i), S(i, i - 1), S(i, i));
    for (int j = lo; j < i; ++j) {
      fc x, y, r, s;
      float c;
      if (j == lo) { x = fsub(S(lo, lo), sigma); y = S(lo + 1, lo); }
      else { x = S(j, j - 1); y = S(j + 1, j - 1); }
      rot_f(x, y, &c, &s, &r);
      if (j > lo) { S(j, j - 1) = r; S(j + 1, j - 1) = f2(0.0f, 0.0f); }
      for (int col = j; col <= i; ++col) {
        fc p = S(j, col), q = S(j + 1, col);
        S(j, col) = fadd(fscl(p, c), fmul(s, q));
        S(j + 1, col) = fsub(fscl(q, c), fmul(fconj(s), p));
      }
      int qend = j + 2 < i ? j + 2 : i;
      for (int row = lo; row <= qend; ++row) {
        fc p = S(row, j), q = S(row, j + 1);
        S(row, j) = fadd(fscl(p, c), fmul(fconj(s), q));
        S(row, j + 1) = fsub(fscl(q, c), fmul(s, p));
      }
    }
  }
}

/* FP32 estimates of every matrix of the batch (2n floats per matrix), as the
 * GPU estimator computes them, with deflation tolerance `tol` (1e-5 there);
 * sweeps (NULL or one per matrix): the FP32 QR's sweeps. */
void model_estimates_batched(int n, int batch, const double* A, float* est, float tol, long* sweeps) {
  fc* h = malloc(sizeof(fc) * (size_t)n * n);
  fc* v = malloc(sizeof(fc) * (size_t)n);
  for (int j = 0; j < batch; ++j) {
    const double* src = A + (size_t)j * 2 * n * n;
    double amax = 0.0;
    for (size_t e = 0; e < (size_t)2 * n * n; ++e) amax = fmax(amax, fabs(src[e]));
    float* out = est + (size_t)j * 2 * n;
    long dummy = 0;
    long* sw = sweeps ? &sweeps[j] : &dummy;
    *sw = 0;
    if (amax == 0.0 || !isfinite(amax)) {
      for (int i = 0; i < 2 * n; ++i) out[i] = 0.0f;
      continue;
    }
    int top;
    frexp(amax, &top);
    top -= 1; /* amax in [2^top, 2^(top+1)) */
    double sc = ldexp(1.0, -top);
    for (size_t e = 0; e < (size_t)n * n; ++e) h[e] = f2((float)(src[2 * e] * sc), (float)(src[2 * e + 1] * sc));
    hessenberg_f(n, h, v);
    qr_f(n, h, out, (float)ldexp(1.0, top), tol, sw);
  }
  free(h);
  free(v);
}

#undef S

/* ---- Scaled rotations (options bit 2; not used by the library yet).
 * The matrix is kept as K with the true entry H(r,c) = K(r,c) * dc[c] / dr[r]
 * (real row and column scale factors). A rotation G = [c s; -conj(s) c]
 * applied to rows j, j+1 becomes k_j += alpha k_{j+1}, k_{j+1} += beta k_j with
 * dr_j, dr_{j+1} divided by c, and applied to columns j, j+1 becomes
 * k_j += gamma k_{j+1}, k_{j+1} += delta k_j with dc_j, dc_{j+1} multiplied by
 * c: two complex multiply-adds per element pair (8 FP64 operations) instead of
 * the 12 of the plain rotation. Shifts, rotations and deflation tests read the
 * true entries through the scale factors; a row or column whose factor leaves
 * [2^-150, 2^150] is rescaled to 1 (O(n) work, counted). */
#define HT(r, c) zscale(H(r, c), dc[c] / dr[r])

static int negligible_s(int n, const zc* a, const double* dr, const double* dc, int k, int lo, int hi,
                        double smlnum, double tol) {
  zc hk = HT(k, k - 1);
  double h1 = zabs1(hk);
  if (h1 <= smlnum) return 1;
  zc dkk = HT(k, k), dk1 = HT(k - 1, k - 1);
  double tst = zabs1(dk1) + zabs1(dkk);
  if (tst == 0.0) {
    if (k - 2 >= lo) tst += zabs1(HT(k - 1, k - 2));
    if (k + 1 <= hi) tst += zabs1(HT(k + 1, k));
  }
  if (h1 > tol * tst) return 0;
  double hu = zabs1(HT(k - 1, k));
  double ab = fmax(h1, hu), ba = fmin(h1, hu);
  double dd = zabs1(zsub(dk1, dkk)), d1 = zabs1(dkk);
  double aa = fmax(d1, dd), bb = fmin(d1, dd), s = aa + ab;
  return ba * (ab / s) <= fmax(smlnum, tol * (bb * (aa / s)));
}

static void rescale_row(int n, zc* a, double* dr, int r, long long* rescales) {
  double f = 1.0 / dr[r];
  for (int c = 0; c < n; ++c) H(r, c) = zscale(H(r, c), f);
  dr[r] = 1.0;
  ++*rescales;
}
static void rescale_col(int n, zc* a, double* dc, int c, long long* rescales) {
  double f = dc[c];
  for (int r = 0; r < n; ++r) H(r, c) = zscale(H(r, c), f);
  dc[c] = 1.0;
  ++*rescales;
}

static int qr_scaled(int n, zc* a, zc* w, const float* est, unsigned char* used, long* sweeps, long long* work,
                     long long* rescales) {
  double smlnum = kSafeMin * ((double)n / kUlp);
  int itmax = 30 * (n > 10 ? n : 10);
  int i = n - 1, lo = 0, its = 0, kdefl = 0;
  double dr[64], dc[64]; /* the library's orders: n <= 64 */
  if (n > 64) return 1;
  for (int k = 0; k < n; ++k) { used[k] = 0; dr[k] = dc[k] = 1.0; }
  const double big = 0x1p150, small = 0x1p-150;
  for (;;) {
    for (;;) {
      int hit = lo;
      for (int k = i; k > lo; --k)
        if (negligible_s(n, a, dr, dc, k, lo, i, smlnum, kUlp)) { hit = k; break; }
      lo = hit;
      if (lo < i) break;
      w[i] = HT(i, i);
      if (est) {
        int k = nearest(est, n, used, w[i]);
        if (k >= 0) used[k] = 1;
      }
      i -= 1; lo = 0; its = 0; kdefl = 0;
      if (i < 0) break;
    }
    if (i < 0) return 0;
    if (its > itmax) {
      for (int k = 0; k <= i; ++k) w[k] = HT(k, k);
      return 1;
    }
    ++its; ++kdefl; ++*sweeps;
    zc sigma;
    if (kdefl % (2 * kPeriod) == 0) {
      zc d = HT(i, i);
      sigma = z(d.re + kWeight * zabs1(HT(i, i - 1)), d.im);
    } else if (kdefl % kPeriod == 0) {
      zc d = HT(lo, lo);
      sigma = z(d.re + kWeight * zabs1(HT(lo + 1, lo)), d.im);
    } else {
      sigma = wilkinson(HT(i - 1, i - 1), HT(i - 1, i), HT(i, i - 1), HT(i, i));
      if (est && its == 1) {
        int k = nearest(est, n, used, sigma);
        if (k >= 0) sigma = z(est[2 * k], est[2 * k + 1]);
      }
    }
    for (int j = lo; j < i; ++j) {
      zc x, y, r, s;
      double c;
      if (j == lo) { x = zsub(HT(lo, lo), sigma); y = HT(lo + 1, lo); }
      else { x = HT(j, j - 1); y = HT(j + 1, j - 1); }
      make_rot(x, y, &c, &s, &r);
      *work += (i - j + 1) + ((j + 2 < i ? j + 2 : i) - lo + 1);
      if (c == 0.0) {
        /* exact swap-like rotation: apply it the plain way (rare) */
        for (int col = j; col <= i; ++col) {
          zc p = HT(j, col), q = HT(j + 1, col);
          H(j, col) = zscale(zmul(s, q), dr[j] / dc[col]);
          H(j + 1, col) = zscale(zsub(z(0.0, 0.0), zmul(zconj(s), p)), dr[j + 1] / dc[col]);
        }
      } else {
        /* left: rows j, j+1 with dr' = dr / c: k_j += alpha k_{j+1}, k_{j+1} += beta k_j */
        zc alpha = zscale(s, dr[j] / (c * dr[j + 1]));
        zc beta = zscale(zconj(s), -dr[j + 1] / (c * dr[j]));
        for (int col = j; col <= i; ++col) {
          zc p = H(j, col), q = H(j + 1, col);
          H(j, col) = zadd(p, zmul(alpha, q));
          H(j + 1, col) = zadd(q, zmul(beta, p));
        }
        dr[j] /= c;
        dr[j + 1] /= c;
      }
      if (j > lo) {
        H(j, j - 1) = zscale(r, dr[j] / dc[j - 1]);
        H(j + 1, j - 1) = z(0.0, 0.0);
      }
      int qend = j + 2 < i ? j + 2 : i;
      if (c == 0.0) {
        for (int row = lo; row <= qend; ++row) {
          zc p = HT(row, j), q = HT(row, j + 1);
          H(row, j) = zscale(zmul(zconj(s), q), dr[row] / dc[j]);
          H(row, j + 1) = zscale(zsub(z(0.0, 0.0), zmul(s, p)), dr[row] / dc[j + 1]);
        }
      } else {
        /* right: columns j, j+1 with dc' = dc * c: k_j += gamma k_{j+1}, k_{j+1} += delta k_j */
        zc gamma = zscale(zconj(s), dc[j + 1] / (c * dc[j]));
        zc delta = zscale(s, -dc[j] / (c * dc[j + 1]));
        for (int row = lo; row <= qend; ++row) {
          zc p = H(row, j), q = H(row, j + 1);
          H(row, j) = zadd(p, zmul(gamma, q));
          H(row, j + 1) = zadd(q, zmul(delta, p));
        }
        dc[j] *= c;
        dc[j + 1] *= c;
      }
      for (int k = j; k <= j + 1; ++k) {
        if (dr[k] > big) rescale_row(n, a, dr, k, rescales);
        if (dc[k] < small) rescale_col(n, a, dc, k, rescales);
      }
    }
  }
}

#undef HT

/* Batch driver: A and w as in the oracle (column-major buffers, w[j*n + i]);
 * est: NULL or 2n floats per matrix; flag and sweeps per matrix. */
void model_zgeev_batched_opts(int n, int batch, const double* A, double* w, const float* est, const double* lam,
                              double tol, int* flag, long* sweeps, long long* work, int options, int* trace,
                              long trace_cap, long long* rescales) {
  zc* a = malloc(sizeof(zc) * (size_t)n * n);
  zc* v = malloc(sizeof(zc) * (size_t)n);
  unsigned char* used = malloc((size_t)n);
  for (int j = 0; j < batch; ++j) {
    const double* src = A + (size_t)j * 2 * n * n;
    for (size_t e = 0; e < (size_t)n * n; ++e) a[e] = z(src[2 * e], src[2 * e + 1]);
    if (options & 8)
      hessenberg_elementary(n, a);
    else
      hessenberg(n, a, v);
    sweeps[j] = 0;
    work[j] = 0;
    if (rescales) rescales[j] = 0;
    if (options & 4) {
      long long dummy = 0;
      flag[j] = qr_scaled(n, a, (zc*)(w + (size_t)j * 2 * n), est ? est + (size_t)j * 2 * n : NULL, used,
                          &sweeps[j], &work[j], rescales ? &rescales[j] : &dummy);
    } else {
      flag[j] = qr(n, a, (zc*)(w + (size_t)j * 2 * n), est ? est + (size_t)j * 2 * n : NULL,
                   lam ? lam + (size_t)j * 2 * n : NULL, tol, used, &sweeps[j], &work[j], options,
                   trace ? trace + (size_t)j * trace_cap : NULL, trace_cap);
    }
  }
  free(a);
  free(v);
  free(used);
}

void model_zgeev_batched(int n, int batch, const double* A, double* w, const float* est, int* flag, long* sweeps) {
  long long* work = malloc(sizeof(long long) * (size_t)(batch > 0 ? batch : 1));
  model_zgeev_batched_opts(n, batch, A, w, est, NULL, kUlp, flag, sweeps, work, 0, NULL, 0, NULL);
  free(work);
}
