/*
 * TEST INFRASTRUCTURE — CPU model of this library's eigenvalue iteration.
 * Never linked into or called by the product library.
 *
 * Serial, one matrix at a time, column-major storage a[c*n + r], no
 * pre-scaling (inputs of moderate size). It restates the mathematics of the
 * GPU path (tokura_zgeev_batched_gb300/csrc/zgeev_lane.cuh: hessenberg,
 * negligible_subdiag, nearest_estimate, qr_eigenvalues; zgeev_device.cuh:
 * make_rot, wilkinson_shift) without its lane layout, so that tests can count
 * sweeps per eigenvalue with and without shift hints and compare eigenvalues
 * and flags with LAPACK. The reference's own algorithm is restated separately
 * (ref_algorithm.c).
 */
#include <math.h>
#include <stdlib.h>

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
static zc zsqrt(zc v) {
  double m = hypot(v.re, v.im);
  if (m == 0.0) return z(0.0, 0.0);
  double t = sqrt(0.5 * (m + fabs(v.re)));
  double h = v.im / (2.0 * t);
  return v.re >= 0.0 ? z(t, h) : z(fabs(h), copysign(t, v.im));
}

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

/* Ahues-Tisseur deflation test of subdiagonal entry k of the block [lo, hi]. */
static int negligible(int n, const zc* a, int k, int lo, int hi, double smlnum) {
  zc hk = H(k, k - 1);
  double h1 = zabs1(hk);
  if (h1 <= smlnum) return 1;
  zc dkk = H(k, k), dk1 = H(k - 1, k - 1);
  double tst = zabs1(dk1) + zabs1(dkk);
  if (tst == 0.0) {
    if (k - 2 >= lo) tst += zabs1(H(k - 1, k - 2));
    if (k + 1 <= hi) tst += zabs1(H(k + 1, k));
  }
  if (h1 > kUlp * tst) return 0;
  double hu = zabs1(H(k - 1, k));
  double ab = fmax(h1, hu), ba = fmin(h1, hu);
  double dd = zabs1(zsub(dk1, dkk)), d1 = zabs1(dkk);
  double aa = fmax(d1, dd), bb = fmin(d1, dd), s = aa + ab;
  return ba * (ab / s) <= fmax(smlnum, kUlp * (bb * (aa / s)));
}

/* Eigenvalue of [[a, b], [c, d]] nearer to d, in a scaled form. */
static zc wilkinson(zc a, zc b, zc c, zc d) {
  zc bc = zmul(b, c);
  if (bc.re == 0.0 && bc.im == 0.0) return d;
  zc x = zscale(zsub(a, d), 0.5);
  double sc = fmax(zabs1(x), sqrt(zabs1(bc)));
  zc xs = zscale(x, 1.0 / sc), bcs = zscale(bc, 1.0 / (sc * sc));
  zc y = zsqrt(zadd(zmul(xs, xs), bcs));
  if (xs.re * y.re + xs.im * y.im < 0.0) y = z(-y.re, -y.im);
  zc den = zadd(xs, y);
  if (den.re == 0.0 && den.im == 0.0) return d;
  return zsub(d, zscale(zdiv(bcs, den), sc));
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
 * is the shift of the first sweep after each deflation. Returns the flag (0
 * converged, 1 sweep cap hit) and adds the sweeps made to *sweeps. */
static int qr(int n, zc* a, zc* w, const float* est, unsigned char* used, long* sweeps) {
  double smlnum = kSafeMin * ((double)n / kUlp);
  int itmax = 30 * (n > 10 ? n : 10);
  int i = n - 1, lo = 0, its = 0, kdefl = 0;
  for (int k = 0; k < n; ++k) used[k] = 0;
  for (;;) {
    for (;;) {
      int hit = lo;
      for (int k = i; k > lo; --k)
        if (negligible(n, a, k, lo, i, smlnum)) { hit = k; break; }
      lo = hit;
      if (lo < i) break;
      w[i] = H(i, i);
      if (est) {
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
    ++its; ++kdefl; ++*sweeps;
    zc sigma;
    if (kdefl % (2 * kPeriod) == 0) {
      sigma = z(H(i, i).re + kWeight * zabs1(H(i, i - 1)), H(i, i).im);
    } else if (kdefl % kPeriod == 0) {
      sigma = z(H(lo, lo).re + kWeight * zabs1(H(lo + 1, lo)), H(lo, lo).im);
    } else {
      sigma = wilkinson(H(i - 1, i - 1), H(i - 1, i), H(i, i - 1), H(i, i));
      if (est && its == 1) {
        int k = nearest(est, n, used, sigma);
        if (k >= 0) sigma = z(est[2 * k], est[2 * k + 1]);
      }
    }
    for (int j = lo; j < i; ++j) {
      zc x, y, r, s;
      double c;
      if (j == lo) { x = zsub(H(lo, lo), sigma); y = H(lo + 1, lo); }
      else { x = H(j, j - 1); y = H(j + 1, j - 1); }
      make_rot(x, y, &c, &s, &r);
      if (j > lo) { H(j, j - 1) = r; H(j + 1, j - 1) = z(0.0, 0.0); }
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

/* Batch driver: A and w as in the oracle (column-major buffers, w[j*n + i]);
 * est: NULL or 2n floats per matrix; flag and sweeps per matrix. */
void model_zgeev_batched(int n, int batch, const double* A, double* w, const float* est, int* flag, long* sweeps) {
  zc* a = malloc(sizeof(zc) * (size_t)n * n);
  zc* v = malloc(sizeof(zc) * (size_t)n);
  unsigned char* used = malloc((size_t)n);
  for (int j = 0; j < batch; ++j) {
    const double* src = A + (size_t)j * 2 * n * n;
    for (size_t e = 0; e < (size_t)n * n; ++e) a[e] = z(src[2 * e], src[2 * e + 1]);
    hessenberg(n, a, v);
    sweeps[j] = 0;
    flag[j] = qr(n, a, (zc*)(w + (size_t)j * 2 * n), est ? est + (size_t)j * 2 * n : NULL, used, &sweeps[j]);
  }
  free(a);
  free(v);
  free(used);
}
