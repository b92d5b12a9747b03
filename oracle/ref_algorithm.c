/*
 * TEST INFRASTRUCTURE — CPU restatement of the reference's GPU algorithm.
 * Never linked into or called by the product library.
 *
 * Serial, one matrix at a time, column-major storage a[c*n + r]. Each function
 * states the reference code it follows (paths inside hirokitokura/
 * tokura_zgeev_batched). The reference's kernels interleave 32 matrices per
 * warp and split loops over threadIdx.y; those are execution details and are
 * not restated. Its numerical choices are kept, including the quirks:
 *   - deflation tests the real parts only (the imaginary test is a no-op,
 *     tokura_zhseqr_MWB_kernel.cuh:133-166);
 *   - a bulge is started at the top of every unreduced block of size >= 3 in
 *     each sweep (:221-451), with the shift taken from the block's trailing
 *     2x2 but chosen closest to the block's TOP diagonal entry (:302-309), and
 *     ad hoc shifts at iteration counts = -1 mod 47 / 25 / 20 (:278-301);
 *   - the sweep cap is n^4 (:655), and 2x2 blocks are finished by the
 *     closed-form (a + d +- sqrt((d - a)^2 + 4bc))/2 (:30-84).
 * Used to pin the reference's accuracy and flag behaviour against LAPACK.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

typedef struct { double re, im; } cplx;

static cplx cx(double r, double i) { cplx z = {r, i}; return z; }
static cplx cadd(cplx a, cplx b) { return cx(a.re + b.re, a.im + b.im); }
static cplx csub(cplx a, cplx b) { return cx(a.re - b.re, a.im - b.im); }
static cplx cmul(cplx a, cplx b) { return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re); }
static cplx cconj(cplx a) { return cx(a.re, -a.im); }
static cplx cscale(cplx a, double s) { return cx(a.re * s, a.im * s); }
static double cnorm2(cplx a) { return a.re * a.re + a.im * a.im; }

#define AT(a, n, r, c) (a)[(size_t)(c) * (n) + (r)]

/* Householder reduction to Hessenberg form with H = I - 2 v v^H, ||v|| = 1
 * (tokura_zgehrd_MWB_kernel.cuh:51-133 builds v; :159-287 applies it from the
 * left to columns r-1..n-1 and from the right to all rows). */
static void ref_zgehrd(int n, cplx* a, cplx* v) {
  for (int r = 1; r < n - 1; ++r) {
    double tail = 0.0; /* sum of |x_i|^2 below the first element */
    for (int i = r + 1; i < n; ++i) tail += cnorm2(AT(a, n, i, r - 1));
    if (tail == 0.0) continue; /* the reference's vector becomes zero: identity */
    cplx x0 = AT(a, n, r, r - 1);
    double xnorm = sqrt(cnorm2(x0) + tail);
    double ax0 = sqrt(cnorm2(x0));
    double f = ax0 > 0.0 ? xnorm / ax0 : 0.0; /* compute_alpha: NaN/Inf scale -> 0 */
    cplx alpha = cx(-f * x0.re, -f * x0.im);
    v[r] = csub(x0, alpha);
    double vn = sqrt(cnorm2(v[r]) + tail);
    double inv = (vn + 1.0 == 1.0) ? 0.0 : 1.0 / vn;
    v[r] = cscale(v[r], inv);
    for (int i = r + 1; i < n; ++i) v[i] = cscale(AT(a, n, i, r - 1), inv);
    for (int c = r - 1; c < n; ++c) {
      cplx w = cx(0, 0);
      for (int i = r; i < n; ++i) w = cadd(w, cmul(cconj(v[i]), AT(a, n, i, c)));
      w = cscale(w, 2.0);
      for (int i = n - 1; i >= r; --i) AT(a, n, i, c) = csub(AT(a, n, i, c), cmul(v[i], w));
    }
    for (int q = 0; q < n; ++q) {
      cplx w = cx(0, 0);
      for (int j = r; j < n; ++j) w = cadd(w, cmul(AT(a, n, q, j), v[j]));
      w = cscale(w, 2.0);
      for (int j = n - 1; j >= r; --j) AT(a, n, q, j) = csub(AT(a, n, q, j), cmul(w, cconj(v[j])));
    }
  }
}

/* Closed-form eigenvalues of the 2x2 block at (k, k) (tokura_zhseqr_MWB_kernel.cuh:30-84). */
static void ref_eig22(int n, const cplx* a, int k, cplx* e0, cplx* e1) {
  cplx a00 = AT(a, n, k, k), a11 = AT(a, n, k + 1, k + 1);
  cplx a10 = AT(a, n, k + 1, k), a01 = AT(a, n, k, k + 1);
  cplx d = csub(a11, a00);
  cplx in = cadd(cmul(d, d), cscale(cmul(a10, a01), 4.0));
  double m = sqrt(in.re * in.re + in.im * in.im);
  cplx root = cx(sqrt(0.5 * (in.re + m)), sqrt(0.5 * (-in.re + m)));
  if (in.im < 0.0) root.im = -root.im;
  cplx s = cadd(a11, a00);
  *e1 = cscale(cadd(s, root), 0.5);
  *e0 = cscale(csub(s, root), 0.5);
}

/* Real-part-only negligibility test (tokura_zhseqr_MWB_kernel.cuh:133-166). */
static int ref_ignore(cplx h, cplx s) {
  double t = s.re == 0.0 ? 1.0 : s.re;
  return fabs(h.re) + fabs(t) == fabs(t);
}

/* Applies the 2-vector reflector I - tau v v^H to rows (p, p+1) for columns
 * c0..c1-1 and to columns (p, p+1) for rows r0..r1-1. */
static void ref_reflect(int n, cplx* a, int p, cplx v0, cplx v1, double tau, int c0, int c1, int r0, int r1) {
  for (int c = c0; c < c1; ++c) {
    cplx w = cadd(cmul(cconj(v0), AT(a, n, p, c)), cmul(cconj(v1), AT(a, n, p + 1, c)));
    w = cscale(w, tau);
    AT(a, n, p + 1, c) = csub(AT(a, n, p + 1, c), cmul(v1, w));
    AT(a, n, p, c) = csub(AT(a, n, p, c), cmul(v0, w));
  }
  for (int q = r0; q < r1; ++q) {
    cplx w = cadd(cmul(AT(a, n, q, p), v0), cmul(AT(a, n, q, p + 1), v1));
    w = cscale(w, tau);
    AT(a, n, q, p + 1) = csub(AT(a, n, q, p + 1), cmul(w, cconj(v1)));
    AT(a, n, q, p) = csub(AT(a, n, q, p), cmul(w, cconj(v0)));
  }
}

/* Next entry of zero_index at or after i that is non-zero (block end). */
static int block_end(const int* zi, int n, int i) {
  for (; i < n + 1; ++i)
    if (zi[i] != 0) return zi[i];
  return n;
}

/* Single-shift QR on the Hessenberg matrix (tokura_zhseqr_MWB_kernel.cuh:611-791).
 * Returns the flag (0 converged, 1 sweep cap n^4 reached), writes w[i] and the
 * number of passes of the kernel's sweep loop (its counter `its`, :654-657) to
 * *its_out. */
static int ref_zhseqr(int n, cplx* a, cplx* w, long long* its_out) {
  int* zi = (int*)calloc((size_t)n + 1, sizeof(int));
  zi[n] = n;
  long long cap = (long long)n * n * n * n, its = 0;
  int prev_done = 0, iteration = 0;
  while (its != cap) {
    ++its;
    for (int i = 2; i < n; ++i) AT(a, n, i, i - 2) = cx(0, 0);
    for (int d = n - 1; d > 0; --d) {
      if (zi[d] != 0) continue;
      cplx hd = AT(a, n, d, d), hp = AT(a, n, d - 1, d - 1);
      cplx s = cx(0.5 * (fabs(hd.re) + fabs(hp.re)), 0.5 * (fabs(hd.im) + fabs(hp.im)));
      if (ref_ignore(AT(a, n, d, d - 1), s)) zi[d] = d;
    }
    int done = 0, prev = n;
    for (int d = n - 1; d > 0; --d) {
      if (zi[d] != 0) {
        AT(a, n, d, d - 1) = cx(0, 0);
        if (prev - d < 3) done += prev - d;
        prev = d;
      }
    }
    if (prev < 3) done += prev;
    if (done == n) break;
    ++iteration;
    if (prev_done != done) iteration = 0;
    prev_done = done;
    /* bulge generation at every block start (:221-451) */
    for (int d = 0; d + 2 < n; ++d) {
      int start = ((zi[d] != 0) || d == 0) && zi[d + 1] == 0 && zi[d + 2] == 0;
      if (!start) continue;
      int sub = block_end(zi, n, d + 3);
      cplx tau;
      if ((iteration + 1) % 47 == 0) {
        tau = cx(0, 0);
      } else if ((iteration + 1) % 25 == 0 || (iteration + 1) % 20 != 0) {
        cplx e0, e1;
        ref_eig22(n, a, sub - 2, &e0, &e1);
        cplx top = AT(a, n, d, d);
        double n0 = cnorm2(csub(top, e0)), n1 = cnorm2(csub(top, e1));
        if ((iteration + 1) % 25 == 0)
          tau = n0 < n1 ? e1 : e0;
        else
          tau = n0 < n1 ? e0 : e1;
      } else {
        tau = cx(-AT(a, n, d, d).re, -AT(a, n, d, d).im);
      }
      if (sqrt(cnorm2(AT(a, n, d + 1, d))) == 0.0) continue;
      cplx v0 = csub(AT(a, n, d, d), tau), v1 = AT(a, n, d + 1, d);
      double vn = sqrt(cnorm2(v0) + cnorm2(v1));
      double av0 = sqrt(cnorm2(v0));
      double f = vn / av0;
      v0 = csub(v0, cx(-f * v0.re, -f * v0.im));
      double half = 0.5 * (cnorm2(v0) + cnorm2(v1));
      if (half + 1.0 == 1.0) continue;
      double t = 1.0 / half;
      if (isnan(half) || isnan(t) || isnan(v0.re) || isnan(v1.im) || isinf(t) || isinf(v0.re) || isinf(v1.im))
        continue;
      int mmin = sub < d + 4 ? sub : d + 4;
      ref_reflect(n, a, d, v0, v1, t, d, sub, d, mmin);
    }
    /* bulge chasing (:454-609) */
    int startd = 0;
    for (int d = 0; d + 2 < n; ++d) {
      if (zi[d + 1] != 0)
        startd = d + 1;
      else if (zi[d + 2] != 0)
        startd = d + 2;
      if (!(zi[d + 1] == 0 && zi[d + 2] == 0)) continue;
      int sub = block_end(zi, n, d + 3);
      cplx v0 = AT(a, n, d + 1, d), v1 = AT(a, n, d + 2, d);
      double vn = sqrt(cnorm2(v0) + cnorm2(v1));
      double av0 = sqrt(cnorm2(v0));
      double f = vn / av0;
      v0 = csub(v0, cx(-f * v0.re, -f * v0.im));
      double nrm = cnorm2(v0) + cnorm2(v1);
      if (nrm == 0.0) continue;
      double t = 2.0 / nrm;
      if (isnan(t) || isnan(v0.re) || isnan(v1.im) || isinf(t) || isinf(v0.re) || isinf(v1.im)) continue;
      int mmin = sub < d + 5 ? sub : d + 5;
      ref_reflect(n, a, d + 1, v0, v1, t, d, sub, startd, mmin);
    }
  }
  int flag = (its == cap) ? 1 : 0;
  *its_out = its;
  for (int s = n - 1; s >= 0;) {
    if (zi[s] != 0 || s == 0) {
      w[s] = AT(a, n, s, s);
      s -= 1;
    } else {
      cplx e0, e1;
      ref_eig22(n, a, s - 1, &e0, &e1);
      w[s] = e1;
      w[s - 1] = e0;
      s -= 2;
    }
  }
  free(zi);
  return flag;
}

/* Reference algorithm on `batch` column-major matrices (A is copied, not
 * modified); sweeps (may be NULL): passes of the sweep loop per matrix. */
int ref_zgeev_batched_sweeps(int n, int batch, const double* A, double* w, int* flag, long long* sweeps) {
  cplx* a = (cplx*)malloc(sizeof(cplx) * (size_t)n * n);
  cplx* v = (cplx*)malloc(sizeof(cplx) * (size_t)n);
  if (!a || !v) {
    free(a);
    free(v);
    return -1;
  }
  for (int k = 0; k < batch; ++k) {
    memcpy(a, A + (size_t)k * n * n * 2, sizeof(cplx) * (size_t)n * n);
    ref_zgehrd(n, a, v);
    long long its = 0;
    flag[k] = ref_zhseqr(n, a, (cplx*)(w + (size_t)k * n * 2), &its);
    if (sweeps) sweeps[k] = its;
  }
  free(a);
  free(v);
  return 0;
}

int ref_zgeev_batched(int n, int batch, const double* A, double* w, int* flag) {
  return ref_zgeev_batched_sweeps(n, batch, A, w, flag, NULL);
}
