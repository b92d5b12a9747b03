// Device building blocks of the batched eigenvalue-only ZGEEV path for sm_103a.
//
// Execution model (GB300): FP64 runs at ~2 lane-FMAs per clock per SM and a
// warp instruction costs the same whether 1 or 32 lanes are active. The
// kernels therefore give every matrix to a small "lane group" of L = 1, 2, 4
// or 8 lanes of one warp (32/L matrices per warp), so that all 32 lanes do
// useful FP64 work, and they keep FP64 instruction count minimal:
//   * Householder Hessenberg reduction with v[0] = 1 and a real tau
//     (replaces tokura_zgehrd_MWB_kernel.cuh:51-287 of the reference),
//   * single-shift complex QR with complex Givens rotations (12 FP64 ops per
//     element pair), Wilkinson shifts (or FP32 estimates as first shifts,
//     zgeev_estimate.cuh), ad hoc shifts and the Ahues-Tisseur deflation
//     test (replaces tokura_zhseqr_MWB_kernel.cuh:221-791).
//
// Data layout: each warp owns one "tile" of up to 32/L matrices, staged
// from the caller's column-major A into the caller's workspace in
// tile-interleaved order: element (r, c) of matrix slot t of a tile of
// width tw sits at tile[(c*n + r)*tw + t]. A warp load of the same element
// of all its matrices is one contiguous 16*tw-byte segment.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "zgeev_debug.cuh"

namespace tzg {

constexpr int kMaxN = 64;
// LAPACK-style constants (double precision): ulp = 2^-52, safe minimum = 2^-1022.
constexpr double kUlp = 2.220446049250313080847e-16;
constexpr double kSafeMin = 2.225073858507201383090e-308;
// Ad hoc shift period and weight (single-shift QR practice, LAPACK zlahqr).
constexpr int kExceptionalPeriod = 10;
constexpr double kExceptionalWeight = 0.75;

__device__ __forceinline__ double cabs1(double2 z) { return fabs(z.x) + fabs(z.y); }

// Tests on FP64 values done with integer instructions. The FP64 pipe is the
// bottleneck of every solver here (about 2 FP64 lane-instructions per SM per
// clock on this GPU), and a floating-point comparison occupies it like an
// FMA; the integer pipe is idle by comparison. Zero tests ignore the sign bit
// (-0.0 counts as zero). For non-negative doubles (+0.0 up to +inf) the order
// of the values is the order of their bit patterns read as signed 64-bit
// integers; -0.0 reads as negative, below every non-negative value, as a
// "less than" wants.
__device__ __forceinline__ bool is_zero(double2 z) {
  const unsigned long long bits =
      (unsigned long long)__double_as_longlong(z.x) | (unsigned long long)__double_as_longlong(z.y);
  return (bits << 1) == 0;
}
__device__ __forceinline__ bool is_zero(double x) { return ((unsigned long long)__double_as_longlong(x) << 1) == 0; }
__device__ __forceinline__ bool nonneg_lt(double a, double b) { return __double_as_longlong(a) < __double_as_longlong(b); }
__device__ __forceinline__ bool nonneg_le(double a, double b) {
  return __double_as_longlong(a) <= __double_as_longlong(b);
}
__device__ __forceinline__ double2 cadd(double2 a, double2 b) { return make_double2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ double2 csub(double2 a, double2 b) { return make_double2(a.x - b.x, a.y - b.y); }
__device__ __forceinline__ double2 cmul(double2 a, double2 b) {
  return make_double2(fma(a.x, b.x, -a.y * b.y), fma(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ double2 cscale(double2 a, double s) { return make_double2(a.x * s, a.y * s); }

// Biased exponent field of |x| (0 for zero/denormal, 2047 for inf/nan).
__device__ __forceinline__ int dexp_field(double x) {
  return (__double2hiint(x) >> 20) & 0x7ff;
}
// 2^e as a double for e in the normal range.
__device__ __forceinline__ double pow2(int e) { return __hiloint2double((e + 1023) << 20, 0); }

// Compile-time lane count tag (for dispatch from a runtime lane width).
template <int L>
struct Lanes {
  static constexpr int value = L;
};

// Lane group of L consecutive lanes of one warp cooperating on one matrix.
template <int L>
struct Group {
  unsigned mask;
  int rank;
  __device__ __forceinline__ Group() {
    const int lane = threadIdx.x & 31;
    rank = lane & (L - 1);
    mask = (L == 32) ? 0xffffffffu : (((1u << L) - 1u) << (lane & ~(L - 1)));
  }
  __device__ __forceinline__ void sync() const {
    if (L > 1) __syncwarp(mask);
  }
  // Butterfly reductions: every lane ends with the bitwise-identical value.
  __device__ __forceinline__ double sum(double v) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v += __shfl_xor_sync(mask, v, o);
    return v;
  }
  __device__ __forceinline__ int imax(int v) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(mask, v, o));
    return v;
  }
  __device__ __forceinline__ int ior(int v) const {
#pragma unroll
    for (int o = L / 2; o > 0; o >>= 1) v |= __shfl_xor_sync(mask, v, o);
    return v;
  }
};

// View of one matrix inside an interleaved tile: element (r, c) at p[(c*n + r)*rs].
struct MatView {
  double2* p;
  int n;
  int rs;  // stride between consecutive rows (= tile width)
  __device__ __forceinline__ double2* at(int r, int c) const {
#ifdef TOKURA_DEBUG_BOUNDS
    if (dbg_out(r, c, n)) return p;
#endif
    return p + (c * n + r) * rs;
  }
  // Start of a strided run that may be empty (not checked: a run is checked by
  // TZG_DBG_RUN on its first and last elements when it has any).
  __device__ __forceinline__ double2* ptr(int r, int c) const { return p + (c * n + r) * rs; }
};

// Complex Givens rotation G = [c s; -conj(s) c] (c real) with G * [x; y] = [rr; 0].
// The matrix is pre-scaled so |x|,|y| <= ~2^7; if |x|^2 * (|x|^2+|y|^2) underflows
// then x is below 2^-250 relative to the matrix and is treated as zero.
struct Rot {
  double c;
  double2 s;
};
__device__ __forceinline__ Rot make_rot(double2 x, double2 y, double2& rr) {
  Rot g;
  const double p = fma(x.x, x.x, x.y * x.y);
  const double q = fma(y.x, y.x, y.y * y.y);
  const double nn = p + q;
  const double pn = p * nn;
  if (is_zero(q)) {  // nothing to annihilate (also covers x = y = 0)
    g.c = 1.0;
    g.s = make_double2(0.0, 0.0);
    rr = x;
  } else if (nonneg_lt(pn, 1e-290)) {  // x negligible: swap-like rotation
    const double rq = rsqrt(q);
    g.c = 0.0;
    g.s = make_double2(y.x * rq, -y.y * rq);  // conj(y)/|y|
    rr = make_double2(q * rq, 0.0);          // |y|
  } else {
    const double R = rsqrt(pn);  // 1/(|x| * N)
    g.c = p * R;                 // |x| / N
    // s = x * conj(y) * R
    const double2 xy = make_double2(fma(x.x, y.x, x.y * y.y), fma(x.y, y.x, -x.x * y.y));
    g.s = make_double2(xy.x * R, xy.y * R);
    const double f = nn * R;  // N / |x|
    rr = make_double2(x.x * f, x.y * f);
  }
  return g;
}

// Left application to a row pair: [a; b] <- G [a; b].
__device__ __forceinline__ void rot_left(const Rot& g, double2& a, double2& b) {
  const double2 a0 = a, b0 = b;
  a.x = fma(g.c, a0.x, fma(g.s.x, b0.x, -g.s.y * b0.y));
  a.y = fma(g.c, a0.y, fma(g.s.x, b0.y, g.s.y * b0.x));
  b.x = fma(g.c, b0.x, -fma(g.s.x, a0.x, g.s.y * a0.y));
  b.y = fma(g.c, b0.y, -fma(g.s.x, a0.y, -g.s.y * a0.x));
}
// Right application to a column pair: [a b] <- [a b] G^H.
__device__ __forceinline__ void rot_right(const Rot& g, double2& a, double2& b) {
  const double2 a0 = a, b0 = b;
  // a' = c a + conj(s) b ; b' = c b - s a
  a.x = fma(g.c, a0.x, fma(g.s.x, b0.x, g.s.y * b0.y));
  a.y = fma(g.c, a0.y, fma(g.s.x, b0.y, -g.s.y * b0.x));
  b.x = fma(g.c, b0.x, -fma(g.s.x, a0.x, -g.s.y * a0.y));
  b.y = fma(g.c, b0.y, -fma(g.s.x, a0.y, g.s.y * a0.x));
}

// Applies G (kRight = false: [a; b] <- G [a; b]) or G^H from the right
// (kRight = true: [a b] <- [a b] G^H) to `count` element pairs p[t*step],
// p[t*step + pair]. Pair t+1 is loaded before pair t is stored, so memory
// latency overlaps the 12 FP64 instructions of each pair.
template <bool kRight>
__device__ __forceinline__ void rotate_pairs(const Rot& g, double2* p, int count, int step, int pair) {
  if (count <= 0) return;
  double2 a = p[0], b = p[pair];
  for (int t = 1; t < count; ++t) {
    double2* pn = p + step;
    const double2 an = pn[0], bn = pn[pair];
    if (kRight) rot_right(g, a, b); else rot_left(g, a, b);
    p[0] = a;
    p[pair] = b;
    a = an;
    b = bn;
    p = pn;
  }
  if (kRight) rot_right(g, a, b); else rot_left(g, a, b);
  p[0] = a;
  p[pair] = b;
}

// Number of t >= 0 with first + t*step <= last.
__device__ __forceinline__ int strided_count(int first, int last, int step) {
  return first <= last ? (last - first) / step + 1 : 0;
}

// Eigenvalue of [a b; c d] closest to d (Wilkinson shift), in a
// cancellation-free form: d - bc / (x + sqrt(x^2 + bc)), x = (a - d)/2, with
// the root's sign chosen so that |x + sqrt(.)| is maximal (Re(conj(x) y) >= 0).
// x and bc are first scaled by an exact power of two 2^-k, k taken from the
// exponent fields, so that the larger of the scaled |x|_1, |bc|_1 lies in
// [1, 4): squaring then neither overflows nor underflows, and with the sign
// rule |x + y|^2 >= |x|^2 + |x^2 + bc| >= max(|x|^2, |bc|) >= 1/2, so the
// quotient is bc * conj(x + y) times 2^k / |x + y|^2. One square root (of
// |x^2 + bc|^2), one reciprocal square root (the principal root of
// x^2 + bc) and one division in all.
__device__ __forceinline__ double2 wilkinson_shift(double2 a, double2 b, double2 c, double2 d) {
  const double2 bc = cmul(b, c);
  if (is_zero(bc)) return d;
  const double2 x = make_double2(0.5 * (a.x - d.x), 0.5 * (a.y - d.y));
  // |x|_1 in [2^ex, 2^(ex+1)), |bc|_1 in [2^eb, 2^(eb+1)); k = max(ex, floor(eb/2)) lies in [-512, 1023].
  const int k = max(dexp_field(cabs1(x)) - 1023, (dexp_field(cabs1(bc)) - 1023) >> 1);
  const double is = pow2(-k);
  const double2 xs = cscale(x, is);
  const double2 bcs = cscale(cscale(bc, is), is);  // bc * 2^-2k in two exact steps
  const double2 zz = make_double2(fma(xs.x, xs.x, fma(-xs.y, xs.y, bcs.x)), fma(2.0 * xs.x, xs.y, bcs.y));
  // Principal square root of zz from u = (|zz| + |Re zz|)/2: sqrt(u) and Im zz / (2 sqrt(u)).
  const double u = 0.5 * (sqrt(fma(zz.x, zz.x, zz.y * zz.y)) + fabs(zz.x));
  double2 y = make_double2(0.0, 0.0);
  if (!is_zero(u)) {
    const double r = rsqrt(u);
    const double t = u * r, h = 0.5 * zz.y * r;
    // Re zz = -0.0 takes the second form, which gives the same root then.
    y = !signbit(zz.x) ? make_double2(t, h) : make_double2(fabs(h), copysign(t, zz.y));
  }
  // A zero Re(conj(x) y) of either sign leaves |x + y| the same for both roots.
  if (signbit(fma(xs.x, y.x, xs.y * y.y))) y = make_double2(-y.x, -y.y);
  const double2 den = cadd(xs, y);
  const double f = pow2(k) / fma(den.x, den.x, den.y * den.y);
  // d - (bcs conj(den) / |den|^2) * 2^k
  const double2 num = make_double2(fma(bcs.x, den.x, bcs.y * den.y), fma(bcs.y, den.x, -bcs.x * den.y));
  return make_double2(fma(-num.x, f, d.x), fma(-num.y, f, d.y));
}

}  // namespace tzg
