// Single-precision eigenvalue estimates used as shift hints by the FP64 QR.
//
// GB300 runs FP32 about 60x faster than FP64, so a complete FP32 eigenvalue
// computation costs a few percent of the FP64 one. Its eigenvalues (relative
// accuracy ~1e-6, set by FP32's backward error) are handed to the FP64 QR,
// which uses the nearest unused estimate as the shift of the first sweep after
// each deflation: that sweep brings the bottom subdiagonal down by about the
// estimate's error and one or two Wilkinson sweeps finish the eigenvalue,
// ~2.65 sweeps per eigenvalue instead of ~3.37 with Wilkinson shifts alone
// (CPU model of both iterations, oracle/model_qr.c, complex Gaussian, n = 64). The estimates only
// steer the iteration; the FP64 result and its accuracy come from the FP64
// QR as before, and a bad or missing estimate costs at most one sweep.
//
// Shape: one warp per matrix, the matrix in shared memory (column-major,
// leading dimension n + 1), all 32 lanes splitting each column/row update,
// decisions taken from warp-uniform values. The estimates are stored in the
// scale of the FP64 kernel's staged matrix (see stage_and_scale).
#pragma once

#include "zgeev_lane.cuh"

namespace tzg {

constexpr float kUlpF = 5.9604644775390625e-08f;     // 2^-24
constexpr float kSafeMinF = 1.1754943508222875e-38f;  // 2^-126
constexpr int kEstimateSweepCap = 30;                 // per eigenvalue; estimates only
// Deflation threshold of the FP32 QR, relative like the FP64 one: 1e-5
// instead of FP32's ulp (6e-8). A subdiagonal entry of that size moves the
// eigenvalues by about its square for separated ones, below the FP32 noise
// of the estimates (~7e-7 relative), and stopping there saves the last,
// noise-limited sweeps (CPU model oracle/model_qr.c at n = 64: 2.62 -> 2.31 FP32
// sweeps per eigenvalue, while the FP64 QR it steers needs 2.61 -> 2.65).
constexpr float kEstimateTol = 1e-5f;

__device__ __forceinline__ float cabs1f(float2 z) { return fabsf(z.x) + fabsf(z.y); }
__device__ __forceinline__ float2 cmulf(float2 a, float2 b) {
  return make_float2(fmaf(a.x, b.x, -a.y * b.y), fmaf(a.x, b.y, a.y * b.x));
}
__device__ __forceinline__ float2 csubf(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// 2^e as a float for e in [-126, 127].
__device__ __forceinline__ float pow2f(int e) { return __int_as_float((e + 127) << 23); }

__device__ __forceinline__ float warp_sumf(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Eigenvalue of [a b; c d] nearest d (Wilkinson), scaled like wilkinson_shift.
__device__ __forceinline__ float2 wilkinson_shift_f(float2 a, float2 b, float2 c, float2 d) {
  const float2 bc = cmulf(b, c);
  if (bc.x == 0.0f && bc.y == 0.0f) return d;
  const float2 x = make_float2(0.5f * (a.x - d.x), 0.5f * (a.y - d.y));
  const float sc = fmaxf(cabs1f(x), sqrtf(cabs1f(bc)));
  if (!(sc > 0.0f) || !(sc < 3.0e38f)) return d;
  const float is = 1.0f / sc;
  const float2 xs = make_float2(x.x * is, x.y * is);
  const float2 bcs = make_float2(bc.x * is * is, bc.y * is * is);
  const float2 z = make_float2(fmaf(xs.x, xs.x, -xs.y * xs.y) + bcs.x, 2.0f * xs.x * xs.y + bcs.y);
  const float m = hypotf(z.x, z.y);
  float2 y = make_float2(0.0f, 0.0f);
  if (m > 0.0f) {
    const float t = sqrtf(0.5f * (m + fabsf(z.x)));
    const float h = z.y / (2.0f * t);
    y = z.x >= 0.0f ? make_float2(t, h) : make_float2(fabsf(h), copysignf(t, z.y));
  }
  if (xs.x * y.x + xs.y * y.y < 0.0f) y = make_float2(-y.x, -y.y);
  const float2 den = make_float2(xs.x + y.x, xs.y + y.y);
  const float dd = fmaf(den.x, den.x, den.y * den.y);
  if (!(dd > 0.0f)) return d;
  // corr = bcs / den
  const float2 corr = make_float2(fmaf(bcs.x, den.x, bcs.y * den.y) / dd, fmaf(bcs.y, den.x, -bcs.x * den.y) / dd);
  return make_float2(d.x - corr.x * sc, d.y - corr.y * sc);
}

struct RotF {
  float c;
  float2 s;
};

// G = [c s; -conj(s) c] with G [x; y] = [rr; 0].
__device__ __forceinline__ RotF make_rot_f(float2 x, float2 y, float2& rr) {
  RotF g;
  const float p = fmaf(x.x, x.x, x.y * x.y);
  const float q = fmaf(y.x, y.x, y.y * y.y);
  const float nn = p + q;
  const float pn = p * nn;
  if (q == 0.0f) {
    g.c = 1.0f;
    g.s = make_float2(0.0f, 0.0f);
    rr = x;
  } else if (pn < 1e-30f) {
    const float rq = rsqrtf(q);
    g.c = 0.0f;
    g.s = make_float2(y.x * rq, -y.y * rq);
    rr = make_float2(q * rq, 0.0f);
  } else {
    const float R = rsqrtf(pn);
    g.c = p * R;
    const float2 xy = make_float2(fmaf(x.x, y.x, x.y * y.y), fmaf(x.y, y.x, -x.x * y.y));
    g.s = make_float2(xy.x * R, xy.y * R);
    const float f = nn * R;
    rr = make_float2(x.x * f, x.y * f);
  }
  return g;
}

// Shared-memory view: (r, c) at p[c*ld + r].
struct SMat {
  float2* p;
  int n;
  int ld;
  __device__ __forceinline__ float2* at(int r, int c) const {
#ifdef TOKURA_DEBUG_BOUNDS
    if (dbg_out(r, c, n)) return p;
#endif
    return p + c * ld + r;
  }
};

__device__ __forceinline__ bool negligible_f(const SMat& S, int k, int lo, int hi, float smlnum) {
  const float h1 = cabs1f(*S.at(k, k - 1));
  if (h1 <= smlnum) return true;
  const float2 dkk = *S.at(k, k), dk1 = *S.at(k - 1, k - 1);
  float tst = cabs1f(dk1) + cabs1f(dkk);
  if (tst == 0.0f) {
    if (k - 2 >= lo) tst += cabs1f(*S.at(k - 1, k - 2));
    if (k + 1 <= hi) tst += cabs1f(*S.at(k + 1, k));
  }
  if (h1 > kEstimateTol * tst) return false;
  const float hu = cabs1f(*S.at(k - 1, k));
  const float ab = fmaxf(h1, hu), ba = fminf(h1, hu);
  const float dd = cabs1f(csubf(dk1, dkk)), d1 = cabs1f(dkk);
  const float aa = fmaxf(d1, dd), bb = fminf(d1, dd);
  const float s = aa + ab;
  return ba * (ab / s) <= fmaxf(smlnum, kEstimateTol * (bb * (aa / s)));
}

// Householder Hessenberg reduction of S by the whole warp (reflector data
// stays below the subdiagonal and is never read by the QR below).
__device__ __forceinline__ void hessenberg_f(const SMat& S, int lane) {
  const int n = S.n;
  const int ld = S.ld;
  for (int r = 0; r + 2 < n; ++r) {
    const int m = n - r - 1;
    float2* x = S.at(r + 1, r);
    float s2 = 0.0f;
    for (int i = 1 + lane; i < m; i += 32) s2 = fmaf(x[i].x, x[i].x, fmaf(x[i].y, x[i].y, s2));
    s2 = warp_sumf(s2);
    if (s2 == 0.0f) continue;
    const float2 x0 = x[0];
    const float a0sq = fmaf(x0.x, x0.x, x0.y * x0.y);
    const float tot = a0sq + s2;
    const float rxn = rsqrtf(tot);
    const float xn = tot * rxn;
    float tau;
    float2 cg, alpha;
    if (a0sq > 0.0f) {
      const float ra0 = rsqrtf(a0sq);
      const float d = a0sq * ra0 + xn;
      const float ig = ra0 / d;
      cg = make_float2(x0.x * ig, -x0.y * ig);
      const float f = -xn * ra0;
      alpha = make_float2(x0.x * f, x0.y * f);
      tau = d * rxn;
    } else {
      cg = make_float2(rxn, 0.0f);
      alpha = make_float2(-xn, 0.0f);
      tau = 1.0f;
    }
    for (int i = 1 + lane; i < m; i += 32) x[i] = cmulf(x[i], cg);
    __syncwarp();
    // Left: column c (one per lane) -= tau v (v^H column).
    for (int c = r + 1 + lane; c < n; c += 32) {
      float2* col = S.at(r + 1, c);
      float2 w = col[0];
      for (int i = 1; i < m; ++i) {
        const float2 v = x[i], a = col[i];
        w.x = fmaf(v.x, a.x, fmaf(v.y, a.y, w.x));
        w.y = fmaf(v.x, a.y, fmaf(-v.y, a.x, w.y));
      }
      const float2 t = make_float2(w.x * tau, w.y * tau);
      col[0] = csubf(col[0], t);
      for (int i = 1; i < m; ++i) col[i] = csubf(col[i], cmulf(x[i], t));
    }
    __syncwarp();
    // Right: row q (one per lane) -= tau (row v) v^H.
    for (int q = lane; q < n; q += 32) {
      float2* row = S.at(q, r + 1);
      float2 w = row[0];
      for (int i = 1; i < m; ++i) {
        const float2 v = x[i], a = row[i * ld];
        w.x = fmaf(v.x, a.x, fmaf(-v.y, a.y, w.x));
        w.y = fmaf(v.x, a.y, fmaf(v.y, a.x, w.y));
      }
      const float2 t = make_float2(w.x * tau, w.y * tau);
      row[0] = csubf(row[0], t);
      for (int i = 1; i < m; ++i) {
        const float2 v = x[i];
        // row[i] -= t * conj(v)
        row[i * ld] = make_float2(row[i * ld].x - fmaf(t.x, v.x, t.y * v.y), row[i * ld].y - fmaf(t.y, v.x, -t.x * v.y));
      }
    }
    __syncwarp();
    if (lane == 0) x[0] = alpha;
    __syncwarp();
  }
}

// Single-shift QR of the Hessenberg S (eigenvalues only); est[i] = T_ii * f.
__device__ __forceinline__ void qr_estimates(const SMat& S, int lane, float f, float2* __restrict__ est) {
  const int n = S.n;
  const float smlnum = kSafeMinF * ((float)n / kUlpF);
  int i = n - 1, lo = 0, its = 0, kdefl = 0;
  while (true) {
    for (;;) {
      int hit = lo;
      for (int k = i - lane; k > lo; k -= 32) {
        if (negligible_f(S, k, lo, i, smlnum)) {
          hit = k;
          break;
        }
      }
      lo = __reduce_max_sync(0xffffffffu, hit);
      if (lo < i) break;
      if (lane == 0) {
        const float2 d = *S.at(i, i);
        est[i] = make_float2(d.x * f, d.y * f);
      }
      i -= 1;
      lo = 0;
      its = 0;
      kdefl = 0;
      if (i < 0) break;
    }
    if (i < 0) break;
    if (its >= kEstimateSweepCap) {  // give up: the current diagonal serves as estimates
      for (int k = lane; k <= i; k += 32) {
        const float2 d = *S.at(k, k);
        est[k] = make_float2(d.x * f, d.y * f);
      }
      break;
    }
    ++its;
    ++kdefl;
    float2 sigma;
    if (kdefl % (2 * kExceptionalPeriod) == 0) {
      const float2 d = *S.at(i, i);
      sigma = make_float2(d.x + 0.75f * cabs1f(*S.at(i, i - 1)), d.y);
    } else if (kdefl % kExceptionalPeriod == 0) {
      const float2 d = *S.at(lo, lo);
      sigma = make_float2(d.x + 0.75f * cabs1f(*S.at(lo + 1, lo)), d.y);
    } else {
      sigma = wilkinson_shift_f(*S.at(i - 1, i - 1), *S.at(i - 1, i), *S.at(i, i - 1), *S.at(i, i));
    }
    for (int j = lo; j < i; ++j) {
      float2 x, y, rr;
      if (j == lo) {
        x = csubf(*S.at(lo, lo), sigma);
        y = *S.at(lo + 1, lo);
      } else {
        x = *S.at(j, j - 1);
        y = *S.at(j + 1, j - 1);
      }
      const RotF g = make_rot_f(x, y, rr);
      __syncwarp();
      if (j > lo && lane == 0) *S.at(j, j - 1) = rr;
      for (int c = j + lane; c <= i; c += 32) {  // rows j, j+1
        float2* pa = S.at(j, c);
        const float2 a = pa[0], b = pa[1];
        pa[0] = make_float2(fmaf(g.c, a.x, fmaf(g.s.x, b.x, -g.s.y * b.y)), fmaf(g.c, a.y, fmaf(g.s.x, b.y, g.s.y * b.x)));
        pa[1] = make_float2(fmaf(g.c, b.x, -fmaf(g.s.x, a.x, g.s.y * a.y)),
                            fmaf(g.c, b.y, -fmaf(g.s.x, a.y, -g.s.y * a.x)));
      }
      __syncwarp();
      const int qend = min(j + 1, i);
      for (int q = lo + lane; q <= qend; q += 32) {  // columns j, j+1
        float2* pa = S.at(q, j);
        const float2 a = pa[0], b = pa[S.ld];
        pa[0] = make_float2(fmaf(g.c, a.x, fmaf(g.s.x, b.x, g.s.y * b.y)), fmaf(g.c, a.y, fmaf(g.s.x, b.y, -g.s.y * b.x)));
        pa[S.ld] = make_float2(fmaf(g.c, b.x, -fmaf(g.s.x, a.x, -g.s.y * a.y)),
                               fmaf(g.c, b.y, -fmaf(g.s.x, a.y, g.s.y * a.x)));
      }
      if (j + 2 <= i && lane == 31) {  // bulge row: its column-j entry is zero before the rotation
        float2* pb = S.at(j + 2, j);
        const float2 b = pb[S.ld];
        pb[0] = make_float2(fmaf(g.s.x, b.x, g.s.y * b.y), fmaf(g.s.x, b.y, -g.s.y * b.x));
        pb[S.ld] = make_float2(g.c * b.x, g.c * b.y);
      }
      __syncwarp();
    }
  }
}

// Estimates for one matrix read through `src` (same sources as the FP64
// path); S is this warp's shared-memory area of n*(n+1) float2.
template <class Src>
__device__ __forceinline__ void estimate_matrix(const Src& src, int n, float2* smem, float2* __restrict__ est) {
  const int lane = threadIdx.x & 31;
  const int nn = n * n;
  int emax = 0;
  for (int e = lane; e < nn; e += 32) {
    const double2 z = src.load(e, n);
    emax = max(emax, max(dexp_field(z.x), dexp_field(z.y)));
  }
  emax = __reduce_max_sync(0xffffffffu, emax);
  if (emax == 0x7ff || emax == 0) {  // the FP64 path returns before its QR
    for (int i = lane; i < n; i += 32) est[i] = make_float2(0.0f, 0.0f);
    return;
  }
  const int top = emax - 1023;                       // largest |Re|,|Im| in [2^top, 2^(top+1))
  const int shift64 = (top > 60 || top < -60) ? top : 0;  // the FP64 staging's exponent shift
  const double sc = top > 1022 ? 0.5 * pow2(-1022) : pow2(-top);  // entries now below 2 in magnitude
  const SMat S{smem, n, n + 1};
  for (int e = lane; e < nn; e += 32) {
    const int c = e / n;
    const double2 z = src.load(e, n);
    *S.at(e - c * n, c) = make_float2((float)(z.x * sc), (float)(z.y * sc));
  }
  __syncwarp();
  hessenberg_f(S, lane);
  qr_estimates(S, lane, pow2f(top - shift64), est);
  __syncwarp();
}

// One warp per block; persistent over the batch, estimates for matrix j at est + j*n.
template <class Batch>
__global__ void __launch_bounds__(32) zgeev_estimate_kernel(int n, int batch, Batch B, float2* __restrict__ est) {
  extern __shared__ float2 estimate_smem[];
  for (long long j = blockIdx.x; j < batch; j += gridDim.x) {
    if (!B.valid(j)) continue;
    estimate_matrix(B.src(j), n, estimate_smem, est + j * n);
  }
}

// Launches the estimator on `stream`: every SM gets as many one-warp blocks
// as its shared memory allows.
template <class Batch>
cudaError_t launch_estimates(int n, int batch, const Batch& B, float2* est, cudaStream_t stream) {
  const size_t smem = sizeof(float2) * (size_t)n * (n + 1);
  int dev = 0, sms = 0, per_sm = 0;
  cudaError_t err = cudaGetDevice(&dev);
  if (err == cudaSuccess) err = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (err == cudaSuccess)
    err = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, zgeev_estimate_kernel<Batch>, 32, smem);
  if (err != cudaSuccess) return err;
  if (per_sm < 1) per_sm = 1;
  long long blocks = (long long)sms * per_sm;
  if (blocks > batch) blocks = batch;
  zgeev_estimate_kernel<Batch><<<(unsigned)blocks, 32, smem, stream>>>(n, batch, B, est);
  return cudaGetLastError();
}

}  // namespace tzg
