// Device helpers shared by the single-sector Lanczos (lanczos.cu) and the
// batched sweep (batch.cu): double-float accumulation on the FP32 pipes, the
// tridiagonal Sturm count and bounds, inverse iteration.
#pragma once

#include <cfloat>
#include <cstdint>

// SpMV with double-float accumulation, for FP32-valued CSR. The vector x is
// given as FP32 pairs (hi, lo) with hi + lo = x to 2^-48; each product v*hi is
// split exactly into a sum of two floats with an FMA (Dekker), v*lo is added
// to the low part, and the running sum is kept as an unevaluated pair updated
// with Knuth's TwoSum. Every operation runs on the FP32 pipes: on GB300 the
// FP64 pipe is ~1/64 of the FP32 rate, so one FP64 FMA per nonzero would cap
// this HBM-bound kernel. Rounding per accumulated product is ~2^-48 relative,
// i.e. FP64-class; the result is converted to FP64 once per row.
__device__ __forceinline__ void two_sum(float a, float b, float& s, float& e) {
  s = a + b;
  const float bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
__device__ __forceinline__ void df_add_prod(float& ah, float& al, float v, float xh, float xl) {
  const float p = v * xh;
  const float pe = fmaf(v, xh, -p);
  const float t = fmaf(v, xl, pe);
  float s, e;
  two_sum(ah, p, s, e);
  ah = s;
  al += e + t;
}
template <int LPR>
__device__ __forceinline__ void df_seg_reduce(float& ah, float& al) {
#pragma unroll
  for (int o = LPR / 2; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, ah, o, LPR);
    const float ol = __shfl_xor_sync(0xffffffffu, al, o, LPR);
    float s, e;
    two_sum(ah, oh, s, e);
    ah = s;
    al = al + ol + e;
  }
}

// (ah, al) += (bh, bl) in double-float.
__device__ __forceinline__ void df_add(float& ah, float& al, float bh, float bl) {
  float s, e;
  two_sum(ah, bh, s, e);
  ah = s;
  al = al + bl + e;
}

// K6: tridiagonal eigen-solve. Sturm count: eigenvalues of T (diag a, off-diag
// b[1..m-1]) below x, with the usual tiny-pivot guard.
static __device__ int sturm_count(const double* a, const double* b, int m, double x, double pivmin) {
  int c = 0;
  double q = a[0] - x;
  if (fabs(q) <= pivmin) q = -pivmin;
  c += q < 0;
  for (int i = 1; i < m; i++) {
    q = (a[i] - x) - b[i] * b[i] / q;
    if (fabs(q) <= pivmin) q = -pivmin;
    c += q < 0;
  }
  return c;
}

static __device__ void gersh(const double* a, const double* b, int m, double* lo, double* hi, double* pivmin) {
  double l = a[0], h = a[0], bm = 0;
  for (int i = 0; i < m; i++) {
    const double r = (i > 0 ? fabs(b[i]) : 0) + (i + 1 < m ? fabs(b[i + 1]) : 0);
    l = fmin(l, a[i] - r);
    h = fmax(h, a[i] + r);
    if (i > 0) bm = fmax(bm, b[i] * b[i]);
  }
  const double w = fmax(fabs(l), fabs(h));
  *lo = l - 2 * DBL_EPSILON * w - 1e-300;
  *hi = h + 2 * DBL_EPSILON * w + 1e-300;
  *pivmin = DBL_MIN * fmax(1.0, bm);
}


// Eigenvector for eigenvalue lam by inverse iteration with a partially pivoted
// tridiagonal LU (one thread; m <= a few thousand). work: 5 m doubles.
static __device__ void tri_inverse_iteration(const double* a, const double* b, int m, double lam, double* y,
                                             double* work) {
  double* d = work;            // diagonal of U
  double* u1 = work + m;       // first superdiagonal
  double* u2 = work + 2 * m;   // second superdiagonal (fill from pivoting)
  double* l = work + 3 * m;    // multipliers
  int* piv = reinterpret_cast<int*>(work + 4 * m);
  double anorm = 0;
  for (int i = 0; i < m; i++) anorm = fmax(anorm, fabs(a[i]) + (i ? fabs(b[i]) : 0) + (i + 1 < m ? fabs(b[i + 1]) : 0));
  const double tiny = DBL_EPSILON * fmax(anorm, 1e-300);
  // factor T - lam I = P L U
  for (int i = 0; i < m; i++) {
    d[i] = a[i] - lam;
    u1[i] = (i + 1 < m) ? b[i + 1] : 0;
    u2[i] = 0;
  }
  for (int i = 0; i + 1 < m; i++) {
    const double sub = b[i + 1];
    if (fabs(d[i]) >= fabs(sub)) {
      piv[i] = 0;
      const double f = (d[i] != 0) ? sub / d[i] : 0;
      l[i] = f;
      d[i + 1] -= f * u1[i];
    } else {
      piv[i] = 1;
      const double f = d[i] / sub;
      l[i] = f;
      // swap rows i and i+1
      const double t0 = d[i], t1 = u1[i];
      d[i] = sub;
      u1[i] = d[i + 1];
      u2[i] = (i + 2 < m) ? u1[i + 1] : 0;
      d[i + 1] = t1 - f * u1[i];
      if (i + 2 < m) u1[i + 1] = -f * u2[i];
      (void)t0;
    }
  }
  for (int i = 0; i < m; i++)
    if (fabs(d[i]) < tiny) d[i] = (d[i] < 0 ? -tiny : tiny);
  for (int i = 0; i < m; i++) y[i] = 1.0 / sqrt((double)m) * (1.0 + 0.01 * (i % 7));
  for (int itn = 0; itn < 4; itn++) {
    // forward: apply P and L
    for (int i = 0; i + 1 < m; i++) {
      if (piv[i]) {
        const double t = y[i];
        y[i] = y[i + 1];
        y[i + 1] = t - l[i] * y[i];
      } else {
        y[i + 1] -= l[i] * y[i];
      }
    }
    // back substitution with U
    for (int i = m - 1; i >= 0; i--) {
      double s = y[i];
      if (i + 1 < m) s -= u1[i] * y[i + 1];
      if (i + 2 < m) s -= u2[i] * y[i + 2];
      y[i] = s / d[i];
    }
    double nrm = 0;
    for (int i = 0; i < m; i++) nrm += y[i] * y[i];
    nrm = sqrt(nrm);
    for (int i = 0; i < m; i++) y[i] /= nrm;
  }
  // sign convention: largest-magnitude component positive
  int im = 0;
  for (int i = 1; i < m; i++)
    if (fabs(y[i]) > fabs(y[im])) im = i;
  if (y[im] < 0)
    for (int i = 0; i < m; i++) y[i] = -y[i];
}

