// K3 SpMV, K4/K5 Lanczos steps with full FP64 reorthogonalization, K6 the
// tridiagonal eigensolver, K7 the Ritz vector, and the Rayleigh quotients.
//
// Replaces Mat::operator* (BLQH_without_spin/matrix.cpp:244-267),
// lhamil::coeff_explicit_update (lanczos_hamiltonian.cpp:453-579), lhamil::diag
// with LAPACK dsyevd (lanczos_hamiltonian.cpp:581-606, matrix.cpp:288-305),
// eigenstates_reconstruction (:610-644) and ground_state_energy (:646-656).
//
// Differences by design (the physics answer is the same):
//   * the Krylov basis is kept in HBM, so the ground state is one GEMV over it
//     instead of a second Lanczos pass, and it is not complex-conjugated (the
//     reference's conjugated reconstruction is an eigenvector only in real
//     sectors);
//   * with reorth = 1 every new vector, after the three-term step, is
//     orthogonalized against all previous ones by one classical Gram-Schmidt
//     pass, so no ghost Ritz values appear and the run stops at convergence or
//     at an invariant subspace (dim < lambda);
//   * all scalars (alpha, beta, Gram-Schmidt coefficients, stop flag) stay in
//     device memory; the host polls the stop flag once per chunk of steps.
#include <algorithm>
#include <cfloat>
#include <cstdio>
#include <cmath>
#include <cstring>

#include "../../include/blqh_gpu_debug.h"
#include "krylov.cuh"
#include "sector.cuh"

double rayleigh_regen_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params& p, const double* d_psi,
                           bool want_complex);
void spin_observables_impl(blqh_ctx* ctx, const blqh_basis* B, const double* psi, int cplx, double* out);
double spin_rayleigh_regen_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_spin& p, const double* x);
int hamil_build_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params& p, int prec, blqh_csr* M);
void free_csr(blqh_csr* m);

namespace {

constexpr int UPD_THREADS = 256;

// device scalar block layout (doubles), per Lanczos object
struct Scal {
  double* alpha;  // [mmax]
  double* beta;   // [mmax+1]; beta[0] = 0 internally
  double* h;      // [2*(mmax+1)] Gram-Schmidt coefficients (re, im)
  double* h2;     // [2*(mmax+1)] second pass
  double* nrm;    // [4]: |w|^2 before, after pass 1, final
  double* ritz;   // [mmax] lowest Ritz value at checks
  int* flags;     // [8]: stop, pass2, steps, breakdown, a full-pass coefficient not small (FP64 update),
                  //      the tridiagonal size of the last convergence check's Ritz value
};

// ---------------------------------------------------------------------------
// SpMV: LPR lanes per row, FP64 accumulation. y = H x - b * xprev.
template <class VT>
__device__ __forceinline__ double2 ld_val(const VT* v, int64_t k);
template <>
__device__ __forceinline__ double2 ld_val<double>(const double* v, int64_t k) {
  return make_double2(__ldg(v + k), 0.0);
}
template <>
__device__ __forceinline__ double2 ld_val<float>(const float* v, int64_t k) {
  return make_double2((double)__ldg(v + k), 0.0);
}
template <>
__device__ __forceinline__ double2 ld_val<double2>(const double2* v, int64_t k) {
  return __ldg(v + k);
}
template <>
__device__ __forceinline__ double2 ld_val<float2>(const float2* v, int64_t k) {
  float2 f = __ldg(v + k);
  return make_double2((double)f.x, (double)f.y);
}

template <class VT, bool CPLX, int LPR>
__global__ void __launch_bounds__(256) k_spmv(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                              const VT* __restrict__ val, const double* __restrict__ x,
                                              double* __restrict__ y, int64_t dim, const double* bptr,
                                              const double* __restrict__ xprev, const int* stop) {
  if (stop && *stop) return;
  // warp-uniform iteration: every lane of a warp runs the same number of row
  // rounds, so the segmented shuffles below always see all 32 lanes.
  const int lane = threadIdx.x & 31;
  constexpr int GPW = 32 / LPR;  // rows per warp per round
  const int gi = lane / LPR, sub = lane % LPR;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const double b = bptr ? *bptr : 0.0;
  for (int64_t rb = warp * GPW; rb < dim; rb += nwarps * GPW) {
    const int64_t r = rb + gi;
    const bool ok = r < dim;
    const int64_t s = ok ? rp[r] : 0, e = ok ? rp[r + 1] : 0;
    double ar = 0.0, ai = 0.0;
    int64_t k = s + sub;
#pragma unroll 4
    for (; k < e; k += LPR) {
      const int32_t c = __ldg(col + k);
      const double2 v = ld_val<VT>(val, k);
      if (CPLX) {
        const double2 xv = __ldg(reinterpret_cast<const double2*>(x) + c);
        ar += v.x * xv.x - v.y * xv.y;
        ai += v.x * xv.y + v.y * xv.x;
      } else {
        ar += v.x * __ldg(x + c);
      }
    }
#pragma unroll
    for (int o = LPR / 2; o > 0; o >>= 1) {
      ar += __shfl_xor_sync(0xffffffffu, ar, o, LPR);
      if (CPLX) ai += __shfl_xor_sync(0xffffffffu, ai, o, LPR);
    }
    if (ok && sub == 0) {
      if (CPLX) {
        double2 o = make_double2(ar, ai);
        if (xprev) {
          const double2 p = reinterpret_cast<const double2*>(xprev)[r];
          o.x -= b * p.x;
          o.y -= b * p.y;
        }
        reinterpret_cast<double2*>(y)[r] = o;
      } else {
        y[r] = xprev ? ar - b * xprev[r] : ar;
      }
    }
  }
}

// ---------------------------------------------------------------------------
// SpMV with double-float accumulation for FP32-valued CSR (helpers in krylov.cuh).
template <bool CPLX, int LPR>
__global__ void __launch_bounds__(256) k_spmv_df(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                                 const float* __restrict__ val, const float2* __restrict__ xs,
                                                 double* __restrict__ y, int64_t dim, const double* bptr,
                                                 const double* __restrict__ xprev, const int* stop) {
  if (stop && *stop) return;
  const int lane = threadIdx.x & 31;
  constexpr int GPW = 32 / LPR;
  const int gi = lane / LPR, sub = lane % LPR;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  const double b = bptr ? *bptr : 0.0;
  for (int64_t rb = warp * GPW; rb < dim; rb += nwarps * GPW) {
    const int64_t r = rb + gi;
    const bool ok = r < dim;
    const int64_t s = ok ? rp[r] : 0, e = ok ? rp[r + 1] : 0;
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
#pragma unroll 4
    for (int64_t k = s + sub; k < e; k += LPR) {
      const int32_t c = __ldg(col + k);
      if (CPLX) {
        const float2 v = __ldg(reinterpret_cast<const float2*>(val) + k);
        const float4 x = __ldg(reinterpret_cast<const float4*>(xs) + c);  // (re hi, re lo, im hi, im lo)
        df_add_prod(rh, rl, v.x, x.x, x.y);
        df_add_prod(rh, rl, -v.y, x.z, x.w);
        df_add_prod(ih, il, v.x, x.z, x.w);
        df_add_prod(ih, il, v.y, x.x, x.y);
      } else {
        const float v = __ldg(val + k);
        const float2 x = __ldg(xs + c);
        df_add_prod(rh, rl, v, x.x, x.y);
      }
    }
    df_seg_reduce<LPR>(rh, rl);
    if (CPLX) df_seg_reduce<LPR>(ih, il);
    if (ok && sub == 0) {
      const double re = (double)rh + (double)rl;
      if (CPLX) {
        double2 o = make_double2(re, (double)ih + (double)il);
        if (xprev) {
          const double2 p = reinterpret_cast<const double2*>(xprev)[r];
          o.x -= b * p.x;
          o.y -= b * p.y;
        }
        reinterpret_cast<double2*>(y)[r] = o;
      } else {
        y[r] = xprev ? re - b * xprev[r] : re;
      }
    }
  }
}

// Real FP32-valued CSR, double-float accumulation, 16-byte loads: each lane
// takes four consecutive nonzeros (one int4 of columns, one float4 of values)
// per step, so a warp keeps 512 B of matrix stream in flight per load pair and
// issues the four gathers of x back to back. The unaligned head (< 4 entries
// before a 16-byte boundary) and tail of each row are loaded one by one.
template <int LPR>
__global__ void __launch_bounds__(256) k_spmv_df_v4(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                                    const float* __restrict__ val, const float2* __restrict__ xs,
                                                    double* __restrict__ y, int64_t dim, const double* bptr,
                                                    const double* __restrict__ xprev, const int* stop) {
  if (stop && *stop) return;
  const int lane = threadIdx.x & 31;
  constexpr int GPW = 32 / LPR;
  const int gi = lane / LPR, sub = lane % LPR;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  // Each warp takes chunks of 32 consecutive rows; lane k keeps the sum of row
  // base + k, and the FP64 epilogue runs once per chunk with all lanes busy
  // (an FP64 instruction costs the same with one active lane as with 32).
  for (int64_t base = warp * 32; base < dim; base += nwarps * 32) {
   float mh = 0.f, ml = 0.f;
   for (int rd = 0; rd < LPR; rd++) {
    const int64_t r = base + rd * GPW + gi;
    const bool ok = r < dim;
    const int64_t s = ok ? __ldg(rp + r) : 0, e = ok ? __ldg(rp + r + 1) : 0;
    float ah = 0.f, al = 0.f;
    const int64_t a4 = (s + 3) & ~(int64_t)3;   // first 16-byte aligned index
    const int64_t b4 = e & ~(int64_t)3;         // end of the aligned body
    const int64_t hend = a4 < e ? a4 : e;
    if (s + sub < hend) {
      const int64_t k = s + sub;
      const float2 x = __ldg(xs + __ldg(col + k));
      df_add_prod(ah, al, __ldg(val + k), x.x, x.y);
    }
    if (b4 > a4) {
      const int4* c4 = reinterpret_cast<const int4*>(col);
      const float4* v4 = reinterpret_cast<const float4*>(val);
      for (int64_t q = (a4 >> 2) + sub; q < (b4 >> 2); q += LPR) {
        const int4 c = __ldg(c4 + q);
        const float4 v = __ldg(v4 + q);
        const float2 x0 = __ldg(xs + c.x), x1 = __ldg(xs + c.y), x2 = __ldg(xs + c.z), x3 = __ldg(xs + c.w);
        df_add_prod(ah, al, v.x, x0.x, x0.y);
        df_add_prod(ah, al, v.y, x1.x, x1.y);
        df_add_prod(ah, al, v.z, x2.x, x2.y);
        df_add_prod(ah, al, v.w, x3.x, x3.y);
      }
      if (b4 + sub < e) {
        const int64_t k = b4 + sub;
        const float2 x = __ldg(xs + __ldg(col + k));
        df_add_prod(ah, al, __ldg(val + k), x.x, x.y);
      }
    }
    df_seg_reduce<LPR>(ah, al);
    // every lane of a segment holds its row's sum; lane k collects row base + k
    const int src = (lane % GPW) * LPR;
    const float th = __shfl_sync(0xffffffffu, ah, src), tl = __shfl_sync(0xffffffffu, al, src);
    if (lane / GPW == rd) {
      mh = th;
      ml = tl;
    }
   }
   const int64_t r = base + lane;
   if (r < dim) {
     const double re = (double)mh + (double)ml;
     y[r] = xprev ? re - *bptr * xprev[r] : re;
   }
  }
}

// x (FP64) -> (hi, lo) FP32 pairs for the double-float SpMV.
__global__ void k_split(const double* __restrict__ x, float2* __restrict__ xs, int64_t n, const int* stop) {
  if (stop && *stop) return;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    const float hi = (float)v;
    xs[i] = make_float2(hi, (float)(v - (double)hi));
  }
}

// ---------------------------------------------------------------------------
// Gram-Schmidt dots: part[blk][k] = sum_{r in tile blk} conj(V_k[r]) w[r] for k
// in [k0, k1), on tiles of GS_ROWS rows (one warp per vector at a time), and the
// tile's |w|^2. cond: run only when the second pass was requested (flags[1]).
constexpr int GS_ROWS = 1024;

__device__ __forceinline__ double block_sum_256(double v, double* red) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); i++) s += red[i];
  __syncthreads();
  return s;  // valid in thread 0
}

template <bool CPLX>
__global__ void __launch_bounds__(256) k_dots(const double* __restrict__ V, int64_t dim, int k0, int k1,
                                              const double* __restrict__ w, double* __restrict__ part, int stride,
                                              double* __restrict__ part_norm, const int* flags, int cond) {
  if (flags[0] || (cond && !flags[1])) return;
  constexpr int VW = CPLX ? 2 : 1;
  __shared__ double ws[GS_ROWS * VW];
  __shared__ double red[8];
  const int64_t r0 = (int64_t)blockIdx.x * GS_ROWS;
  const int64_t rem = dim - r0;
  const int nr = (int)(rem < GS_ROWS ? rem : GS_ROWS);
  double nn = 0;
  for (int t = threadIdx.x; t < GS_ROWS * VW; t += blockDim.x) {
    const double v = (t < nr * VW) ? w[r0 * VW + t] : 0.0;
    ws[t] = v;
    nn += v * v;
  }
  const double tot = block_sum_256(nn, red);
  if (threadIdx.x == 0 && part_norm) part_norm[blockIdx.x] = tot;
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = k0 + wid; k < k1; k += (int)(blockDim.x >> 5)) {
    const double* vk = V + ((int64_t)k * dim + r0) * VW;
    double sr = 0, si = 0;
    if (CPLX) {
      for (int t = lane; t < nr; t += 32) {
        const double2 a = reinterpret_cast<const double2*>(vk)[t];
        const double br = ws[2 * t], bi = ws[2 * t + 1];
        sr += a.x * br + a.y * bi;
        si += a.x * bi - a.y * br;
      }
    } else {
      for (int t = lane; t < nr; t += 32) sr += vk[t] * ws[t];
    }
    for (int o = 16; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      if (CPLX) si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) {
      part[((int64_t)blockIdx.x * stride + k) * 2] = sr;
      part[((int64_t)blockIdx.x * stride + k) * 2 + 1] = si;
    }
  }
}

// One block per coefficient k (plus one for |w|^2 in stage 1): sums the tile
// partials in a fixed order (deterministic).
// stage 1: h = dots, alpha_j = Re h[j], nrm[0] = |w|^2
// stage 2: h2 = dots (second pass), alpha_j += Re h2[j]
__global__ void k_reduce_dots(const double* part, int nblk, int stride, int k0, int k1, const double* part_norm,
                              Scal S, int j, int stage) {
  if (S.flags[0] || (stage == 2 && !S.flags[1])) return;
  __shared__ double red[8];
  const int kb = blockIdx.x;
  const bool is_norm = kb >= k1 - k0;
  if (is_norm && (stage != 1 || !part_norm)) return;
  double a = 0, b = 0;
  if (!is_norm) {
    const int k = k0 + kb;
    for (int blk = threadIdx.x; blk < nblk; blk += blockDim.x) {
      a += part[((int64_t)blk * stride + k) * 2];
      b += part[((int64_t)blk * stride + k) * 2 + 1];
    }
  } else {
    for (int blk = threadIdx.x; blk < nblk; blk += blockDim.x) a += part_norm[blk];
  }
  a = block_sum_256(a, red);
  b = block_sum_256(b, red);
  if (threadIdx.x != 0) return;
  if (is_norm) {
    S.nrm[0] = a;
    return;
  }
  const int k = k0 + kb;
  double* h = (stage == 1) ? S.h : S.h2;
  h[2 * k] = a;
  h[2 * k + 1] = b;
  // the full pass's correction is summed on the FP32 pipes only while every
  // coefficient is below 2^-30 |w| (see k_update)
  if (stage == 2 && a * a + b * b > 0x1p-60 * S.nrm[1]) atomicOr(S.flags + 4, 1);
  if (k == j) {
    if (stage == 1) S.alpha[j] = a;
    else S.alpha[j] += a;
  }
}

// FP32 value with the 24 leading significant bits of x (truncated), from its
// bit pattern with integer operations only (GB300's FP64 pipe issues ~2 lane
// operations per clock per SM; this keeps the correction below off it).
// |x| < 2^-126 gives 0; |x| < 2^128 is assumed (Krylov vectors have |x| <= 1).
__device__ __forceinline__ float f64_lead_f32(double x) {
  const unsigned long long bits = (unsigned long long)__double_as_longlong(x);
  const unsigned hw = (unsigned)(bits >> 32), lw = (unsigned)bits;
  const int e = (int)((hw >> 20) & 0x7FFu) - 896;  // FP32 biased exponent
  const unsigned f = (hw & 0x80000000u) | ((unsigned)e << 23) | (__funnelshift_l(lw, hw, 3) & 0x7FFFFFu);
  return e > 0 ? __uint_as_float(f) : 0.0f;
}

// w -= sum_k h[k] V_k over k in [k0, k1); partial |w|^2 per block.
// The full pass (cond = 1) after the three-term step removes components that
// are round-off sized (|h_k| <= 2^-30 |w|, checked by k_reduce_dots; flags[4]
// is set otherwise): the correction sum_k h_k V_k is then accumulated in FP32
// from FP32-truncated coefficients and vector entries (relative error ~2^-22
// of a correction <= 2^-30 |w|, below FP64's rounding of w) and subtracted
// from w in FP64. The local step (cond = 0) and a flagged pass use FP64 FMAs.
template <bool CPLX>
__global__ void __launch_bounds__(UPD_THREADS) k_update(const double* __restrict__ V, int64_t dim, int k0, int k1,
                                                        const double* __restrict__ hcoef, double* __restrict__ w,
                                                        double* __restrict__ part_norm, const int* flags, int cond) {
  if (flags[0] || (cond && !flags[1])) return;
  extern __shared__ double hs[];
  const int nk = k1 - k0;
  const bool lowp = cond && !flags[4];
  float* hf = reinterpret_cast<float*>(hs + 2 * nk);
  for (int t = threadIdx.x; t < 2 * nk; t += blockDim.x) {
    const double c = hcoef[2 * k0 + t];
    hs[t] = c;
    hf[t] = f64_lead_f32(c);
  }
  __syncthreads();
  double nn = 0;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < dim) {
    if (CPLX) {
      double2 acc = reinterpret_cast<const double2*>(w)[r];
      if (lowp) {
        float dr = 0.f, di = 0.f;
        for (int k = 0; k < nk; k++) {
          const double2 v = reinterpret_cast<const double2*>(V)[(int64_t)(k0 + k) * dim + r];
          const float vr = f64_lead_f32(v.x), vi = f64_lead_f32(v.y);
          const float hr = hf[2 * k], hi = hf[2 * k + 1];
          dr = fmaf(hr, vr, fmaf(-hi, vi, dr));
          di = fmaf(hr, vi, fmaf(hi, vr, di));
        }
        acc.x -= (double)dr;
        acc.y -= (double)di;
      } else {
        for (int k = 0; k < nk; k++) {
          const double2 v = reinterpret_cast<const double2*>(V)[(int64_t)(k0 + k) * dim + r];
          const double hr = hs[2 * k], hi = hs[2 * k + 1];
          acc.x -= hr * v.x - hi * v.y;
          acc.y -= hr * v.y + hi * v.x;
        }
      }
      reinterpret_cast<double2*>(w)[r] = acc;
      nn = acc.x * acc.x + acc.y * acc.y;
    } else {
      double acc = w[r];
      if (lowp) {
        float d0 = 0.f, d1 = 0.f;
        int k = 0;
        for (; k + 2 <= nk; k += 2) {
          d0 = fmaf(hf[2 * k], f64_lead_f32(V[(int64_t)(k0 + k) * dim + r]), d0);
          d1 = fmaf(hf[2 * k + 2], f64_lead_f32(V[(int64_t)(k0 + k + 1) * dim + r]), d1);
        }
        if (k < nk) d0 = fmaf(hf[2 * k], f64_lead_f32(V[(int64_t)(k0 + k) * dim + r]), d0);
        acc -= (double)(d0 + d1);
      } else {
        int k = 0;
        for (; k + 4 <= nk; k += 4) {
          const double v0 = V[(int64_t)(k0 + k) * dim + r], v1 = V[(int64_t)(k0 + k + 1) * dim + r];
          const double v2 = V[(int64_t)(k0 + k + 2) * dim + r], v3 = V[(int64_t)(k0 + k + 3) * dim + r];
          acc -= hs[2 * k] * v0;
          acc -= hs[2 * k + 2] * v1;
          acc -= hs[2 * k + 4] * v2;
          acc -= hs[2 * k + 6] * v3;
        }
        for (; k < nk; k++) acc -= hs[2 * k] * V[(int64_t)(k0 + k) * dim + r];
      }
      w[r] = acc;
      nn = acc * acc;
    }
  }
  __shared__ double red[UPD_THREADS / 32];
  const double tot = block_sum_256(nn, red);
  if (threadIdx.x == 0) part_norm[blockIdx.x] = tot;
}

// ---------------------------------------------------------------------------
// Gram-Schmidt on FP32 planes (FP32 values with double-float accumulation).
// Next to each FP64 Krylov vector V_k the library keeps two FP32 planes, Vh_k =
// the leading 24 bits of V_k (truncated, f64_lead_f32) and Vl_k = the rest
// rounded to FP32, so that Vh + Vl = V_k to 2^-48. The full Gram-Schmidt pass
// then runs on GB300's FP32 pipes (its FP64 pipe issues ~2 lane operations per
// clock per SM, which capped the FP64 dots at ~35 % of HBM bandwidth):
//   * dots conj(V_k) w in double-float from (Vh, Vl) and the split of w
//     (error <= ~2^-46 sum |V_k| |w|, FP64-class): 8 bytes per entry;
//   * the correction of k_update's FP32 path reads Vh only: 4 bytes per entry
//     instead of 8, with the same values it used before.
// Rows of a plane are padded to a multiple of 4 floats (zero-filled).

// (hi, lo) planes of one vector: hi = leading 24 bits of x, lo = the rest rounded.
__global__ void k_planes(const double* __restrict__ x, float* __restrict__ vh, float* __restrict__ vl, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = x[i];
    const float h = f64_lead_f32(v);
    vh[i] = h;
    vl[i] = (float)(v - (double)h);
  }
}

// (ah, al) += (vh + vl) (wh + wl) in double-float (the vl wl term, ~2^-48 of the
// product, is dropped).
__device__ __forceinline__ void df_prod_split(float& ah, float& al, float vh, float vl, float wh, float wl) {
  const float p = vh * wh;
  const float pe = fmaf(vh, wh, -p);
  const float t = fmaf(vh, wl, fmaf(vl, wh, pe));
  float s, e;
  two_sum(ah, p, s, e);
  ah = s;
  al += e + t;
}

// part[blk][k] = conj(V_k) w over the tile blk of GS_ROWS rows, for k in
// [k0, k1), from the planes (row stride ld floats). One warp per vector at a
// time, 16-byte loads. cond: run only when the second pass was requested.
template <bool CPLX>
__global__ void __launch_bounds__(256) k_dots_df(const float* __restrict__ Vh, const float* __restrict__ Vl,
                                                 int64_t ld, int64_t dim, int k0, int k1,
                                                 const double* __restrict__ w, double* __restrict__ part, int stride,
                                                 const int* flags, int cond) {
  if (flags[0] || (cond && !flags[1])) return;
  constexpr int VW = CPLX ? 2 : 1;
  constexpr int TF = GS_ROWS * VW;  // floats of a plane tile
  __shared__ __align__(16) float wh[TF];
  __shared__ __align__(16) float wl[TF];
  const int64_t e0 = (int64_t)blockIdx.x * TF;
  const int64_t n = dim * VW;
  const int ne = (int)(n - e0 < TF ? n - e0 : TF);
  for (int t = threadIdx.x; t < TF; t += blockDim.x) {
    const double v = t < ne ? w[e0 + t] : 0.0;
    const float h = (float)v;
    wh[t] = h;
    wl[t] = (float)(v - (double)h);
  }
  __syncthreads();
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = k0 + wid; k < k1; k += (int)(blockDim.x >> 5)) {
    const float* ph = Vh + (int64_t)k * ld + e0;
    const float* pl = Vl + (int64_t)k * ld + e0;
    float sh = 0.f, sl = 0.f, ih = 0.f, il = 0.f;
#pragma unroll 2
    for (int t = lane * 4; t < ne; t += 128) {  // the row padding keeps t + 3 inside the plane
      const float4 h4 = __ldcs(reinterpret_cast<const float4*>(ph + t));
      const float4 l4 = __ldcs(reinterpret_cast<const float4*>(pl + t));
      const float4 a4 = *reinterpret_cast<const float4*>(wh + t);
      const float4 b4 = *reinterpret_cast<const float4*>(wl + t);
      if (CPLX) {  // two entries (re, im): conj(v) w = (vr wr + vi wi, vr wi - vi wr)
        df_prod_split(sh, sl, h4.x, l4.x, a4.x, b4.x);
        df_prod_split(sh, sl, h4.y, l4.y, a4.y, b4.y);
        df_prod_split(ih, il, h4.x, l4.x, a4.y, b4.y);
        df_prod_split(ih, il, -h4.y, -l4.y, a4.x, b4.x);
        df_prod_split(sh, sl, h4.z, l4.z, a4.z, b4.z);
        df_prod_split(sh, sl, h4.w, l4.w, a4.w, b4.w);
        df_prod_split(ih, il, h4.z, l4.z, a4.w, b4.w);
        df_prod_split(ih, il, -h4.w, -l4.w, a4.z, b4.z);
      } else {
        df_prod_split(sh, sl, h4.x, l4.x, a4.x, b4.x);
        df_prod_split(sh, sl, h4.y, l4.y, a4.y, b4.y);
        df_prod_split(sh, sl, h4.z, l4.z, a4.z, b4.z);
        df_prod_split(sh, sl, h4.w, l4.w, a4.w, b4.w);
      }
    }
    df_seg_reduce<32>(sh, sl);
    if (CPLX) df_seg_reduce<32>(ih, il);
    if (lane == 0) {
      part[((int64_t)blockIdx.x * stride + k) * 2] = (double)sh + (double)sl;
      part[((int64_t)blockIdx.x * stride + k) * 2 + 1] = CPLX ? (double)ih + (double)il : 0.0;
    }
  }
}

// k_update with planes: four consecutive entries of w per thread (two complex
// rows). The FP32 path reads Vh (16-byte loads); the FP64 path (the local step,
// or a flagged pass) reads V. Same arithmetic, in the same order, as k_update.
template <bool CPLX>
__global__ void __launch_bounds__(UPD_THREADS) k_update_pl(const double* __restrict__ V,
                                                           const float* __restrict__ Vh, int64_t ld, int64_t dim,
                                                           int k0, int k1, const double* __restrict__ hcoef,
                                                           double* __restrict__ w, double* __restrict__ part_norm,
                                                           const int* flags, int cond) {
  if (flags[0] || (cond && !flags[1])) return;
  extern __shared__ double hs[];
  const int nk = k1 - k0;
  const bool lowp = cond && !flags[4];
  float* hf = reinterpret_cast<float*>(hs + 2 * nk);
  for (int t = threadIdx.x; t < 2 * nk; t += blockDim.x) {
    const double c = hcoef[2 * k0 + t];
    hs[t] = c;
    hf[t] = f64_lead_f32(c);
  }
  __syncthreads();
  constexpr int VW = CPLX ? 2 : 1;
  const int64_t n = dim * VW;
  const int64_t e0 = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) * 4;
  double nn = 0;
  if (e0 < n) {
    const int ne = (int)(n - e0 < 4 ? n - e0 : 4);  // 4, or the tail (complex: even)
    double a[4];
#pragma unroll
    for (int q = 0; q < 4; q++) a[q] = q < ne ? w[e0 + q] : 0.0;
    if (lowp) {
      if (CPLX) {
        float dr0 = 0.f, di0 = 0.f, dr1 = 0.f, di1 = 0.f;
#pragma unroll 4
        for (int k = 0; k < nk; k++) {
          const float4 v = __ldcs(reinterpret_cast<const float4*>(Vh + (int64_t)(k0 + k) * ld + e0));
          const float hr = hf[2 * k], hi = hf[2 * k + 1];
          dr0 = fmaf(hr, v.x, fmaf(-hi, v.y, dr0));
          di0 = fmaf(hr, v.y, fmaf(hi, v.x, di0));
          dr1 = fmaf(hr, v.z, fmaf(-hi, v.w, dr1));
          di1 = fmaf(hr, v.w, fmaf(hi, v.z, di1));
        }
        a[0] -= (double)dr0;
        a[1] -= (double)di0;
        a[2] -= (double)dr1;
        a[3] -= (double)di1;
      } else {
        float d0[4] = {0.f, 0.f, 0.f, 0.f}, d1[4] = {0.f, 0.f, 0.f, 0.f};  // even and odd k
        int k = 0;
#pragma unroll 2
        for (; k + 2 <= nk; k += 2) {
          const float4 v0 = __ldcs(reinterpret_cast<const float4*>(Vh + (int64_t)(k0 + k) * ld + e0));
          const float4 v1 = __ldcs(reinterpret_cast<const float4*>(Vh + (int64_t)(k0 + k + 1) * ld + e0));
          const float h0 = hf[2 * k], h1 = hf[2 * k + 2];
          d0[0] = fmaf(h0, v0.x, d0[0]);
          d0[1] = fmaf(h0, v0.y, d0[1]);
          d0[2] = fmaf(h0, v0.z, d0[2]);
          d0[3] = fmaf(h0, v0.w, d0[3]);
          d1[0] = fmaf(h1, v1.x, d1[0]);
          d1[1] = fmaf(h1, v1.y, d1[1]);
          d1[2] = fmaf(h1, v1.z, d1[2]);
          d1[3] = fmaf(h1, v1.w, d1[3]);
        }
        if (k < nk) {
          const float4 v0 = __ldcs(reinterpret_cast<const float4*>(Vh + (int64_t)(k0 + k) * ld + e0));
          const float h0 = hf[2 * k];
          d0[0] = fmaf(h0, v0.x, d0[0]);
          d0[1] = fmaf(h0, v0.y, d0[1]);
          d0[2] = fmaf(h0, v0.z, d0[2]);
          d0[3] = fmaf(h0, v0.w, d0[3]);
        }
#pragma unroll
        for (int q = 0; q < 4; q++) a[q] -= (double)(d0[q] + d1[q]);
      }
    } else {
      for (int k = 0; k < nk; k++) {
        const double* vk = V + (int64_t)(k0 + k) * n + e0;
        const double hr = hs[2 * k], hi = hs[2 * k + 1];
        if (CPLX) {
#pragma unroll
          for (int q = 0; q < 4; q += 2)
            if (q < ne) {
              const double vr = vk[q], vi = vk[q + 1];
              a[q] -= hr * vr - hi * vi;
              a[q + 1] -= hr * vi + hi * vr;
            }
        } else {
#pragma unroll
          for (int q = 0; q < 4; q++)
            if (q < ne) a[q] -= hr * vk[q];
        }
      }
    }
#pragma unroll
    for (int q = 0; q < 4; q++)
      if (q < ne) {
        w[e0 + q] = a[q];
        nn += a[q] * a[q];
      }
  }
  __shared__ double red[UPD_THREADS / 32];
  const double tot = block_sum_256(nn, red);
  if (threadIdx.x == 0) part_norm[blockIdx.x] = tot;
}

// <psi|H|psi> with each FP64 element carried as v32 + res (FP32 value and the
// FP32 rest of the builder's FP64 value, 2^-48 relative): y = H32 psi comes
// from the double-float SpMV; here one warp per row sums res * psi_hi in FP32
// (the rest is 2^-24 of the element, so FP32 keeps 2^-48 of the total) and
// adds Re(conj(psi_r) (y_r + that sum)) in FP64 into a block partial. Rows go
// to warps in a fixed grid-stride order: the result is reproducible.
template <bool CPLX>
__global__ void __launch_bounds__(256) k_rq_res(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                                                const void* __restrict__ res, const float2* __restrict__ xs,
                                                const double* __restrict__ psi, const double* __restrict__ y,
                                                int64_t dim, double* __restrict__ part) {
  __shared__ double red[8];
  const int lane = threadIdx.x & 31;
  const int64_t wg = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  double acc = 0;
  for (int64_t r = wg; r < dim; r += nw) {
    const int64_t a = rp[r], e = rp[r + 1];
    float sr = 0.f, si = 0.f;
    for (int64_t k = a + lane; k < e; k += 32) {
      const int c = __ldg(col + k);
      if (CPLX) {
        const float2 rv = __ldg(reinterpret_cast<const float2*>(res) + k);
        const float4 x = __ldg(reinterpret_cast<const float4*>(xs) + c);  // (re hi, re lo, im hi, im lo)
        sr = fmaf(rv.x, x.x, fmaf(-rv.y, x.z, sr));
        si = fmaf(rv.x, x.z, fmaf(rv.y, x.x, si));
      } else {
        sr = fmaf(__ldg(reinterpret_cast<const float*>(res) + k), __ldg(xs + c).x, sr);
      }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      if (CPLX) si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) {
      if (CPLX) acc += psi[2 * r] * (y[2 * r] + (double)sr) + psi[2 * r + 1] * (y[2 * r + 1] + (double)si);
      else acc += psi[r] * (y[r] + (double)sr);
    }
  }
  const double t = block_sum_256(acc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = t;
}

// After pass 1: |w|^2 and whether a second Gram-Schmidt pass is needed (the
// norm dropped below 1/sqrt(2) of its value before the pass); after pass 2:
// the final |w|^2. which: 1 = after pass 1, 2 = after pass 2.
// beta_{j+1} = |w| from the final |w|^2, the step count, and the breakdown test
// (one thread).
__device__ __forceinline__ void beta_from(Scal S, int j, double nrm2, double breakdown_tol) {
  const double b = sqrt(nrm2);
  S.beta[j + 1] = b;
  S.flags[2] = j + 1;
  const double scale = fabs(S.alpha[j]) + S.beta[j];
  if (!(b > breakdown_tol * (scale > 0 ? scale : 1.0))) {
    S.flags[3] = 1;
    S.flags[0] = 1;
  }
}

// After pass 1: |w|^2 and whether a second Gram-Schmidt pass is needed (the
// norm dropped below 1/sqrt(2) of its value before the pass); after pass 2:
// the final |w|^2. which: 1 = after pass 1, 2 = after pass 2. With
// breakdown_tol > 0 this is the step's last norm: it also sets beta_{j+1}.
__global__ void k_norm_step(const double* part_norm, int nblk, Scal S, int j, int which, int always_pass2,
                            double breakdown_tol) {
  if (S.flags[0]) return;
  if (which == 2 && !S.flags[1]) {  // no second pass: the final norm is pass 1's
    if (breakdown_tol > 0 && threadIdx.x == 0) beta_from(S, j, S.nrm[1], breakdown_tol);
    return;
  }
  __shared__ double red[8];
  double a = 0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) a += part_norm[b];
  a = block_sum_256(a, red);
  if (threadIdx.x != 0) return;
  S.nrm[1] = a;
  if (which == 1) {
    S.flags[1] = always_pass2 ? 1 : (a < 0.5 * S.nrm[0]) ? 1 : 0;
    S.flags[4] = 0;
  }
  if (breakdown_tol > 0) beta_from(S, j, a, breakdown_tol);
}

// V_{j+1} = w / beta_{j+1}
// (and its FP32 planes when vh is set, and its (hi, lo) split for the next
// double-float SpMV when xs is set, as k_split would write it)
__global__ void k_scale(const double* __restrict__ w, double* __restrict__ vout, int64_t n, Scal S, int j,
                        float* __restrict__ vh, float* __restrict__ vl, float2* __restrict__ xs) {
  if (S.flags[0]) return;
  const double inv = 1.0 / S.beta[j + 1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const double v = w[i] * inv;
    vout[i] = v;
    if (xs) {
      const float hi = (float)v;
      xs[i] = make_float2(hi, (float)(v - (double)hi));
    }
    if (vh) {
      const float h = f64_lead_f32(v);
      vh[i] = h;
      vl[i] = (float)(v - (double)h);
    }
  }
}

// ---------------------------------------------------------------------------
// K6: tridiagonal eigen-solve (Sturm count, bounds, inverse iteration in krylov.cuh).
// Lowest eigenvalue by parallel multisection (one block); optional
// convergence test against the previous check, which sets the stop flag.
// One warp. FP64 on GB300 runs at a small fraction of the FP32 rate and a
// block-wide multisection of 256 Sturm counts per round cost ~0.5 ms per call,
// so the bracket starts from the previous check: by interlacing the lowest
// Ritz value only moves down as the tridiagonal grows, so one point just above
// it and 31 at geometric distances below it (2^-52 .. 2^8 of the spectrum's
// scale) bracket it in one round; then 32-point multisection to 2 ulp. The first check, or a
// probe that fails to bracket, starts from the Gershgorin interval.
// With `staged`, alpha and beta are first copied into shared memory (every
// Sturm sweep then reads them at shared-memory latency, not L2's).
__device__ __forceinline__ void stage_tri(const double*& a, const double*& b, int m, int staged) {
  if (!staged) return;
  extern __shared__ double tri_sm[];
  for (int i = threadIdx.x; i < m; i += blockDim.x) {
    tri_sm[i] = a[i];
    tri_sm[m + i] = b[i];
  }
  __syncthreads();
  a = tri_sm;
  b = tri_sm + m;
}

__global__ void k_tri_lowest(Scal S, int check_conv, double tol, int slot, int staged) {
  const int m = S.flags[2];
  if (m <= 0) return;
  const int lane = threadIdx.x & 31;
  const double* A_ = S.alpha;
  const double* B_ = S.beta;
  stage_tri(A_, B_, m, staged);
  double glo = 0, ghi = 0, pm = 0;
  gersh(A_, B_, m, &glo, &ghi, &pm);  // every lane (same values)
  double lo = glo, hi = ghi;
  const double prev = slot > 0 ? S.ritz[slot - 1] : 0.0;
  if (slot > 0 && prev >= glo && prev <= ghi) {
    const double scale = fmax(ghi - glo, fabs(prev));
    // lane 0 just above prev (an eigenvalue lies below it), lanes 1..31 below
    const double x = lane == 0 ? prev + scale * 0x1p-48 : prev - scale * ldexp(1.0, 2 * (lane - 1) - 52);
    const unsigned hit = __ballot_sync(0xffffffffu, sturm_count(A_, B_, m, x, pm) >= 1);
    // counts grow with x, i.e. towards lane 0: the lanes with a hit are 0 .. L-1
    const int L = __popc(hit);
    const double xa = __shfl_sync(0xffffffffu, x, L > 0 ? L - 1 : 0);
    const double xb = __shfl_sync(0xffffffffu, x, L < 32 ? L : 31);
    if (L > 0 && L < 32 && hit == ((1u << L) - 1u)) {
      hi = xa;
      lo = xb;
    }
  }
  for (int it = 0; it < 16; it++) {
    if (hi - lo <= 2 * DBL_EPSILON * fmax(fabs(lo), fabs(hi))) break;
    const double x = lo + (hi - lo) * (lane + 1) / 33.0;
    const unsigned hit = __ballot_sync(0xffffffffu, sturm_count(A_, B_, m, x, pm) >= 1);
    const int f = hit ? __ffs(hit) - 1 : 32;  // first point with an eigenvalue below it
    const double xf = __shfl_sync(0xffffffffu, x, f < 32 ? f : 31);
    const double nhi = f < 32 ? xf : hi;
    const double xprev = __shfl_sync(0xffffffffu, x, f > 0 ? f - 1 : 0);
    const double nlo = f > 0 ? xprev : lo;
    if (nhi == hi && nlo == lo) break;
    hi = nhi;
    lo = nlo;
  }
  if (lane == 0) {
    const double e = 0.5 * (lo + hi);
    S.ritz[slot] = e;
    S.flags[5] = m;  // the tridiagonal size this value belongs to
    if (check_conv && slot > 0 && !S.flags[0]) {
      if (fabs(e - prev) <= tol) S.flags[0] = 1;
    }
  }
}

// Lowest eigenvalue of the m x m tridiagonal (one warp): 32-point multisection
// from the Gershgorin interval to 2 ulp: *out. When the last convergence check
// (ritz[last], recorded for size flags[5]) already found it for this m, that
// value is taken instead (the same 2-ulp multisection).
__global__ void k_tri_min(const double* a, const double* b, int m, double* out, int staged, const double* ritz,
                          const int* flags, int last) {
  if (last >= 0 && flags[5] == m) {
    if (threadIdx.x == 0) *out = ritz[last];
    return;
  }
  stage_tri(a, b, m, staged);
  const int lane = threadIdx.x & 31;
  double lo = 0, hi = 0, pm = 0;
  gersh(a, b, m, &lo, &hi, &pm);
  for (int it = 0; it < 24; it++) {
    if (hi - lo <= 2 * DBL_EPSILON * fmax(fabs(lo), fabs(hi))) break;
    const double x = lo + (hi - lo) * (lane + 1) / 33.0;
    const unsigned hit = __ballot_sync(0xffffffffu, sturm_count(a, b, m, x, pm) >= 1);
    const int f = hit ? __ffs(hit) - 1 : 32;
    const double xf = __shfl_sync(0xffffffffu, x, f < 32 ? f : 31);
    const double xp = __shfl_sync(0xffffffffu, x, f > 0 ? f - 1 : 0);
    const double nhi = f < 32 ? xf : hi, nlo = f > 0 ? xp : lo;
    if (nhi == hi && nlo == lo) break;
    hi = nhi;
    lo = nlo;
  }
  if (lane == 0) *out = 0.5 * (lo + hi);
}

// All eigenvalues (ascending) by bisection, one thread per index.
__global__ void k_tri_all(const double* a, const double* b, int m, double* eig) {
  __shared__ double lo0, hi0, pm;
  if (threadIdx.x == 0) gersh(a, b, m, &lo0, &hi0, &pm);
  __syncthreads();
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < m; k += gridDim.x * blockDim.x) {
    double lo = lo0, hi = hi0;
    for (int it = 0; it < 200; it++) {
      const double mid = 0.5 * (lo + hi);
      if (mid <= lo || mid >= hi) break;
      if (sturm_count(a, b, m, mid, pm) > k) hi = mid;
      else lo = mid;
    }
    eig[k] = 0.5 * (lo + hi);
  }
}

// Eigenvector for eigenvalue *lam_p by inverse iteration (single thread).
// With `staged` (one warp): alpha, beta, the factors and the vector live in
// shared memory (8 m doubles) and only the result is written out.
__global__ void k_tri_vec(const double* a, const double* b, int m, const double* lam_p, double* y, double* work,
                          int staged) {
  if (blockIdx.x != 0) return;
  if (!staged) {
    if (threadIdx.x == 0) tri_inverse_iteration(a, b, m, *lam_p, y, work);
    return;
  }
  stage_tri(a, b, m, staged);
  extern __shared__ double tri_sm[];
  double* sy = tri_sm + 2 * m;
  double* swork = tri_sm + 3 * m;
  if (threadIdx.x == 0) tri_inverse_iteration(a, b, m, *lam_p, sy, swork);
  __syncthreads();
  for (int i = threadIdx.x; i < m; i += blockDim.x) y[i] = sy[i];
}

// psi[r] = sum_l y[l] V_l[r] (GEMV over the Krylov basis); partial |psi|^2.
template <bool CPLX>
__global__ void k_ritz(const double* __restrict__ V, int64_t dim, int m, const double* __restrict__ y,
                       double* __restrict__ psi, double* __restrict__ part_norm) {
  extern __shared__ double ys[];
  for (int t = threadIdx.x; t < m; t += blockDim.x) ys[t] = y[t];
  __syncthreads();
  double nn = 0;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < dim) {
    if (CPLX) {
      double2 acc = make_double2(0, 0);
      for (int k = 0; k < m; k++) {
        const double2 v = reinterpret_cast<const double2*>(V)[(int64_t)k * dim + r];
        acc.x += ys[k] * v.x;
        acc.y += ys[k] * v.y;
      }
      reinterpret_cast<double2*>(psi)[r] = acc;
      nn = acc.x * acc.x + acc.y * acc.y;
    } else {
      double acc = 0;
      for (int k = 0; k < m; k++) acc += ys[k] * V[(int64_t)k * dim + r];
      psi[r] = acc;
      nn = acc * acc;
    }
  }
  __shared__ double red[8];
  for (int o = 16; o > 0; o >>= 1) nn += __shfl_xor_sync(0xffffffffu, nn, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = nn;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < (int)(blockDim.x / 32); i++) s += red[i];
    part_norm[blockIdx.x] = s;
  }
}

// Device start vector: u - 1/2 with u uniform in (0, 1) from splitmix64 of
// (seed, index) (Steele, Lea, Flood 2014), so the start costs no host work.
__global__ void k_rand_fill(double* x, int64_t n, uint64_t seed) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    uint64_t z = seed * 0x9E3779B97F4A7C15ULL + (uint64_t)(i + 1) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    z ^= z >> 31;
    x[i] = ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0) - 0.5;
  }
}

// out = conj(psi) (interleaved complex; a copy when real).
__global__ void k_conj(const double* __restrict__ psi, double* __restrict__ out, int64_t n, int cplx) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = (cplx && (i & 1)) ? -psi[i] : psi[i];
}

__global__ void k_sum(const double* part, int n, double* out) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    double s = 0;
    for (int i = 0; i < n; i++) s += part[i];
    *out = s;
  }
}

__global__ void k_scale_by_norm(double* v, int64_t n, const double* nrm2) {
  const double inv = 1.0 / sqrt(*nrm2);
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] *= inv;
}

// partial Re<a, b> over blocks (real or interleaved complex, n doubles)
__global__ void k_dot_partial(const double* a, const double* b, int64_t n, int cplx, double* part) {
  double s = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    s += a[i] * b[i];  // Re(conj(a) b) = ar br + ai bi for interleaved complex
  (void)cplx;
  __shared__ double red[8];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0;
    for (int i = 0; i < (int)(blockDim.x / 32); i++) t += red[i];
    part[blockIdx.x] = t;
  }
}

}  // namespace

// ---------------------------------------------------------------------------
// MT19937 (Matsumoto & Nishimura 1998) and its 64-bit variant (Nishimura 2000),
// written from the published algorithms: the streams std::mt19937 and the
// reference's genrand64_real3 produce for a given seed.
namespace {
struct MT32 {
  uint32_t s[624];
  int i = 624;
  explicit MT32(uint32_t seed) {
    s[0] = seed;
    for (int k = 1; k < 624; k++) s[k] = 1812433253u * (s[k - 1] ^ (s[k - 1] >> 30)) + (uint32_t)k;
  }
  uint32_t next() {
    if (i >= 624) {
      for (int k = 0; k < 624; k++) {
        const uint32_t y = (s[k] & 0x80000000u) | (s[(k + 1) % 624] & 0x7fffffffu);
        s[k] = s[(k + 397) % 624] ^ (y >> 1) ^ ((y & 1u) ? 0x9908b0dfu : 0u);
      }
      i = 0;
    }
    uint32_t y = s[i++];
    y ^= y >> 11;
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= y >> 18;
    return y;
  }
};
struct MT64 {
  uint64_t s[312];
  int i = 312;
  explicit MT64(uint64_t seed) {
    s[0] = seed;
    for (int k = 1; k < 312; k++) s[k] = 6364136223846793005ULL * (s[k - 1] ^ (s[k - 1] >> 62)) + (uint64_t)k;
  }
  uint64_t next() {
    if (i >= 312) {
      for (int k = 0; k < 312; k++) {
        const uint64_t y = (s[k] & 0xFFFFFFFF80000000ULL) | (s[(k + 1) % 312] & 0x7FFFFFFFULL);
        s[k] = s[(k + 156) % 312] ^ (y >> 1) ^ ((y & 1ULL) ? 0xB5026F5AA96619E9ULL : 0ULL);
      }
      i = 0;
    }
    uint64_t x = s[i++];
    x ^= (x >> 29) & 0x5555555555555555ULL;
    x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
    x ^= (x << 37) & 0xFFF7EEE000000000ULL;
    x ^= x >> 43;
    return x;
  }
  double real3() { return ((double)(next() >> 12) + 0.5) * (1.0 / 4503599627370496.0); }
};

// The reference writes phi_0[i] = complex<double>(draw() - 0.5, draw() - 0.5)
// (lanczos_hamiltonian.cpp:468-476, matrix.cpp:54-70); GCC, which builds it,
// evaluates the two arguments right to left, so the imaginary part is drawn
// first (its recorded Lanczos coefficients in complex sectors agree with this
// order only). Complex sectors follow that order; real sectors, which the
// library runs in real arithmetic, take one draw per entry.
void fill_start(uint64_t seed, int rng, int64_t dim, int cplx, double* out) {
  const int64_t n = dim * (cplx ? 2 : 1);
  double nrm = 0;
  MT32 g32((uint32_t)seed);
  MT64 g64(rng == 0 ? 0 : seed);
  auto draw = [&]() { return rng == 0 ? g32.next() * 1.0 / 4294967295.0 - 0.5 : g64.real3() - 0.5; };
  for (int64_t i = 0; i < n; i += (cplx ? 2 : 1)) {
    if (cplx) {
      out[i + 1] = draw();
      out[i] = draw();
      nrm += out[i] * out[i] + out[i + 1] * out[i + 1];
    } else {
      out[i] = draw();
      nrm += out[i] * out[i];
    }
  }
  nrm = sqrt(nrm);
  for (int64_t i = 0; i < n; i++) out[i] /= nrm;
}
}  // namespace

// ---------------------------------------------------------------------------
struct blqh_lanczos {
  blqh_ctx* ctx = nullptr;
  const blqh_csr* M = nullptr;
  blqh_lanczos_opts o{};
  int64_t dim = 0;
  int cplx = 0, vw = 1;
  int mmax = 0;
  double* V = nullptr;     // [(mmax+1) * dim * vw]
  double* w = nullptr;     // [dim * vw]
  double* psi = nullptr;   // [dim * vw]
  double* scal = nullptr;  // scalar block
  Scal S{};
  double* part = nullptr;  // dot partials [nblk_dot * (mmax+1) * 2]
  double* pnorm = nullptr; // [max(nblk_dot, nblk_upd)]
  double* work = nullptr;  // tridiagonal work [5*mmax + ...]
  double* y = nullptr;     // [mmax] Ritz coefficients
  float2* xs = nullptr;    // [dim * vw] (hi, lo) split of the SpMV input (double-float accumulation)
  float* Vh = nullptr;     // [(mmax+1) * pld] FP32 planes of V for the Gram-Schmidt pass (or null)
  float* Vl = nullptr;
  int64_t pld = 0;         // plane row stride (floats): dim * vw rounded up to a multiple of 4
  int nblk_dot = 0, nblk_upd = 0;
  int steps = 0;
  int last_check = -1;  // ritz[] slot of the last convergence check of the last run (-1: none)
  bool started = false, iterated = false, have_psi = false;
};

namespace {

void free_lanczos(blqh_lanczos* L) {
  if (!L) return;
  dev_free(L->xs);
  dev_free(L->Vh);
  dev_free(L->Vl);
  dev_free(L->V);
  dev_free(L->w);
  dev_free(L->psi);
  dev_free(L->scal);
  dev_free(L->part);
  dev_free(L->pnorm);
  dev_free(L->work);
  dev_free(L->y);
  delete L;
}

int spmv_lpr(double mean_row) {
  if (mean_row >= 96) return 32;
  if (mean_row >= 40) return 16;
  if (mean_row >= 16) return 8;
  return 4;
}

template <class VT, bool CPLX>
void spmv_t(blqh_ctx* ctx, const blqh_csr* M, const double* x, double* y, const double* bptr, const double* xprev,
            const int* stop) {
  const int lpr = M->lanes_per_row;
  const int threads = 256;
  const int64_t groups = M->dim;
  int64_t blocks = (groups * lpr + threads - 1) / threads;
  const int64_t cap = (int64_t)ctx->num_sms * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  auto rp = M->d_row_ptr;
  auto cl = M->d_col;
  auto vl = reinterpret_cast<const VT*>(M->d_val);
  switch (lpr) {
    case 32: k_spmv<VT, CPLX, 32><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, x, y, M->dim, bptr, xprev, stop); break;
    case 16: k_spmv<VT, CPLX, 16><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, x, y, M->dim, bptr, xprev, stop); break;
    case 8: k_spmv<VT, CPLX, 8><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, x, y, M->dim, bptr, xprev, stop); break;
    default: k_spmv<VT, CPLX, 4><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, x, y, M->dim, bptr, xprev, stop); break;
  }
}

template <bool CPLX>
void spmv_df_t(blqh_ctx* ctx, const blqh_csr* M, const float2* xs, double* y, const double* bptr,
               const double* xprev, const int* stop) {
  if (M->blk_state > 0 && blocked_mode() >= 0) {
    blocked_spmv(ctx, M, xs, y, bptr, xprev, stop);
    return;
  }
  const int lpr = M->lanes_per_row;
  const int threads = 256;
  int64_t blocks = (M->dim * lpr + threads - 1) / threads;
  const int64_t cap = (int64_t)ctx->num_sms * 16;
  if (blocks > cap) blocks = cap;
  if (blocks < 1) blocks = 1;
  auto rp = M->d_row_ptr;
  auto cl = M->d_col;
  auto vl = reinterpret_cast<const float*>(M->d_val);
  if (!CPLX && lpr >= 8) {
    if (lpr == 32)
      k_spmv_df_v4<32><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, xs, y, M->dim, bptr, xprev, stop);
    else if (lpr == 16)
      k_spmv_df_v4<16><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, xs, y, M->dim, bptr, xprev, stop);
    else
      k_spmv_df_v4<8><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, xs, y, M->dim, bptr, xprev, stop);
    return;
  }
  switch (lpr) {
    case 32: k_spmv_df<CPLX, 32><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, xs, y, M->dim, bptr, xprev, stop); break;
    case 16: k_spmv_df<CPLX, 16><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, xs, y, M->dim, bptr, xprev, stop); break;
    case 8: k_spmv_df<CPLX, 8><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, xs, y, M->dim, bptr, xprev, stop); break;
    default: k_spmv_df<CPLX, 4><<<(int)blocks, threads, 0, ctx->stream>>>(rp, cl, vl, xs, y, M->dim, bptr, xprev, stop); break;
  }
}

// y = H x - b xprev. With an FP32-valued CSR and a split buffer xs, the product
// accumulates in double-float (k_spmv_df); otherwise in native FP64 (k_spmv).
void spmv_dev(blqh_ctx* ctx, const blqh_csr* M, const double* x, double* y, const double* bptr = nullptr,
              const double* xprev = nullptr, const int* stop = nullptr, float2* xs = nullptr,
              bool xs_ready = false) {
  if (xs && M->precision == BLQH_VAL_FP32) {
    const int64_t n = M->dim * (M->is_complex ? 2 : 1);
    if (!xs_ready) {  // else the caller's previous kernel left x's split in xs
      TimerScope tm(ctx, TM_MISC);
      k_split<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(x, xs, n, stop);
      count_launch(ctx, TM_MISC);
    }
    TimerScope ts(ctx, TM_SPMV);
    if (M->is_complex) spmv_df_t<true>(ctx, M, xs, y, bptr, xprev, stop);
    else spmv_df_t<false>(ctx, M, xs, y, bptr, xprev, stop);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_SPMV);
    return;
  }
  TimerScope ts(ctx, TM_SPMV);
  if (M->is_complex) {
    if (M->precision == BLQH_VAL_FP64) spmv_t<double2, true>(ctx, M, x, y, bptr, xprev, stop);
    else spmv_t<float2, true>(ctx, M, x, y, bptr, xprev, stop);
  } else {
    if (M->precision == BLQH_VAL_FP64) spmv_t<double, false>(ctx, M, x, y, bptr, xprev, stop);
    else spmv_t<float, false>(ctx, M, x, y, bptr, xprev, stop);
  }
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_SPMV);
}

// Dynamic shared memory of the tridiagonal kernels: `per` doubles per Lanczos
// step when that fits in 48 KB, else 0 (they then read global memory).
int tri_smem(const blqh_lanczos* L, int per) {
  const size_t b = (size_t)per * (L->mmax + 1) * sizeof(double);
  return b <= 48 * 1024 ? (int)b : 0;
}

template <bool CPLX>
void gs_pass(blqh_lanczos* L, int k0, int k1, int j, int stage) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  const int stride = L->mmax + 1;
  const int cond = (stage == 2);
  if (L->Vh && stage == 2)  // the full pass on the FP32 planes (the local step stays in FP64)
    k_dots_df<CPLX><<<L->nblk_dot, 256, 0, st>>>(L->Vh, L->Vl, L->pld, L->dim, k0, k1, L->w, L->part, stride,
                                                 L->S.flags, cond);
  else
    k_dots<CPLX><<<L->nblk_dot, 256, 0, st>>>(L->V, L->dim, k0, k1, L->w, L->part, stride, L->pnorm, L->S.flags,
                                              cond);
  k_reduce_dots<<<k1 - k0 + 1, 256, 0, st>>>(L->part, L->nblk_dot, stride, k0, k1, L->pnorm, L->S, j, stage);
  const double* hc = (stage == 1) ? L->S.h : L->S.h2;
  const size_t hsm = 2 * (k1 - k0) * (sizeof(double) + sizeof(float));
  if (L->Vh)
    k_update_pl<CPLX><<<L->nblk_upd, UPD_THREADS, hsm, st>>>(L->V, L->Vh, L->pld, L->dim, k0, k1, hc, L->w,
                                                             L->pnorm, L->S.flags, cond);
  else
    k_update<CPLX><<<L->nblk_upd, UPD_THREADS, hsm, st>>>(L->V, L->dim, k0, k1, hc, L->w, L->pnorm, L->S.flags,
                                                          cond);
  count_launch(ctx, TM_REORTH, 3);
}

template <bool CPLX>
void lanczos_step(blqh_lanczos* L, int j) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = L->dim * L->vw;
  double* vj = L->V + (int64_t)j * n;
  const double* vprev = j > 0 ? L->V + (int64_t)(j - 1) * n : nullptr;
  // from the second step on, the previous step's k_scale left v_j's split in xs
  spmv_dev(ctx, L->M, vj, L->w, j > 0 ? L->S.beta + j : nullptr, vprev, L->S.flags, L->xs, j > 0);
  {
    TimerScope ts(ctx, TM_REORTH);
    // three-term step: the SpMV removed beta_j v_{j-1}; remove the v_j component
    // (alpha_j). With reorth, one classical Gram-Schmidt pass against every stored
    // vector follows; taking the local step first keeps that pass from having to
    // be repeated (the norm drop of the alpha_j removal no longer enters it).
    gs_pass<CPLX>(L, j, j + 1, j, 1);
    // the step's last norm step also sets beta_{j+1} (breakdown below 1e-13 of |alpha_j| + beta_j)
    k_norm_step<<<1, 256, 0, st>>>(L->pnorm, L->nblk_upd, L->S, j, 1, L->o.reorth ? 1 : 0,
                                    L->o.reorth ? 0.0 : 1e-13);
    if (L->o.reorth) {
      gs_pass<CPLX>(L, 0, j + 1, j, 2);
      k_norm_step<<<1, 256, 0, st>>>(L->pnorm, L->nblk_upd, L->S, j, 2, 0, 1e-13);
    }
    k_scale<<<grid_for(ctx, n, 256, 8), 256, 0, st>>>(L->w, L->V + (int64_t)(j + 1) * n, n, L->S, j,
                                                      L->Vh ? L->Vh + (int64_t)(j + 1) * L->pld : nullptr,
                                                      L->Vl ? L->Vl + (int64_t)(j + 1) * L->pld : nullptr,
                                                      L->M->precision == BLQH_VAL_FP32 ? L->xs : nullptr);
    count_launch(ctx, TM_REORTH, L->o.reorth ? 3 : 2);
  }
}

void iterate_impl(blqh_lanczos* L) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  if (!L->started) {
    const int64_t n = L->dim * L->vw;
    if (L->o.rng == 2) {
      TimerScope tm(ctx, TM_MISC);
      const int blocks = grid_for(ctx, n, 256, 4);
      k_rand_fill<<<grid_for(ctx, n, 256, 8), 256, 0, st>>>(L->V, n, L->o.seed);
      k_dot_partial<<<blocks, 256, 0, st>>>(L->V, L->V, n, 0, L->pnorm);
      k_sum<<<1, 1, 0, st>>>(L->pnorm, blocks, L->S.nrm + 2);
      k_scale_by_norm<<<grid_for(ctx, n, 256, 8), 256, 0, st>>>(L->V, n, L->S.nrm + 2);
      BLQH_TRY_CUDA(ctx, cudaGetLastError());
      count_launch(ctx, TM_MISC, 4);
    } else {
      std::vector<double> x(n);
      fill_start(L->o.seed, L->o.rng, L->dim, L->cplx, x.data());
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(L->V, x.data(), x.size() * 8, cudaMemcpyHostToDevice, st));
      BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(st));
    }
    L->started = true;
  }
  if (L->Vh) {  // planes of the start vector (the steps write the others)
    TimerScope tm(ctx, TM_MISC);
    const int64_t n = L->dim * L->vw;
    k_planes<<<grid_for(ctx, n, 256, 8), 256, 0, st>>>(L->V, L->Vh, L->Vl, n);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_MISC);
  }
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(L->S.flags, 0, 4 * sizeof(int), st));
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(L->S.flags + 5, 0xFF, sizeof(int), st));  // no check's size yet
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(L->S.beta, 0, sizeof(double), st));
  const int chunk = std::max(1, L->o.check_every);
  const bool conv = L->o.tol > 0;
  int* hflags = reinterpret_cast<int*>(ctx->pinned);
  cudaEvent_t ev[2];
  cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming);
  cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming);
  int launched_chunks = 0;
  int j = 0;
  bool stop = false;
  while (j < L->mmax && !stop) {
    const int jend = std::min(L->mmax, j + chunk);
    for (; j < jend; j++) {
      if (L->cplx) lanczos_step<true>(L, j);
      else lanczos_step<false>(L, j);
    }
    if (conv) {  // with tol = 0 the recurrence runs to max_steps: no check needed
      TimerScope tm(ctx, TM_MISC);
      k_tri_lowest<<<1, 32, tri_smem(L, 2), st>>>(L->S, 1, L->o.tol, launched_chunks, tri_smem(L, 2) > 0);
      BLQH_TRY_CUDA(ctx, cudaGetLastError());
      count_launch(ctx, TM_MISC);
    }
    int* slot = hflags + 4 * (launched_chunks & 1);
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(slot, L->S.flags, 4 * sizeof(int), cudaMemcpyDeviceToHost, st));
    BLQH_TRY_CUDA(ctx, cudaEventRecord(ev[launched_chunks & 1], st));
    launched_chunks++;
    // wait for the previous chunk's flags (the current chunk keeps the GPU busy)
    if (launched_chunks >= 2) {
      const int prev = (launched_chunks - 2) & 1;
      BLQH_TRY_CUDA(ctx, cudaEventSynchronize(ev[prev]));
      if (hflags[4 * prev]) stop = true;
    }
  }
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(st));
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  int f[4];
  BLQH_TRY_CUDA(ctx, cudaMemcpy(f, L->S.flags, sizeof(f), cudaMemcpyDeviceToHost));
  L->steps = f[2];
  L->last_check = conv && launched_chunks > 0 ? launched_chunks - 1 : -1;
  L->iterated = true;
  L->have_psi = false;
}

void ritz_impl(blqh_lanczos* L) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  const int m = L->steps;
  TimerScope tm(ctx, TM_MISC);
  // only the lowest Ritz pair is needed here (blqh_lanczos_eig gives them all)
  k_tri_min<<<1, 32, tri_smem(L, 2), st>>>(L->S.alpha, L->S.beta, m, L->work + 6 * L->mmax, tri_smem(L, 2) > 0,
                                            L->S.ritz, L->S.flags, L->last_check);
  k_tri_vec<<<1, 32, tri_smem(L, 8), st>>>(L->S.alpha, L->S.beta, m, L->work + 6 * L->mmax, L->y, L->work,
                                            tri_smem(L, 8) > 0);
  const int blocks = (int)((L->dim + 255) / 256);
  if (L->cplx)
    k_ritz<true><<<blocks, 256, m * sizeof(double), st>>>(L->V, L->dim, m, L->y, L->psi, L->pnorm);
  else
    k_ritz<false><<<blocks, 256, m * sizeof(double), st>>>(L->V, L->dim, m, L->y, L->psi, L->pnorm);
  k_sum<<<1, 1, 0, st>>>(L->pnorm, blocks, L->S.nrm + 2);
  k_scale_by_norm<<<grid_for(ctx, L->dim * L->vw, 256, 8), 256, 0, st>>>(L->psi, L->dim * L->vw, L->S.nrm + 2);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_MISC, 5);
  L->have_psi = true;
}

// <x|H|x> with the stored CSR values (x normalized, on the device).
double rq_stored(blqh_lanczos* L, const double* x) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  spmv_dev(ctx, L->M, x, L->w);
  const int64_t n = L->dim * L->vw;
  const int blocks = grid_for(ctx, n, 256, 4);
  TimerScope tm(ctx, TM_MISC);
  k_dot_partial<<<blocks, 256, 0, st>>>(x, L->w, n, L->cplx, L->pnorm);
  k_sum<<<1, 1, 0, st>>>(L->pnorm, blocks, L->S.nrm + 3);
  count_launch(ctx, TM_MISC, 2);
  double e = 0;
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(&e, L->S.nrm + 3, 8, cudaMemcpyDeviceToHost, st));
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(st));
  return e;
}

// K10 for the SpMV of a matrix of at least 2^15 rows: the row kernel at 4, 8,
// 16 and 32 lanes per row and, for FP32 values with double-float accumulation,
// the blocked kernel (spmv_blocked.cu) are timed on this matrix (x = 0, three
// products each); the choice is cached per class as (lanes, blocked).
// BLQH_SPMV_BLOCKED=1 forces the blocked kernel, =0 rules it out.
void tune_spmv(blqh_lanczos* L) {
  blqh_csr* M = const_cast<blqh_csr*>(L->M);
  blqh_ctx* ctx = L->ctx;
  const int bm = blocked_mode();
  const bool can_blk = M->precision == BLQH_VAL_FP32 && L->xs && bm >= 0;
  if (can_blk && bm == 1) {
    blocked_prepare(ctx, M);
    return;
  }
  if (M->dim < (1 << 15) || !tune_enabled()) {
    if (can_blk && M->dim >= (1 << 15)) blocked_prepare(ctx, M);
    return;
  }
  const int mode = M->precision == BLQH_VAL_FP32 ? (L->o.accumulate ? 1 : 2) : 0;
  const std::string key = tune_key("spmv", mode, M->is_complex, M->dim, M->mean_row, 1);
  int lpr = 0, blk = 0;
  if (!tune_lookup(key, &lpr, &blk)) {
    const int64_t n = L->dim * L->vw;
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(L->V, 0, n * 8, ctx->stream));
    cudaEvent_t e0, e1;
    BLQH_TRY_CUDA(ctx, cudaEventCreate(&e0));
    BLQH_TRY_CUDA(ctx, cudaEventCreate(&e1));
    auto time3 = [&]() {
      spmv_dev(ctx, M, L->V, L->w, nullptr, nullptr, nullptr, L->xs);  // warm-up
      BLQH_TRY_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
      for (int r = 0; r < 3; r++) spmv_dev(ctx, M, L->V, L->w, nullptr, nullptr, nullptr, L->xs);
      BLQH_TRY_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaEventSynchronize(e1));
      float ms = 0;
      BLQH_TRY_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
      return (double)ms;
    };
    double best = 1e30;
    if (M->blk_state > 0) blocked_release(M);
    for (int c : {4, 8, 16, 32}) {
      M->lanes_per_row = c;
      const double ms = time3();
      if (ms < best) {
        best = ms;
        lpr = c;
      }
    }
    M->lanes_per_row = lpr;
    if (can_blk && blocked_prepare(ctx, M)) {
      const double ms = time3();
      if (blocked_error(ctx, M) == BLQH_OK && ms < best) {
        best = ms;
        blk = 1;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tune_store(key, lpr, blk, best / 3);
  }
  M->lanes_per_row = lpr;
  if (blk && can_blk) blocked_prepare(ctx, M);
  else if (M->blk_state > 0) blocked_release(M);
}

// The full Gram-Schmidt pass of FP32-valued runs (accumulate = 0) works on FP32
// planes of the Krylov basis; BLQH_GS_FP64=1 keeps it in FP64.
bool gs_planes_enabled() {
  const char* e = getenv("BLQH_GS_FP64");
  return !(e && e[0] == '1');
}

// BLQH_RQ_REGEN=1 finishes FP32-valued runs with the regenerated FP64 elements
// (the row generator again) instead of the stored FP32 rests.
bool regen_forced() {
  const char* e = getenv("BLQH_RQ_REGEN");
  return e && e[0] == '1';
}

// <psi|H|psi> from the FP32 values and their stored FP32 rests (k_rq_res).
double rayleigh_res_impl(blqh_lanczos* L) {
  blqh_ctx* ctx = L->ctx;
  const blqh_csr* M = L->M;
  TimerScope ts(ctx, TM_BUILD);
  spmv_dev(ctx, M, L->psi, L->w, nullptr, nullptr, nullptr, L->xs);  // y = H32 psi; xs = (hi, lo) of psi
  const int grid = grid_for(ctx, M->dim * 32, 256, 8);
  if (M->is_complex)
    k_rq_res<true><<<grid, 256, 0, ctx->stream>>>(M->d_row_ptr, M->d_col, M->d_res, L->xs, L->psi, L->w, M->dim,
                                                  L->pnorm);
  else
    k_rq_res<false><<<grid, 256, 0, ctx->stream>>>(M->d_row_ptr, M->d_col, M->d_res, L->xs, L->psi, L->w, M->dim,
                                                   L->pnorm);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_BUILD);
  std::vector<double> h(grid);
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(h.data(), L->pnorm, grid * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  double e = 0;
  for (int b = 0; b < grid; b++) e += h[b];
  return e;
}

blqh_lanczos* create_impl(blqh_ctx* ctx, const blqh_csr* M, const blqh_lanczos_opts& o) {
  blqh_lanczos* L = new blqh_lanczos();
  L->ctx = ctx;
  L->M = M;
  L->o = o;
  L->dim = M->dim;
  L->cplx = M->is_complex;
  L->vw = L->cplx ? 2 : 1;
  L->mmax = (int)std::min<int64_t>(o.max_steps, M->dim);
  const_cast<blqh_csr*>(M)->lanes_per_row = spmv_lpr(M->mean_row);
  const int upd_smem = 2 * (L->mmax + 1) * (int)(sizeof(double) + sizeof(float));
  smem_attr_at_least(k_update<false>, upd_smem);
  smem_attr_at_least(k_update<true>, upd_smem);
  smem_attr_at_least(k_update_pl<false>, upd_smem);
  smem_attr_at_least(k_update_pl<true>, upd_smem);
  try {
    const int64_t n = L->dim * L->vw;
    L->V = dalloc<double>(ctx, (size_t)(L->mmax + 1) * n);
    L->w = dalloc<double>(ctx, n);
    L->psi = dalloc<double>(ctx, n);
    const int m = L->mmax;
    const size_t ns = (size_t)m + (m + 1) + 2 * (m + 1) + 2 * (m + 1) + 4 + m + 4;
    L->scal = dalloc<double>(ctx, ns);
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(L->scal, 0, ns * 8, ctx->stream));
    double* p = L->scal;
    L->S.alpha = p;
    p += m;
    L->S.beta = p;
    p += m + 1;
    L->S.h = p;
    p += 2 * (m + 1);
    L->S.h2 = p;
    p += 2 * (m + 1);
    L->S.nrm = p;
    p += 4;
    L->S.ritz = p;
    p += m;
    L->S.flags = reinterpret_cast<int*>(p);
    L->nblk_dot = (int)((L->dim + GS_ROWS - 1) / GS_ROWS);
    L->nblk_upd = (int)((L->dim + UPD_THREADS - 1) / UPD_THREADS);
    L->part = dalloc<double>(ctx, (size_t)L->nblk_dot * (m + 1) * 2);
    // block partials of the dot, update and norm kernels, and of k_rq_res (at most 8 blocks per SM)
    L->pnorm = dalloc<double>(ctx, std::max<int64_t>(std::max<int64_t>(std::max(L->nblk_dot, L->nblk_upd),
                                                                       (L->dim + 255) / 256),
                                                     (int64_t)ctx->num_sms * 8) +
                                       1024);
    L->work = dalloc<double>(ctx, 8 * (size_t)m + 16);
    L->y = dalloc<double>(ctx, m + 1);
    if (M->precision == BLQH_VAL_FP32 && o.accumulate == 0) L->xs = dalloc<float2>(ctx, n + 2);
    if (M->precision == BLQH_VAL_FP32 && o.accumulate == 0 && o.reorth && gs_planes_enabled()) {
      // the planes double the Krylov basis' memory; without room for them the
      // run keeps the FP64 Gram-Schmidt kernels
      const int64_t pld = (n + 3) & ~(int64_t)3;
      try {
        L->Vh = dalloc<float>(ctx, (size_t)(L->mmax + 1) * pld);
        L->Vl = dalloc<float>(ctx, (size_t)(L->mmax + 1) * pld);
      } catch (const BlqhError& e) {
        if (e.code != BLQH_ERR_NOMEM) throw;
        dev_free(L->Vh);
        dev_free(L->Vl);
        L->Vh = L->Vl = nullptr;
        ctx->last_error.clear();
      }
      if (L->Vh) {
        L->pld = pld;
        BLQH_TRY_CUDA(ctx, cudaMemsetAsync(L->Vh, 0, (size_t)(L->mmax + 1) * pld * sizeof(float), ctx->stream));
        BLQH_TRY_CUDA(ctx, cudaMemsetAsync(L->Vl, 0, (size_t)(L->mmax + 1) * pld * sizeof(float), ctx->stream));
        L->nblk_upd = (int)((n + 4 * UPD_THREADS - 1) / (4 * UPD_THREADS));
      }
    }
    tune_spmv(L);
  } catch (const BlqhError&) {
    free_lanczos(L);
    throw;
  }
  return L;
}

}  // namespace

extern "C" {

int blqh_spmv(blqh_ctx* ctx, const blqh_csr* m, const double* x, double* y) {
  if (!ctx || !m || !x || !y) return BLQH_ERR_ARG;
  double* dx = nullptr;
  double* dy = nullptr;
  float2* xs = nullptr;
  int rc = BLQH_OK;
  try {
    const int64_t n = m->dim * (m->is_complex ? 2 : 1);
    dx = dalloc<double>(ctx, n);
    dy = dalloc<double>(ctx, n);
    if (m->precision == BLQH_VAL_FP32) xs = dalloc<float2>(ctx, n + 2);
    if (xs && blocked_mode() == 1) blocked_prepare(ctx, const_cast<blqh_csr*>(m));
    const_cast<blqh_csr*>(m)->lanes_per_row = spmv_lpr(m->mean_row);
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(dx, x, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    spmv_dev(ctx, m, dx, dy, nullptr, nullptr, nullptr, xs);
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(y, dy, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    rc = blocked_error(ctx, m);
  } catch (const BlqhError& e) {
    rc = e.code;
  }
  dev_free(dx);
  dev_free(dy);
  dev_free(xs);
  return rc;
}

int blqh_lanczos_create(blqh_ctx* ctx, const blqh_csr* m, const blqh_lanczos_opts* o, blqh_lanczos** out) {
  if (!ctx || !m || !o || !out) return BLQH_ERR_ARG;
  *out = nullptr;
  if (o->max_steps < 1 || o->max_steps > BLQH_MAX_LAMBDA || o->check_every < 1 || o->rng < 0 || o->rng > 2) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_lanczos_create: max_steps in [1, 4096], check_every >= 1, rng 0, 1 or 2");
    return BLQH_ERR_ARG;
  }
  try {
    *out = create_impl(ctx, m, *o);
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_set_start(blqh_lanczos* L, const double* x) {
  if (!L || !x) return BLQH_ERR_ARG;
  blqh_ctx* ctx = L->ctx;
  try {
    const int64_t n = L->dim * L->vw;
    double nrm = 0;
    for (int64_t i = 0; i < n; i++) nrm += x[i] * x[i];
    if (!(nrm > 0) || !std::isfinite(nrm)) {
      set_error(ctx, BLQH_ERR_ARG, "blqh_lanczos_set_start: start vector is zero or not finite");
      return BLQH_ERR_ARG;
    }
    std::vector<double> h(x, x + n);
    const double inv = 1.0 / sqrt(nrm);
    for (auto& v : h) v *= inv;
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(L->V, h.data(), n * 8, cudaMemcpyHostToDevice, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    L->started = true;
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_iterate(blqh_lanczos* L, int* steps_done) {
  if (!L) return BLQH_ERR_ARG;
  try {
    cudaSetDevice(L->ctx->device);
    iterate_impl(L);
  } catch (const BlqhError& e) {
    return e.code;
  }
  if (const int rc = blocked_error(L->ctx, L->M)) return rc;
  if (steps_done) *steps_done = L->steps;
  return BLQH_OK;
}

int blqh_lanczos_coeffs(blqh_lanczos* L, double* alpha, double* beta) {
  if (!L) return BLQH_ERR_ARG;
  if (!L->iterated) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_coeffs: call blqh_lanczos_iterate first");
    return BLQH_ERR_STATE;
  }
  blqh_ctx* ctx = L->ctx;
  try {
    const int m = L->steps;
    if (alpha) BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(alpha, L->S.alpha, m * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (beta) {
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(beta, L->S.beta, (m + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      beta[0] = 1.0;
    }
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_eig(blqh_lanczos* L, double* eigenvalues, double* psi0) {
  if (!L) return BLQH_ERR_ARG;
  if (!L->iterated || L->steps < 1) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_eig: call blqh_lanczos_iterate first");
    return BLQH_ERR_STATE;
  }
  blqh_ctx* ctx = L->ctx;
  try {
    const int m = L->steps;
    k_tri_all<<<1, 256, 0, ctx->stream>>>(L->S.alpha, L->S.beta, m, L->work + 6 * L->mmax);
    k_tri_vec<<<1, 32, tri_smem(L, 8), ctx->stream>>>(L->S.alpha, L->S.beta, m, L->work + 6 * L->mmax, L->y,
                                                      L->work, tri_smem(L, 8) > 0);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_MISC, 2);
    if (eigenvalues)
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(eigenvalues, L->work + 6 * L->mmax, m * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (psi0) BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(psi0, L->y, m * 8, cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_ritz_vector(blqh_lanczos* L, double* psi) {
  if (!L) return BLQH_ERR_ARG;
  if (!L->iterated || L->steps < 1) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_ritz_vector: call blqh_lanczos_iterate first");
    return BLQH_ERR_STATE;
  }
  blqh_ctx* ctx = L->ctx;
  try {
    ritz_impl(L);
    if (psi)
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(psi, L->psi, L->dim * L->vw * 8, cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_rayleigh(blqh_lanczos* L, double* energy) {
  if (!L || !energy) return BLQH_ERR_ARG;
  if (!L->have_psi) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_rayleigh: call blqh_lanczos_ritz_vector first");
    return BLQH_ERR_STATE;
  }
  try {
    *energy = rq_stored(L, L->psi);
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_rayleigh_conj(blqh_lanczos* L, const blqh_basis* b, const blqh_params* p, double* energy) {
  if (!L || !energy || (!b != !p)) return BLQH_ERR_ARG;
  if (!L->have_psi) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_rayleigh_conj: call blqh_lanczos_ritz_vector first");
    return BLQH_ERR_STATE;
  }
  if (b && (b->model != BLQH_MODEL_SPINLESS || b->dim != L->dim)) {
    set_error(L->ctx, BLQH_ERR_ARG, "blqh_lanczos_rayleigh_conj: spinless basis of the matrix's sector expected");
    return BLQH_ERR_ARG;
  }
  blqh_ctx* ctx = L->ctx;
  double* xc = nullptr;
  int rc = BLQH_OK;
  try {
    const int64_t n = L->dim * L->vw;
    xc = dalloc<double>(ctx, n);
    k_conj<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(L->psi, xc, n, L->cplx);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_MISC);
    *energy = b ? rayleigh_regen_impl(ctx, b, *p, xc, L->cplx != 0) : rq_stored(L, xc);
  } catch (const BlqhError& e) {
    rc = e.code;
  }
  dev_free(xc);
  return rc;
}

int blqh_lanczos_rayleigh_fp64(blqh_lanczos* L, const blqh_basis* b, const blqh_params* p, double* energy) {
  if (!L || !b || !p || !energy) return BLQH_ERR_ARG;
  if (!L->have_psi) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_rayleigh_fp64: call blqh_lanczos_ritz_vector first");
    return BLQH_ERR_STATE;
  }
  if (b->model != BLQH_MODEL_SPINLESS) {
    set_error(L->ctx, BLQH_ERR_ARG, "blqh_lanczos_rayleigh_fp64: spinless bases only (use blqh_lanczos_rayleigh)");
    return BLQH_ERR_ARG;
  }
  if (b->dim != L->dim) {
    set_error(L->ctx, BLQH_ERR_ARG, "blqh_lanczos_rayleigh_fp64: basis does not match the matrix");
    return BLQH_ERR_ARG;
  }
  try {
    if (L->M->d_res && L->xs && !regen_forced()) *energy = rayleigh_res_impl(L);
    else *energy = rayleigh_regen_impl(L->ctx, b, *p, L->psi, L->cplx != 0);
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_destroy(blqh_lanczos* L) {
  free_lanczos(L);
  return BLQH_OK;
}

int blqh_start_vector(uint64_t seed, int rng, int64_t dim, int is_complex, double* out) {
  if (!out || dim < 0 || (rng != 0 && rng != 1)) return BLQH_ERR_ARG;
  fill_start(seed, rng, dim, is_complex, out);
  return BLQH_OK;
}

int blqh_ground_state(blqh_ctx* ctx, const blqh_sector* s, const blqh_params* p, int prec,
                      const blqh_lanczos_opts* o, const double* start, double* psi, blqh_result* out) {
  if (!ctx || !s || !p || !o || !out) return BLQH_ERR_ARG;
  blqh_basis* B = nullptr;
  blqh_csr* M = nullptr;
  blqh_lanczos* L = nullptr;
  int rc = blqh_basis_build(ctx, s, &B);
  if (rc == BLQH_OK) rc = blqh_hamil_build(ctx, B, p, prec, &M);
  if (rc == BLQH_OK) rc = blqh_lanczos_create(ctx, M, o, &L);
  if (rc == BLQH_OK && start) rc = blqh_lanczos_set_start(L, start);
  int steps = 0;
  if (rc == BLQH_OK) rc = blqh_lanczos_iterate(L, &steps);
  if (rc == BLQH_OK) rc = blqh_lanczos_ritz_vector(L, psi);
  double e = 0;
  if (rc == BLQH_OK) {
    if (prec == BLQH_VAL_FP64) rc = blqh_lanczos_rayleigh(L, &e);
    else rc = blqh_lanczos_rayleigh_fp64(L, B, p, &e);
  }
  if (rc == BLQH_OK) {
    double r0 = 0;
    cudaMemcpy(&r0, L->work + 6 * L->mmax, 8, cudaMemcpyDeviceToHost);
    out->energy = e;
    out->ritz0 = r0;
    out->steps = steps;
    out->dim = B->dim;
    out->nnz = M->nnz;
  }
  blqh_lanczos_destroy(L);
  blqh_csr_destroy(M);
  blqh_basis_destroy(B);
  return rc;
}

int blqh_lanczos_observables(blqh_lanczos* L, const blqh_basis* b, double* sz, double* sx, double* occ) {
  if (!L || !b) return BLQH_ERR_ARG;
  if (!L->have_psi) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_observables: call blqh_lanczos_ritz_vector first");
    return BLQH_ERR_STATE;
  }
  if (b->dim != L->dim) {
    set_error(L->ctx, BLQH_ERR_ARG, "blqh_lanczos_observables: basis does not match the Hamiltonian");
    return BLQH_ERR_ARG;
  }
  try {
    observables_impl(L->ctx, b, L->psi, L->cplx, sz, sx, occ);
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_rayleigh_fp64_spin(blqh_lanczos* L, const blqh_basis* b, const blqh_params_spin* p,
                                    double* energy) {
  if (!L || !b || !p || !energy) return BLQH_ERR_ARG;
  if (!L->have_psi) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_rayleigh_fp64_spin: call blqh_lanczos_ritz_vector first");
    return BLQH_ERR_STATE;
  }
  if (b->model != BLQH_MODEL_SPINFUL || b->dim != L->dim) {
    set_error(L->ctx, BLQH_ERR_ARG, "blqh_lanczos_rayleigh_fp64_spin: spinful basis of the matrix's sector expected");
    return BLQH_ERR_ARG;
  }
  try {
    *energy = spin_rayleigh_regen_impl(L->ctx, b, *p, L->psi);
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_observables_spin(blqh_lanczos* L, const blqh_basis* b, double* out) {
  if (!L || !b || !out) return BLQH_ERR_ARG;
  if (!L->have_psi) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_observables_spin: call blqh_lanczos_ritz_vector first");
    return BLQH_ERR_STATE;
  }
  if (b->model != BLQH_MODEL_SPINFUL || b->dim != L->dim) {
    set_error(L->ctx, BLQH_ERR_ARG, "blqh_lanczos_observables_spin: spinful basis of the matrix's sector expected");
    return BLQH_ERR_ARG;
  }
  try {
    spin_observables_impl(L->ctx, b, L->psi, L->cplx, out);
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_debug_spmv_layout(const blqh_csr* M) {
  if (!M) return -1;
  return M->blk_state > 0 ? (M->blk_dict > 0 ? 2 : 1) : 0;
}

}  // extern "C"
