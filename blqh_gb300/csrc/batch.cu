// K9: batched sweep. Many (sector, parameter point) instances of uneven
// dimension advance in ONE persistent kernel: each thread block takes the next
// instance from a device work queue (ordered by decreasing cost), runs its
// whole Lanczos recurrence with full FP64 reorthogonalization, solves its
// tridiagonal and forms its ground state, then takes the next instance. The
// instance's SpMV input vector lives in shared memory (as FP32 pairs for the
// double-float product when the values are FP32, as FP64 otherwise), so the
// gathers of the SpMV never leave the SM; the Krylov basis streams from HBM.
// No block waits for another block: there is no grid barrier and no spin.
//
// Replaces the sweep loops of the reference's drivers (BLQH_without_spin/
// main.cpp:77-115 over momentum sectors, :134-181 over layer distance), which
// call basis::init, lhamil::set_hamil, coeff_explicit_update, diag,
// eigenstates_reconstruction and ground_state_energy once per point
// (lanczos_hamiltonian.cpp:87-656). Per step: the three-term step (remove the
// components along v_j and v_{j-1}), then one full classical Gram-Schmidt
// pass against every stored vector, and a further pass when the norm fell
// below 1/sqrt(2) of its value after the three-term step (the
// Daniel-Gragg-Kaufman-Stewart criterion). The lowest Ritz pair comes from
// Sturm multisection and inverse iteration; the finisher is the FP64
// regenerated Rayleigh quotient for FP32 values, the stored FP64 CSR otherwise.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <tuple>
#include <vector>

#include "krylov.cuh"
#include "sector.cuh"

namespace {

// One instance as the persistent kernel sees it.
struct BInst {
  const int64_t* rp;
  const int32_t* col;
  const void* val;
  int64_t dim;
  int cplx, fp32, xsmem;
  int number;     // position in the caller's list (start-vector stream)
  double* V;      // [(lam + 1) * N], N = dim * (cplx ? 2 : 1)
  double* w;      // [N]
  double* psi;    // [N]
  double* ab;     // alpha [lam], beta [lam + 1] (beta[0] = 0)
  double* res;    // [5]: energy, lowest Ritz value, residual estimate, steps, repeated Gram-Schmidt passes
  double* xg;     // [N] staging of the SpMV input in global memory when it does not fit shared memory
};

constexpr int RED = 66;  // doubles of the block-reduction area

// Shared-memory layout (doubles): red | hs, h2 [2 (lam+1)] | ta [lam] | tb [lam+1] | ys [lam] |
// tri work [6 lam] | scal [8] | x area (rounded to 32 bytes: the x area takes 16-byte loads).
__host__ __device__ inline int batch_fixed_doubles(int lam) {
  return (RED + 4 * (lam + 1) + 9 * lam + 1 + 8 + 3) / 4 * 4;
}

// Per-instance device storage, in doubles from the instance's block (each array 256-byte aligned).
struct Lay {
  size_t V, w, psi, ab, res, xg, total;
};
inline Lay instance_layout(int64_t N, int lam, bool xsmem) {
  auto up = [](size_t v) { return (v + 31) / 32 * 32; };
  Lay L;
  L.V = 0;
  L.w = up((size_t)N * (lam + 1));
  L.psi = up(L.w + N);
  L.ab = up(L.psi + N);
  L.res = L.ab + 2 * lam + 1;
  L.xg = up(L.res + 5);
  L.total = up(L.xg + (xsmem ? 0 : (size_t)N));
  return L;
}

template <int NT>
__device__ __forceinline__ void block_sum2(double& a, double& b, double* red) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  if (lane == 0) {
    red[2 * wid] = a;
    red[2 * wid + 1] = b;
  }
  __syncthreads();
  if (wid == 0) {
    double x = lane < NT / 32 ? red[2 * lane] : 0.0, y = lane < NT / 32 ? red[2 * lane + 1] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      x += __shfl_xor_sync(0xffffffffu, x, o);
      y += __shfl_xor_sync(0xffffffffu, y, o);
    }
    if (lane == 0) {
      red[64] = x;
      red[65] = y;
    }
  }
  __syncthreads();
  a = red[64];
  b = red[65];
}

// w = H x (rq = false), or the partial Re <x, H x> of this thread (rq = true,
// FP64 values only). x: FP32 pairs (hi, lo) per double when F32, FP64
// otherwise; in shared or global memory. F32: w receives the unevaluated
// (hi, lo) pair of every component (same 8 bytes); converting here would cost
// every lane of a row group an FP64 instruction, so run_instance converts them
// lane-parallel.
template <int NT, int LPR, bool CPLX, bool F32>
__device__ __forceinline__ double bspmv(const BInst& I, const void* __restrict__ x, double* __restrict__ w,
                                        bool rq) {
  constexpr int NG = NT / LPR;
  const int grp = threadIdx.x / LPR, sub = threadIdx.x % LPR;
  double dot = 0.0;
  for (int64_t rb = 0; rb < I.dim; rb += NG) {
    const int64_t r = rb + grp;
    const bool ok = r < I.dim;
    const int64_t s = ok ? __ldg(I.rp + r) : 0, e = ok ? __ldg(I.rp + r + 1) : 0;
    if (F32) {
      float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
#pragma unroll 4
      for (int64_t k = s + sub; k < e; k += LPR) {
        const int32_t c = __ldg(I.col + k);
        if (CPLX) {
          const float2 v = __ldg(reinterpret_cast<const float2*>(I.val) + k);
          const float4 xv = reinterpret_cast<const float4*>(x)[c];
          df_add_prod(rh, rl, v.x, xv.x, xv.y);
          df_add_prod(rh, rl, -v.y, xv.z, xv.w);
          df_add_prod(ih, il, v.x, xv.z, xv.w);
          df_add_prod(ih, il, v.y, xv.x, xv.y);
        } else {
          const float v = __ldg(reinterpret_cast<const float*>(I.val) + k);
          const float2 xv = reinterpret_cast<const float2*>(x)[c];
          df_add_prod(rh, rl, v, xv.x, xv.y);
        }
      }
      df_seg_reduce<LPR>(rh, rl);
      if (CPLX) df_seg_reduce<LPR>(ih, il);
      if (ok && sub == 0) {
        float2* wp = reinterpret_cast<float2*>(w);
        if (CPLX) {
          wp[2 * r] = make_float2(rh, rl);
          wp[2 * r + 1] = make_float2(ih, il);
        } else {
          wp[r] = make_float2(rh, rl);
        }
      }
    } else {
      double ar = 0.0, ai = 0.0;
#pragma unroll 4
      for (int64_t k = s + sub; k < e; k += LPR) {
        const int32_t c = __ldg(I.col + k);
        if (CPLX) {
          const double2 v = __ldg(reinterpret_cast<const double2*>(I.val) + k);
          const double2 xv = reinterpret_cast<const double2*>(x)[c];
          ar += v.x * xv.x - v.y * xv.y;
          ai += v.x * xv.y + v.y * xv.x;
        } else {
          ar += __ldg(reinterpret_cast<const double*>(I.val) + k) * reinterpret_cast<const double*>(x)[c];
        }
      }
#pragma unroll
      for (int o = LPR / 2; o > 0; o >>= 1) {
        ar += __shfl_xor_sync(0xffffffffu, ar, o, LPR);
        if (CPLX) ai += __shfl_xor_sync(0xffffffffu, ai, o, LPR);
      }
      if (ok && sub == 0) {
        if (rq) {
          if (CPLX) {
            const double2 p = reinterpret_cast<const double2*>(x)[r];
            dot += p.x * ar + p.y * ai;
          } else {
            dot += reinterpret_cast<const double*>(x)[r] * ar;
          }
        } else if (CPLX) {
          reinterpret_cast<double2*>(w)[r] = make_double2(ar, ai);
        } else {
          w[r] = ar;
        }
      }
    }
  }
  return dot;
}

// h[k] = <V_k, w> for k < nk (complex: conj(V_k) w), one warp per vector.
// Two independent accumulator sets per lane keep two loads and FMA chains in flight.
template <int NT, bool CPLX>
__device__ __forceinline__ void cgs_dots(const double* __restrict__ V, int64_t N, int nk,
                                         const double* __restrict__ w, double* h) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  for (int k = wid; k < nk; k += NT / 32) {
    const double* vk = V + (int64_t)k * N;
    double sr = 0.0, si = 0.0, tr = 0.0, ti = 0.0;
    if (CPLX) {
      const double2* a2 = reinterpret_cast<const double2*>(vk);
      const double2* b2 = reinterpret_cast<const double2*>(w);
      const int64_t n2 = N / 2;
      int64_t i = lane;
      for (; i + 32 < n2; i += 64) {
        const double2 a = a2[i], b = b2[i], c = a2[i + 32], d = b2[i + 32];
        sr += a.x * b.x + a.y * b.y;
        si += a.x * b.y - a.y * b.x;
        tr += c.x * d.x + c.y * d.y;
        ti += c.x * d.y - c.y * d.x;
      }
      if (i < n2) {
        const double2 a = a2[i], b = b2[i];
        sr += a.x * b.x + a.y * b.y;
        si += a.x * b.y - a.y * b.x;
      }
    } else {
      int64_t i = lane;
      for (; i + 32 < N; i += 64) {
        sr += vk[i] * w[i];
        tr += vk[i + 32] * w[i + 32];
      }
      if (i < N) sr += vk[i] * w[i];
    }
    sr += tr;
    si += ti;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sr += __shfl_xor_sync(0xffffffffu, sr, o);
      si += __shfl_xor_sync(0xffffffffu, si, o);
    }
    if (lane == 0) {
      h[2 * k] = sr;
      h[2 * k + 1] = si;
    }
  }
}

// w -= sum_k V_k h_k; returns this thread's partial |w|^2.
template <int NT, bool CPLX>
__device__ __forceinline__ double cgs_update(const double* __restrict__ V, int64_t N, int nk, const double* h,
                                             double* __restrict__ w) {
  double nn = 0.0;
  if (CPLX) {
    for (int64_t i = threadIdx.x; i < N / 2; i += NT) {
      double2 acc = reinterpret_cast<double2*>(w)[i];
      double2 bcc = make_double2(0.0, 0.0);
      int k = 0;
      for (; k + 2 <= nk; k += 2) {
        const double2 v = reinterpret_cast<const double2*>(V + (int64_t)k * N)[i];
        const double2 u = reinterpret_cast<const double2*>(V + (int64_t)(k + 1) * N)[i];
        const double hr = h[2 * k], hi = h[2 * k + 1], gr = h[2 * k + 2], gi = h[2 * k + 3];
        acc.x -= hr * v.x - hi * v.y;
        acc.y -= hr * v.y + hi * v.x;
        bcc.x -= gr * u.x - gi * u.y;
        bcc.y -= gr * u.y + gi * u.x;
      }
      if (k < nk) {
        const double2 v = reinterpret_cast<const double2*>(V + (int64_t)k * N)[i];
        const double hr = h[2 * k], hi = h[2 * k + 1];
        acc.x -= hr * v.x - hi * v.y;
        acc.y -= hr * v.y + hi * v.x;
      }
      acc.x += bcc.x;
      acc.y += bcc.y;
      reinterpret_cast<double2*>(w)[i] = acc;
      nn += acc.x * acc.x + acc.y * acc.y;
    }
  } else {
    for (int64_t i = threadIdx.x; i < N; i += NT) {
      double acc = w[i], bcc = 0.0;
      int k = 0;
      for (; k + 2 <= nk; k += 2) {
        const double v0 = V[(int64_t)k * N + i], v1 = V[(int64_t)(k + 1) * N + i];
        acc -= h[2 * k] * v0;
        bcc -= h[2 * k + 2] * v1;
      }
      if (k < nk) acc -= h[2 * k] * V[(int64_t)k * N + i];
      acc += bcc;
      w[i] = acc;
      nn += acc * acc;
    }
  }
  return nn;
}

// Write v (FP64) into the SpMV input area: FP32 pairs or FP64.
__device__ __forceinline__ void stage_x(void* x, int64_t i, double v, bool f32) {
  if (f32) {
    const float hi = (float)v;
    reinterpret_cast<float2*>(x)[i] = make_float2(hi, (float)(v - (double)hi));
  } else {
    reinterpret_cast<double*>(x)[i] = v;
  }
}

// u - 1/2, u uniform in (0, 1): splitmix64 (Steele, Lea, Flood 2014) of (seed, stream, index).
__device__ __forceinline__ double splitmix_unit(uint64_t seed, uint64_t stream, uint64_t i) {
  uint64_t z = seed * 0x9E3779B97F4A7C15ULL + stream * 0xD1B54A32D192ED03ULL + (i + 1) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  z ^= z >> 31;
  return ((double)(z >> 11) + 0.5) * (1.0 / 9007199254740992.0) - 0.5;
}

template <int NT, int LPR, bool CPLX, bool F32>
__device__ void run_instance(const BInst& I, int lam, uint64_t seed, double bd_tol, double* sm, void* xs_sm) {
  double* red = sm;
  double* hs = red + RED;
  double* h2 = hs + 2 * (lam + 1);
  double* ta = h2 + 2 * (lam + 1);
  double* tb = ta + lam;
  double* ys = tb + lam + 1;
  double* trw = ys + lam;
  double* scal = trw + 6 * lam;
  void* x = I.xsmem ? xs_sm : static_cast<void*>(I.xg);
  const int64_t N = I.dim * (CPLX ? 2 : 1);

  // start vector: splitmix64 of (seed, instance number, index) - 1/2, normalized
  double nn = 0.0, z0 = 0.0;
  for (int64_t i = threadIdx.x; i < N; i += NT) {
    const double v = splitmix_unit(seed, (uint64_t)I.number, (uint64_t)i);
    I.V[i] = v;
    nn += v * v;
  }
  block_sum2<NT>(nn, z0, red);
  {
    const double inv = 1.0 / sqrt(nn);
    for (int64_t i = threadIdx.x; i < N; i += NT) {
      const double v = I.V[i] * inv;
      I.V[i] = v;
      stage_x(x, i, v, F32);
    }
  }
  if (threadIdx.x == 0) I.ab[lam] = 0.0;  // beta[0]
  __syncthreads();

  int m = lam, passes2 = 0;
  for (int j = 0; j < lam; j++) {
    bspmv<NT, LPR, CPLX, F32>(I, x, I.w, false);
    __syncthreads();
    double n0 = 0.0, z = 0.0;
    if (F32) {
      for (int64_t i = threadIdx.x; i < N; i += NT) {
        const float2 pr = reinterpret_cast<const float2*>(I.w)[i];
        const double v = (double)pr.x + (double)pr.y;
        I.w[i] = v;
        n0 += v * v;
      }
      __syncthreads();
    } else {
      for (int64_t i = threadIdx.x; i < N; i += NT) n0 += I.w[i] * I.w[i];
    }
    // three-term step: remove the components along v_{j-1} and v_j
    const int k0 = j > 0 ? j - 1 : 0, nl = j - k0 + 1;
    cgs_dots<NT, CPLX>(I.V + (int64_t)k0 * N, N, nl, I.w, h2);
    block_sum2<NT>(n0, z, red);  // also orders the dots before the update
    double nloc = cgs_update<NT, CPLX>(I.V + (int64_t)k0 * N, N, nl, h2, I.w);
    z = 0.0;
    block_sum2<NT>(nloc, z, red);
    // full classical Gram-Schmidt pass against V_0..V_j
    cgs_dots<NT, CPLX>(I.V, N, j + 1, I.w, hs);
    __syncthreads();
    double n1 = cgs_update<NT, CPLX>(I.V, N, j + 1, hs, I.w);
    z = 0.0;
    block_sum2<NT>(n1, z, red);
    for (int t = threadIdx.x; t < 2 * nl; t += NT) hs[2 * k0 + t] += h2[t];
    __syncthreads();
    if (n1 < 0.5 * nloc) {
      // the norm fell below 1/sqrt(2) of its value after the three-term step: repeat the pass
      passes2++;
      cgs_dots<NT, CPLX>(I.V, N, j + 1, I.w, h2);
      __syncthreads();
      n1 = cgs_update<NT, CPLX>(I.V, N, j + 1, h2, I.w);
      z = 0.0;
      block_sum2<NT>(n1, z, red);
      for (int t = threadIdx.x; t < 2 * (j + 1); t += NT) hs[t] += h2[t];
      __syncthreads();
    }
    const double alpha = hs[2 * j];
    const double beta = sqrt(n1);
    const double bprev = I.ab[lam + j];
    __syncthreads();
    if (threadIdx.x == 0) {
      I.ab[j] = alpha;
      I.ab[lam + j + 1] = beta;
    }
    const double scale = fabs(alpha) + bprev;
    if (!(beta > bd_tol * (scale > 0 ? scale : 1.0))) {
      m = j + 1;  // invariant subspace: T is exact
      break;
    }
    if (j + 1 == lam) break;
    const double inv = 1.0 / beta;
    double* vn = I.V + (int64_t)(j + 1) * N;
    for (int64_t i = threadIdx.x; i < N; i += NT) {
      const double v = I.w[i] * inv;
      vn[i] = v;
      stage_x(x, i, v, F32);
    }
    __syncthreads();
  }
  __syncthreads();

  // lowest eigenpair of the m x m tridiagonal
  for (int i = threadIdx.x; i < m; i += NT) {
    ta[i] = I.ab[i];
    tb[i] = I.ab[lam + i];
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int lane = threadIdx.x;
    double lo = 0.0, hi = 0.0, pm = 0.0;
    if (lane == 0) gersh(ta, tb, m, &lo, &hi, &pm);
    lo = __shfl_sync(0xffffffffu, lo, 0);
    hi = __shfl_sync(0xffffffffu, hi, 0);
    pm = __shfl_sync(0xffffffffu, pm, 0);
    for (int it = 0; it < 40; it++) {
      const double xv = lo + (hi - lo) * (lane + 1) / 33.0;
      const int c = sturm_count(ta, tb, m, xv, pm);
      const unsigned bal = __ballot_sync(0xffffffffu, c >= 1);
      const int first = bal ? __ffs(bal) - 1 : 32;
      const double nlo = first == 0 ? lo : lo + (hi - lo) * first / 33.0;
      const double nhi = first == 32 ? hi : lo + (hi - lo) * (first + 1) / 33.0;
      lo = nlo;
      hi = nhi;
      if (hi - lo <= 2 * DBL_EPSILON * fmax(fabs(lo), fabs(hi))) break;
    }
    if (lane == 0) {
      scal[0] = 0.5 * (lo + hi);
      tri_inverse_iteration(ta, tb, m, scal[0], ys, trw);
    }
  }
  __syncthreads();
  const double theta = scal[0];
  // ground state psi = sum_k y_k V_k, normalized
  nn = 0.0;
  for (int64_t i = threadIdx.x; i < N; i += NT) {
    double acc = 0.0;
    for (int k = 0; k < m; k++) acc += ys[k] * I.V[(int64_t)k * N + i];
    I.psi[i] = acc;
    nn += acc * acc;
  }
  z0 = 0.0;
  block_sum2<NT>(nn, z0, red);
  {
    const double inv = 1.0 / sqrt(nn);
    for (int64_t i = threadIdx.x; i < N; i += NT) {
      const double v = I.psi[i] * inv;
      I.psi[i] = v;
      if (!F32) stage_x(x, i, v, false);
    }
  }
  __syncthreads();
  double energy = theta;
  if (!F32) {
    // Rayleigh quotient with the stored FP64 CSR
    double d = bspmv<NT, LPR, CPLX, false>(I, x, nullptr, true), zz = 0.0;
    block_sum2<NT>(d, zz, red);
    energy = d;
  }
  if (threadIdx.x == 0) {
    const double bm = I.ab[lam + m];
    I.res[0] = energy;
    I.res[1] = theta;
    I.res[2] = fabs(bm * ys[m - 1]);
    I.res[3] = m;
    I.res[4] = passes2;
  }
  __syncthreads();
}

template <int NT, int LPR>
__global__ void __launch_bounds__(NT) k_batch_lanczos(const BInst* __restrict__ insts, const int* __restrict__ order,
                                                      int n, int lam, uint64_t seed, double bd_tol, int* counter) {
  extern __shared__ __align__(16) double bsm[];
  void* xs_sm = bsm + batch_fixed_doubles(lam);
  __shared__ int s_idx;
  for (;;) {
    if (threadIdx.x == 0) s_idx = atomicAdd(counter, 1);
    __syncthreads();
    const int idx = s_idx;
    __syncthreads();
    if (idx >= n) break;
    const BInst I = insts[order[idx]];
    if (I.cplx) {
      if (I.fp32) run_instance<NT, LPR, true, true>(I, lam, seed, bd_tol, bsm, xs_sm);
      else run_instance<NT, LPR, true, false>(I, lam, seed, bd_tol, bsm, xs_sm);
    } else {
      if (I.fp32) run_instance<NT, LPR, false, true>(I, lam, seed, bd_tol, bsm, xs_sm);
      else run_instance<NT, LPR, false, false>(I, lam, seed, bd_tol, bsm, xs_sm);
    }
  }
}

// res[i][0] = sum of the Rayleigh-quotient block partials of instance i (real parts).
__global__ void k_rq_reduce(const double* __restrict__ part, const int64_t* __restrict__ off,
                            const int* __restrict__ cnt, int n, double* const* res) {
  const int i = blockIdx.x;
  if (i >= n) return;
  __shared__ double red[8];
  double s = 0.0;
  for (int b = threadIdx.x; b < cnt[i]; b += blockDim.x) s += part[2 * (off[i] + b)];
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += red[w];
    res[i][0] = t;
  }
}

using KFn = void (*)(const BInst*, const int*, int, int, uint64_t, double, int*);
KFn batch_kernel(int threads, int lpr) {
#define BLQH_K(T, L) \
  if (threads == T && lpr == L) return k_batch_lanczos<T, L>;
  BLQH_K(256, 4) BLQH_K(256, 8) BLQH_K(256, 16) BLQH_K(256, 32)
  BLQH_K(512, 4) BLQH_K(512, 8) BLQH_K(512, 16) BLQH_K(512, 32)
#undef BLQH_K
  return nullptr;
}

}  // namespace

// ---------------------------------------------------------------------------
struct blqh_batch {
  blqh_ctx* ctx = nullptr;
  blqh_batch_opts o{};
  int n = 0;
  std::vector<blqh_instance> inst;
  std::vector<blqh_basis*> bases;
  std::vector<int> bidx;             // instance -> basis
  std::vector<blqh_csr*> csr;        // null when the sector is empty
  std::vector<RqPlan*> rq;           // mixed precision finisher plans
  std::vector<int64_t> N;            // doubles per vector
  std::vector<size_t> pool_off;      // doubles from the pool start
  double* pool = nullptr;
  BInst* d_inst = nullptr;
  int* d_order = nullptr;
  int* d_counter = nullptr;
  int nrun = 0;                      // instances with dim > 0
  double* d_part = nullptr;          // Rayleigh partials
  int64_t* d_off = nullptr;
  int* d_cnt = nullptr;
  double** d_res = nullptr;
  int nrq = 0;
  int threads = 512, lpr = 16, bps = 1, smem = 0, grid = 0;
  int64_t x_cap = 0;                 // bytes of the shared x area
  double mean_row = 0, mean_dim = 0; // over the running instances (tuning class)
  KFn kern = nullptr;
  cudaGraphExec_t gexec = nullptr;
  cudaEvent_t ev[3] = {nullptr, nullptr, nullptr};  // before the Lanczos launch, after it, after the finisher
  bool solved = false;
  Lay layout(int i) const { return instance_layout(N[i], o.lambda, N[i] * 8 <= x_cap); }
};

namespace {

void batch_free(blqh_batch* b) {
  if (!b) return;
  if (b->gexec) cudaGraphExecDestroy(b->gexec);
  for (auto e : b->ev)
    if (e) cudaEventDestroy(e);
  for (auto* p : b->rq)
    if (p) rq_plan_destroy(p);
  for (auto* m : b->csr) free_csr(m);
  for (auto* s : b->bases) blqh_basis_destroy(s);
  dev_free(b->pool);
  dev_free(b->d_inst);
  dev_free(b->d_order);
  dev_free(b->d_counter);
  dev_free(b->d_part);
  dev_free(b->d_off);
  dev_free(b->d_cnt);
  dev_free(b->d_res);
  delete b;
}

int lpr_for(double mean_row) {
  if (mean_row >= 96) return 32;
  if (mean_row >= 40) return 16;
  if (mean_row >= 12) return 8;
  return 4;
}

// Kernel, shared memory and occupancy for a (threads, lanes per row) shape.
void configure_shape(blqh_batch* b, int threads, int lpr) {
  blqh_ctx* ctx = b->ctx;
  b->threads = threads;
  b->lpr = lpr;
  b->kern = batch_kernel(threads, lpr);
  if (!b->kern) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_batch_create: threads 256 or 512, lanes_per_row 4, 8, 16 or 32");
    throw BlqhError{BLQH_ERR_ARG, "shape"};
  }
  BLQH_TRY_CUDA(ctx, smem_attr_at_least(b->kern, b->smem));
  int bps = 0;
  BLQH_TRY_CUDA(ctx, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, b->kern, b->threads, b->smem));
  b->bps = std::max(1, bps);
  b->grid = std::max(1, std::min(b->nrun, ctx->num_sms * b->bps));
}

// K10 for the batch: each candidate shape runs one round of the most
// expensive instances (one per resident block) for a few Lanczos steps on the
// batch's own data; the fastest per instance-step wins and is cached per class.
void tune_shape(blqh_batch* b) {
  blqh_ctx* ctx = b->ctx;
  bool any_cplx = false;
  for (auto* m : b->csr) any_cplx = any_cplx || (m && m->is_complex);
  const std::string key = tune_key("batch", b->o.value_precision, any_cplx, (int64_t)b->mean_dim, b->mean_row,
                                   b->o.lambda);
  int t = 0, l = 0;
  if (!tune_lookup(key, &t, &l)) {
    const int lam_t = std::min(b->o.lambda, 12);
    double best = 1e30;
    for (int th : {256, 512})
      for (int lp : {4, 8, 16, 32}) {
        if (lp == 4 && b->mean_row >= 24) continue;
        configure_shape(b, th, lp);
        const int nsub = std::min(b->nrun, ctx->num_sms * b->bps);
        double ms_best = 1e30;
        for (int rep = 0; rep < 2; rep++) {
          BLQH_TRY_CUDA(ctx, cudaMemsetAsync(b->d_counter, 0, sizeof(int), ctx->stream));
          BLQH_TRY_CUDA(ctx, cudaEventRecord(b->ev[0], ctx->stream));
          b->kern<<<std::min(b->grid, nsub), b->threads, b->smem, ctx->stream>>>(b->d_inst, b->d_order, nsub, lam_t,
                                                                                 b->o.seed, 1e-13, b->d_counter);
          BLQH_TRY_CUDA(ctx, cudaGetLastError());
          BLQH_TRY_CUDA(ctx, cudaEventRecord(b->ev[1], ctx->stream));
          BLQH_TRY_CUDA(ctx, cudaEventSynchronize(b->ev[1]));
          float ms = 0;
          BLQH_TRY_CUDA(ctx, cudaEventElapsedTime(&ms, b->ev[0], b->ev[1]));
          ms_best = std::min(ms_best, (double)ms);
        }
        const double per = ms_best / nsub;  // time per instance over the round
        if (per < best) {
          best = per;
          t = th;
          l = lp;
        }
      }
    tune_store(key, t, l, best);
  }
  configure_shape(b, t, l);
}

void batch_create_impl(blqh_batch* b) {
  blqh_ctx* ctx = b->ctx;
  const int lam = b->o.lambda;
  // one basis per distinct sector
  std::map<std::tuple<int, int, int, int, int, int, int, int>, int> seen;
  b->bidx.resize(b->n);
  for (int i = 0; i < b->n; i++) {
    const int model = b->inst[i].model;
    const blqh_sector& s = b->inst[i].sector;
    const blqh_sector_spin& ss = b->inst[i].ssector;
    const blqh_sector_mono& ms = b->inst[i].msector;
    const auto key = model == BLQH_MODEL_SPINFUL
                         ? std::make_tuple(1, ss.nphi, ss.nel, ss.nel_up, ss.nel_su, ss.J, ss.K, ss.rep_mode)
                     : model == BLQH_MODEL_MONOLAYER ? std::make_tuple(2, ms.nphi, ms.nel, -1, -1, ms.J, ms.K, ms.rep_mode)
                                                     : std::make_tuple(0, s.nphi, s.nel, s.nel_up, -1, s.J, s.K, s.rep_mode);
    auto it = seen.find(key);
    if (it == seen.end()) {
      blqh_basis* B = nullptr;
      const int rc = model == BLQH_MODEL_SPINFUL     ? blqh_basis_build_spin(ctx, &ss, &B)
                     : model == BLQH_MODEL_MONOLAYER ? blqh_basis_build_mono(ctx, &ms, &B)
                                                     : blqh_basis_build(ctx, &s, &B);
      if (rc != BLQH_OK) throw BlqhError{rc, "basis"};
      it = seen.emplace(key, (int)b->bases.size()).first;
      b->bases.push_back(B);
    }
    b->bidx[i] = it->second;
  }
  // CSR per instance
  b->csr.assign(b->n, nullptr);
  b->N.assign(b->n, 0);
  double nnz_sum = 0, dim_sum = 0;
  int64_t max_n = 0;
  for (int i = 0; i < b->n; i++) {
    const blqh_basis* B = b->bases[b->bidx[i]];
    if (B->dim == 0) continue;
    blqh_csr* M = new blqh_csr;
    M->ctx = ctx;
    b->csr[i] = M;
    if (b->inst[i].model == BLQH_MODEL_SPINFUL) {
      spin_hamil_build_impl(ctx, B, b->inst[i].sparams, M);
    } else if (b->inst[i].model == BLQH_MODEL_MONOLAYER) {
      mono_hamil_build_impl(ctx, B, b->inst[i].mparams, M);
    } else {
      hamil_build_impl(ctx, B, b->inst[i].params, b->o.value_precision, M);
    }
    b->N[i] = M->dim * (M->is_complex ? 2 : 1);
    nnz_sum += (double)M->nnz;
    dim_sum += (double)M->dim;
    max_n = std::max(max_n, b->N[i]);
  }
  // shared memory: the fixed part plus an x area for the instances that fit in it
  int smem_max = 0;
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  const int fixed = batch_fixed_doubles(lam) * 8;
  const int64_t x_cap = std::min<int64_t>(max_n * 8, (int64_t)std::max(0, 96 * 1024 - fixed));
  b->x_cap = x_cap;
  b->smem = fixed + (int)((x_cap + 15) / 16 * 16);
  if (b->smem > smem_max) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_batch_create: lambda too large for shared memory");
    throw BlqhError{BLQH_ERR_UNSUPPORTED, "smem"};
  }
  for (auto& e : b->ev) BLQH_TRY_CUDA(ctx, cudaEventCreate(&e));
  // shape: threads and lanes per row (given, tuned, or the defaults)
  b->mean_row = dim_sum > 0 ? nnz_sum / dim_sum : 0;
  b->mean_dim = b->n ? dim_sum / std::max(1, (int)std::count_if(b->csr.begin(), b->csr.end(), [](blqh_csr* m) {
    return m != nullptr;
  })) : 0;
  configure_shape(b, b->o.threads ? b->o.threads : 256,
                  b->o.lanes_per_row ? b->o.lanes_per_row : lpr_for(b->mean_row));
  // device storage per instance (instance_layout)
  b->pool_off.assign(b->n, 0);
  size_t total = 0;
  for (int i = 0; i < b->n; i++) {
    if (!b->csr[i]) continue;
    b->pool_off[i] = total;
    total += b->layout(i).total;
  }
  b->pool = dalloc<double>(ctx, total + 32);
  std::vector<BInst> hi;
  std::vector<double> cost;
  std::vector<double*> res_ptr;
  for (int i = 0; i < b->n; i++) {
    if (!b->csr[i]) continue;
    const blqh_csr* M = b->csr[i];
    BInst I{};
    I.rp = M->d_row_ptr;
    I.col = M->d_col;
    I.val = M->d_val;
    I.dim = M->dim;
    I.cplx = M->is_complex;
    I.fp32 = M->precision == BLQH_VAL_FP32;
    const int64_t Ni = b->N[i];
    I.xsmem = Ni * 8 <= x_cap;
    I.number = i;
    double* p = b->pool + b->pool_off[i];
    const Lay L = b->layout(i);
    I.V = p + L.V;
    I.w = p + L.w;
    I.psi = p + L.psi;
    I.ab = p + L.ab;
    I.res = p + L.res;
    I.xg = I.xsmem ? nullptr : p + L.xg;
    hi.push_back(I);
    // cost: SpMV bytes and reorthogonalization work over lam steps
    cost.push_back((double)lam * ((double)M->nnz * (I.fp32 ? 8.0 : 12.0) * (I.cplx ? 1.5 : 1.0) +
                                  0.5 * lam * (double)Ni * 16.0));
  }
  b->nrun = (int)hi.size();
  std::vector<int> order(b->nrun);
  for (int k = 0; k < b->nrun; k++) order[k] = k;
  std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return cost[a] > cost[c]; });
  b->d_inst = dalloc<BInst>(ctx, std::max(1, b->nrun));
  b->d_order = dalloc<int>(ctx, std::max(1, b->nrun));
  b->d_counter = dalloc<int>(ctx, 1);
  if (b->nrun) {
    BLQH_TRY_CUDA(ctx, cudaMemcpy(b->d_inst, hi.data(), hi.size() * sizeof(BInst), cudaMemcpyHostToDevice));
    BLQH_TRY_CUDA(ctx, cudaMemcpy(b->d_order, order.data(), order.size() * sizeof(int), cudaMemcpyHostToDevice));
  }
  b->grid = std::max(1, std::min(b->nrun, ctx->num_sms * b->bps));
  if (b->o.threads == 0 && b->o.lanes_per_row == 0 && tune_enabled() && b->nrun > 0) tune_shape(b);
  // mixed precision: one regenerated Rayleigh quotient per instance
  b->rq.assign(b->n, nullptr);
  if (b->o.value_precision == BLQH_VAL_FP32) {
    std::vector<int64_t> off;
    std::vector<int> cnt;
    int64_t tot = 0;
    int k = 0;  // position among the running instances
    for (int i = 0; i < b->n; i++) {
      if (!b->csr[i]) continue;
      const int kk = k++;
      if (b->csr[i]->precision != BLQH_VAL_FP32) continue;  // spinful: FP64 values, finished in the kernel
      res_ptr.push_back(hi[kk].res);
      b->rq[i] = rq_plan_create(ctx, b->bases[b->bidx[i]], b->inst[i].params);
      off.push_back(tot);
      cnt.push_back(rq_plan_grid(b->rq[i]));
      tot += rq_plan_grid(b->rq[i]);
    }
    b->nrq = (int)off.size();
    b->d_part = dalloc<double>(ctx, 2 * std::max<int64_t>(1, tot));
    b->d_off = dalloc<int64_t>(ctx, std::max(1, b->nrq));
    b->d_cnt = dalloc<int>(ctx, std::max(1, b->nrq));
    b->d_res = dalloc<double*>(ctx, std::max(1, b->nrq));
    if (b->nrq) {
      BLQH_TRY_CUDA(ctx, cudaMemcpy(b->d_off, off.data(), off.size() * 8, cudaMemcpyHostToDevice));
      // (res_ptr lists the instances with a plan, in plan order)
      BLQH_TRY_CUDA(ctx, cudaMemcpy(b->d_cnt, cnt.data(), cnt.size() * 4, cudaMemcpyHostToDevice));
      BLQH_TRY_CUDA(ctx, cudaMemcpy(b->d_res, res_ptr.data(), res_ptr.size() * sizeof(double*),
                                    cudaMemcpyHostToDevice));
    }
  }
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
}

// Timing event on the context stream; inside a stream capture it must be an
// external record node (a plain record there only orders work).
void record_ev(blqh_ctx* ctx, cudaEvent_t e) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  BLQH_TRY_CUDA(ctx, cudaStreamIsCapturing(ctx->stream, &st));
  if (st == cudaStreamCaptureStatusActive)
    BLQH_TRY_CUDA(ctx, cudaEventRecordWithFlags(e, ctx->stream, cudaEventRecordExternal));
  else
    BLQH_TRY_CUDA(ctx, cudaEventRecord(e, ctx->stream));
}

// Every launch of one solve, in stream order.
void batch_enqueue(blqh_batch* b) {
  blqh_ctx* ctx = b->ctx;
  if (!b->nrun) return;
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(b->d_counter, 0, sizeof(int), ctx->stream));
  record_ev(ctx, b->ev[0]);
  b->kern<<<b->grid, b->threads, b->smem, ctx->stream>>>(b->d_inst, b->d_order, b->nrun, b->o.lambda, b->o.seed,
                                                         1e-13, b->d_counter);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  record_ev(ctx, b->ev[1]);
  count_launch(ctx, TM_SPMV);
  if (b->o.value_precision == BLQH_VAL_FP32) {
    int64_t off = 0;
    for (int i = 0; i < b->n; i++) {
      if (!b->rq[i]) continue;
      const double* psi = b->pool + b->pool_off[i] + b->layout(i).psi;
      rq_plan_launch(ctx, b->rq[i], psi, b->d_part + 2 * off);
      off += rq_plan_grid(b->rq[i]);
    }
    k_rq_reduce<<<b->nrq, 256, 0, ctx->stream>>>(b->d_part, b->d_off, b->d_cnt, b->nrq, b->d_res);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_MISC);
  }
  record_ev(ctx, b->ev[2]);
}

void batch_solve_impl(blqh_batch* b) {
  blqh_ctx* ctx = b->ctx;
  if (b->o.use_graph && b->nrun) {
    if (!b->gexec) {
      const bool timing = ctx->timing;
      ctx->timing = false;  // no timer events inside the capture
      cudaGraph_t g = nullptr;
      BLQH_TRY_CUDA(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
      try {
        batch_enqueue(b);
      } catch (...) {
        cudaStreamEndCapture(ctx->stream, &g);
        if (g) cudaGraphDestroy(g);
        ctx->timing = timing;
        throw;
      }
      BLQH_TRY_CUDA(ctx, cudaStreamEndCapture(ctx->stream, &g));
      ctx->timing = timing;
      const cudaError_t e = cudaGraphInstantiate(&b->gexec, g, 0);
      cudaGraphDestroy(g);
      BLQH_TRY_CUDA(ctx, e);
    }
    BLQH_TRY_CUDA(ctx, cudaGraphLaunch(b->gexec, ctx->stream));
  } else {
    TimerScope ts(ctx, TM_SPMV);
    batch_enqueue(b);
  }
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  for (auto* p : b->rq)
    if (p) {
      const int rc = rq_plan_check(ctx, p);
      if (rc) throw BlqhError{rc, "rq"};
    }
  b->solved = true;
}

}  // namespace

extern "C" {

int blqh_batch_create(blqh_ctx* ctx, const blqh_instance* inst, int n, const blqh_batch_opts* o, blqh_batch** out) {
  if (!ctx || !o || !out || n < 0 || (n > 0 && !inst)) return BLQH_ERR_ARG;
  *out = nullptr;
  if (o->lambda < 2 || o->lambda > 1024 ||
      (o->value_precision != BLQH_VAL_FP32 && o->value_precision != BLQH_VAL_FP64)) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_batch_create: lambda in [2, 1024], value_precision FP32 or FP64");
    return BLQH_ERR_ARG;
  }
  for (int i = 0; i < n; i++)
    if (inst[i].model != BLQH_MODEL_SPINLESS && inst[i].model != BLQH_MODEL_SPINFUL &&
        inst[i].model != BLQH_MODEL_MONOLAYER) {
      set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_batch_create: unknown model");
      return BLQH_ERR_UNSUPPORTED;
    }
  blqh_batch* b = new blqh_batch;
  b->ctx = ctx;
  b->o = *o;
  b->n = n;
  b->inst.assign(inst, inst + n);
  try {
    cudaSetDevice(ctx->device);
    batch_create_impl(b);
  } catch (const BlqhError& e) {
    batch_free(b);
    return e.code;
  }
  *out = b;
  return BLQH_OK;
}

int blqh_batch_solve(blqh_batch* b) {
  if (!b) return BLQH_ERR_ARG;
  try {
    cudaSetDevice(b->ctx->device);
    batch_solve_impl(b);
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_batch_results(const blqh_batch* b, blqh_batch_result* out) {
  if (!b || !out) return BLQH_ERR_ARG;
  if (!b->solved) {
    set_error(b->ctx, BLQH_ERR_STATE, "blqh_batch_results: call blqh_batch_solve first");
    return BLQH_ERR_STATE;
  }
  for (int i = 0; i < b->n; i++) {
    blqh_batch_result r{};
    const blqh_csr* M = b->csr[i];
    if (!M) {
      r.energy = r.ritz0 = NAN;
      out[i] = r;
      continue;
    }
    double res[5];
    const double* d = b->pool + b->pool_off[i] + b->layout(i).res;
    if (cudaMemcpy(res, d, sizeof(res), cudaMemcpyDeviceToHost) != cudaSuccess) {
      set_error(b->ctx, BLQH_ERR_CUDA, "blqh_batch_results: copy failed");
      return BLQH_ERR_CUDA;
    }
    r.energy = res[0];
    r.ritz0 = res[1];
    r.resid = res[2];
    r.steps = (int)res[3];
    r.second_passes = (int)res[4];
    r.dim = M->dim;
    r.nnz = M->nnz;
    out[i] = r;
  }
  return BLQH_OK;
}

int blqh_batch_ground_state(const blqh_batch* b, int i, double* psi) {
  if (!b || !psi || i < 0 || i >= b->n) return BLQH_ERR_ARG;
  if (!b->solved || !b->csr[i]) {
    set_error(b->ctx, BLQH_ERR_STATE, "blqh_batch_ground_state: instance not solved (or empty sector)");
    return BLQH_ERR_STATE;
  }
  const double* d = b->pool + b->pool_off[i] + b->layout(i).psi;
  if (cudaMemcpy(psi, d, b->N[i] * 8, cudaMemcpyDeviceToHost) != cudaSuccess) {
    set_error(b->ctx, BLQH_ERR_CUDA, "blqh_batch_ground_state: copy failed");
    return BLQH_ERR_CUDA;
  }
  return BLQH_OK;
}

int blqh_batch_shape(const blqh_batch* b, int* threads, int* lanes_per_row, int* blocks_per_sm) {
  if (!b) return BLQH_ERR_ARG;
  if (threads) *threads = b->threads;
  if (lanes_per_row) *lanes_per_row = b->lpr;
  if (blocks_per_sm) *blocks_per_sm = b->bps;
  return BLQH_OK;
}

int blqh_batch_timing(const blqh_batch* b, double* lanczos_ms, double* finish_ms, int* launches) {
  if (!b) return BLQH_ERR_ARG;
  if (!b->solved || !b->nrun) {
    set_error(b->ctx, BLQH_ERR_STATE, "blqh_batch_timing: no solve has run");
    return BLQH_ERR_STATE;
  }
  float a = 0.f, c = 0.f;
  if (cudaEventElapsedTime(&a, b->ev[0], b->ev[1]) != cudaSuccess ||
      cudaEventElapsedTime(&c, b->ev[1], b->ev[2]) != cudaSuccess) {
    cudaGetLastError();
    set_error(b->ctx, BLQH_ERR_CUDA, "blqh_batch_timing: event timing unavailable");
    return BLQH_ERR_CUDA;
  }
  if (lanczos_ms) *lanczos_ms = a;
  if (finish_ms) *finish_ms = c;
  if (launches) *launches = 1 + (b->o.value_precision == BLQH_VAL_FP32 ? b->nrq + 1 : 0);
  return BLQH_OK;
}

int blqh_batch_destroy(blqh_batch* b) {
  batch_free(b);
  return BLQH_OK;
}

int blqh_batch_run(blqh_ctx* ctx, const blqh_instance* inst, int n, const blqh_batch_opts* o,
                   blqh_batch_result* out) {
  if (!out && n > 0) return BLQH_ERR_ARG;
  blqh_batch* b = nullptr;
  int rc = blqh_batch_create(ctx, inst, n, o, &b);
  if (rc == BLQH_OK) rc = blqh_batch_solve(b);
  if (rc == BLQH_OK) rc = blqh_batch_results(b, out);
  blqh_batch_destroy(b);
  return rc;
}

}  // extern "C"
