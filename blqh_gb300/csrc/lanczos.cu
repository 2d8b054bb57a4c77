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
  int* flags;     // [4]: stop, pass2, steps, breakdown
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

// ---------------------------------------------------------------------------
// Column-tiled streaming SpMV (real, FP32 values, double-float accumulation).
//
// The gathers of x are what limits the plain CSR kernel: every nonzero asks L2
// for a 32-byte sector to use 8 bytes of it, and the rate of those requests
// saturates L1 -> L2 before HBM does. Here one persistent block per SM owns a
// contiguous range of rpb rows, and x is walked in column blocks ("tiles") of
// w entries, each staged once per block into shared memory.
//
// Matrix layout (built once per matrix by prepare_tiles): for row block b and
// column block cb, tile t = b * nb + cb holds the entries of those rows whose
// columns fall in the block, row-major, as FP32 values and 16-bit column
// offsets from the block start (6 bytes per nonzero). Tiles are stored in the
// order t, each padded to a multiple of 8 entries, so a block's matrix stream
// is one contiguous, 16-byte aligned range. toff[t][rl] (stride tstride, a
// multiple of 4) is row rl's first entry inside tile t; tstart[t] the tile's
// first entry.
//
// The stream is fetched by one thread with cp.async.bulk into a ring of
// `stages` shared-memory buffers of `chunk` entries, each completed through an
// mbarrier transaction count, so DRAM reads run ahead of the arithmetic
// whatever the row lengths. Consumers split each chunk evenly by entries (see
// k_spmv_stream), gather x from the shared tile and add into the rows' running
// double-float sums in shared memory. Every wait on an mbarrier
// is bounded; on expiry the block records an error, waits (bounded) for its
// copies in flight and returns.
constexpr int TILE_THREADS = 1024;
constexpr int TILE_PAD = 8;  // tile lengths are padded to this many entries (16 bytes of tcol)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Bounded wait: false once about `limit` cycles have passed without completion.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, long long limit) {
  const long long t0 = clock64();
  while (!mbar_try_wait(bar, parity))
    if (clock64() - t0 > limit) return false;
  return true;
}
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// seg[r][cb] = (first entry of row r with column >= cb * w) - row start.
__global__ void k_tile_seg(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t dim, int w,
                           int nb, uint16_t* __restrict__ seg) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = rp[r], e = rp[r + 1];
    uint16_t* sr = seg + r * (nb + 1);
    int64_t k = s;
    for (int cb = 0; cb <= nb; cb++) {
      const int64_t lim = (int64_t)cb * w;
      while (k < e && col[k] < lim) k++;
      sr[cb] = (uint16_t)(k - s);
    }
    sr[nb] = (uint16_t)(e - s);
  }
}

// toff for one tile per block (block exclusive scan of the rows' entry counts
// in the tile); tlen[tile] = padded tile length; *count += true tile length.
__global__ void __launch_bounds__(TILE_THREADS) k_tile_offsets(const uint16_t* __restrict__ seg, int64_t dim,
                                                              int nb, int rpb, int tstride,
                                                              uint32_t* __restrict__ toff,
                                                              int64_t* __restrict__ tlen,
                                                              unsigned long long* count, int* overflow) {
  __shared__ int64_t wsum[TILE_THREADS / 32];
  const int tile = blockIdx.x;
  const int b = tile / nb, cb = tile - b * nb;
  const int64_t r0 = (int64_t)b * rpb;
  const int64_t rem = dim - r0;
  const int nrows = (int)(rem < rpb ? (rem > 0 ? rem : 0) : rpb);
  const int per = (nrows + TILE_THREADS - 1) / TILE_THREADS;
  const int lo = threadIdx.x * per, hi = min(lo + per, nrows);
  int64_t local = 0;
  for (int rl = lo; rl < hi; rl++) {
    const uint16_t* sr = seg + (r0 + rl) * (nb + 1) + cb;
    local += sr[1] - sr[0];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t x = local;
  for (int o = 1; o < 32; o <<= 1) {
    const int64_t yv = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += yv;
  }
  if (lane == 31) wsum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t v = wsum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const int64_t yv = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += yv;
    }
    wsum[lane] = v;
  }
  __syncthreads();
  int64_t run = (wid ? wsum[wid - 1] : 0) + x - local;
  const int64_t total = wsum[TILE_THREADS / 32 - 1];
  uint32_t* to = toff + (int64_t)tile * tstride;
  for (int rl = lo; rl < hi; rl++) {
    to[rl] = (uint32_t)run;
    const uint16_t* sr = seg + (r0 + rl) * (nb + 1) + cb;
    run += sr[1] - sr[0];
  }
  for (int rl = nrows + threadIdx.x; rl < tstride; rl += TILE_THREADS) to[rl] = (uint32_t)total;
  if (threadIdx.x == 0) {
    tlen[tile] = (total + TILE_PAD - 1) / TILE_PAD * TILE_PAD;
    atomicAdd(count, (unsigned long long)total);
    if (total > 0x7fffffffll) atomicOr(overflow, 1);
  }
}

__global__ void k_tile_copy(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                            const float* __restrict__ val, const uint16_t* __restrict__ seg,
                            const uint32_t* __restrict__ toff, const int64_t* __restrict__ tstart, int64_t dim,
                            int w, int nb, int rpb, int tstride, float* __restrict__ tval,
                            uint16_t* __restrict__ tcol) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t b = r / rpb, rl = r - b * rpb, s = rp[r];
    const uint16_t* sr = seg + r * (nb + 1);
    for (int cb = 0; cb < nb; cb++) {
      const int64_t tile = b * nb + cb;
      int64_t dst = tstart[tile] + toff[tile * tstride + rl];
      for (int64_t k = s + sr[cb]; k < s + sr[cb + 1]; k++, dst++) {
        tval[dst] = val[k];
        tcol[dst] = (uint16_t)(col[k] - cb * w);
      }
    }
  }
}

// Shared memory of k_spmv_stream, in bytes from the dynamic base (each part
// 128-byte aligned): barriers, row accumulators, the tile's row offsets, the x
// tile, the ring.
struct StreamSmem {
  int bar, acc, tofs, xt, ring, total;
};
__host__ __device__ inline StreamSmem stream_smem(int w, int rpb, int tstride, int chunk, int stages) {
  auto up = [](int v) { return (v + 127) / 128 * 128; };
  StreamSmem m;
  m.bar = 0;
  m.acc = 128;
  m.tofs = m.acc + up(rpb * 8);
  m.xt = m.tofs + up(tstride * 4);
  m.ring = m.xt + up(w * 8);
  m.total = m.ring + stages * up(chunk * 6);
  return m;
}

__device__ __forceinline__ void acc_add(float2* acc, int row, float h, float l) {
  float2 cur = acc[row];
  df_add(cur.x, cur.y, h, l);
  acc[row] = cur;
}

// Consumers take the chunk by entries, not by rows ("merge path"): lane t of
// the block owns entries [EPL t, EPL t + EPL) of the chunk, finds the row of
// its first entry by binary search in the tile's row offsets, and walks its
// entries keeping one double-float partial per row segment. A row segment
// that starts and ends inside the lane's entries belongs to the lane alone
// and is added to the row's accumulator at once. The first and the last
// segment of a lane may be shared with neighbouring lanes: a warp-level
// segmented suffix sum over the lanes' first segments joins them, and the lane
// where the row starts adds the joined value. A row continuing from an
// earlier warp (or chunk) is not added by the warp but parked in a slot per
// warp, and warp 0 adds the slots after a block barrier. Every thread does the
// same amount of work whatever the row lengths.
template <int EPL, int NT>
__global__ void __launch_bounds__(NT, 1)
    k_spmv_stream(const float* __restrict__ tval, const uint16_t* __restrict__ tcol,
                  const uint32_t* __restrict__ toff, const int64_t* __restrict__ tstart, int w, int nb, int rpb,
                  int tstride, int stages, const float2* __restrict__ xs, double* __restrict__ y, int64_t dim,
                  const double* bptr, const double* __restrict__ xprev, const int* stop, int* err) {
  static_assert(EPL % 4 == 0 && EPL <= 32 && NT % 32 == 0 && NT <= 1024, "entries per lane, threads");
  constexpr int chunk = EPL * NT;
  if (stop && *stop) return;
  extern __shared__ __align__(128) unsigned char ssm[];
  const StreamSmem L = stream_smem(w, rpb, tstride, chunk, stages);
  uint64_t* bars = reinterpret_cast<uint64_t*>(ssm + L.bar);
  float2* acc = reinterpret_cast<float2*>(ssm + L.acc);
  uint32_t* tofs = reinterpret_cast<uint32_t*>(ssm + L.tofs);
  float2* xt = reinterpret_cast<float2*>(ssm + L.xt);
  __shared__ int park_row[NT / 32];
  __shared__ float2 park_val[NT / 32];
  const int stage_bytes = (chunk * 6 + 127) / 128 * 128;
  const long long limit = 2000000000ll;  // about one second
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;

  const int64_t r0 = (int64_t)blockIdx.x * rpb;
  const int64_t rem = dim - r0;
  const int nrows = (int)(rem < rpb ? (rem > 0 ? rem : 0) : rpb);
  const int64_t t0 = (int64_t)blockIdx.x * nb;  // first tile of the block

  // producer state (thread 0): next tile and offset to fetch, chunks issued
  int p_cb = 0;
  int64_t p_q = 0;
  int64_t issued = 0;
  auto issue_next = [&](int64_t g) {
    while (p_cb < nb) {
      const int64_t len = __ldg(tstart + t0 + p_cb + 1) - __ldg(tstart + t0 + p_cb);
      if (p_q < len) break;
      p_cb++;
      p_q = 0;
    }
    if (p_cb >= nb) return;
    const int64_t len = __ldg(tstart + t0 + p_cb + 1) - __ldg(tstart + t0 + p_cb);
    const int64_t n = (len - p_q < chunk) ? (len - p_q) : chunk;
    const int64_t base = __ldg(tstart + t0 + p_cb) + p_q;
    const int st = (int)(g % stages);
    unsigned char* dst = ssm + L.ring + st * stage_bytes;
    mbar_expect_tx(bars + st, (uint32_t)(n * 6));
    bulk_g2s(dst, tval + base, (uint32_t)(n * 4), bars + st);
    bulk_g2s(dst + chunk * 4, tcol + base, (uint32_t)(n * 2), bars + st);
    p_q += n;
    issued = g + 1;
  };

  if (threadIdx.x == 0) {
    for (int st = 0; st < stages; st++) mbar_init(bars + st, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_proxy_async();
  }
  for (int t = threadIdx.x; t < nrows; t += blockDim.x) acc[t] = make_float2(0.f, 0.f);
  if (threadIdx.x < NT / 32) park_row[threadIdx.x] = -1;
  __syncthreads();
  if (threadIdx.x == 0)
    for (int64_t g = 0; g < stages; g++) issue_next(g);

  int64_t g = 0;  // chunks consumed
  bool failed = false;
  for (int cb = 0; cb < nb && !failed; cb++) {
    const int64_t tile = t0 + cb;
    const int64_t len = __ldg(tstart + tile + 1) - __ldg(tstart + tile);
    if (len == 0) continue;
    const int64_t c0 = (int64_t)cb * w;
    const int64_t cr = dim - c0;
    const int tw = (int)(cr < w ? cr : w);
    __syncthreads();  // the previous tile's x and offsets are no longer read
    for (int t = threadIdx.x; t < tw; t += blockDim.x) xt[t] = __ldg(xs + c0 + t);
    for (int t = threadIdx.x; t <= nrows; t += blockDim.x) tofs[t] = __ldg(toff + tile * tstride + t);
    __syncthreads();
    const int64_t tot = tofs[nrows];  // true entry count of the tile
    for (int64_t q0 = 0; q0 < len; q0 += chunk, g++) {
      const int st = (int)(g % stages);
      const bool ok_wait = mbar_wait_bounded(bars + st, (uint32_t)((g / stages) & 1), limit);
      const bool okw = __all_sync(0xffffffffu, ok_wait);
      const int nv = (int)(q0 < tot ? ((q0 + chunk < tot) ? chunk : tot - q0) : 0);  // valid entries
      if (okw && (warp * 32) * EPL < nv) {
        const unsigned char* sb = ssm + L.ring + st * stage_bytes;
        const int i0 = threadIdx.x * EPL;
        // this lane's entries
        float v[EPL];
        uint32_t c[EPL];
#pragma unroll
        for (int q = 0; q < EPL / 4; q++) {
          const float4 a = reinterpret_cast<const float4*>(sb)[threadIdx.x * (EPL / 4) + q];
          v[4 * q] = a.x;
          v[4 * q + 1] = a.y;
          v[4 * q + 2] = a.z;
          v[4 * q + 3] = a.w;
          const uint2 cc = reinterpret_cast<const uint2*>(sb + chunk * 4)[threadIdx.x * (EPL / 4) + q];
          c[4 * q] = cc.x & 0xffffu;
          c[4 * q + 1] = cc.x >> 16;
          c[4 * q + 2] = cc.y & 0xffffu;
          c[4 * q + 3] = cc.y >> 16;
        }
        // first segment (frow, fh, fl); last segment (orow, oh, ol) when the lane has several rows
        int frow = -1, orow = -1;
        float fh = 0.f, fl = 0.f, oh = 0.f, ol = 0.f;
        if (i0 < nv) {
          const uint32_t p0 = (uint32_t)(q0 + i0);
          int lo = 0, hi = nrows;  // tofs[lo] <= p0 < tofs[hi]
          while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (tofs[mid] <= p0) lo = mid;
            else hi = mid;
          }
          int r = lo;
          uint32_t rend = tofs[r + 1];
          float ah = 0.f, al = 0.f;
          bool first = true;
#pragma unroll
          for (int u = 0; u < EPL; u++) {
            if (i0 + u < nv) {
              const uint32_t pos = p0 + u;
              while (pos >= rend) {  // row r ended before this entry
                if (first) {
                  frow = r;
                  fh = ah;
                  fl = al;
                  first = false;
                } else if (ah != 0.f || al != 0.f) {
                  acc_add(acc, r, ah, al);  // the row lies inside this lane's entries
                }
                r++;
                rend = tofs[r + 1];
                ah = 0.f;
                al = 0.f;
              }
              const float2 x = xt[c[u]];
              df_add_prod(ah, al, v[u], x.x, x.y);
            }
          }
          if (first) {
            frow = r;
            fh = ah;
            fl = al;
          } else {
            orow = r;
            oh = ah;
            ol = al;
          }
        }
        // segmented suffix sum over the lanes' first segments: P_l = F_l + P_{l+1}
        // while lane l holds a single row that continues into lane l+1
        const bool single = orow < 0;
        const int nfrow = __shfl_down_sync(0xffffffffu, frow, 1);
        const bool open0 = single && frow >= 0 && lane < 31 && nfrow == frow;
        float ph = fh, pl = fl;
        bool open = open0;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const float qh = __shfl_down_sync(0xffffffffu, ph, d);
          const float ql = __shfl_down_sync(0xffffffffu, pl, d);
          const bool qo = __shfl_down_sync(0xffffffffu, open ? 1 : 0, d) != 0;
          if (open && lane + d < 32) df_add(ph, pl, qh, ql);
          open = open && lane + d < 32 && qo;
        }
        const float nph = __shfl_down_sync(0xffffffffu, ph, 1), npl = __shfl_down_sync(0xffffffffu, pl, 1);
        // the row of each lane's outgoing segment, and of the previous lane's
        const int key_out = single ? frow : orow;
        const int prev_out = __shfl_up_sync(0xffffffffu, key_out, 1);
        const bool absorbed = lane > 0 && frow >= 0 && prev_out == frow;  // F joins the previous lane's chain
        // a row already begun before this warp's first entry is parked for the fix-up
        const bool from_before = lane == 0 && frow >= 0 && (int64_t)tofs[frow] < q0 + (int64_t)(warp * 32) * EPL;
        if (frow >= 0 && !absorbed) {
          // the chain that starts with this lane's first segment: P (single lanes) or F alone
          float th = single ? ph : fh, tl = single ? pl : fl;
          if (from_before) {
            park_row[warp] = frow;
            park_val[warp] = make_float2(th, tl);
          } else if (th != 0.f || tl != 0.f) {
            acc_add(acc, frow, th, tl);
          }
        }
        if (!single) {
          // the lane's last row starts inside its entries; it may continue into the next lanes
          float th = oh, tl = ol;
          if (lane < 31 && nfrow == orow) df_add(th, tl, nph, npl);
          if (th != 0.f || tl != 0.f) acc_add(acc, orow, th, tl);
        }
      }
      __syncthreads();
      // fix-up: rows that continue from an earlier warp (at most one per warp), in warp order
      if (warp == 0) {
        const int prow = lane < NT / 32 ? park_row[lane] : -1;
        const float2 pv = lane < NT / 32 ? park_val[lane] : make_float2(0.f, 0.f);
        float ph = (prow >= 0) ? pv.x : 0.f, pl = (prow >= 0) ? pv.y : 0.f;
        const int nrow = __shfl_down_sync(0xffffffffu, prow, 1);
        bool open = prow >= 0 && lane < 31 && nrow == prow;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
          const float qh = __shfl_down_sync(0xffffffffu, ph, d);
          const float ql = __shfl_down_sync(0xffffffffu, pl, d);
          const bool qo = __shfl_down_sync(0xffffffffu, open ? 1 : 0, d) != 0;
          if (open && lane + d < 32) df_add(ph, pl, qh, ql);
          open = open && lane + d < 32 && qo;
        }
        const int prev = __shfl_up_sync(0xffffffffu, prow, 1);
        if (prow >= 0 && !(lane > 0 && prev == prow) && (ph != 0.f || pl != 0.f)) acc_add(acc, prow, ph, pl);
        if (lane < NT / 32) park_row[lane] = -1;
      }
      // the stage is free once every thread is past it; a failed wait anywhere ends the block
      if (__syncthreads_or(!ok_wait)) {
        failed = true;
        break;
      }
      if (threadIdx.x == 0) {
        fence_proxy_async();
        issue_next(g + stages);
      }
    }
  }
  if (failed) {
    if (threadIdx.x == 0) {
      atomicOr(err, 1);
      // drain: every chunk issued but not consumed completes its barrier phase
      for (int64_t h = g; h < issued; h++)
        mbar_wait_bounded(bars + (h % stages), (uint32_t)((h / stages) & 1), limit);
    }
    return;
  }
  __syncthreads();
  const double b = bptr ? *bptr : 0.0;
  for (int t = threadIdx.x; t < nrows; t += blockDim.x) {
    const float2 a = acc[t];
    const double re = (double)a.x + (double)a.y;
    const int64_t r = r0 + t;
    y[r] = xprev ? re - b * xprev[r] : re;
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
constexpr int GS_ROWS = 256;

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
  if (k == j) {
    if (stage == 1) S.alpha[j] = a;
    else S.alpha[j] += a;
  }
}

// w -= sum_k h[k] V_k over k in [k0, k1); partial |w|^2 per block.
template <bool CPLX>
__global__ void __launch_bounds__(UPD_THREADS) k_update(const double* __restrict__ V, int64_t dim, int k0, int k1,
                                                        const double* __restrict__ hcoef, double* __restrict__ w,
                                                        double* __restrict__ part_norm, const int* flags, int cond) {
  if (flags[0] || (cond && !flags[1])) return;
  extern __shared__ double hs[];
  const int nk = k1 - k0;
  for (int t = threadIdx.x; t < 2 * nk; t += blockDim.x) hs[t] = hcoef[2 * k0 + t];
  __syncthreads();
  double nn = 0;
  const int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (r < dim) {
    if (CPLX) {
      double2 acc = reinterpret_cast<const double2*>(w)[r];
      for (int k = 0; k < nk; k++) {
        const double2 v = reinterpret_cast<const double2*>(V)[(int64_t)(k0 + k) * dim + r];
        const double hr = hs[2 * k], hi = hs[2 * k + 1];
        acc.x -= hr * v.x - hi * v.y;
        acc.y -= hr * v.y + hi * v.x;
      }
      reinterpret_cast<double2*>(w)[r] = acc;
      nn = acc.x * acc.x + acc.y * acc.y;
    } else {
      double acc = w[r];
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
      w[r] = acc;
      nn = acc * acc;
    }
  }
  __shared__ double red[UPD_THREADS / 32];
  const double tot = block_sum_256(nn, red);
  if (threadIdx.x == 0) part_norm[blockIdx.x] = tot;
}

// After pass 1: |w|^2 and whether a second Gram-Schmidt pass is needed (the
// norm dropped below 1/sqrt(2) of its value before the pass); after pass 2:
// the final |w|^2. which: 1 = after pass 1, 2 = after pass 2.
__global__ void k_norm_step(const double* part_norm, int nblk, Scal S, int j, int which, int always_pass2,
                            double breakdown_tol) {
  if (S.flags[0]) return;
  if (which == 2 && !S.flags[1]) return;  // final norm comes from pass 1 when no second pass
  __shared__ double red[8];
  double a = 0;
  for (int b = threadIdx.x; b < nblk; b += blockDim.x) a += part_norm[b];
  a = block_sum_256(a, red);
  if (threadIdx.x != 0) return;
  S.nrm[1] = a;
  if (which == 1) S.flags[1] = always_pass2 ? 1 : (a < 0.5 * S.nrm[0]) ? 1 : 0;
}

__global__ void k_beta(Scal S, int j, double breakdown_tol) {
  if (S.flags[0]) return;
  const double b = sqrt(S.nrm[1]);
  S.beta[j + 1] = b;
  S.flags[2] = j + 1;
  const double scale = fabs(S.alpha[j]) + S.beta[j];
  if (!(b > breakdown_tol * (scale > 0 ? scale : 1.0))) {
    S.flags[3] = 1;
    S.flags[0] = 1;
  }
}

// V_{j+1} = w / beta_{j+1}
__global__ void k_scale(const double* __restrict__ w, double* __restrict__ vout, int64_t n, Scal S, int j) {
  if (S.flags[0]) return;
  const double inv = 1.0 / S.beta[j + 1];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    vout[i] = w[i] * inv;
}

// ---------------------------------------------------------------------------
// K6: tridiagonal eigen-solve (Sturm count, bounds, inverse iteration in krylov.cuh).
// Lowest eigenvalue by parallel multisection (one block); optional
// convergence test against the previous check, which sets the stop flag.
__global__ void k_tri_lowest(Scal S, int check_conv, double tol, int slot) {
  const int m = S.flags[2];
  if (m <= 0) return;
  __shared__ double lo, hi, pm;
  __shared__ int best;
  if (threadIdx.x == 0) gersh(S.alpha, S.beta, m, &lo, &hi, &pm);
  __syncthreads();
  for (int it = 0; it < 12; it++) {
    const double x = lo + (hi - lo) * (threadIdx.x + 1) / (blockDim.x + 1);
    const int c = sturm_count(S.alpha, S.beta, m, x, pm);
    if (threadIdx.x == 0) best = blockDim.x;
    __syncthreads();
    if (c >= 1) atomicMin(&best, (int)threadIdx.x);
    __syncthreads();
    const double nlo = (best == 0) ? lo : lo + (hi - lo) * best / (blockDim.x + 1);
    const double nhi = (best == (int)blockDim.x) ? hi : lo + (hi - lo) * (best + 1) / (blockDim.x + 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      lo = nlo;
      hi = nhi;
    }
    __syncthreads();
    if (hi - lo <= 2 * DBL_EPSILON * fmax(fabs(lo), fabs(hi))) break;
  }
  if (threadIdx.x == 0) {
    const double e = 0.5 * (lo + hi);
    S.ritz[slot] = e;
    if (check_conv && slot > 0 && !S.flags[0]) {
      const double prev = S.ritz[slot - 1];
      if (fabs(e - prev) <= tol) S.flags[0] = 1;
    }
  }
}

// Lowest eigenvalue of the m x m tridiagonal by multisection (one block): *out.
__global__ void k_tri_min(const double* a, const double* b, int m, double* out) {
  __shared__ double lo, hi, pm;
  __shared__ int best;
  if (threadIdx.x == 0) gersh(a, b, m, &lo, &hi, &pm);
  __syncthreads();
  for (int it = 0; it < 12; it++) {
    const double x = lo + (hi - lo) * (threadIdx.x + 1) / (blockDim.x + 1);
    const int c = sturm_count(a, b, m, x, pm);
    if (threadIdx.x == 0) best = blockDim.x;
    __syncthreads();
    if (c >= 1) atomicMin(&best, (int)threadIdx.x);
    __syncthreads();
    const double nlo = (best == 0) ? lo : lo + (hi - lo) * best / (blockDim.x + 1);
    const double nhi = (best == (int)blockDim.x) ? hi : lo + (hi - lo) * (best + 1) / (blockDim.x + 1);
    __syncthreads();
    if (threadIdx.x == 0) {
      lo = nlo;
      hi = nhi;
    }
    __syncthreads();
    if (hi - lo <= 2 * DBL_EPSILON * fmax(fabs(lo), fabs(hi))) break;
  }
  if (threadIdx.x == 0) *out = 0.5 * (lo + hi);
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
__global__ void k_tri_vec(const double* a, const double* b, int m, const double* lam_p, double* y, double* work) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  tri_inverse_iteration(a, b, m, *lam_p, y, work);
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

void fill_start(uint64_t seed, int rng, int64_t dim, int cplx, double* out) {
  const int64_t n = dim * (cplx ? 2 : 1);
  double nrm = 0;
  if (rng == 0) {
    MT32 g((uint32_t)seed);
    for (int64_t i = 0; i < n; i++) {
      out[i] = g.next() * 1.0 / 4294967295.0 - 0.5;
      nrm += out[i] * out[i];
    }
  } else {
    MT64 g(seed);
    for (int64_t i = 0; i < n; i++) {
      out[i] = g.real3() - 0.5;
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
  int nblk_dot = 0, nblk_upd = 0;
  int steps = 0;
  bool started = false, iterated = false, have_psi = false;
};

namespace {

void free_lanczos(blqh_lanczos* L) {
  if (!L) return;
  dev_free(L->xs);
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

// Column-tiled layout for k_spmv_stream (real FP32 CSR): rows split evenly
// over one block per SM; the x tile as wide as shared memory allows next to
// the row accumulators, the tile's row offsets and the ring. Built only for
// matrices of at least BLQH_TILE_MIN_DIM rows (unset: never). On the
// Nphi=16, dim 647079 matrix it measured 1.41 ms per product against 0.88 ms
// for k_spmv_df_v4 (its consumers are latency- and issue-bound), so it is an
// opt-in variant. BLQH_STREAM_EPL and BLQH_STREAM_STAGES set the entries per
// lane (8, 16, 32) and the ring depth (default 8 and 2).
void prepare_tiles(blqh_ctx* ctx, blqh_csr* M) {
  auto env_int = [](const char* name, long long dflt) {
    const char* v = getenv(name);
    return v ? atoll(v) : dflt;
  };
  const int64_t min_dim = env_int("BLQH_TILE_MIN_DIM", -1);
  if (min_dim < 0) return;
  if (M->tile_tried || M->is_complex || M->precision != BLQH_VAL_FP32 || M->dim < min_dim) return;
  M->tile_tried = true;
  // (entries per lane, threads): (8, 1024), (16, 512) or (32, 256)
  int epl = (int)env_int("BLQH_STREAM_EPL", 8);
  if (epl != 8 && epl != 16 && epl != 32) epl = 8;
  const int nt = 8192 / epl;
  const int chunk = epl * nt;
  int stages = (int)env_int("BLQH_STREAM_STAGES", 2);
  stages = stages < 2 ? 2 : (stages > 8 ? 8 : stages);
  int smem = 0;
  cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  const int64_t rpb = (M->dim + ctx->num_sms - 1) / ctx->num_sms;
  if (rpb > 16384) return;
  const int tstride = (int)((rpb + 1 + 3) / 4 * 4);
  const StreamSmem fixed = stream_smem(0, (int)rpb, tstride, chunk, stages);
  int64_t w = ((int64_t)smem - fixed.total - 1024) / 8;  // 1 KB for the kernel's static shared memory
  if (w > 65536) w = 65536;  // 16-bit column offsets
  w = (w / 256) * 256;
  if (w < 4096) return;
  const int64_t nb = (M->dim + w - 1) / w;
  M->tile_w = (int)w;
  M->tile_nb = (int)nb;
  M->tile_rpb = (int)rpb;
  M->tile_stride = tstride;
  M->tile_epl = epl;
  M->tile_stages = stages;
  M->tile_blocks = (int)((M->dim + rpb - 1) / rpb);
  const int64_t tiles = (int64_t)M->tile_blocks * nb;
  uint16_t* seg = nullptr;
  int64_t* tlen = nullptr;
  int* over = nullptr;
  unsigned long long* count = nullptr;
  bool ok = false;
  try {
    seg = dalloc<uint16_t>(ctx, (size_t)M->dim * (nb + 1));
    k_tile_seg<<<grid_for(ctx, M->dim, 256, 8), 256, 0, ctx->stream>>>(M->d_row_ptr, M->d_col, M->dim, M->tile_w,
                                                                      M->tile_nb, seg);
    M->d_toff = dalloc<uint32_t>(ctx, (size_t)tiles * tstride);
    M->d_tstart = dalloc<int64_t>(ctx, tiles + 1);
    tlen = dalloc<int64_t>(ctx, tiles + 1);
    over = dalloc<int>(ctx, 1);
    count = dalloc<unsigned long long>(ctx, 1);
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(over, 0, sizeof(int), ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(tlen, 0, (tiles + 1) * sizeof(int64_t), ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(count, 0, sizeof(unsigned long long), ctx->stream));
    k_tile_offsets<<<(int)tiles, TILE_THREADS, 0, ctx->stream>>>(seg, M->dim, M->tile_nb, M->tile_rpb, tstride,
                                                                 M->d_toff, tlen, count, over);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    int64_t total = 0;
    scan_exclusive_i64(ctx, tlen, M->d_tstart, tiles + 1, &total);
    int ov = 0;
    unsigned long long cnt = 0;
    BLQH_TRY_CUDA(ctx, cudaMemcpy(&ov, over, sizeof(int), cudaMemcpyDeviceToHost));
    BLQH_TRY_CUDA(ctx, cudaMemcpy(&cnt, count, sizeof(cnt), cudaMemcpyDeviceToHost));
    if (getenv("BLQH_DEBUG"))
      fprintf(stderr, "blqh tiles: dim %lld rpb %lld w %lld nb %lld tiles %lld padded %lld nnz %lld/%llu ov %d\n",
              (long long)M->dim, (long long)rpb, (long long)w, (long long)nb, (long long)tiles, (long long)total,
              (long long)M->nnz, cnt, ov);
    if (!ov && (int64_t)cnt == M->nnz) {
      // padded entries (and TILE_PAD past the end) are zero: they are fetched, never used
      M->d_tval = dalloc<float>(ctx, total + TILE_PAD);
      M->d_tcol = dalloc<uint16_t>(ctx, total + TILE_PAD);
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_tval, 0, (total + TILE_PAD) * sizeof(float), ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_tcol, 0, (total + TILE_PAD) * sizeof(uint16_t), ctx->stream));
      k_tile_copy<<<grid_for(ctx, M->dim, 256, 8), 256, 0, ctx->stream>>>(
          M->d_row_ptr, M->d_col, reinterpret_cast<const float*>(M->d_val), seg, M->d_toff, M->d_tstart, M->dim,
          M->tile_w, M->tile_nb, M->tile_rpb, tstride, M->d_tval, M->d_tcol);
      BLQH_TRY_CUDA(ctx, cudaGetLastError());
      M->d_terr = dalloc<int>(ctx, 1);  // the stream kernel's error word
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_terr, 0, sizeof(int), ctx->stream));
      ok = true;
    }
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int sm_bytes = stream_smem((int)w, (int)rpb, tstride, chunk, stages).total;
    if (epl == 8)
      BLQH_TRY_CUDA(ctx, cudaFuncSetAttribute(k_spmv_stream<8, 1024>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_bytes));
    else if (epl == 16)
      BLQH_TRY_CUDA(ctx, cudaFuncSetAttribute(k_spmv_stream<16, 512>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_bytes));
    else
      BLQH_TRY_CUDA(ctx, cudaFuncSetAttribute(k_spmv_stream<32, 256>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm_bytes));
  } catch (const BlqhError&) {
    dev_free(seg);
    dev_free(tlen);
    dev_free(over);
    dev_free(count);
    throw;
  }
  dev_free(seg);
  dev_free(tlen);
  dev_free(over);
  dev_free(count);
  if (ok) {
    M->tiled = true;
    count_launch(ctx, TM_MISC, 6);
  } else {
    dev_free(M->d_toff);
    dev_free(M->d_tstart);
    M->d_toff = nullptr;
    M->d_tstart = nullptr;
  }
}

// Error word of the streaming SpMV: a bounded wait that expired.
int stream_error(blqh_ctx* ctx, const blqh_csr* M) {
  if (!M->tiled || !M->d_terr) return 0;
  int e = 0;
  cudaMemcpy(&e, M->d_terr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e) {
    set_error(ctx, BLQH_ERR_CUDA, "SpMV: a shared-memory ring wait expired");
    cudaMemset(M->d_terr, 0, sizeof(int));
    return BLQH_ERR_CUDA;
  }
  return 0;
}

template <bool CPLX>
void spmv_df_t(blqh_ctx* ctx, const blqh_csr* M, const float2* xs, double* y, const double* bptr,
               const double* xprev, const int* stop) {
  if (!CPLX && M->tiled) {
    const int chunk = 8192;
    const int sm_bytes = stream_smem(M->tile_w, M->tile_rpb, M->tile_stride, chunk, M->tile_stages).total;
#define BLQH_STREAM(E, T)                                                                                      \
  k_spmv_stream<E, T><<<M->tile_blocks, T, sm_bytes, ctx->stream>>>(                                           \
      M->d_tval, M->d_tcol, M->d_toff, M->d_tstart, M->tile_w, M->tile_nb, M->tile_rpb, M->tile_stride,       \
      M->tile_stages, xs, y, M->dim, bptr, xprev, stop, M->d_terr)
    if (M->tile_epl == 8) BLQH_STREAM(8, 1024);
    else if (M->tile_epl == 16) BLQH_STREAM(16, 512);
    else BLQH_STREAM(32, 256);
#undef BLQH_STREAM
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
              const double* xprev = nullptr, const int* stop = nullptr, float2* xs = nullptr) {
  if (xs && M->precision == BLQH_VAL_FP32) {
    const int64_t n = M->dim * (M->is_complex ? 2 : 1);
    k_split<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(x, xs, n, stop);
    count_launch(ctx, TM_MISC);
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

template <bool CPLX>
void gs_pass(blqh_lanczos* L, int k0, int k1, int j, int stage) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  const int stride = L->mmax + 1;
  const int cond = (stage == 2);
  k_dots<CPLX><<<L->nblk_dot, 256, 0, st>>>(L->V, L->dim, k0, k1, L->w, L->part, stride, L->pnorm, L->S.flags,
                                            cond);
  k_reduce_dots<<<k1 - k0 + 1, 256, 0, st>>>(L->part, L->nblk_dot, stride, k0, k1, L->pnorm, L->S, j, stage);
  const double* hc = (stage == 1) ? L->S.h : L->S.h2;
  k_update<CPLX><<<L->nblk_upd, UPD_THREADS, 2 * (k1 - k0) * sizeof(double), st>>>(L->V, L->dim, k0, k1, hc, L->w,
                                                                                 L->pnorm, L->S.flags, cond);
  count_launch(ctx, TM_REORTH, 3);
}

template <bool CPLX>
void lanczos_step(blqh_lanczos* L, int j) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  const int64_t n = L->dim * L->vw;
  double* vj = L->V + (int64_t)j * n;
  const double* vprev = j > 0 ? L->V + (int64_t)(j - 1) * n : nullptr;
  spmv_dev(ctx, L->M, vj, L->w, j > 0 ? L->S.beta + j : nullptr, vprev, L->S.flags, L->xs);
  {
    TimerScope ts(ctx, TM_REORTH);
    // three-term step: the SpMV removed beta_j v_{j-1}; remove the v_j component
    // (alpha_j). With reorth, one classical Gram-Schmidt pass against every stored
    // vector follows; taking the local step first keeps that pass from having to
    // be repeated (the norm drop of the alpha_j removal no longer enters it).
    gs_pass<CPLX>(L, j, j + 1, j, 1);
    k_norm_step<<<1, 256, 0, st>>>(L->pnorm, L->nblk_upd, L->S, j, 1, L->o.reorth ? 1 : 0, 0.0);
    if (L->o.reorth) {
      gs_pass<CPLX>(L, 0, j + 1, j, 2);
      k_norm_step<<<1, 256, 0, st>>>(L->pnorm, L->nblk_upd, L->S, j, 2, 0, 0.0);
    }
    k_beta<<<1, 1, 0, st>>>(L->S, j, 1e-13);
    k_scale<<<grid_for(ctx, n, 256, 8), 256, 0, st>>>(L->w, L->V + (int64_t)(j + 1) * n, n, L->S, j);
    count_launch(ctx, TM_REORTH, L->o.reorth ? 4 : 3);
  }
}

void iterate_impl(blqh_lanczos* L) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  if (!L->started) {
    const int64_t n = L->dim * L->vw;
    if (L->o.rng == 2) {
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
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(L->S.flags, 0, 4 * sizeof(int), st));
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
    k_tri_lowest<<<1, 256, 0, st>>>(L->S, conv ? 1 : 0, L->o.tol, launched_chunks);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_MISC);
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
  L->iterated = true;
  L->have_psi = false;
}

void ritz_impl(blqh_lanczos* L) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  const int m = L->steps;
  // only the lowest Ritz pair is needed here (blqh_lanczos_eig gives them all)
  k_tri_min<<<1, 256, 0, st>>>(L->S.alpha, L->S.beta, m, L->work + 6 * L->mmax);
  k_tri_vec<<<1, 1, 0, st>>>(L->S.alpha, L->S.beta, m, L->work + 6 * L->mmax, L->y, L->work);
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

double rq_stored(blqh_lanczos* L) {
  blqh_ctx* ctx = L->ctx;
  cudaStream_t st = ctx->stream;
  spmv_dev(ctx, L->M, L->psi, L->w);
  const int64_t n = L->dim * L->vw;
  const int blocks = grid_for(ctx, n, 256, 4);
  k_dot_partial<<<blocks, 256, 0, st>>>(L->psi, L->w, n, L->cplx, L->pnorm);
  k_sum<<<1, 1, 0, st>>>(L->pnorm, blocks, L->S.nrm + 3);
  count_launch(ctx, TM_MISC, 2);
  double e = 0;
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(&e, L->S.nrm + 3, 8, cudaMemcpyDeviceToHost, st));
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(st));
  return e;
}

// K10 for the row SpMV: lanes per row timed on this matrix (x = 0, three
// products each) for matrices of at least 2^15 rows, cached per class.
void tune_spmv(blqh_lanczos* L) {
  blqh_csr* M = const_cast<blqh_csr*>(L->M);
  if (M->dim < (1 << 15) || M->tiled || !tune_enabled()) return;
  blqh_ctx* ctx = L->ctx;
  const int mode = M->precision == BLQH_VAL_FP32 ? (L->o.accumulate ? 1 : 2) : 0;
  const std::string key = tune_key("spmv", mode, M->is_complex, M->dim, M->mean_row, 0);
  int lpr = 0, unused = 0;
  if (!tune_lookup(key, &lpr, &unused)) {
    const int64_t n = L->dim * L->vw;
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(L->V, 0, n * 8, ctx->stream));
    cudaEvent_t e0, e1;
    BLQH_TRY_CUDA(ctx, cudaEventCreate(&e0));
    BLQH_TRY_CUDA(ctx, cudaEventCreate(&e1));
    double best = 1e30;
    for (int c : {4, 8, 16, 32}) {
      M->lanes_per_row = c;
      spmv_dev(ctx, M, L->V, L->w, nullptr, nullptr, nullptr, L->xs);  // warm-up
      BLQH_TRY_CUDA(ctx, cudaEventRecord(e0, ctx->stream));
      for (int r = 0; r < 3; r++) spmv_dev(ctx, M, L->V, L->w, nullptr, nullptr, nullptr, L->xs);
      BLQH_TRY_CUDA(ctx, cudaEventRecord(e1, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaEventSynchronize(e1));
      float ms = 0;
      BLQH_TRY_CUDA(ctx, cudaEventElapsedTime(&ms, e0, e1));
      if (ms < best) {
        best = ms;
        lpr = c;
      }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    tune_store(key, lpr, 0, best / 3);
  }
  M->lanes_per_row = lpr;
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
  const int upd_smem = 2 * (L->mmax + 1) * (int)sizeof(double);
  cudaFuncSetAttribute(k_update<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, upd_smem);
  cudaFuncSetAttribute(k_update<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, upd_smem);
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
    L->pnorm = dalloc<double>(ctx, std::max<int64_t>(std::max(L->nblk_dot, L->nblk_upd), (L->dim + 255) / 256) + 1024);
    L->work = dalloc<double>(ctx, 8 * (size_t)m + 16);
    L->y = dalloc<double>(ctx, m + 1);
    if (M->precision == BLQH_VAL_FP32 && o.accumulate == 0) {
      L->xs = dalloc<float2>(ctx, n);
      prepare_tiles(ctx, const_cast<blqh_csr*>(M));
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
    if (m->precision == BLQH_VAL_FP32) xs = dalloc<float2>(ctx, n);
    if (xs) prepare_tiles(ctx, const_cast<blqh_csr*>(m));
    const_cast<blqh_csr*>(m)->lanes_per_row = spmv_lpr(m->mean_row);
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(dx, x, n * 8, cudaMemcpyHostToDevice, ctx->stream));
    spmv_dev(ctx, m, dx, dy, nullptr, nullptr, nullptr, xs);
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(y, dy, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    rc = stream_error(ctx, m);
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
  if (const int rc = stream_error(L->ctx, L->M)) return rc;
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
    k_tri_vec<<<1, 1, 0, ctx->stream>>>(L->S.alpha, L->S.beta, m, L->work + 6 * L->mmax, L->y, L->work);
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
    *energy = rq_stored(L);
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_lanczos_rayleigh_fp64(blqh_lanczos* L, const blqh_basis* b, const blqh_params* p, double* energy) {
  if (!L || !b || !p || !energy) return BLQH_ERR_ARG;
  if (!L->have_psi) {
    set_error(L->ctx, BLQH_ERR_STATE, "blqh_lanczos_rayleigh_fp64: call blqh_lanczos_ritz_vector first");
    return BLQH_ERR_STATE;
  }
  if (b->dim != L->dim) {
    set_error(L->ctx, BLQH_ERR_ARG, "blqh_lanczos_rayleigh_fp64: basis does not match the matrix");
    return BLQH_ERR_ARG;
  }
  try {
    *energy = rayleigh_regen_impl(L->ctx, b, *p, L->psi, L->cplx != 0);
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

int blqh_debug_spmv_layout(const blqh_csr* M) {
  if (!M) return -1;
  return M->tiled ? 1 : 0;
}

}  // extern "C"
