// Row-block x column-tile SpMV for FP32-valued CSR (real and complex),
// double-float accumulation (y = H x - b xprev, the Lanczos product of
// Mat::operator*, BLQH_without_spin/matrix.cpp:244-267).
//
// Why: the row-parallel CSR kernel gathers x[col] from L2 for every nonzero,
// one 32-byte sector for 8 or 16 useful bytes, and the L1 processes about one
// such divergent line per clock per SM; at Nphi = 16 that caps the product near
// 40 % of HBM bandwidth. Here x is read from shared memory instead.
//
// Layout (built once per matrix by blocked_prepare): rows are split into
// blocks of rpb rows (one CTA each), a block's rows into BL_WARPS contiguous
// groups of rpw rows (one warp each, so no two warps ever add into the same
// row), and columns into tiles of w entries. The entries of group g whose
// columns fall in tile t form segment (g, t), stored in row-then-column order
// as a 32-bit key (row within the block << 16 | column within the tile) and
// the FP32 value (float2 when complex): 8 or 12 bytes per nonzero against the
// CSR's 8 or 12 plus row pointers. A group's segments are consecutive in t,
// each starting on a multiple of 4 entries (16-byte loads).
//
// Kernel: one CTA per row block, BL_WARPS warps. x tiles are double-buffered
// in shared memory by cp.async.bulk (one thread issues, an mbarrier per
// buffer completes them, every wait bounded); tile t + 2 is fetched once all
// warps are past tile t. Each warp walks its segments in chunks of 256
// entries (8 consecutive entries per lane), keeping the next two chunks in
// flight in registers across tile boundaries, so HBM stays busy while tiles
// turn over. Within a chunk a lane sums runs of equal rows; the runs that
// cross lanes are joined by a segmented suffix sum over the warp, and one lane
// per row adds the row's part into the block's accumulators in shared memory
// (double-float). The summation order is fixed, so results are reproducible.
#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "blqh_internal.h"
#include "krylov.cuh"

namespace {

constexpr int BL_WARPS = 16;
constexpr int BL_THREADS = BL_WARPS * 32;
constexpr int BL_EPL = 8;                  // entries per lane per chunk
constexpr int BL_CHUNK = 32 * BL_EPL;      // entries per warp chunk
constexpr int BL_XBYTES = 65536;           // bytes per x tile buffer
constexpr int BL_SMEM_FIXED = 128 + 2 * BL_XBYTES;
constexpr long long BL_WAIT_LIMIT = 2000000000ll;  // clock64 cycles, about one second

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
// false once about `limit` cycles have passed without completion
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

// ---------------------------------------------------------------------------
// Layout construction.

// rowseg[r][t] = (first entry of row r with column >= t w) - row start, t = 0..nb.
__global__ void k_bl_rowseg(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t dim, int w,
                            int nb, uint16_t* __restrict__ rowseg, int* over) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = rp[r], e = rp[r + 1];
    if (e - s > 65535) {
      atomicOr(over, 1);
      continue;
    }
    uint16_t* sr = rowseg + r * (nb + 1);
    int64_t k = s;
    for (int t = 0; t < nb; t++) {
      const int64_t lim = (int64_t)t * w;
      while (k < e && col[k] < lim) k++;
      sr[t] = (uint16_t)(k - s);
    }
    sr[nb] = (uint16_t)(e - s);
  }
}

struct Group {
  int64_t r0, r1;  // global rows of the group
};
__device__ __forceinline__ Group group_rows(int64_t g, int64_t dim, int rpb, int rpw) {
  const int64_t b = g / BL_WARPS, wp = g - b * BL_WARPS;
  const int64_t bend = min(dim, (b + 1) * (int64_t)rpb);
  Group G;
  G.r0 = min(bend, b * (int64_t)rpb + wp * rpw);
  G.r1 = min(bend, G.r0 + rpw);
  return G;
}

// Pass 0: segment lengths (true and padded to 4). Pass 1: copy the entries.
// One block per group, one thread per tile; the thread walks the group's rows.
template <bool CPLX>
__global__ void k_bl_fill(int pass, const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                          const void* __restrict__ val, const uint16_t* __restrict__ rowseg, int64_t dim, int w,
                          int nb, int rpb, int rpw, int32_t* __restrict__ blen, int64_t* __restrict__ plen,
                          const int64_t* __restrict__ bstart, uint32_t* __restrict__ keys, void* __restrict__ vals) {
  const int64_t g = blockIdx.x;
  const Group G = group_rows(g, dim, rpb, rpw);
  const int64_t rb0 = (g / BL_WARPS) * (int64_t)rpb;
  for (int t = threadIdx.x; t < nb; t += blockDim.x) {
    int64_t run = pass ? bstart[g * nb + t] : 0;
    for (int64_t r = G.r0; r < G.r1; r++) {
      const uint16_t* sr = rowseg + r * (nb + 1);
      const int64_t s = rp[r] + sr[t], e = rp[r] + sr[t + 1];
      if (pass) {
        const uint32_t rk = (uint32_t)(r - rb0) << 16;
        for (int64_t k = s; k < e; k++, run++) {
          keys[run] = rk | (uint32_t)(col[k] - (int64_t)t * w);
          if (CPLX) reinterpret_cast<float2*>(vals)[run] = reinterpret_cast<const float2*>(val)[k];
          else reinterpret_cast<float*>(vals)[run] = reinterpret_cast<const float*>(val)[k];
        }
      } else {
        run += e - s;
      }
    }
    if (!pass) {
      blen[g * nb + t] = (int32_t)run;
      plen[g * nb + t] = (run + 3) & ~(int64_t)3;
    }
  }
}

// ---------------------------------------------------------------------------
// The product.

struct BlArgs {
  const uint32_t* keys;
  const void* vals;
  const int64_t* bstart;
  const int32_t* blen;
  int w, nb, rpb, rpw;
  int64_t dim;
  int* err;
};

template <bool CPLX>
struct Slot {
  uint4 k[BL_EPL / 4];
  float4 v[CPLX ? BL_EPL / 2 : BL_EPL / 4];
};

template <bool CPLX>
__device__ __forceinline__ void load_slot(Slot<CPLX>& s, const BlArgs& A, int64_t pos, int n, int lane) {
  const int o = lane * BL_EPL;
  if (o < n) {
    const uint4* kp = reinterpret_cast<const uint4*>(A.keys + pos + o);
    const float4* vp = reinterpret_cast<const float4*>(reinterpret_cast<const char*>(A.vals) +
                                                       (pos + o) * (CPLX ? 8 : 4));
#pragma unroll
    for (int q = 0; q < BL_EPL / 4; q++) s.k[q] = __ldcs(kp + q);
#pragma unroll
    for (int q = 0; q < (CPLX ? BL_EPL / 2 : BL_EPL / 4); q++) s.v[q] = __ldcs(vp + q);
  }
}

__device__ __forceinline__ uint32_t key_at(const uint4* k, int u) {
  const uint4 q = k[u >> 2];
  switch (u & 3) {
    case 0: return q.x;
    case 1: return q.y;
    case 2: return q.z;
    default: return q.w;
  }
}
__device__ __forceinline__ float val_at(const float4* v, int u) {
  const float4 q = v[u >> 2];
  switch (u & 3) {
    case 0: return q.x;
    case 1: return q.y;
    case 2: return q.z;
    default: return q.w;
  }
}
__device__ __forceinline__ float2 cval_at(const float4* v, int u) {
  const float4 q = v[u >> 1];
  return (u & 1) ? make_float2(q.z, q.w) : make_float2(q.x, q.y);
}

// Running sums of a run: NC double-float pairs (1 real, 2 complex).
template <int NC>
struct Run {
  float h[NC], l[NC];
  __device__ __forceinline__ void zero() {
#pragma unroll
    for (int c = 0; c < NC; c++) h[c] = l[c] = 0.f;
  }
  __device__ __forceinline__ bool nonzero() const {
    bool z = false;
#pragma unroll
    for (int c = 0; c < NC; c++) z = z || h[c] != 0.f || l[c] != 0.f;
    return z;
  }
  __device__ __forceinline__ void add(const Run& o) {
#pragma unroll
    for (int c = 0; c < NC; c++) df_add(h[c], l[c], o.h[c], o.l[c]);
  }
  __device__ __forceinline__ Run shfl_down(int d) const {
    Run o;
#pragma unroll
    for (int c = 0; c < NC; c++) {
      o.h[c] = __shfl_down_sync(0xffffffffu, h[c], d);
      o.l[c] = __shfl_down_sync(0xffffffffu, l[c], d);
    }
    return o;
  }
};

template <int NC>
__device__ __forceinline__ void acc_add(float2* acc, int row, const Run<NC>& r) {
#pragma unroll
  for (int c = 0; c < NC; c++) {
    float2 cur = acc[row * NC + c];
    df_add(cur.x, cur.y, r.h[c], r.l[c]);
    acc[row * NC + c] = cur;
  }
}

// One chunk of a warp: n valid entries (lane l holds entries 8l .. 8l+7).
template <bool CPLX>
__device__ __forceinline__ void process_chunk(const Slot<CPLX>& s, int n, const void* xb, float2* acc, int lane) {
  constexpr int NC = CPLX ? 2 : 1;
  int frow = -1, orow = -1, cur = -1;
  Run<NC> F, O, R;
  F.zero();
  O.zero();
  R.zero();
  const int o = lane * BL_EPL;
#pragma unroll
  for (int u = 0; u < BL_EPL; u++) {
    if (o + u < n) {
      const uint32_t key = key_at(s.k, u);
      const int row = (int)(key >> 16);
      const uint32_t c = key & 0xffffu;
      if (row != cur) {
        if (cur >= 0) {
          if (frow < 0) {
            frow = cur;
            F = R;
          } else {
            acc_add<NC>(acc, cur, R);  // the row lies inside this lane's entries
          }
        }
        cur = row;
        R.zero();
      }
      if (CPLX) {
        const float2 v = cval_at(s.v, u);
        const float4 x = reinterpret_cast<const float4*>(xb)[c];  // (re hi, re lo, im hi, im lo)
        df_add_prod(R.h[0], R.l[0], v.x, x.x, x.y);
        df_add_prod(R.h[0], R.l[0], -v.y, x.z, x.w);
        df_add_prod(R.h[NC - 1], R.l[NC - 1], v.x, x.z, x.w);
        df_add_prod(R.h[NC - 1], R.l[NC - 1], v.y, x.x, x.y);
      } else {
        const float2 x = reinterpret_cast<const float2*>(xb)[c];
        df_add_prod(R.h[0], R.l[0], val_at(s.v, u), x.x, x.y);
      }
    }
  }
  if (cur >= 0) {
    if (frow < 0) {
      frow = cur;
      F = R;
    } else {
      orow = cur;
      O = R;
    }
  }
  // Runs that cross lanes. P_l = F_l + P_{l+1} while lane l holds a single run
  // that continues into lane l+1 (segmented suffix sum by pointer jumping).
  const bool single = orow < 0;
  const int nfrow = __shfl_down_sync(0xffffffffu, frow, 1);
  bool open = single && frow >= 0 && lane < 31 && nfrow == frow;
  Run<NC> P = F;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const Run<NC> Q = P.shfl_down(d);
    const bool qo = __shfl_down_sync(0xffffffffu, open ? 1 : 0, d) != 0;
    if (open && lane + d < 32) P.add(Q);
    open = open && lane + d < 32 && qo;
  }
  const Run<NC> NP = P.shfl_down(1);
  const int key_out = single ? frow : orow;
  const int prev_out = __shfl_up_sync(0xffffffffu, key_out, 1);
  const bool absorbed = lane > 0 && frow >= 0 && prev_out == frow;  // joined to the previous lane's run
  if (frow >= 0 && !absorbed) {
    const Run<NC>& T = single ? P : F;
    if (T.nonzero()) acc_add<NC>(acc, frow, T);
  }
  if (!single) {
    Run<NC> T = O;
    if (lane < 31 && nfrow == orow) T.add(NP);
    if (T.nonzero()) acc_add<NC>(acc, orow, T);
  }
  __syncwarp();  // the accumulators are read again by the warp's next chunk
}

template <bool CPLX>
__global__ void __launch_bounds__(BL_THREADS, 1)
    k_spmv_blocked(BlArgs A, const float2* __restrict__ xs, double* __restrict__ y, const double* bptr,
                   const double* __restrict__ xprev, const int* stop) {
  constexpr int NC = CPLX ? 2 : 1;
  constexpr int XE = CPLX ? 16 : 8;  // bytes per x entry
  if (stop && *stop) return;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  unsigned char* xbuf = smem + 128;
  float2* acc = reinterpret_cast<float2*>(smem + BL_SMEM_FIXED);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int64_t r0 = (int64_t)blockIdx.x * A.rpb;
  const int nrows = (int)min((int64_t)A.rpb, A.dim - r0);
  const int nb = A.nb;

  auto issue = [&](int t) {
    const int64_t c0 = (int64_t)t * A.w;
    const int64_t n = min((int64_t)A.w, A.dim - c0);
    const uint32_t bytes = (uint32_t)((n * XE + 15) & ~(int64_t)15);  // the split buffer has 16 bytes of slack
    uint64_t* bar = bars + (t & 1);
    mbar_expect_tx(bar, bytes);
    bulk_g2s(xbuf + (t & 1) * BL_XBYTES, reinterpret_cast<const char*>(xs) + c0 * XE, bytes, bar);
  };

  if (threadIdx.x == 0) {
    mbar_init(bars, 1);
    mbar_init(bars + 1, 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_proxy_async();
  }
  for (int i = threadIdx.x; i < nrows * NC; i += BL_THREADS) acc[i] = make_float2(0.f, 0.f);
  __syncthreads();
  if (threadIdx.x == 0) {
    issue(0);
    if (nb > 1) issue(1);
  }

  // The warp's chunk stream: segments t = 0 .. nb-1 of group g, 256 entries at
  // a time. Three register slots hold consecutive chunks; the slots take turns
  // (no copies between them, which would wait for loads in flight), and the
  // start and length of the next segment are read one segment ahead.
  const int64_t g = (int64_t)blockIdx.x * BL_WARPS + warp;
  const int64_t* bst = A.bstart + g * nb;
  const int32_t* bln = A.blen + g * nb;
  int it_t = -1, it_rem = 0;
  int64_t it_pos = 0;
  int64_t nx_pos = bst[0];
  int nx_len = bln[0];
  auto next_chunk = [&](int& ct, int64_t& cpos, int& cn) {
    while (it_rem == 0) {
      if (it_t + 1 >= nb) {
        ct = nb;
        cpos = 0;
        cn = 0;
        return;
      }
      it_t++;
      it_pos = nx_pos;
      it_rem = nx_len;
      if (it_t + 1 < nb) {
        nx_pos = bst[it_t + 1];
        nx_len = bln[it_t + 1];
      }
    }
    ct = it_t;
    cpos = it_pos;
    cn = it_rem < BL_CHUNK ? it_rem : BL_CHUNK;
    it_pos += cn;
    it_rem -= cn;
  };
  Slot<CPLX> s0, s1, s2;
  int t0, t1, t2, n0, n1, n2;
  int64_t p0, p1, p2;
  next_chunk(t0, p0, n0);
  load_slot<CPLX>(s0, A, p0, n0, lane);
  next_chunk(t1, p1, n1);
  load_slot<CPLX>(s1, A, p1, n1, lane);
  next_chunk(t2, p2, n2);
  load_slot<CPLX>(s2, A, p2, n2, lane);

  bool failed = false;
  int ok_upto = -1;                  // last tile whose copy this thread saw complete
  int issued_upto = nb > 1 ? 1 : 0;  // last tile whose copy was issued (thread 0)
  int turn = 0;                      // slot holding the next chunk
  for (int t = 0; t < nb; t++) {
    if (!mbar_wait_bounded(bars + (t & 1), (uint32_t)((t >> 1) & 1), BL_WAIT_LIMIT)) failed = true;
    else ok_upto = t;
    const void* xb = xbuf + (t & 1) * BL_XBYTES;
    // in bounds whatever the buffer holds
    for (;;) {
      if (turn == 0) {
        if (t0 != t) break;
        process_chunk<CPLX>(s0, n0, xb, acc, lane);
        next_chunk(t0, p0, n0);
        load_slot<CPLX>(s0, A, p0, n0, lane);
        turn = 1;
      } else if (turn == 1) {
        if (t1 != t) break;
        process_chunk<CPLX>(s1, n1, xb, acc, lane);
        next_chunk(t1, p1, n1);
        load_slot<CPLX>(s1, A, p1, n1, lane);
        turn = 2;
      } else {
        if (t2 != t) break;
        process_chunk<CPLX>(s2, n2, xb, acc, lane);
        next_chunk(t2, p2, n2);
        load_slot<CPLX>(s2, A, p2, n2, lane);
        turn = 0;
      }
    }
    // every warp is past tile t: its buffer takes tile t + 2
    failed = __syncthreads_or(failed) != 0;
    if (failed) break;
    if (threadIdx.x == 0 && t + 2 < nb) {
      fence_proxy_async();
      issue(t + 2);
      issued_upto = t + 2;
    }
  }
  if (failed) {
    if (threadIdx.x == 0) {
      atomicOr(A.err, 1);
      // no copy may land after the block exits: wait (bounded) for those not seen complete
      for (int t = ok_upto + 1; t <= issued_upto; t++)
        mbar_wait_bounded(bars + (t & 1), (uint32_t)((t >> 1) & 1), BL_WAIT_LIMIT);
    }
    return;
  }
  const double b = bptr ? *bptr : 0.0;
  for (int i = threadIdx.x; i < nrows; i += BL_THREADS) {
    const int64_t r = r0 + i;
    if (CPLX) {
      const float2 re = acc[2 * i], im = acc[2 * i + 1];
      double2 o = make_double2((double)re.x + (double)re.y, (double)im.x + (double)im.y);
      if (xprev) {
        const double2 p = reinterpret_cast<const double2*>(xprev)[r];
        o.x -= b * p.x;
        o.y -= b * p.y;
      }
      reinterpret_cast<double2*>(y)[r] = o;
    } else {
      const float2 a = acc[i];
      const double v = (double)a.x + (double)a.y;
      y[r] = xprev ? v - b * xprev[r] : v;
    }
  }
}

int smem_bytes(const blqh_csr* M) {
  return BL_SMEM_FIXED + M->blk_rpb * (M->is_complex ? 16 : 8);
}

}  // namespace

int blocked_mode() {
  const char* e = getenv("BLQH_SPMV_BLOCKED");
  if (!e || !e[0]) return 0;
  return e[0] == '0' ? -1 : 1;
}

// Builds the blocked layout of an FP32-valued matrix. Returns true when it
// exists afterwards. Rows longer than 65535 entries, or too many rows for one
// block's accumulators, leave the matrix on the row-parallel kernel.
bool blocked_prepare(blqh_ctx* ctx, blqh_csr* M) {
  if (M->blk_state != 0) return M->blk_state > 0;
  M->blk_state = -1;
  if (M->precision != BLQH_VAL_FP32 || M->dim < 1 || M->nnz < 1) return false;
  const int cplx = M->is_complex;
  int smem = 0;
  cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  const int per_row = cplx ? 16 : 8;
  const int64_t rpb_max = std::min<int64_t>(65535, (int64_t)(smem - BL_SMEM_FIXED) / per_row);
  if (rpb_max < BL_WARPS) return false;
  int64_t rpb = (M->dim + ctx->num_sms - 1) / ctx->num_sms;
  if (rpb > rpb_max) rpb = rpb_max;
  const int64_t blocks = (M->dim + rpb - 1) / rpb;
  const int64_t rpw = (rpb + BL_WARPS - 1) / BL_WARPS;
  const int w = BL_XBYTES / (cplx ? 16 : 8);
  const int64_t nb = (M->dim + w - 1) / w;
  const int64_t groups = blocks * BL_WARPS;
  const int64_t segs = groups * nb;
  uint16_t* rowseg = nullptr;
  int64_t* plen = nullptr;
  int* over = nullptr;
  try {
    rowseg = dalloc<uint16_t>(ctx, (size_t)M->dim * (nb + 1));
    over = dalloc<int>(ctx, 1);
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(over, 0, sizeof(int), ctx->stream));
    k_bl_rowseg<<<grid_for(ctx, M->dim, 256, 8), 256, 0, ctx->stream>>>(M->d_row_ptr, M->d_col, M->dim, w, (int)nb,
                                                                       rowseg, over);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    M->d_blen = dalloc<int32_t>(ctx, segs);
    M->d_bstart = dalloc<int64_t>(ctx, segs + 1);
    plen = dalloc<int64_t>(ctx, segs + 1);
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(plen, 0, (segs + 1) * sizeof(int64_t), ctx->stream));
    auto fill = [&](int pass) {
      if (cplx)
        k_bl_fill<true><<<(unsigned)groups, 128, 0, ctx->stream>>>(
            pass, M->d_row_ptr, M->d_col, M->d_val, rowseg, M->dim, w, (int)nb, (int)rpb, (int)rpw, M->d_blen, plen,
            M->d_bstart, M->d_bkey, M->d_bval);
      else
        k_bl_fill<false><<<(unsigned)groups, 128, 0, ctx->stream>>>(
            pass, M->d_row_ptr, M->d_col, M->d_val, rowseg, M->dim, w, (int)nb, (int)rpb, (int)rpw, M->d_blen, plen,
            M->d_bstart, M->d_bkey, M->d_bval);
      BLQH_TRY_CUDA(ctx, cudaGetLastError());
    };
    fill(0);
    int ov = 0;
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(&ov, over, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    int64_t total = 0;
    scan_exclusive_i64(ctx, plen, M->d_bstart, segs + 1, &total);  // synchronizes
    if (!ov) {
      const int64_t cap = total + 2 * BL_EPL;  // a lane's last 16-byte load may run past the padded end
      M->d_bkey = dalloc<uint32_t>(ctx, cap);
      M->d_bval = dalloc<float>(ctx, cap * (cplx ? 2 : 1));
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_bkey, 0, cap * sizeof(uint32_t), ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_bval, 0, cap * sizeof(float) * (cplx ? 2 : 1), ctx->stream));
      fill(1);
      M->d_berr = dalloc<int>(ctx, 1);
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_berr, 0, sizeof(int), ctx->stream));
      M->blk_w = w;
      M->blk_nb = (int)nb;
      M->blk_rpb = (int)rpb;
      M->blk_rpw = (int)rpw;
      M->blk_blocks = (int)blocks;
      M->blk_entries = total;
      const int sm = smem_bytes(M);
      if (cplx)
        BLQH_TRY_CUDA(ctx, cudaFuncSetAttribute(k_spmv_blocked<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
      else
        BLQH_TRY_CUDA(ctx, cudaFuncSetAttribute(k_spmv_blocked<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm));
      M->blk_state = 1;
      count_launch(ctx, TM_MISC, 3);
    }
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } catch (const BlqhError&) {
    dev_free(rowseg);
    dev_free(plen);
    dev_free(over);
    blocked_release(M);
    throw;
  }
  dev_free(rowseg);
  dev_free(plen);
  dev_free(over);
  if (M->blk_state != 1) {
    blocked_release(M);
    M->blk_state = -1;
  }
  if (getenv("BLQH_DEBUG"))
    fprintf(stderr, "blqh blocked spmv: dim %lld nnz %lld rpb %lld rpw %lld w %d nb %lld blocks %lld entries %lld\n",
            (long long)M->dim, (long long)M->nnz, (long long)rpb, (long long)rpw, w, (long long)nb,
            (long long)blocks, (long long)M->blk_entries);
  return M->blk_state > 0;
}

// Frees the blocked layout (the matrix goes back to the row-parallel kernel).
void blocked_release(blqh_csr* M) {
  dev_free(M->d_bkey);
  dev_free(M->d_bval);
  dev_free(M->d_bstart);
  dev_free(M->d_blen);
  dev_free(M->d_berr);
  M->d_bkey = nullptr;
  M->d_bval = nullptr;
  M->d_bstart = nullptr;
  M->d_blen = nullptr;
  M->d_berr = nullptr;
  if (M->blk_state > 0) M->blk_state = -1;
}

// y = H x - b xprev with the blocked layout; xs is x split into FP32 pairs
// (with 16 bytes of slack past its end).
void blocked_spmv(blqh_ctx* ctx, const blqh_csr* M, const float2* xs, double* y, const double* bptr,
                  const double* xprev, const int* stop) {
  BlArgs A;
  A.keys = M->d_bkey;
  A.vals = M->d_bval;
  A.bstart = M->d_bstart;
  A.blen = M->d_blen;
  A.w = M->blk_w;
  A.nb = M->blk_nb;
  A.rpb = M->blk_rpb;
  A.rpw = M->blk_rpw;
  A.dim = M->dim;
  A.err = M->d_berr;
  const int sm = smem_bytes(M);
  if (M->is_complex)
    k_spmv_blocked<true><<<M->blk_blocks, BL_THREADS, sm, ctx->stream>>>(A, xs, y, bptr, xprev, stop);
  else
    k_spmv_blocked<false><<<M->blk_blocks, BL_THREADS, sm, ctx->stream>>>(A, xs, y, bptr, xprev, stop);
}

// Error word of the blocked SpMV: a bounded wait that expired (cleared when read).
int blocked_error(blqh_ctx* ctx, const blqh_csr* M) {
  if (M->blk_state <= 0 || !M->d_berr) return 0;
  int e = 0;
  cudaMemcpy(&e, M->d_berr, sizeof(int), cudaMemcpyDeviceToHost);
  if (e) {
    set_error(ctx, BLQH_ERR_CUDA, "SpMV: a shared-memory tile wait expired");
    cudaMemset(M->d_berr, 0, sizeof(int));
    return BLQH_ERR_CUDA;
  }
  return 0;
}
