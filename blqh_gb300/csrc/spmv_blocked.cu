// Row-block x column-tile SpMV for FP32-valued CSR (real and complex),
// double-float accumulation (y = H x - b xprev, the Lanczos product of
// Mat::operator*, BLQH_without_spin/matrix.cpp:244-267).
//
// Why: the row-parallel CSR kernel gathers x[col] from L2 for every nonzero,
// one 32-byte sector for 8 or 16 useful bytes, and the L1 processes about one
// such divergent line per clock per SM; at Nphi = 16 that caps the product near
// 40 % of HBM bandwidth. Here x is read from shared memory instead.
//
// Layout (built once per matrix by blocked_prepare). Rows are split into
// blocks of rpb rows (one CTA each) and columns into tiles of w entries (x of
// one tile fills a 64 KB shared buffer). For block b and tile t, the block's
// rows with entries in the tile are sorted by that entry count (descending)
// and cut into slices of 32 rows; a slice of length L (its first row's count)
// is stored column-major in L steps of 32 lanes: lane l of step k holds entry
// k of the slice's row l (2-byte column within the tile, FP32 value, or
// float2 when complex; zero past the row's end). A slice header holds the 32
// rows (16-bit row within the block, 0xFFFF for an empty lane) and L. The
// slices of (b, t) are split over the CTA's warps in contiguous ranges of
// about equal cost, a step counting 1 and a slice end 2 (the warp that takes
// the short slices at the end of the count order has more ends per step).
// Within one tile a row belongs to one slice only, so a
// lane adds its row's partial sum into the block's accumulator without races
// (across tiles, see the kernel below). A row's entries are summed in column
// order and its tiles in tile order, so the result is reproducible. Storage:
// 6 bytes (10 complex) per padded entry plus 66 bytes per slice, against the
// CSR's 8 (12) plus row pointers; sorting keeps the padding to a few percent.
//
// Kernel: one CTA per row block. x tiles are double-buffered in shared memory
// by cp.async.bulk (an mbarrier per buffer completes them, every wait
// bounded). Warps move through the tiles on their own: the last warp to finish
// tile t (a counter in shared memory) fetches tile t + 2 into the freed buffer;
// the first warp to begin tile t prefetches the matrix entries of tile t + 1
// into L2 (cp.async.bulk.prefetch.L2). Each
// warp walks its steps eight at a time (all loads first), one double-float
// running sum per lane, and adds it into the row's accumulator at the end of
// each slice.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <type_traits>

#include "blqh_internal.h"
#include "krylov.cuh"

namespace {

constexpr int BL_XBYTES = 65536;  // bytes per x tile buffer
constexpr int BL_SMEM_FIXED = 128 + 2 * BL_XBYTES;
constexpr int BL_STEPS = 8;       // steps loaded at once per warp
constexpr long long BL_WAIT_LIMIT = 2000000000ll;  // clock64 cycles, about one second
constexpr int PLAN_THREADS = 256;
// Dictionary form (real matrices): the off-diagonal values of a Hamiltonian
// sector are sums of a few interaction-table entries times +-1 and 1/sqrt(Dl Dr)
// orbit factors, so they take few distinct FP32 values (about 460 at Nphi = 16,
// (J, K) = (0, 0), 2.4e8 entries). An entry is then one 32-bit word: its
// column within the 4096-wide tile (12 bits) and the index of its value in a
// table held in shared memory, 4 bytes against 6 for (2-byte column, FP32
// value). The diagonal (a different value in every row) is kept apart. This
// form is read by k_spmv_ring (below), whose tiles are 4096 columns wide.
constexpr int BL_DICT_CAP = 2048;          // values the table holds (index 0 is 0.0f, the padding)
constexpr int BL_DICT_SLOTS = 1 << 14;     // hash slots while the table is built
constexpr uint32_t BL_DICT_EMPTY = 0xFFFFFFFFu;  // a NaN pattern no matrix value has

template <bool CPLX>
struct BlShape {
  static constexpr int warps = CPLX ? 16 : 32;
  static constexpr int threads = warps * 32;
  static constexpr int xe = CPLX ? 16 : 8;  // bytes per x entry (FP32 pairs)
  static constexpr int w = BL_XBYTES / xe;  // tile width in columns
  static constexpr int ve = CPLX ? 8 : 4;   // bytes per value
  // Real: warps move through the tiles independently, even and odd tiles add
  // into separate accumulators. Complex (twice the accumulator): a block
  // barrier after every tile.
  static constexpr bool indep = !CPLX;
  static constexpr int nacc = indep ? 2 : 1;
};

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
// L2 prefetch of [p, p + bytes): rounded out to 16 bytes (every array has 16
// bytes of slack at both ends of its use), in requests of at most 64 KB.
__device__ __forceinline__ void l2_prefetch(const void* p, int64_t bytes) {
  if (bytes <= 0) return;
  uintptr_t a = reinterpret_cast<uintptr_t>(p) & ~(uintptr_t)15;
  const uintptr_t e = (reinterpret_cast<uintptr_t>(p) + (uintptr_t)bytes + 15) & ~(uintptr_t)15;
  for (; a < e; a += 65536) {
    const uint32_t n = (uint32_t)((e - a) < 65536 ? (e - a) : 65536);
    asm volatile("cp.async.bulk.prefetch.L2.global [%0], %1;" ::"l"(a), "r"(n) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Layout construction.

// rowseg[t][r] = (first entry of row r with column >= t w) - row start, t = 0..nb
// (tile-major: the plan's CTA for tile t reads consecutive rows).
// dpos (dictionary form, else null): offset of the diagonal entry within row r, 0xFFFF if the row has none.
// tstart[t]: first column of tile t (nb + 1 entries, tstart[nb] = dim).
__global__ void k_bl_rowseg(const int64_t* __restrict__ rp, const int32_t* __restrict__ col, int64_t dim,
                            const int32_t* __restrict__ tstart, int nb, uint16_t* __restrict__ rowseg, int* over,
                            uint16_t* __restrict__ dpos) {
  int longest = 0;
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x) {
    const int64_t s = rp[r], e = rp[r + 1];
    if (e - s > 65535) {
      atomicOr(over, 1);
      continue;
    }
    longest = max(longest, (int)(e - s));
    if (dpos) {  // columns of a row ascend: binary search for r
      int64_t lo = s, hi = e;
      while (lo < hi) {
        const int64_t mid = (lo + hi) >> 1;
        if (col[mid] < r) lo = mid + 1;
        else hi = mid;
      }
      dpos[r] = (lo < e && col[lo] == r) ? (uint16_t)(lo - s) : (uint16_t)0xFFFF;
    }
    int64_t k = s;
    for (int t = 0; t < nb; t++) {
      const int64_t lim = tstart[t];
      while (k < e && col[k] < lim) k++;
      rowseg[(int64_t)t * dim + r] = (uint16_t)(k - s);
    }
    rowseg[(int64_t)nb * dim + r] = (uint16_t)(e - s);
  }
  for (int o = 16; o > 0; o >>= 1) longest = max(longest, __shfl_xor_sync(0xffffffffu, longest, o));
  if ((threadIdx.x & 31) == 0) atomicMax(over + 1, longest);  // over[1]: the longest row
}

// 32-bit integer hash (the "lowbias32" finalizer from C. Wellons' hash prospector).
__device__ __forceinline__ uint32_t dict_hash(uint32_t k) {
  k ^= k >> 16;
  k *= 0x7feb352du;
  k ^= k >> 15;
  k *= 0x846ca68bu;
  k ^= k >> 16;
  return k & (BL_DICT_SLOTS - 1);
}

// Distinct off-diagonal values (FP32 bit patterns) into an open-addressing
// table, one warp per row. cnt[0] = values inserted, cnt[1] = 1 if the table
// filled up. A plain load that finds the key ends the probe; an empty slot is
// claimed with atomicCAS (a stale empty read only costs a failed CAS).
__global__ void k_dict_insert(const int64_t* __restrict__ rp, const int32_t* __restrict__ col,
                              const float* __restrict__ val, int64_t dim, uint32_t* table, int* cnt) {
  const int lane = threadIdx.x & 31;
  const int64_t warp = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nwarps = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t r = warp; r < dim; r += nwarps) {
    const int64_t s = rp[r], e = rp[r + 1];
    for (int64_t k = s + lane; k < e; k += 32) {
      if (col[k] == r) continue;
      const uint32_t key = __float_as_uint(val[k]);
      uint32_t h = dict_hash(key);
      int probe = 0;
      for (; probe < BL_DICT_SLOTS; probe++) {
        const uint32_t cur = *(volatile const uint32_t*)(table + h);
        if (cur == key) break;
        if (cur == BL_DICT_EMPTY) {
          const uint32_t prev = atomicCAS(table + h, BL_DICT_EMPTY, key);
          if (prev == BL_DICT_EMPTY) {
            atomicAdd(cnt, 1);
            break;
          }
          if (prev == key) break;
        }
        h = (h + 1) & (BL_DICT_SLOTS - 1);
      }
      if (probe == BL_DICT_SLOTS) atomicOr(cnt + 1, 1);
    }
  }
}

// One block: index 1, 2, ... to the occupied slots in slot order; dict[idx] =
// value, idx_of[slot] = idx; dict[0] = 0 (the padding entries' value).
__global__ void __launch_bounds__(PLAN_THREADS) k_dict_index(const uint32_t* __restrict__ table,
                                                              uint32_t* __restrict__ idx_of, float* __restrict__ dict) {
  constexpr int PER = BL_DICT_SLOTS / PLAN_THREADS;
  __shared__ uint32_t wsum[PLAN_THREADS / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int h0 = threadIdx.x * PER;
  uint32_t n = 0;
  for (int i = 0; i < PER; i++) n += table[h0 + i] != BL_DICT_EMPTY;
  uint32_t x = n;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[wid] = x;
  __syncthreads();
  uint32_t before = x - n;
  for (int i = 0; i < wid; i++) before += wsum[i];
  uint32_t idx = 1 + before;
  for (int i = 0; i < PER; i++) {
    const uint32_t key = table[h0 + i];
    if (key == BL_DICT_EMPTY) continue;
    idx_of[h0 + i] = idx;
    if (idx < (uint32_t)BL_DICT_CAP) dict[idx] = __uint_as_float(key);
    idx++;
  }
  if (threadIdx.x == 0) dict[0] = 0.0f;
}

__device__ __forceinline__ uint32_t dict_lookup(const uint32_t* table, const uint32_t* idx_of, uint32_t key) {
  uint32_t h = dict_hash(key);
  for (int probe = 0; probe < BL_DICT_SLOTS && table[h] != key; probe++) h = (h + 1) & (BL_DICT_SLOTS - 1);
  return idx_of[h];
}

// diag[r] = the row's diagonal value (0 if it has none).
__global__ void k_dict_diag(const int64_t* __restrict__ rp, const float* __restrict__ val,
                            const uint16_t* __restrict__ dpos, int64_t dim, float* __restrict__ diag) {
  for (int64_t r = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; r < dim; r += (int64_t)gridDim.x * blockDim.x)
    diag[r] = dpos[r] != 0xFFFF ? val[rp[r] + dpos[r]] : 0.0f;
}

struct PlanArgs {
  const int64_t* rp;
  const int32_t* col;
  const void* val;
  const uint16_t* rowseg;
  const int32_t* tstart;  // first column of each tile
  int64_t dim;
  int w, nb, rpb, warps;
  int cmax;  // largest possible count of a row in a tile: min(w, longest row)
  // warp ranges balance steps + slice_cost x slices: a slice's end (the row's
  // partial sum into the accumulator, the next headers) costs a warp about as
  // much as slice_cost steps, and warps that hold the short slices wait for
  // no one when the ranges count it
  int slice_cost;
  // pass 0 outputs
  int64_t* nslice;  // [bt]
  int64_t* nstep;   // [bt]
  // pass 1 inputs (exclusive scans of the above) and outputs
  const int64_t* slice0;  // [bt + 1]
  const int64_t* step0;   // [bt + 1]
  int32_t* split;         // [bt][2 (warps + 1)]: slice offsets, then step offsets, per warp
  uint16_t* hdr;          // [slices][32]
  uint16_t* slen;         // [slices]
  uint16_t* cols;         // [steps][32]
  void* vals;             // [steps][32]
  // dictionary form (else null): diagonal offsets, the value table, packed entries
  const uint16_t* dpos;
  const uint32_t* dtab;
  const uint32_t* didx;
  uint32_t* ents;         // [steps * 32], quad layout within each warp's range
  int colbits;            // bits of the column within the tile in a packed entry
  // dictionary form: each (block, tile) stream cut into chunks ("units") of at
  // most chunk_cap bytes (entries, headers, lengths), each split over the warps
  int chunk_cap;
  int* over;              // set when a single slice exceeds chunk_cap
  int64_t* nchunk;        // pass 0: chunks of (b, t)
  const int64_t* uchunk0; // pass 1: first unit of (b, t) (exclusive scan of nchunk)
  int32_t* usplit;        // [units][2 (warps + 1)]: slice offsets, then step offsets, per warp, chunk-relative
  int32_t* utile;         // [units] tile of the unit
  int64_t* ustep0;        // [units + 1] first step of the unit
  int64_t* uslice0;       // [units + 1] first slice of the unit
};

// Shared memory of k_bl_plan: histogram and bucket starts [cmax + 1] each,
// counts and sorted rows [rpb] each (16-bit), step prefix per slice.
__host__ __device__ inline int plan_smem(int cmax, int rpb) {
  // histogram, bucket starts, counts, sorted rows, step prefix; then chunk bounds
  // and per-slice warp ranges (dictionary form)
  return (2 * (cmax + 1)) * 4 + 2 * ((rpb * 2 + 15) / 16) * 16 + 4 * (rpb / 32 + 3) * 4;
}

// Chunks of one (block, tile) stream: consecutive slices while entries (128 B
// per step), headers and lengths (66 B per slice) stay within cap bytes.
// cb (optional) receives the chunk bounds; returns the count (>= 1).
__device__ inline int plan_chunks(const int32_t* pre, int ns, int cap, int32_t* cb, int* over) {
  int n = 0;
  int64_t bytes = 0;
  if (cb) cb[0] = 0;
  for (int s = 0; s < ns; s++) {
    const int64_t sb = (int64_t)(pre[s + 1] - pre[s]) * 128 + 66;
    if (sb > cap) atomicOr(over, 1);
    if (bytes > 0 && bytes + sb > cap) {
      n++;
      if (cb) cb[n] = s;
      bytes = 0;
    }
    bytes += sb;
  }
  n++;
  if (cb) cb[n] = ns;
  return n;
}

// Exclusive scan of one value per thread over the block; *total gets the sum.
__device__ __forceinline__ uint32_t block_scan(uint32_t v, uint32_t* wsum, uint32_t* total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) wsum[wid] = x;
  __syncthreads();
  if (wid == 0) {
    uint32_t t = lane < PLAN_THREADS / 32 ? wsum[lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    if (lane < PLAN_THREADS / 32) wsum[lane] = t;
  }
  __syncthreads();
  const uint32_t before = (wid ? wsum[wid - 1] : 0) + x - v;
  *total = wsum[PLAN_THREADS / 32 - 1];
  __syncthreads();
  return before;
}

// One CTA per (block b, tile t): the block's rows with entries in tile t,
// bucket-sorted by entry count (descending), cut into slices of 32.
// Pass 0 counts slices and steps; pass 1 writes headers, splits and entries.
template <bool CPLX>
__global__ void __launch_bounds__(PLAN_THREADS) k_bl_plan(int pass, PlanArgs P) {
  extern __shared__ __align__(16) unsigned char sm[];
  uint32_t* hist = reinterpret_cast<uint32_t*>(sm);
  uint32_t* start = hist + (P.cmax + 1);
  const int rows16 = ((P.rpb * 2 + 15) / 16) * 16;
  uint16_t* cnt = reinterpret_cast<uint16_t*>(sm + 2 * (P.cmax + 1) * 4);
  uint16_t* sorted = reinterpret_cast<uint16_t*>(sm + 2 * (P.cmax + 1) * 4 + rows16);
  int32_t* pre = reinterpret_cast<int32_t*>(sm + 2 * (P.cmax + 1) * 4 + 2 * rows16);
  __shared__ uint32_t wsum[PLAN_THREADS / 32];
  const int64_t bt = blockIdx.x;
  const int b = (int)(bt / P.nb), t = (int)(bt - (int64_t)b * P.nb);
  const int64_t r0 = (int64_t)b * P.rpb;
  const int nrows = (int)min((int64_t)P.rpb, P.dim - r0);
  for (int c = threadIdx.x; c <= P.cmax; c += PLAN_THREADS) hist[c] = 0;
  __syncthreads();
  const uint16_t* seg0 = P.rowseg + (int64_t)t * P.dim + r0;  // tile t and t + 1, this block's rows
  const uint16_t* seg1 = seg0 + P.dim;
  for (int i = threadIdx.x; i < nrows; i += PLAN_THREADS) {
    int c = (int)seg1[i] - (int)seg0[i];
    if (P.dpos) {  // the diagonal is stored apart
      const int dp = P.dpos[r0 + i];
      if (dp != 0xFFFF && dp >= (int)seg0[i] && dp < (int)seg1[i]) c--;
    }
    cnt[i] = (uint16_t)c;
    if (c > 0) atomicAdd(&hist[c], 1u);
  }
  __syncthreads();
  // start[c] = rows with a larger count (values cmax .. 1 in descending order, a run per thread)
  const int per = (P.cmax + PLAN_THREADS - 1) / PLAN_THREADS;
  const int j0 = threadIdx.x * per, j1 = min(P.cmax, j0 + per);
  uint32_t loc = 0;
  for (int j = j0; j < j1; j++) loc += hist[P.cmax - j];
  uint32_t nz = 0;
  uint32_t run = block_scan(loc, wsum, &nz);
  for (int j = j0; j < j1; j++) {
    start[P.cmax - j] = run;
    run += hist[P.cmax - j];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < nrows; i += PLAN_THREADS)
    if (cnt[i] > 0) sorted[atomicAdd(&start[cnt[i]], 1u)] = (uint16_t)i;
  __syncthreads();
  const int ns = ((int)nz + 31) / 32;
  // step prefix over the slices (a slice's length is its first row's count)
  const int sper = (ns + PLAN_THREADS - 1) / PLAN_THREADS;
  const int q0 = threadIdx.x * sper, q1 = min(ns, q0 + sper);
  uint32_t sl = 0;
  for (int q = q0; q < q1; q++) sl += cnt[sorted[32 * q]];
  uint32_t steps = 0;
  uint32_t srun = block_scan(sl, wsum, &steps);
  for (int q = q0; q < q1; q++) {
    pre[q] = (int32_t)srun;
    srun += cnt[sorted[32 * q]];
  }
  if (threadIdx.x == 0) pre[ns] = (int32_t)steps;
  if (pass == 0) {
    if (P.nchunk) __syncthreads();  // every thread's part of pre[] is written (uniform branch)
    if (threadIdx.x == 0) {
      P.nslice[bt] = ns;
      P.nstep[bt] = steps;
      if (P.nchunk) P.nchunk[bt] = plan_chunks(pre, ns, P.chunk_cap, nullptr, P.over);
    }
    return;
  }
  __syncthreads();
  // warp ranges of contiguous slices with about equal step counts
  __shared__ int32_t spl[2 * (32 + 1)];
  int32_t* sp = P.split + bt * 2 * (P.warps + 1);
  for (int wp = threadIdx.x; wp <= P.warps; wp += PLAN_THREADS) {
    int s = ns;
    if (wp < P.warps) {
      const int64_t cost = (int64_t)steps + (int64_t)P.slice_cost * ns;
      const int64_t target = (cost * wp + P.warps - 1) / P.warps;
      int lo = 0, hi = ns;  // first s with pre[s] + slice_cost s >= target
      while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (pre[mid] + (int64_t)P.slice_cost * mid < target) lo = mid + 1;
        else hi = mid;
      }
      s = lo;
    }
    sp[wp] = s;
    sp[P.warps + 1 + wp] = pre[s];
    spl[wp] = s;
    spl[P.warps + 1 + wp] = pre[s];
  }
  const int64_t s0 = P.slice0[bt], k0 = P.step0[bt];
  if (P.ents) {
    // chunks, their warp splits, and per slice the step range of its warp
    const int rs = P.rpb / 32 + 3;
    int32_t* cb = pre + rs;        // [nch + 1] chunk bounds (slices)
    int32_t* wst = cb + rs;        // per slice: first step (tile-relative) of its warp's range
    int32_t* wn = wst + rs;        // per slice: steps of its warp's range
    __shared__ int nch;
    __syncthreads();
    if (threadIdx.x == 0) nch = plan_chunks(pre, ns, P.chunk_cap, cb, P.over);
    __syncthreads();
    const int W = P.warps;
    const int64_t uc0 = P.uchunk0[bt];
    for (int c = threadIdx.x; c < nch; c += PLAN_THREADS) {
      const int a = cb[c], z = cb[c + 1];
      const int bs = pre[a], cs = pre[z] - bs;
      int32_t* us = P.usplit + (uc0 + c) * 2 * (W + 1);
      int prev = a;
      for (int wp = 0; wp <= W; wp++) {
        int sx = z;
        if (wp < W) {
          const int64_t target = ((int64_t)cs * wp + W - 1) / W;
          int lo = a, hi = z;  // first s with pre[s] - bs >= target
          while (lo < hi) {
            const int mid = (lo + hi) >> 1;
            if (pre[mid] - bs < target) lo = mid + 1;
            else hi = mid;
          }
          sx = lo;
        }
        us[wp] = sx - a;
        us[W + 1 + wp] = pre[sx] - bs;
        if (wp > 0)
          for (int q = prev; q < sx; q++) {
            wst[q] = pre[prev];
            wn[q] = pre[sx] - pre[prev];
          }
        prev = sx;
      }
      P.utile[uc0 + c] = t;
      P.ustep0[uc0 + c] = k0 + bs;
      P.uslice0[uc0 + c] = s0 + a;
    }
    __syncthreads();
    // Dictionary form. Within a warp's step range [ws, we) of n steps the first
    // 4 floor(n / 4) steps are stored in quads: quad q holds, per lane, that
    // lane's entries of steps 4q .. 4q + 3 as 16 contiguous bytes, the 32 lanes
    // one after another (512 bytes per quad); the remaining n mod 4 steps are
    // stored step by step (32 words each). Same storage as step-major order.
    for (int q = threadIdx.x; q < ns * 32; q += PLAN_THREADS) {
      const int s = q >> 5, l = q & 31;
      const int idx = 32 * s + l;
      const int i = idx < (int)nz ? sorted[idx] : -1;
      P.hdr[(s0 + s) * 32 + l] = i >= 0 ? (uint16_t)i : (uint16_t)0xFFFF;
      if (l == 0) P.slen[s0 + s] = (uint16_t)(pre[s + 1] - pre[s]);
      if (i < 0) continue;
      const int ws = wst[s], n = wn[s];  // the step range of the warp that takes slice s
      const int nq4 = n & ~3;
      const int64_t base = (k0 + ws) * 32;
      const int64_t src = P.rp[r0 + i];
      const int a = seg0[i], e = seg1[i];
      const int dp = P.dpos[r0 + i];
      int k = pre[s] - ws;  // step of this entry within the warp's range
      for (int u = a; u < e; u++) {
        if (u == dp) continue;
        const uint32_t key = __float_as_uint(reinterpret_cast<const float*>(P.val)[src + u]);
        const uint32_t c = (uint32_t)(P.col[src + u] - P.tstart[t]);
        const int64_t pos = k < nq4 ? base + (k >> 2) * 128 + l * 4 + (k & 3) : base + nq4 * 32 + (k - nq4) * 32 + l;
        P.ents[pos] = c | (dict_lookup(P.dtab, P.didx, key) << P.colbits);
        k++;
      }
    }
    return;
  }
  for (int q = threadIdx.x; q < ns * 32; q += PLAN_THREADS) {
    const int s = q >> 5, l = q & 31;
    const int idx = 32 * s + l;
    const int i = idx < (int)nz ? sorted[idx] : -1;
    P.hdr[(s0 + s) * 32 + l] = i >= 0 ? (uint16_t)i : (uint16_t)0xFFFF;
    if (l == 0) P.slen[s0 + s] = (uint16_t)(pre[s + 1] - pre[s]);
    if (i < 0) continue;
    const int64_t src = P.rp[r0 + i] + seg0[i];
    const int c = cnt[i];
    const int64_t dst0 = k0 + pre[s];
    for (int k = 0; k < c; k++) {
      const int64_t d = (dst0 + k) * 32 + l;
      P.cols[d] = (uint16_t)(P.col[src + k] - P.tstart[t]);
      if (CPLX) reinterpret_cast<float2*>(P.vals)[d] = reinterpret_cast<const float2*>(P.val)[src + k];
      else reinterpret_cast<float*>(P.vals)[d] = reinterpret_cast<const float*>(P.val)[src + k];
    }
  }
}

// ---------------------------------------------------------------------------
// The product.

struct BlArgs {
  const uint16_t* cols;
  const void* vals;
  const uint16_t* hdr;
  const uint16_t* slen;
  const int64_t* slice0;
  const int64_t* step0;
  const int32_t* split;
  int nb, rpb;
  int pf;  // tiles of matrix data prefetched into L2 ahead of the leading warp
  int64_t dim;
  int* err;
};

template <bool CPLX>
__device__ __forceinline__ void acc_add(float2* acc, int row, const float* h, const float* l) {
#pragma unroll
  for (int c = 0; c < (CPLX ? 2 : 1); c++) {
    float2 cur = acc[row * (CPLX ? 2 : 1) + c];
    df_add(cur.x, cur.y, h[c], l[c]);
    acc[row * (CPLX ? 2 : 1) + c] = cur;
  }
}

template <bool CPLX>
__global__ void __launch_bounds__(BlShape<CPLX>::threads, 1)
    k_spmv_blocked(BlArgs A, const float2* __restrict__ xs, double* __restrict__ y, const double* bptr,
                   const double* __restrict__ xprev, const int* stop) {
  using S = BlShape<CPLX>;
  constexpr int NC = CPLX ? 2 : 1;
  if (stop && *stop) return;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* bars = reinterpret_cast<uint64_t*>(smem);
  unsigned char* xbuf = smem + 128;
  float2* acc = reinterpret_cast<float2*>(smem + BL_SMEM_FIXED);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int b = blockIdx.x;
  const int64_t r0 = (int64_t)b * A.rpb;
  const int nrows = (int)min((int64_t)A.rpb, A.dim - r0);
  const int nb = A.nb;

  auto issue = [&](int t) {
    const int64_t c0 = (int64_t)t * S::w;
    const int64_t n = min((int64_t)S::w, A.dim - c0);
    const uint32_t bytes = (uint32_t)((n * S::xe + 15) & ~(int64_t)15);  // the split buffer has 16 bytes of slack
    uint64_t* bar = bars + (t & 1);
    mbar_expect_tx(bar, bytes);
    bulk_g2s(xbuf + (t & 1) * BL_XBYTES, reinterpret_cast<const char*>(xs) + c0 * S::xe, bytes, bar);
  };
  auto prefetch = [&](int t) {  // matrix data of (b, t) into L2
    const int64_t bt = (int64_t)b * nb + t;
    const int64_t k0 = A.step0[bt], k1 = A.step0[bt + 1];
    const int64_t s0 = A.slice0[bt], s1 = A.slice0[bt + 1];
    l2_prefetch(A.cols + k0 * 32, (k1 - k0) * 64);
    l2_prefetch(reinterpret_cast<const char*>(A.vals) + k0 * 32 * S::ve, (k1 - k0) * 32 * S::ve);
    l2_prefetch(A.hdr + s0 * 32, (s1 - s0) * 64);
  };

  __shared__ unsigned int s_done[2];  // warps done with a tile, per buffer (monotonic)
  __shared__ unsigned int s_begun;    // warps that began a tile (monotonic)
  __shared__ int s_issued[2];         // copies issued, per buffer
  __shared__ volatile int s_fail;     // a bounded wait expired somewhere in the block
  if (threadIdx.x == 0) {
    mbar_init(bars, 1);
    mbar_init(bars + 1, 1);
    s_done[0] = s_done[1] = 0;
    s_begun = 0;
    s_issued[0] = 1;
    s_issued[1] = nb > 1 ? 1 : 0;
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_proxy_async();
  }
  for (int i = threadIdx.x; i < A.rpb * NC * S::nacc; i += S::threads) acc[i] = make_float2(0.f, 0.f);
  __syncthreads();
  if (threadIdx.x == 0) {
    issue(0);
    if (nb > 1) issue(1);
    for (int q = 0; q < A.pf && q < nb; q++) prefetch(q);  // then tile t + pf when tile t begins
  }

  auto process_tile = [&](int t, float2* acc_t) {
    const unsigned char* xb = xbuf + (t & 1) * BL_XBYTES;
    const int64_t bt = (int64_t)b * nb + t;
    const int32_t* sp = A.split + bt * 2 * (S::warps + 1);
    const int64_t sbase = A.slice0[bt];
    const int sa = sp[warp], se = sp[warp + 1];
    const int64_t kbeg = A.step0[bt] + sp[S::warps + 1 + warp];
    int rem = sp[S::warps + 2 + warp] - sp[S::warps + 1 + warp];  // steps of this warp in the tile
    if (sa < se) {
      // slice lengths of the next 32 slices, one per lane; rows of the next four
      int s = sa;
      int lens = s + lane < se ? A.slen[sbase + s + lane] : 0;
      int row = A.hdr[(sbase + s) * 32 + lane];
      int r1 = s + 1 < se ? A.hdr[(sbase + s + 1) * 32 + lane] : 0xFFFF;
      int r2 = s + 2 < se ? A.hdr[(sbase + s + 2) * 32 + lane] : 0xFFFF;
      int r3 = s + 3 < se ? A.hdr[(sbase + s + 3) * 32 + lane] : 0xFFFF;
      int lbase = s;  // slice whose length lane 0 of `lens` holds
      int left = __shfl_sync(0xffffffffu, lens, 0);
      float h[NC], l[NC];
#pragma unroll
      for (int c = 0; c < NC; c++) h[c] = l[c] = 0.f;
      const uint16_t* pc = A.cols + kbeg * 32 + lane;
      const float2* pv2 = reinterpret_cast<const float2*>(A.vals) + kbeg * 32 + lane;
      const float* pv1 = reinterpret_cast<const float*>(A.vals) + kbeg * 32 + lane;
      // one group of up to BL_STEPS steps: all loads, then the products
      auto group = [&](auto full) {
        uint32_t cc[BL_STEPS];
        float2 vv[BL_STEPS];
#pragma unroll
        for (int u = 0; u < BL_STEPS; u++) {
          cc[u] = 0;
          vv[u] = make_float2(0.f, 0.f);
          if (decltype(full)::value || u < rem) {
            cc[u] = __ldcs(pc + u * 32);
            if (CPLX) vv[u] = __ldcs(pv2 + u * 32);
            else vv[u].x = __ldcs(pv1 + u * 32);
          }
        }
#pragma unroll
        for (int u = 0; u < BL_STEPS; u++) {
          if (decltype(full)::value || u < rem) {
            if (CPLX) {
              const float4 x = reinterpret_cast<const float4*>(xb)[cc[u]];  // (re hi, re lo, im hi, im lo)
              df_add_prod(h[0], l[0], vv[u].x, x.x, x.y);
              df_add_prod(h[0], l[0], -vv[u].y, x.z, x.w);
              df_add_prod(h[NC - 1], l[NC - 1], vv[u].x, x.z, x.w);
              df_add_prod(h[NC - 1], l[NC - 1], vv[u].y, x.x, x.y);
            } else {
              const float2 x = reinterpret_cast<const float2*>(xb)[cc[u]];
              df_add_prod(h[0], l[0], vv[u].x, x.x, x.y);
            }
            if (--left == 0) {  // end of slice s (warp-uniform)
              if (row != 0xFFFF) acc_add<CPLX>(acc_t, row, h, l);
#pragma unroll
              for (int c = 0; c < NC; c++) h[c] = l[c] = 0.f;
              s++;
              row = r1;
              r1 = r2;
              r2 = r3;
              r3 = s + 3 < se ? A.hdr[(sbase + s + 3) * 32 + lane] : 0xFFFF;
              if (s - lbase == 32) {
                lbase = s;
                lens = s + lane < se ? A.slen[sbase + s + lane] : 0;
              }
              left = __shfl_sync(0xffffffffu, lens, (s - lbase) & 31);
            }
          }
        }
        pc += BL_STEPS * 32;
        pv1 += BL_STEPS * 32;
        pv2 += BL_STEPS * 32;
        rem -= BL_STEPS;
      };
      while (rem >= BL_STEPS) group(std::true_type());
      if (rem > 0) group(std::false_type());
    }
  };

  if (!S::indep) {
    for (int t = 0; t < nb; t++) {
      if (threadIdx.x == 0 && A.pf > 0 && t + A.pf < nb) prefetch(t + A.pf);
      bool ok = !s_fail && mbar_wait_bounded(bars + (t & 1), (uint32_t)((t >> 1) & 1), BL_WAIT_LIMIT);
      ok = __all_sync(0xffffffffu, ok);  // the warp's lanes agree (process_tile shuffles)
      if (!ok) s_fail = 1;
      else process_tile(t, acc);
      __syncthreads();  // every warp is past tile t: its buffer takes tile t + 2
      if (s_fail) break;
      if (threadIdx.x == 0 && t + 2 < nb) {
        fence_proxy_async();
        issue(t + 2);
        s_issued[t & 1]++;
      }
    }
  } else {
    // Warps move through the tiles independently; the last warp to finish tile
    // t refills its buffer with tile t + 2.
    for (int t = 0; t < nb; t++) {
      // the first warp to reach tile t prefetches the matrix data of tile t + pf
      if (lane == 0 && atomicAdd(&s_begun, 1u) == (unsigned int)(S::warps * t) && A.pf > 0 && t + A.pf < nb)
        prefetch(t + A.pf);
      bool ok = !s_fail && mbar_wait_bounded(bars + (t & 1), (uint32_t)((t >> 1) & 1), BL_WAIT_LIMIT);
      if (!__all_sync(0xffffffffu, ok)) {  // the warp's lanes agree (process_tile shuffles)
        s_fail = 1;
        break;
      }
      process_tile(t, acc + (S::indep ? (t & 1) * A.rpb * NC : 0));
      __syncwarp();
      if (lane == 0) {
        __threadfence_block();  // this warp's reads of the buffer come first
        const unsigned int old = atomicAdd(&s_done[t & 1], 1u);
        if (old == (unsigned int)(S::warps * ((t >> 1) + 1) - 1) && t + 2 < nb && !s_fail) {
          __threadfence_block();
          fence_proxy_async();
          issue(t + 2);
          atomicAdd(&s_issued[t & 1], 1);
        }
      }
    }
  }
  __syncthreads();
  if (s_fail) {
    if (threadIdx.x == 0) {
      atomicOr(A.err, 1);
      // no copy may land after the block exits: the last copy issued into each
      // buffer completes after the earlier ones (bounded wait)
      for (int i = 0; i < 2; i++)
        if (s_issued[i] > 0) mbar_wait_bounded(bars + i, (uint32_t)((s_issued[i] - 1) & 1), BL_WAIT_LIMIT);
    }
    return;
  }
  const double bv = bptr ? *bptr : 0.0;
  for (int i = threadIdx.x; i < nrows; i += S::threads) {
    const int64_t r = r0 + i;
    if (CPLX) {
      const float2 re = acc[2 * i], im = acc[2 * i + 1];
      double2 o = make_double2((double)re.x + (double)re.y, (double)im.x + (double)im.y);
      if (xprev) {
        const double2 p = reinterpret_cast<const double2*>(xprev)[r];
        o.x -= bv * p.x;
        o.y -= bv * p.y;
      }
      reinterpret_cast<double2*>(y)[r] = o;
    } else {
      const float2 a = acc[i], c = acc[A.rpb + i];  // even and odd tiles
      const double v = ((double)a.x + (double)a.y) + ((double)c.x + (double)c.y);
      y[r] = xprev ? v - bv * xprev[r] : v;
    }
  }
}

// The product in dictionary form (real matrices), fed by bulk copies.
//
// Every global read of the loop goes through the tensor-memory-access path. A
// row block's work is a queue of units: each (block, tile) stream (packed
// entries, slice headers, slice lengths) is cut into chunks of at most one
// stage, each with its own split over the 32 warps, in tile order. For unit i
// one thread issues cp.async.bulk copies of its stream (and its split) into
// stage i mod S (S = 2 or 3 stages), completed on that stage's mbarrier; x's
// 4096-column tile (32 KB) is copied into one of two buffers when the tile two
// back is finished. Warps read entries (16-byte quad loads), x, the value table
// and headers from shared memory only and never wait on a global load; every
// mbarrier wait is bounded. The block finishes a unit before the next (within
// a tile a row belongs to one slice, so to one unit), so one double-float
// accumulator per row suffices; the diagonal (kept apart) is added at the end.
struct RingArgs {
  const uint32_t* ents;
  const uint16_t* hdr;
  const uint16_t* slen;
  const int32_t* usplit;   // [units][2 (W + 1)]
  const int32_t* utile;    // [units]
  const int64_t* ustep0;   // [units + 1]
  const int64_t* uslice0;  // [units + 1]
  const int64_t* uchunk0;  // [blocks * tiles + 1]: first unit of (b, t)
  const float* dict;
  const float* diag;
  int ndict, nb, rpb, stage, nstage, pf;
  int64_t dim;
  int* err;
};

constexpr int BL_RING_XBYTES = 32768;  // x tile: 4096 columns of FP32 pairs
constexpr int BL_RING_W = BL_RING_XBYTES / 8;
constexpr int BL_RING_COL_BITS = 12;
constexpr uint32_t BL_RING_COL_MASK = (1u << BL_RING_COL_BITS) - 1u;
constexpr int BL_RING_FIXED = 128 + 2 * BL_RING_XBYTES;  // barriers, x buffers
constexpr int BL_RING_MAXSTAGE = 3;

// Byte windows of unit u inside its stage: entries, headers, slice lengths and
// the warp split, each copied from a 16-byte aligned window that covers it.
struct StageMap {
  int64_t e_src, h_src, l_src, p_src;   // byte offsets in the source arrays
  uint32_t e_n, h_n, l_n, p_n;          // bytes (multiples of 16)
  uint32_t l_skip, p_skip;              // elements before the unit's own in the l / p windows
  __host__ __device__ uint32_t total() const { return e_n + h_n + l_n + p_n; }
};
__host__ __device__ inline StageMap stage_map(int64_t k0, int64_t k1, int64_t s0, int64_t s1, int64_t u, int W) {
  StageMap m;
  m.e_src = k0 * 128;
  m.e_n = (uint32_t)((k1 - k0) * 128);
  m.h_src = s0 * 64;
  m.h_n = (uint32_t)((s1 - s0) * 64);
  const int64_t la = (s0 * 2) & ~(int64_t)15, le = (s1 * 2 + 15) & ~(int64_t)15;
  m.l_src = la;
  m.l_n = (uint32_t)(le - la);
  m.l_skip = (uint32_t)((s0 * 2 - la) / 2);
  const int64_t pb = u * 2 * (W + 1) * 4;
  const int64_t pa = pb & ~(int64_t)15, pe = (pb + 2 * (W + 1) * 4 + 15) & ~(int64_t)15;
  m.p_src = pa;
  m.p_n = (uint32_t)(pe - pa);
  m.p_skip = (uint32_t)((pb - pa) / 4);
  return m;
}

__global__ void __launch_bounds__(BlShape<false>::threads, 1)
    k_spmv_ring(RingArgs A, const float2* __restrict__ xs, double* __restrict__ y, const double* bptr,
                const double* __restrict__ xprev, const int* stop) {
  constexpr int W = BlShape<false>::warps;
  if (stop && *stop) return;
  extern __shared__ __align__(128) unsigned char smem[];
  uint64_t* xbar = reinterpret_cast<uint64_t*>(smem);  // [2]
  uint64_t* sbar = xbar + 2;                           // [BL_RING_MAXSTAGE]
  unsigned char* xbuf = smem + 128;
  float2* acc = reinterpret_cast<float2*>(smem + BL_RING_FIXED);
  // the same offsets as smem_need(): accumulators, value table, stages, each 16-byte aligned
  const int acc_bytes = (A.rpb * 8 + 15) & ~15;
  float* sdict = reinterpret_cast<float*>(smem + BL_RING_FIXED + acc_bytes);
  unsigned char* stg = smem + BL_RING_FIXED + acc_bytes + ((A.ndict * 4 + 15) & ~15);
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int b = blockIdx.x;
  const int64_t r0 = (int64_t)b * A.rpb;
  const int nrows = (int)min((int64_t)A.rpb, A.dim - r0);
  const int nb = A.nb, NS = A.nstage;
  const int64_t u0 = A.uchunk0[(int64_t)b * nb];
  const int nu = (int)(A.uchunk0[(int64_t)(b + 1) * nb] - u0);

  auto map_of = [&](int i) {
    const int64_t u = u0 + i;
    return stage_map(A.ustep0[u], A.ustep0[u + 1], A.uslice0[u], A.uslice0[u + 1], u, W);
  };
  auto issue_x = [&](int t) {  // x tile t into buffer t & 1
    const int64_t c0 = (int64_t)t * BL_RING_W;
    const int64_t n = min((int64_t)BL_RING_W, A.dim - c0);
    const uint32_t xb = (uint32_t)((n * 8 + 15) & ~(int64_t)15);  // the split x has 16 bytes of slack
    mbar_expect_tx(xbar + (t & 1), xb);
    bulk_g2s(xbuf + (t & 1) * BL_RING_XBYTES, reinterpret_cast<const char*>(xs) + c0 * 8, xb, xbar + (t & 1));
  };
  auto issue_u = [&](int i) {  // unit i's stream into stage i mod NS
    const int q = i % NS;
    const StageMap m = map_of(i);
    mbar_expect_tx(sbar + q, m.total());
    unsigned char* d = stg + (size_t)q * A.stage;
    if (m.e_n) bulk_g2s(d, reinterpret_cast<const char*>(A.ents) + m.e_src, m.e_n, sbar + q);
    if (m.h_n) bulk_g2s(d + m.e_n, reinterpret_cast<const char*>(A.hdr) + m.h_src, m.h_n, sbar + q);
    if (m.l_n) bulk_g2s(d + m.e_n + m.h_n, reinterpret_cast<const char*>(A.slen) + m.l_src, m.l_n, sbar + q);
    bulk_g2s(d + m.e_n + m.h_n + m.l_n, reinterpret_cast<const char*>(A.usplit) + m.p_src, m.p_n, sbar + q);
  };
  auto prefetch = [&](int i) {
    const StageMap m = map_of(i);
    l2_prefetch(reinterpret_cast<const char*>(A.ents) + m.e_src, m.e_n);
    l2_prefetch(reinterpret_cast<const char*>(A.hdr) + m.h_src, m.h_n);
  };

  __shared__ int s_xissued[2], s_sissued[BL_RING_MAXSTAGE];
  __shared__ volatile int s_fail;
  if (threadIdx.x == 0) {
    for (int i = 0; i < 2 + BL_RING_MAXSTAGE; i++) mbar_init(xbar + i, 1);
    for (int i = 0; i < 2; i++) s_xissued[i] = 0;
    for (int i = 0; i < BL_RING_MAXSTAGE; i++) s_sissued[i] = 0;
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    fence_proxy_async();
  }
  for (int i = threadIdx.x; i < A.rpb; i += BlShape<false>::threads) acc[i] = make_float2(0.f, 0.f);
  for (int i = threadIdx.x; i < A.ndict; i += BlShape<false>::threads) sdict[i] = A.dict[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int t = 0; t < 2 && t < nb; t++) {
      issue_x(t);
      s_xissued[t]++;
    }
    for (int i = 0; i < NS && i < nu; i++) {
      issue_u(i);
      s_sissued[i]++;
    }
    for (int i = NS; i < NS + A.pf && i < nu; i++) prefetch(i);
  }

  for (int i = 0; i < nu; i++) {
    const int q = i % NS;
    const int t = A.utile[u0 + i];
    const bool ok = mbar_wait_bounded(xbar + (t & 1), (uint32_t)((t >> 1) & 1), BL_WAIT_LIMIT) &&
                    mbar_wait_bounded(sbar + q, (uint32_t)((i / NS) & 1), BL_WAIT_LIMIT);
    if (!ok) s_fail = 1;
    __syncthreads();
    if (s_fail) break;
    if (threadIdx.x == 0 && i + NS + A.pf < nu) prefetch(i + NS + A.pf);
    {
      const float2* xb = reinterpret_cast<const float2*>(xbuf + (t & 1) * BL_RING_XBYTES);
      const StageMap m = map_of(i);
      const unsigned char* d = stg + (size_t)q * A.stage;
      const uint32_t* ent = reinterpret_cast<const uint32_t*>(d);
      const uint16_t* hd = reinterpret_cast<const uint16_t*>(d + m.e_n);
      const uint16_t* sl = reinterpret_cast<const uint16_t*>(d + m.e_n + m.h_n) + m.l_skip;
      const int32_t* sp = reinterpret_cast<const int32_t*>(d + m.e_n + m.h_n + m.l_n) + m.p_skip;
      const int sa = sp[warp], se = sp[warp + 1];
      if (sa < se) {
        const int kw = sp[W + 1 + warp];
        const int rem = sp[W + 2 + warp] - kw;
        const uint32_t* pe = ent + (size_t)kw * 32;
        const uint4* pq = reinterpret_cast<const uint4*>(pe) + lane;
        int s = sa;
        int row = hd[s * 32 + lane];
        int left = sl[s];
        float h = 0.f, l = 0.f;
        auto consume = [&](uint32_t e) {
          const float2 x = xb[e & BL_RING_COL_MASK];
          df_add_prod(h, l, sdict[e >> BL_RING_COL_BITS], x.x, x.y);
          if (--left == 0) {  // end of slice s (warp-uniform)
            if (row != 0xFFFF) acc_add<false>(acc, row, &h, &l);
            h = l = 0.f;
            if (++s < se) {
              row = hd[s * 32 + lane];
              left = sl[s];
            }
          }
        };
        const int nq = rem >> 2;
        for (int qq = 0; qq < nq; qq++) {
          const uint4 e = pq[qq * 32];
          consume(e.x);
          consume(e.y);
          consume(e.z);
          consume(e.w);
        }
        for (int k = nq * 4; k < rem; k++) consume(pe[(size_t)nq * 128 + (k - nq * 4) * 32 + lane]);
      }
    }
    __syncthreads();  // every warp is past unit i: its stage takes unit i + NS
    if (threadIdx.x == 0) {
      fence_proxy_async();
      if (i + NS < nu) {
        issue_u(i + NS);
        s_sissued[q]++;
      }
      // the last unit of tile t frees x buffer t & 1 for tile t + 2
      const bool last_of_tile = i + 1 == nu || A.utile[u0 + i + 1] != t;
      if (last_of_tile && t + 2 < nb) {
        issue_x(t + 2);
        s_xissued[t & 1]++;
      }
    }
  }
  __syncthreads();
  if (s_fail) {
    if (threadIdx.x == 0) {
      atomicOr(A.err, 1);
      // no copy may land after the block exits: wait (bounded) for the last one issued into each buffer
      for (int k = 0; k < 2; k++)
        if (s_xissued[k] > 0) mbar_wait_bounded(xbar + k, (uint32_t)((s_xissued[k] - 1) & 1), BL_WAIT_LIMIT);
      for (int k = 0; k < NS; k++)
        if (s_sissued[k] > 0) mbar_wait_bounded(sbar + k, (uint32_t)((s_sissued[k] - 1) & 1), BL_WAIT_LIMIT);
    }
    return;
  }
  const double bv = bptr ? *bptr : 0.0;
  for (int i = threadIdx.x; i < nrows; i += BlShape<false>::threads) {
    const int64_t r = r0 + i;
    const float2 a = acc[i];
    const float2 xr = xs[r];
    const double v = ((double)a.x + (double)a.y) + (double)A.diag[r] * ((double)xr.x + (double)xr.y);
    y[r] = xprev ? v - bv * xprev[r] : v;
  }
}

int64_t smem_need(bool cplx, int ndict, int64_t rpb, int64_t stage, int nstage);
int smem_bytes(const blqh_csr* M) {
  return (int)smem_need(M->is_complex != 0, M->blk_dict, M->blk_rpb, M->blk_stage, M->blk_nstage);
}

template <bool CPLX>
void plan(blqh_ctx* ctx, int pass, const PlanArgs& P, int64_t nbt, int sm) {
  k_bl_plan<CPLX><<<(unsigned)nbt, PLAN_THREADS, sm, ctx->stream>>>(pass, P);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
}

}  // namespace

// BLQH_SPMV_DICT=1 builds real matrices in dictionary form (k_spmv_ring); by
// default they keep the (2-byte column, FP32 value) form, whose kernel measured
// faster on GB300 (0.59 ms against 0.75 ms per product at Nphi = 16).
static bool dict_enabled() {
  const char* e = getenv("BLQH_SPMV_DICT");
  return e && e[0] == '1';
}

// Steps one slice end is worth when the plan balances the warps' ranges
// (measured at Nphi = 16: 0.586 ms per product with 0, 0.475 ms with 2;
// BLQH_SPLIT_SLICE_COST overrides).
static int split_slice_cost() {
  const char* e = getenv("BLQH_SPLIT_SLICE_COST");
  const int v = e ? atoi(e) : 2;
  return v < 0 ? 0 : (v > 64 ? 64 : v);
}

int blocked_mode() {
  const char* e = getenv("BLQH_SPMV_BLOCKED");
  if (!e || !e[0]) return 0;
  return e[0] == '0' ? -1 : 1;
}

// Builds the blocked layout of an FP32-valued matrix. Returns true when it
// exists afterwards. Rows longer than 65535 entries, or too many rows for one
// block's accumulators, leave the matrix on the row-parallel kernel.
namespace {

// Shared memory of the product for a layout: x buffers, accumulators, and in
// dictionary form the value table and the two stages.
int64_t smem_need(bool cplx, int ndict, int64_t rpb, int64_t stage, int nstage) {
  if (ndict) return BL_RING_FIXED + ((rpb * 8 + 15) & ~15) + ((ndict * 4 + 15) & ~15) + nstage * stage;
  return BL_SMEM_FIXED + rpb * 16;  // real: two FP32-pair accumulators, complex: one complex
}

// Stages of the dictionary form (2 or 3; BLQH_RING_STAGES overrides the default 3).
int ring_stages() {
  const char* e = getenv("BLQH_RING_STAGES");
  const int v = e ? atoi(e) : 3;
  return v == 2 ? 2 : 3;
}

// One attempt at the blocked layout; use_dict selects the dictionary form
// (real matrices). Returns 1 built, 0 not built, -1 retry without the dictionary.
int blocked_prepare_impl(blqh_ctx* ctx, blqh_csr* M, bool use_dict) {
  const bool cplx = M->is_complex != 0;
  int smem = 0;
  cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  const int warps = cplx ? BlShape<true>::warps : BlShape<false>::warps;
  uint16_t* rowseg = nullptr;
  int64_t* cnt = nullptr;
  int* over = nullptr;
  uint32_t* dtab = nullptr;  // dictionary form: hash table, slot indices, diagonal offsets
  uint32_t* didx = nullptr;
  uint16_t* dpos = nullptr;
  auto free_tmp = [&]() {
    dev_free(rowseg);
    dev_free(cnt);
    dev_free(over);
    dev_free(dtab);
    dev_free(didx);
    dev_free(dpos);
    rowseg = nullptr;
    cnt = nullptr;
    over = nullptr;
    dtab = didx = nullptr;
    dpos = nullptr;
  };
  int result = 0;
  try {
    over = dalloc<int>(ctx, 8);  // [0] row too long, [1] longest row, [2..3] dictionary, [4] slice over a stage
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(over, 0, 8 * sizeof(int), ctx->stream));
    int ndict = 0;
    if (use_dict) {
      // distinct off-diagonal values; the dictionary form only when they fit the table
      dtab = dalloc<uint32_t>(ctx, BL_DICT_SLOTS);
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(dtab, 0xFF, BL_DICT_SLOTS * sizeof(uint32_t), ctx->stream));
      k_dict_insert<<<grid_for(ctx, M->dim * 32, 256, 8), 256, 0, ctx->stream>>>(
          M->d_row_ptr, M->d_col, reinterpret_cast<const float*>(M->d_val), M->dim, dtab, over + 2);
      BLQH_TRY_CUDA(ctx, cudaGetLastError());
      int dc[2] = {0, 0};
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(dc, over + 2, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (dc[1] || dc[0] + 1 > BL_DICT_CAP) {
        free_tmp();
        return -1;
      }
      ndict = dc[0] + 1;
      didx = dalloc<uint32_t>(ctx, BL_DICT_SLOTS);
      dpos = dalloc<uint16_t>(ctx, M->dim + 8);
      M->d_bdict = dalloc<float>(ctx, BL_DICT_CAP);
      k_dict_index<<<1, PLAN_THREADS, 0, ctx->stream>>>(dtab, didx, M->d_bdict);
      BLQH_TRY_CUDA(ctx, cudaGetLastError());
    }
    const int w = ndict ? BL_RING_W : (cplx ? BlShape<true>::w : BlShape<false>::w);
    // rows per block: one block per SM when the accumulators fit
    const int64_t rpb_cap = ndict ? (smem - BL_RING_FIXED - BL_DICT_CAP * 4 - 2 * 40960 - 1024) / 8
                                  : (smem - BL_SMEM_FIXED - 1024) / 16;
    const int64_t rpb_max = std::min<int64_t>(65535, rpb_cap);
    if (rpb_max < 32) {
      free_tmp();
      return ndict ? -1 : 0;
    }
    int64_t rpb = (M->dim + ctx->num_sms - 1) / ctx->num_sms;
    if (rpb > rpb_max) rpb = rpb_max;
    const int64_t blocks = (M->dim + rpb - 1) / rpb;
    // dictionary form: stages share what the x buffers, accumulators and value table leave
    const int nstage = ndict ? ring_stages() : 0;
    const int64_t stage_cap =
        ndict ? ((smem - 1024 - BL_RING_FIXED - ((rpb * 8 + 15) & ~15) - ((ndict * 4 + 15) & ~15)) / nstage) &
                    ~(int64_t)127
              : 0;
    if (ndict && stage_cap < 8192) {
      free_tmp();
      return -1;
    }
    std::vector<int32_t> ts;
    for (int64_t c = 0; c < M->dim; c += w) ts.push_back((int32_t)c);
    ts.push_back((int32_t)M->dim);
    const int64_t nb = (int64_t)ts.size() - 1;
    const int64_t nbt = blocks * nb;
    M->d_btstart = dalloc<int32_t>(ctx, nb + 1);
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(M->d_btstart, ts.data(), (nb + 1) * sizeof(int32_t), cudaMemcpyHostToDevice,
                                       ctx->stream));
    rowseg = dalloc<uint16_t>(ctx, (size_t)M->dim * (nb + 1));
    k_bl_rowseg<<<grid_for(ctx, M->dim, 256, 8), 256, 0, ctx->stream>>>(M->d_row_ptr, M->d_col, M->dim, M->d_btstart,
                                                                       (int)nb, rowseg, over, dpos);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    int ovl[2] = {0, 0};
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(ovl, over, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    const int cmax = std::max(1, std::min(w, ovl[1]));
    const int plan_sm = plan_smem(cmax, (int)rpb);
    if (ovl[0] || plan_sm > smem) {
      free_tmp();
      return ndict ? -1 : 0;
    }
    cnt = dalloc<int64_t>(ctx, 2 * (nbt + 1));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(cnt, 0, 2 * (nbt + 1) * sizeof(int64_t), ctx->stream));
    M->d_bslice0 = dalloc<int64_t>(ctx, nbt + 1);
    M->d_bstep0 = dalloc<int64_t>(ctx, nbt + 1);
    M->d_bsplit = dalloc<int32_t>(ctx, nbt * 2 * (warps + 1) + 16);
    PlanArgs P{};
    P.rp = M->d_row_ptr;
    P.col = M->d_col;
    P.val = M->d_val;
    P.rowseg = rowseg;
    P.tstart = M->d_btstart;
    P.dim = M->dim;
    P.w = w;
    P.nb = (int)nb;
    P.rpb = (int)rpb;
    P.warps = warps;
    P.cmax = cmax;
    P.slice_cost = ndict ? 0 : split_slice_cost();
    P.dpos = dpos;
    P.nslice = cnt;
    P.nstep = cnt + nbt + 1;
    int64_t* nch = nullptr;
    if (ndict) {
      nch = dalloc<int64_t>(ctx, nbt + 1);
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(nch, 0, (nbt + 1) * sizeof(int64_t), ctx->stream));
      M->d_uchunk0 = dalloc<int64_t>(ctx, nbt + 1);
      P.nchunk = nch;
      P.chunk_cap = (int)(stage_cap - 512);  // room for the length and split windows
      P.over = over + 4;
    }
    if (cplx) {
      BLQH_TRY_CUDA(ctx, smem_attr_at_least(k_bl_plan<true>, plan_sm));
      plan<true>(ctx, 0, P, nbt, plan_sm);
    } else {
      BLQH_TRY_CUDA(ctx, smem_attr_at_least(k_bl_plan<false>, plan_sm));
      plan<false>(ctx, 0, P, nbt, plan_sm);
    }
    int64_t units = 0;
    if (ndict) {
      int ov = 0;
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(&ov, over + 4, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      if (ov) {  // one slice alone exceeds a stage
        dev_free(nch);
        free_tmp();
        return -1;
      }
      scan_exclusive_i64(ctx, nch, M->d_uchunk0, nbt + 1, &units);
      dev_free(nch);
      M->d_usplit = dalloc<int32_t>(ctx, units * 2 * (warps + 1) + 16);
      M->d_utile = dalloc<int32_t>(ctx, units + 1);
      M->d_ustep0 = dalloc<int64_t>(ctx, units + 1);
      M->d_uslice0 = dalloc<int64_t>(ctx, units + 1);
      P.uchunk0 = M->d_uchunk0;
      P.usplit = M->d_usplit;
      P.utile = M->d_utile;
      P.ustep0 = M->d_ustep0;
      P.uslice0 = M->d_uslice0;
    }
    int64_t slices = 0, steps = 0;
    scan_exclusive_i64(ctx, P.nslice, M->d_bslice0, nbt + 1, &slices);
    scan_exclusive_i64(ctx, P.nstep, M->d_bstep0, nbt + 1, &steps);
    const int ve = cplx ? 8 : 4;
    M->d_bhdr = dalloc<uint16_t>(ctx, slices * 32 + 16);
    M->d_bslen = dalloc<uint16_t>(ctx, slices + 64);
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_bslen, 0, (slices + 64) * 2, ctx->stream));
    if (ndict) {
      // padding words are 0: column 0 with value index 0 (0.0f)
      M->d_bent = dalloc<uint32_t>(ctx, steps * 32 + 16);
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_bent, 0, (steps * 32 + 16) * 4, ctx->stream));
      M->d_bdiag = dalloc<float>(ctx, M->dim + 8);
      k_dict_diag<<<grid_for(ctx, M->dim, 256, 8), 256, 0, ctx->stream>>>(
          M->d_row_ptr, reinterpret_cast<const float*>(M->d_val), dpos, M->dim, M->d_bdiag);
      P.dtab = dtab;
      P.didx = didx;
      P.ents = M->d_bent;
      P.colbits = BL_RING_COL_BITS;
    } else {
      M->d_bcol = dalloc<uint16_t>(ctx, steps * 32 + 16);
      M->d_bval = dalloc<unsigned char>(ctx, (steps * 32 + 16) * ve);
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_bcol, 0, (steps * 32 + 16) * 2, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_bval, 0, (steps * 32 + 16) * ve, ctx->stream));
    }
    P.slice0 = M->d_bslice0;
    P.step0 = M->d_bstep0;
    P.split = M->d_bsplit;
    P.hdr = M->d_bhdr;
    P.slen = M->d_bslen;
    P.cols = M->d_bcol;
    P.vals = M->d_bval;
    if (cplx) plan<true>(ctx, 1, P, nbt, plan_sm);
    else plan<false>(ctx, 1, P, nbt, plan_sm);
    int64_t stage = 0;
    if (ndict) {
      // the sentinels, then the largest stage any unit needs
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(M->d_ustep0 + units, &steps, 8, cudaMemcpyHostToDevice, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(M->d_uslice0 + units, &slices, 8, cudaMemcpyHostToDevice, ctx->stream));
      std::vector<int64_t> hk(units + 1), hs(units + 1);
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(hk.data(), M->d_ustep0, (units + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(hs.data(), M->d_uslice0, (units + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      for (int64_t u = 0; u < units; u++)
        stage = std::max<int64_t>(stage, stage_map(hk[u], hk[u + 1], hs[u], hs[u + 1], u, warps).total());
      stage = (stage + 127) & ~(int64_t)127;
      if (stage > stage_cap) {  // cannot happen with the chunk cap; fall back rather than overflow
        free_tmp();
        return -1;
      }
    }
    M->d_berr = dalloc<int>(ctx, 1);
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(M->d_berr, 0, sizeof(int), ctx->stream));
    M->blk_nb = (int)nb;
    M->blk_rpb = (int)rpb;
    M->blk_blocks = (int)blocks;
    M->blk_steps = steps;
    M->blk_slices = slices;
    M->blk_dict = ndict;
    M->blk_stage = (int)stage;
    M->blk_nstage = nstage;
    M->blk_units = units;
    const int sm = smem_bytes(M);
    if (cplx)
      BLQH_TRY_CUDA(ctx, smem_attr_at_least(k_spmv_blocked<true>, sm));
    else if (ndict)
      BLQH_TRY_CUDA(ctx, smem_attr_at_least(k_spmv_ring, sm));
    else
      BLQH_TRY_CUDA(ctx, smem_attr_at_least(k_spmv_blocked<false>, sm));
    M->blk_state = 1;
    result = 1;
    count_launch(ctx, TM_MISC, ndict ? 6 : 3);
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } catch (const BlqhError&) {
    free_tmp();
    blocked_release(M);
    M->blk_state = -1;
    throw;
  }
  free_tmp();
  if (getenv("BLQH_DEBUG"))
    fprintf(stderr,
            "blqh blocked spmv: dim %lld nnz %lld rpb %d nb %d blocks %d steps %lld slices %lld dict %d stage %d x %d"
            " units %lld\n",
            (long long)M->dim, (long long)M->nnz, M->blk_rpb, M->blk_nb, M->blk_blocks, (long long)M->blk_steps,
            (long long)M->blk_slices, M->blk_dict, M->blk_stage, M->blk_nstage, (long long)M->blk_units);
  return result;
}

}  // namespace

bool blocked_prepare(blqh_ctx* ctx, blqh_csr* M) {
  if (M->blk_state != 0) return M->blk_state > 0;
  M->blk_state = -1;
  if (M->precision != BLQH_VAL_FP32 || M->dim < 1 || M->nnz < 1) return false;
  TimerScope tm(ctx, TM_MISC);
  int r = -1;
  if (!M->is_complex && dict_enabled()) r = blocked_prepare_impl(ctx, M, true);
  if (r < 0) {
    blocked_release(M);
    M->blk_state = -1;
    r = blocked_prepare_impl(ctx, M, false);
  }
  if (r <= 0) {
    blocked_release(M);
    M->blk_state = -1;
  }
  return M->blk_state > 0;
}

// Frees the blocked layout (the matrix goes back to the row-parallel kernel).
void blocked_release(blqh_csr* M) {
  dev_free(M->d_bcol);
  dev_free(M->d_bval);
  dev_free(M->d_bhdr);
  dev_free(M->d_bslen);
  dev_free(M->d_bslice0);
  dev_free(M->d_bstep0);
  dev_free(M->d_bsplit);
  dev_free(M->d_berr);
  dev_free(M->d_bent);
  dev_free(M->d_bdict);
  dev_free(M->d_bdiag);
  dev_free(M->d_btstart);
  M->d_btstart = nullptr;
  dev_free(M->d_usplit);
  dev_free(M->d_utile);
  dev_free(M->d_ustep0);
  dev_free(M->d_uslice0);
  dev_free(M->d_uchunk0);
  M->d_usplit = nullptr;
  M->d_utile = nullptr;
  M->d_ustep0 = nullptr;
  M->d_uslice0 = nullptr;
  M->d_uchunk0 = nullptr;
  M->blk_nstage = 0;
  M->blk_units = 0;
  M->d_bent = nullptr;
  M->d_bdict = nullptr;
  M->d_bdiag = nullptr;
  M->blk_dict = 0;
  M->blk_stage = 0;
  M->d_bcol = nullptr;
  M->d_bval = nullptr;
  M->d_bhdr = nullptr;
  M->d_bslen = nullptr;
  M->d_bslice0 = nullptr;
  M->d_bstep0 = nullptr;
  M->d_bsplit = nullptr;
  M->d_berr = nullptr;
  if (M->blk_state > 0) M->blk_state = -1;
}

// y = H x - b xprev with the blocked layout; xs is x split into FP32 pairs
// (with 16 bytes of slack past its end).
void blocked_spmv(blqh_ctx* ctx, const blqh_csr* M, const float2* xs, double* y, const double* bptr,
                  const double* xprev, const int* stop) {
  BlArgs A;
  A.cols = M->d_bcol;
  A.vals = M->d_bval;
  A.hdr = M->d_bhdr;
  A.slen = M->d_bslen;
  A.slice0 = M->d_bslice0;
  A.step0 = M->d_bstep0;
  A.split = M->d_bsplit;
  A.nb = M->blk_nb;
  A.rpb = M->blk_rpb;
  static const int pf = [] {
    const char* e = getenv("BLQH_BLOCKED_PREFETCH");
    const int v = e ? atoi(e) : 1;
    return v < 0 ? 0 : (v > 8 ? 8 : v);
  }();
  A.pf = pf;
  A.dim = M->dim;
  A.err = M->d_berr;
  const int sm = smem_bytes(M);
  if (M->blk_dict > 0) {
    RingArgs R{M->d_bent, M->d_bhdr, M->d_bslen, M->d_usplit, M->d_utile, M->d_ustep0, M->d_uslice0, M->d_uchunk0,
               M->d_bdict, M->d_bdiag, M->blk_dict, M->blk_nb, M->blk_rpb, M->blk_stage, M->blk_nstage, pf, M->dim,
               M->d_berr};
    k_spmv_ring<<<M->blk_blocks, BlShape<false>::threads, sm, ctx->stream>>>(R, xs, y, bptr, xprev, stop);
  } else if (M->is_complex)
    k_spmv_blocked<true><<<M->blk_blocks, BlShape<true>::threads, sm, ctx->stream>>>(A, xs, y, bptr, xprev, stop);
  else
    k_spmv_blocked<false><<<M->blk_blocks, BlShape<false>::threads, sm, ctx->stream>>>(A, xs, y, bptr, xprev, stop);
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
