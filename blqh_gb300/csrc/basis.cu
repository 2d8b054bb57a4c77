// K1 — sector basis enumeration on the device.
//
// Replaces basis::init / generate / generate_all_density
// (BLQH_without_spin/basis.cpp:61-119, 199-259). The reference inserts every
// state of total momentum J into a std::unordered_map in depth-first order,
// then erases, while iterating the container, each state whose orbit under
// magnetic translations has another member still present; the survivors,
// sorted, are the basis. Which orbit member survives is therefore the one
// visited last in the container's iteration order.
//
// Here:
//   1. every state is enumerated in numeric order by one thread and numbered
//      with its depth-first rank (= its insertion index) from small tables;
//   2. for the reference convention, the container's iteration order is
//      reproduced level by level: libstdc++ keeps a singly linked list in which
//      each bucket's nodes are contiguous, puts a new node first in its bucket
//      (or, for an empty bucket, first in the list) and, on growth to the next
//      listed prime >= twice the bucket count, re-threads the old list in
//      order. Each growth level is a handful of data-parallel passes
//      (bucket minima, group ranks by scan, in-bucket ranks);
//   3. a state survives when it is last in that order among its orbit members
//      (or smallest, for BLQH_REP_MIN); survivors are compacted in numeric order,
//      which is the reference's sorted `id`;
//   4. per representative: orbit period (basis_C), whether the orbit carries
//      momentum K, and a map from every orbit member's dense index to
//      (representative row, translation) used by the Hamiltonian build.
#include <algorithm>
#include <cstring>
#include <unordered_map>

#include "sector.cuh"

namespace {

constexpr uint32_t NONE = 0xFFFFFFFFu;

// --------------------------------------------------------------------------
// Enumeration space in numeric order.
struct EnumSpace {
  int all_density;
  int nphi, nel, L;
  int64_t size;
  // fixed split: colex (= numeric) lists of the layer patterns
  const uint32_t* pat_u;
  const uint32_t* pat_d;
  int64_t cu, cd;
  FastDiv div_cu;  // g / cu (the fixed-split space has fewer than 2^32 states)
  // free split: binomials C(b, k), [(L+1) x (nel+1)]
  const int64_t* binom;
  // fixed split with a momentum J in [0, nphi): only the states with that
  // momentum are enumerated (1/nphi of the product space), in numeric order:
  // lower pattern i (numeric order) with the upper patterns of the residue it
  // needs, taken from pat_ur (upper patterns grouped by residue, numeric order
  // in each group, group r at uoff[r]); pre_d[i] = states before lower pattern i
  int restricted;
  int J;
  const uint32_t* pat_ur;
  const int32_t* uoff;
  const int64_t* pre_d;
  const uint8_t* resid;
};

// Restricted space: the lower pattern index of state g (pre_d[i] <= g < pre_d[i + 1]).
__device__ __forceinline__ int64_t lower_of(const EnumSpace& E, int64_t g) {
  int64_t lo = 0, hi = E.cd;
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (E.pre_d[mid] <= g) lo = mid;
    else hi = mid;
  }
  return lo;
}
// Restricted space: state g, with i its lower pattern index (advanced from a smaller g's).
__device__ __forceinline__ uint64_t valid_state(const EnumSpace& E, int64_t g, int64_t& i) {
  while (E.pre_d[i + 1] <= g) i++;
  const uint32_t d = E.pat_d[i];
  int need = E.J - (int)E.resid[d];
  need += need < 0 ? E.nphi : 0;
  return ((uint64_t)d << E.nphi) | (uint64_t)E.pat_ur[E.uoff[need] + (g - E.pre_d[i])];
}

__device__ __forceinline__ uint64_t enum_state(const EnumSpace& E, int64_t g) {
  if (E.restricted) {
    int64_t i = lower_of(E, g);
    return valid_state(E, g, i);
  }
  if (!E.all_density) {
    const int64_t rd = E.div_cu.div((uint32_t)g), ru = g - rd * E.cu;
    return ((uint64_t)E.pat_d[rd] << E.nphi) | (uint64_t)E.pat_u[ru];
  }
  uint64_t c = 0;
  int k = E.nel;
  for (int b = E.L - 1; b >= 0 && k > 0; b--) {
    const int64_t v = E.binom[b * (E.nel + 1) + k];
    if (v <= g) {
      c |= 1ULL << b;
      g -= v;
      k--;
    }
  }
  return c;
}

__global__ void k_enum_scatter(EnumSpace E, SectorIdx S, uint64_t* keys) {
  for (int64_t g = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; g < E.size; g += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t c = enum_state(E, g);
    const int64_t e = sector_index(S, c);
    if (e >= 0) keys[e] = c;
  }
}

// ---- libstdc++ iteration-order emulation, one growth level ------------------
__global__ void k_lvl_bucket(const uint64_t* keys, const uint32_t* pos, int64_t r, int64_t rn, uint64_t P,
                             uint32_t* bkt, uint32_t* first_old, uint32_t* first_new, uint32_t* cnt,
                             uint32_t* cnt_new) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < rn; e += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t b = (uint32_t)(keys[e] % P);
    bkt[e] = b;
    if (e < r) {
      atomicMin(&first_old[b], pos[e]);
    } else {
      atomicMin(&first_new[b], (uint32_t)e);
      atomicAdd(&cnt_new[b], 1u);
    }
    atomicAdd(&cnt[b], 1u);
  }
}

// Groups (non-empty buckets) in list order: buckets first filled at this level,
// most recent first; then buckets re-threaded from the old list, in decreasing
// position of their first old node. slot = rank key (dense, unique).
__global__ void k_lvl_slots(int64_t r, int64_t rn, uint64_t P, const uint32_t* first_old, const uint32_t* first_new,
                            const uint32_t* cnt, uint32_t* slot_size, uint32_t* gslot) {
  for (int64_t b = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; b < (int64_t)P; b += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t c = cnt[b];
    if (!c) continue;
    int64_t slot;
    if (first_old[b] != NONE) slot = (rn - r) + (r - 1 - (int64_t)first_old[b]);
    else slot = rn - 1 - (int64_t)first_new[b];
    slot_size[slot] = c;
    gslot[b] = (uint32_t)slot;
  }
}

__global__ void k_lvl_members(int64_t rn, const uint32_t* bkt, const int64_t* bstart, uint32_t* cursor,
                              uint32_t* members) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < rn; e += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t b = bkt[e];
    const uint32_t k = atomicAdd(&cursor[b], 1u);
    members[bstart[b] + k] = (uint32_t)e;
  }
}

// Within a group: nodes inserted at this level (latest first), then the
// re-threaded old nodes in reverse of their old order.
__global__ void k_lvl_pos(int64_t r, int64_t rn, const uint32_t* bkt, const int64_t* bstart, const uint32_t* cnt,
                          const uint32_t* cnt_new, const uint32_t* members, const uint32_t* gslot,
                          const int64_t* slot_off, const uint32_t* pos, uint32_t* new_pos) {
  for (int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; e < rn; e += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t b = bkt[e];
    const int64_t s = bstart[b];
    const uint32_t nb = cnt[b];
    uint32_t rank = 0;
    if (e >= r) {
      for (uint32_t k = 0; k < nb; k++) {
        const uint32_t f = members[s + k];
        rank += (f >= r && f > e);
      }
    } else {
      rank = cnt_new[b];
      const uint32_t pe = pos[e];
      for (uint32_t k = 0; k < nb; k++) {
        const uint32_t f = members[s + k];
        rank += (f < r && pos[f] > pe);
      }
    }
    new_pos[e] = (uint32_t)(slot_off[gslot[b]] + rank);
  }
}

// ---- survivor selection and compaction --------------------------------------
constexpr int SEL_BLOCK = 256;
constexpr int SEL_ITEMS = 8;
constexpr int SEL_TILE = SEL_BLOCK * SEL_ITEMS;

__device__ __forceinline__ bool is_survivor(const SectorIdx& S, uint64_t c, int64_t e, int rep_mode,
                                            const uint32_t* pos) {
  if (S.K < 0) return true;
  const uint32_t pe = (rep_mode == BLQH_REP_REFERENCE) ? pos[e] : 0;
  for (int n = 1; n < S.nphi; n++) {
    int par;
    const uint64_t m = inv_translate_bits(c, n, S.nphi, &par);
    if (m == c) continue;
    const int64_t em = sector_index(S, m);
    if (em < 0) continue;
    if (rep_mode == BLQH_REP_MIN) {
      if (m < c) return false;
    } else if (pos[em] > pe) {
      return false;
    }
  }
  return true;
}

__device__ int64_t block_excl_i64(int64_t v, int64_t* total) {
  __shared__ int64_t ws[SEL_BLOCK / 32];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  int64_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    int64_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) ws[wid] = x;
  __syncthreads();
  if (wid == 0) {
    int64_t w = (lane < SEL_BLOCK / 32) ? ws[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      int64_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < SEL_BLOCK / 32) ws[lane] = w;
  }
  __syncthreads();
  const int64_t off = wid ? ws[wid - 1] : 0;
  if (total) *total = ws[SEL_BLOCK / 32 - 1];
  __syncthreads();
  return off + x - v;
}

// phase 0: survivors per tile; phase 1: write them at tile offset (numeric order).
// Pass 0 runs the survivor test, counts the tile's survivors and keeps one bit
// per candidate (a word per thread); pass 1 writes the survivors' states from
// those bits, in candidate order.
__global__ void k_select(EnumSpace E, SectorIdx S, int rep_mode, const uint32_t* pos, int phase, int64_t* tile_cnt,
                         uint32_t* keepbits, uint64_t* ids) {
  static_assert(SEL_ITEMS <= 32, "one keep word per thread");
  const int64_t base = (int64_t)blockIdx.x * SEL_TILE + (int64_t)threadIdx.x * SEL_ITEMS;
  const int64_t word = (int64_t)blockIdx.x * SEL_BLOCK + threadIdx.x;
  uint32_t bitsk = 0;
  int64_t li = (E.restricted && base < E.size) ? lower_of(E, base) : 0;  // lower pattern of g = base
  if (phase == 0) {
    for (int k = 0; k < SEL_ITEMS; k++) {
      const int64_t g = base + k;
      if (g >= E.size) continue;
      const uint64_t c = E.restricted ? valid_state(E, g, li) : enum_state(E, g);
      const int64_t e = sector_index(S, c);
      if (e < 0) continue;
      if (is_survivor(S, c, e, rep_mode, pos)) bitsk |= 1u << k;
    }
    keepbits[word] = bitsk;
  } else {
    bitsk = keepbits[word];
  }
  int64_t total;
  int64_t off = block_excl_i64(__popc(bitsk), &total);
  if (phase == 0) {
    if (threadIdx.x == 0) tile_cnt[blockIdx.x] = total;
    return;
  }
  off += tile_cnt[blockIdx.x];
  for (uint32_t b = bitsk; b; b &= b - 1) {
    const int64_t g = base + __ffs(b) - 1;
    ids[off++] = E.restricted ? valid_state(E, g, li) : enum_state(E, g);
  }
}

// Orbit data per representative; map every orbit member to (row, translation).
__global__ void k_orbits(SectorIdx S, int64_t dim, const uint64_t* ids, uint8_t* period, uint8_t* compat,
                         uint32_t* map) {
  for (int64_t j = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; j < dim; j += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t c = ids[j];
    const int D = orbit_period(c, S.nphi);
    period[j] = (uint8_t)D;
    int par = 0;
    translate_bits(c, D, S.nphi, &par);
    const int64_t dk = (int64_t)D * (S.K < 0 ? 0 : S.K);
    const bool phase_one = (dk % S.nphi) == 0;
    const bool phase_minus = ((2 * dk) % (2 * S.nphi)) == S.nphi;
    compat[j] = (uint8_t)((par == 0 && phase_one) || (par == 1 && phase_minus));
    const int nq = (S.K < 0) ? 1 : D;
    for (int q = 0; q < nq; q++) {
      int p2;
      const uint64_t m = translate_bits(c, q, S.nphi, &p2);
      const int64_t em = sector_index(S, m);
      if (em >= 0) map[em] = ((uint32_t)j << 5) | (uint32_t)q;
    }
  }
}

// ---- host helpers -------------------------------------------------------------
int64_t binom_h(int n, int k) {
  if (k < 0 || k > n) return 0;
  int64_t r = 1;
  for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
  return r;
}

// k-subsets of [0, n) as bit patterns, in lexicographic order of the sorted tuple
// (the order of the reference's depth-first recursion).
void lex_patterns(int n, int k, std::vector<uint32_t>& out) {
  out.clear();
  if (k == 0) {
    out.push_back(0);
    return;
  }
  std::vector<int> o(k);
  for (int i = 0; i < k; i++) o[i] = i;
  while (true) {
    uint32_t p = 0;
    for (int i = 0; i < k; i++) p |= 1u << o[i];
    out.push_back(p);
    int i = k - 1;
    while (i >= 0 && o[i] == n - k + i) i--;
    if (i < 0) break;
    o[i]++;
    for (int t = i + 1; t < k; t++) o[t] = o[t - 1] + 1;
  }
}

struct HostTables {
  std::vector<uint32_t> upA, loB;
  std::vector<uint8_t> resid;
  std::vector<int64_t> PE;
  std::vector<uint32_t> pat_u, pat_d;  // numeric order
  std::vector<int64_t> binom;
  int64_t nvalid = 0, space = 0;
  // fixed split, 0 <= J < nphi: the momentum-restricted enumeration (EnumSpace)
  std::vector<uint32_t> pat_ur;
  std::vector<int32_t> uoff;
  std::vector<int64_t> pre_d;
};

// Numbering tables for the dense index (depth-first rank), see sector_index().
HostTables make_tables(const blqh_sector& s) {
  HostTables T;
  const int nphi = s.nphi, nel = s.nel;
  const int L = 2 * nphi;
  if (s.nel_up >= 0) {
    const int nu = s.nel_up, nd = nel - s.nel_up;
    const int P = 1 << nphi;
    T.resid.assign(P, 0);
    for (int p = 0; p < P; p++) {
      int r = 0;
      for (int b = 0; b < nphi; b++)
        if ((p >> b) & 1) r += b;
      T.resid[p] = (uint8_t)(r % nphi);
    }
    std::vector<uint32_t> lu, ld;
    lex_patterns(nphi, nu, lu);
    lex_patterns(nphi, nd, ld);
    T.upA.assign(P, 0);
    T.loB.assign((size_t)P * nphi, 0);
    const int64_t Cd = (int64_t)ld.size();
    if (s.J >= 0) {
      std::vector<int64_t> cntL(nphi, 0);
      for (uint32_t p : ld) cntL[T.resid[p]]++;
      int64_t acc = 0;
      for (uint32_t p : lu) {
        T.upA[p] = (uint32_t)acc;
        acc += (s.J < nphi) ? cntL[((s.J - T.resid[p]) % nphi + nphi) % nphi] : 0;
      }
      T.nvalid = (s.J < nphi) ? acc : 0;
      std::vector<int64_t> run(nphi, 0);
      for (uint32_t p : ld) {
        for (int r = 0; r < nphi; r++) T.loB[(size_t)p * nphi + r] = (uint32_t)run[r];
        run[T.resid[p]]++;
      }
    } else {
      for (size_t i = 0; i < lu.size(); i++) T.upA[lu[i]] = (uint32_t)(i * Cd);
      for (size_t i = 0; i < ld.size(); i++) T.loB[(size_t)ld[i] * nphi] = (uint32_t)i;
      T.nvalid = (int64_t)lu.size() * Cd;
    }
    T.pat_u = lu;
    T.pat_d = ld;
    std::sort(T.pat_u.begin(), T.pat_u.end());
    std::sort(T.pat_d.begin(), T.pat_d.end());
    T.space = (int64_t)T.pat_u.size() * (int64_t)T.pat_d.size();
    if (s.J >= 0 && s.J < nphi) {
      T.uoff.assign(nphi + 1, 0);
      for (uint32_t p : T.pat_u) T.uoff[T.resid[p] + 1]++;
      for (int r = 0; r < nphi; r++) T.uoff[r + 1] += T.uoff[r];
      T.pat_ur.assign(T.pat_u.size(), 0);
      std::vector<int32_t> fill(T.uoff.begin(), T.uoff.end() - 1);
      for (uint32_t p : T.pat_u) T.pat_ur[fill[T.resid[p]]++] = p;  // numeric order within each residue
      T.pre_d.assign(T.pat_d.size() + 1, 0);
      for (size_t i = 0; i < T.pat_d.size(); i++) {
        const int need = ((s.J - T.resid[T.pat_d[i]]) % nphi + nphi) % nphi;
        T.pre_d[i + 1] = T.pre_d[i] + (T.uoff[need + 1] - T.uoff[need]);
      }
    }
  } else {
    // dp[p][k][r]: k-subsets of [p, L) with sum(orbital mod nphi) == r (mod nphi)
    std::vector<int64_t> dp((size_t)(L + 1) * (nel + 1) * nphi, 0);
    auto D = [&](int p, int k, int r) -> int64_t& { return dp[((size_t)p * (nel + 1) + k) * nphi + r]; };
    D(L, 0, 0) = 1;
    for (int p = L - 1; p >= 0; p--)
      for (int k = 0; k <= nel; k++)
        for (int r = 0; r < nphi; r++) {
          int64_t v = D(p + 1, k, r);
          if (k > 0) v += D(p + 1, k - 1, ((r - p % nphi) % nphi + nphi) % nphi);
          D(p, k, r) = v;
        }
    T.PE.assign((size_t)(nel + 1) * (L + 1) * nphi, 0);
    for (int k = 0; k < nel; k++)
      for (int r = 0; r < nphi; r++) {
        int64_t acc = 0;
        for (int v = 0; v <= L; v++) {
          T.PE[((size_t)k * (L + 1) + v) * nphi + r] = acc;
          if (v < L) {
            if (s.J >= 0) acc += D(v + 1, k, ((r - v % nphi) % nphi + nphi) % nphi);
            else acc += binom_h(L - v - 1, k);
          }
        }
      }
    if (s.J >= 0) T.nvalid = (s.J < nphi) ? D(0, nel, s.J) : 0;
    else T.nvalid = binom_h(L, nel);
    T.binom.assign((size_t)(L + 1) * (nel + 1), 0);
    for (int b = 0; b <= L; b++)
      for (int k = 0; k <= nel; k++) T.binom[(size_t)b * (nel + 1) + k] = binom_h(b, k);
    T.space = binom_h(L, nel);
  }
  return T;
}

SectorIdx host_index(const blqh_sector& s, const HostTables& T) {
  SectorIdx S{};
  S.nphi = s.nphi;
  S.nel = s.nel;
  S.nel_up = s.nel_up;
  S.nel_dn = s.nel - s.nel_up;
  S.J = s.J;
  S.K = s.K;
  S.all_density = s.nel_up < 0;
  S.lmask = (1u << s.nphi) - 1;
  S.nvalid = T.nvalid;
  S.upA = T.upA.data();
  S.loB = T.loB.data();
  S.resid = T.resid.data();
  S.PE = T.PE.data();
  return S;
}

template <class T>
T* upload(blqh_ctx* ctx, const std::vector<T>& v) {
  if (v.empty()) return nullptr;
  T* d = dalloc<T>(ctx, v.size());
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(d, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, ctx->stream));
  return d;
}

// Bucket count libstdc++ grows to for a request of n (std::unordered_map::rehash
// on an empty container), i.e. its listed prime >= n. rehash(n) on an empty map
// asks the container's rehash policy for _M_next_bkt(n) (n >= 1) and then
// allocates and clears that many buckets: ~120 ms of host time for the level
// chain of a 1e7-state sector, during which the GPU waits. The policy's answer
// is taken directly, after checking once that it matches rehash (else rehash).
uint64_t bucket_count_by_rehash(uint64_t n) {
  std::unordered_map<uint64_t, int64_t> m;
  m.rehash(n);
  return m.bucket_count();
}
uint64_t next_bucket_count(uint64_t n) {
  static const bool policy_ok = [] {
    for (uint64_t q : {1ull, 12ull, 13ull, 29ull, 1000ull, 123457ull})
      if (std::__detail::_Prime_rehash_policy()._M_next_bkt(q) != bucket_count_by_rehash(q)) return false;
    return true;
  }();
  if (n >= 1 && policy_ok) return std::__detail::_Prime_rehash_policy()._M_next_bkt(n);
  return bucket_count_by_rehash(n);
}

int check_sector(const blqh_sector& s, std::string& why) {
  if (s.nphi < 2 || s.nphi > BLQH_MAX_NPHI) {
    why = "nphi must be in [2, 16]";
    return BLQH_ERR_UNSUPPORTED;
  }
  if (s.nel < 0 || s.nel > 2 * s.nphi) {
    why = "nel out of range";
    return BLQH_ERR_ARG;
  }
  if (s.nel_up > s.nel || (s.nel_up >= 0 && (s.nel_up > s.nphi || s.nel - s.nel_up > s.nphi))) {
    why = "nel_up out of range";
    return BLQH_ERR_ARG;
  }
  if (s.nel_up < 0 && 2 * s.nphi >= 32) {
    why = "free layer split needs 2*nphi < 32 (the reference keeps these states in 32-bit ints)";
    return BLQH_ERR_UNSUPPORTED;
  }
  if (s.rep_mode != BLQH_REP_REFERENCE && s.rep_mode != BLQH_REP_MIN) {
    why = "unknown rep_mode";
    return BLQH_ERR_ARG;
  }
  return BLQH_OK;
}

void free_basis(blqh_basis* b) {
  if (!b) return;
  dev_free(b->d_id);
  dev_free(b->d_period);
  dev_free(b->d_compat);
  dev_free(b->d_map);
  dev_free(b->d_upA);
  dev_free(b->d_loB);
  dev_free(b->d_resid);
  dev_free(b->d_PE);
  delete b;
}

}  // namespace

// Positions of N keys, inserted in the given order into a libstdc++
// std::unordered_map<unsigned long, long>, in the container's iteration order
// after the last insert (device array of N, owned by the caller).
uint32_t* iteration_positions(blqh_ctx* ctx, const uint64_t* keys, int64_t N) {
  const int BLK = 256;
  // level schedule: the first insert grows the table to next(12); level s then
  // holds until the element count reaches its bucket count P_s.
  std::vector<uint64_t> Ps;
  uint64_t P = next_bucket_count(12);
  Ps.push_back(P);
  while ((int64_t)P < N) {
    P = next_bucket_count(2 * P);
    Ps.push_back(P);
  }
  const uint64_t Pmax = Ps.back();
  DevBufs G;
  uint32_t* pos = G.add(dalloc<uint32_t>(ctx, N));
  uint32_t* npos = G.add(dalloc<uint32_t>(ctx, N));
  uint32_t* bkt = G.add(dalloc<uint32_t>(ctx, N));
  uint32_t* members = G.add(dalloc<uint32_t>(ctx, N));
  uint32_t* slot_size = G.add(dalloc<uint32_t>(ctx, N));
  int64_t* slot_off = G.add(dalloc<int64_t>(ctx, N));
  uint32_t* first_old = G.add(dalloc<uint32_t>(ctx, Pmax));
  uint32_t* first_new = G.add(dalloc<uint32_t>(ctx, Pmax));
  uint32_t* cnt = G.add(dalloc<uint32_t>(ctx, Pmax));
  uint32_t* cnt_new = G.add(dalloc<uint32_t>(ctx, Pmax));
  uint32_t* gslot = G.add(dalloc<uint32_t>(ctx, Pmax));
  uint32_t* cursor = G.add(dalloc<uint32_t>(ctx, Pmax));
  int64_t* bstart = G.add(dalloc<int64_t>(ctx, Pmax));
  int64_t r = 0;
  for (size_t lv = 0; lv < Ps.size() && r < N; lv++) {
    const uint64_t Pl = Ps[lv];
    const int64_t rn = std::min<int64_t>((int64_t)Pl, N);
    cudaStream_t st = ctx->stream;
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(first_old, 0xFF, Pl * 4, st));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(first_new, 0xFF, Pl * 4, st));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(cnt, 0, Pl * 4, st));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(cnt_new, 0, Pl * 4, st));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(cursor, 0, Pl * 4, st));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(slot_size, 0, rn * 4, st));
    k_lvl_bucket<<<grid_for(ctx, rn, BLK), BLK, 0, st>>>(keys, pos, r, rn, Pl, bkt, first_old, first_new, cnt,
                                                        cnt_new);
    k_lvl_slots<<<grid_for(ctx, (int64_t)Pl, BLK), BLK, 0, st>>>(r, rn, Pl, first_old, first_new, cnt, slot_size,
                                                                gslot);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    scan_exclusive_u32_to_i64(ctx, slot_size, slot_off, rn, nullptr);
    scan_exclusive_u32_to_i64(ctx, cnt, bstart, (int64_t)Pl, nullptr);
    k_lvl_members<<<grid_for(ctx, rn, BLK), BLK, 0, st>>>(rn, bkt, bstart, cursor, members);
    k_lvl_pos<<<grid_for(ctx, rn, BLK), BLK, 0, st>>>(r, rn, bkt, bstart, cnt, cnt_new, members, gslot, slot_off,
                                                     pos, npos);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_BASIS, 10);
    std::swap(pos, npos);
    r = rn;
  }
  // hand the result to the caller; the guard frees the other buffer
  for (auto& q : G.ps)
    if (q == pos) q = nullptr;
  return pos;
}

namespace {

void build_basis(blqh_ctx* ctx, blqh_basis* B) {
  const blqh_sector& s = B->sector;
  HostTables T = make_tables(s);
  TimerScope ts(ctx, TM_BASIS);
  B->d_upA = upload(ctx, T.upA);
  B->d_loB = upload(ctx, T.loB);
  B->d_resid = upload(ctx, T.resid);
  B->d_PE = upload(ctx, T.PE);
  B->sx = host_index(s, T);
  B->sx.upA = B->d_upA;
  B->sx.loB = B->d_loB;
  B->sx.resid = B->d_resid;
  B->sx.PE = B->d_PE;
  const SectorIdx S = B->sx;
  const int64_t N = T.nvalid;
  if (N == 0) {
    B->dim = 0;
    return;
  }
  DevBufs G;
  EnumSpace E{};
  E.all_density = S.all_density;
  E.nphi = s.nphi;
  E.nel = s.nel;
  E.L = 2 * s.nphi;
  E.size = T.space;
  E.pat_u = G.add(upload(ctx, T.pat_u));
  E.pat_d = G.add(upload(ctx, T.pat_d));
  E.cu = (int64_t)T.pat_u.size();
  E.cd = (int64_t)T.pat_d.size();
  E.div_cu = FastDiv((uint32_t)(E.cu > 0 ? E.cu : 1));
  if (!T.pre_d.empty() && T.pre_d.back() == N) {  // momentum-restricted enumeration (N states)
    E.restricted = 1;
    E.J = s.J;
    E.pat_ur = G.add(upload(ctx, T.pat_ur));
    E.uoff = G.add(upload(ctx, T.uoff));
    E.pre_d = G.add(upload(ctx, T.pre_d));
    E.resid = B->d_resid;
    E.size = N;
  }
  E.binom = G.add(upload(ctx, T.binom));
  const int BLK = 256;
  const bool emulate = (s.rep_mode == BLQH_REP_REFERENCE) && s.K >= 0;
  uint32_t* pos = nullptr;
  if (emulate) {
    uint64_t* keys = G.add(dalloc<uint64_t>(ctx, N));
    k_enum_scatter<<<grid_for(ctx, E.size, BLK), BLK, 0, ctx->stream>>>(E, S, keys);
    count_launch(ctx, TM_BASIS);
    pos = G.add(iteration_positions(ctx, keys, N));
  }
  // survivors, counted then written per tile in numeric order
  const int64_t ntiles = (E.size + SEL_TILE - 1) / SEL_TILE;
  int64_t* tile_cnt = G.add(dalloc<int64_t>(ctx, ntiles + 1));
  uint32_t* keepbits = G.add(dalloc<uint32_t>(ctx, (size_t)ntiles * SEL_BLOCK));
  k_select<<<(unsigned)ntiles, SEL_BLOCK, 0, ctx->stream>>>(E, S, s.rep_mode, pos, 0, tile_cnt, keepbits, nullptr);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  int64_t dim = 0;
  scan_exclusive_i64(ctx, tile_cnt, tile_cnt, ntiles, &dim);
  B->dim = dim;
  B->d_id = dalloc<uint64_t>(ctx, dim);
  k_select<<<(unsigned)ntiles, SEL_BLOCK, 0, ctx->stream>>>(E, S, s.rep_mode, pos, 1, tile_cnt, keepbits, B->d_id);
  B->d_period = dalloc<uint8_t>(ctx, dim);
  B->d_compat = dalloc<uint8_t>(ctx, dim);
  B->d_map = dalloc<uint32_t>(ctx, N);
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(B->d_map, 0xFF, N * 4, ctx->stream));
  k_orbits<<<grid_for(ctx, dim, BLK), BLK, 0, ctx->stream>>>(S, dim, B->d_id, B->d_period, B->d_compat, B->d_map);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_BASIS, 4);
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

int blqh_basis_build(blqh_ctx* ctx, const blqh_sector* sector, blqh_basis** out) {
  if (!ctx || !sector || !out) return BLQH_ERR_ARG;
  *out = nullptr;
  std::string why;
  int rc = check_sector(*sector, why);
  if (rc != BLQH_OK) {
    set_error(ctx, rc, "blqh_basis_build: " + why);
    return rc;
  }
  blqh_basis* B = new blqh_basis();
  B->ctx = ctx;
  B->sector = *sector;
  try {
    cudaSetDevice(ctx->device);
    build_basis(ctx, B);
  } catch (const BlqhError& e) {
    free_basis(B);
    return e.code;
  }
  *out = B;
  return BLQH_OK;
}

int blqh_basis_size(const blqh_basis* b, int64_t* dim) {
  if (!b || !dim) return BLQH_ERR_ARG;
  *dim = b->dim;
  return BLQH_OK;
}

int blqh_basis_get(blqh_ctx* ctx, const blqh_basis* b, uint64_t* ids, int16_t* periods) {
  if (!ctx || !b) return BLQH_ERR_ARG;
  if (b->dim == 0) return BLQH_OK;
  try {
    if (ids)
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(ids, b->d_id, b->dim * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (periods) {
      std::vector<uint8_t> p(b->dim);
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(p.data(), b->d_period, b->dim, cudaMemcpyDeviceToHost, ctx->stream));
      BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
      for (int64_t i = 0; i < b->dim; i++) periods[i] = (int16_t)p[i];
    }
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_basis_destroy(blqh_basis* b) {
  free_basis(b);
  return BLQH_OK;
}

// Host evaluation of the dense state index (for CPU-side checks of the tables).
int blqh_debug_sector_index(const blqh_sector* s, int64_t n, const uint64_t* states, int64_t* index_out,
                            int64_t* nvalid_out) {
  if (!s || (n && (!states || !index_out))) return BLQH_ERR_ARG;
  std::string why;
  int rc = check_sector(*s, why);
  if (rc != BLQH_OK) {
    set_error(nullptr, rc, why);
    return rc;
  }
  HostTables T = make_tables(*s);
  SectorIdx S = host_index(*s, T);
  for (int64_t i = 0; i < n; i++) index_out[i] = sector_index(S, states[i]);
  if (nvalid_out) *nvalid_out = T.nvalid;
  return BLQH_OK;
}

}  // extern "C"
