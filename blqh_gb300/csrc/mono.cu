// The monolayer (Monolayer/ of the reference): basis and Hamiltonian on the device.
//
// States are nphi bits, bit n = orbital n. C = gcd(nel, nphi) magnetic
// translations move every electron by q = nphi / C orbitals (Monolayer/
// basis.cpp:59-62, 263-289).
//
// Basis (replaces basis::init and generate, basis.cpp:59-119, 216-235): the
// reference inserts every nel-subset of momentum J into a std::unordered_map in
// depth-first order (the lexicographic order of the sorted orbital tuple),
// erases while iterating each state with another member of its translation
// orbit still present, and sorts the survivors. Here every thread unranks its
// candidates from the lexicographic rank, the momentum filter and a scan give
// each inserted state its insertion index, the container's iteration order
// comes from the libstdc++ emulation shared with the bilayer bases
// (iteration_positions), and a state survives when it is last in iteration
// order among its orbit members (the erase-while-iterating rule).
//
// Hamiltonian (replaces lhamil::set_hamil, lanczos_hamiltonian.cpp:77-198):
// one warp per row. Work item w = ((k1 * npairs + p) * T + ti) walks the
// reference's loops in their order: left translation k1, occupied pair p =
// (n, m) in ascending order, hop t = ti - nphi / 2 in [-nphi / 2, nphi / 2].
// Each lane looks the target up in a table of every orbit member (member ->
// representative index and the translations that lead there; one member of an
// orbit is a representative), which gives the column, the right translation k2
// and the period Cr the reference finds by trying each k2 in turn. The warp then
// groups equal columns of a round
// of 32 items, and the lowest lane of each group adds the group's terms one by
// one, in item order, to the column's accumulator in a per-warp open-addressing
// table in shared memory. Every column therefore receives the reference's
// terms in the reference's order, and the values equal the reference's sums.
// The charging energy E_cl * nel joins the diagonal last, as in the reference
// (:187). Pass 0 counts the entries with |value| > 1e-10; pass 1 sorts them by
// column (bitonic, per warp) and writes them.
#include <algorithm>
#include <cmath>
#include <vector>

#include "blqh_internal.h"

namespace {

__device__ __forceinline__ int pc64(uint64_t x) { return __popcll(x); }

// translate (basis.cpp:263-275, inv = 0): rotate left by `bits` within nphi bits;
// inv_translate (basis.cpp:277-289, inv = 1): rotate right. *par = parity of
// c (nel - c), c = electrons in the `bits` orbitals that wrap.
__host__ __device__ __forceinline__ uint64_t mrot(uint64_t c, int bits, int nphi, int nel, int inv, int* par) {
  const uint64_t mask = (1ULL << nphi) - 1, low = (1ULL << bits) - 1;
  const int rev = nphi - bits;
  c &= mask;
#ifdef __CUDA_ARCH__
  const int ncross = __popcll(inv ? (c & low) : (c & (low << rev)));
#else
  const int ncross = __builtin_popcountll(inv ? (c & low) : (c & (low << rev)));
#endif
  *par = (ncross * (nel - ncross)) & 1;
  return inv ? (((c >> bits) | (c << rev)) & mask) : (((c << bits) | (c >> rev)) & mask);
}

__device__ __forceinline__ int64_t find_key(const uint64_t* __restrict__ sorted, int64_t n, uint64_t key) {
  int64_t lo = 0, hi = n;
  while (lo < hi) {
    const int64_t mid = (lo + hi) >> 1;
    if (sorted[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < n && sorted[lo] == key) ? lo : -1;
}

// The g-th nel-subset of [0, nphi) in lexicographic order of the sorted tuple,
// the order of the depth-first generate (basis.cpp:216-235). binom[n * 32 + k] = C(n, k).
__device__ __forceinline__ uint64_t unrank(uint64_t g, int nphi, int nel, const uint64_t* __restrict__ binom) {
  uint64_t c = 0;
  int x = 0;
  for (int i = 0; i < nel; i++) {
    for (;;) {
      const uint64_t cnt = binom[(nphi - 1 - x) * 32 + (nel - 1 - i)];
      if (g < cnt) break;
      g -= cnt;
      x++;
    }
    c |= 1ULL << x;
    x++;
  }
  return c;
}

__device__ __forceinline__ int momentum(uint64_t c) {
  int k = 0;
  for (uint64_t x = c; x; x &= x - 1) k += __ffsll((long long)x) - 1;
  return k;
}

__global__ void k_mono_enum(int64_t total, int nphi, int nel, int J, const uint64_t* __restrict__ binom,
                            uint32_t* __restrict__ ok) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
    ok[g] = (J < 0 || momentum(unrank((uint64_t)g, nphi, nel, binom)) % nphi == J) ? 1u : 0u;
}

__global__ void k_mono_scatter(int64_t total, int nphi, int nel, const uint64_t* __restrict__ binom,
                               const uint32_t* __restrict__ ok, const int64_t* __restrict__ off,
                               uint64_t* __restrict__ keys) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
    if (ok[g]) keys[off[g]] = unrank((uint64_t)g, nphi, nel, binom);
}

// keep[e]: no other member of e's orbit (right rotations by q n, n in [1, C)) is
// later in iteration order (reference survivor, basis.cpp:66-89), or smaller (BLQH_REP_MIN).
__global__ void k_mono_survive(const uint64_t* __restrict__ keys, int64_t N, const uint64_t* __restrict__ skey,
                               const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ pos, int nphi,
                               int nel, int C, int rep_mode, uint32_t* __restrict__ keep) {
  const int q = nphi / C;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t c = keys[e];
    bool live = true;
    for (int n = 1; n < C && live; n++) {
      int par;
      const uint64_t m = mrot(c, q * n, nphi, nel, 1, &par);
      if (m == c) continue;
      const int64_t s = find_key(skey, N, m);
      if (s < 0) continue;
      if (rep_mode == BLQH_REP_MIN) live = !(m < c);
      else live = !(pos[sidx[s]] > pos[e]);
    }
    keep[e] = live ? 1u : 0u;
  }
}

__global__ void k_mono_compact(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ keep,
                               const int64_t* __restrict__ off, int64_t N, uint64_t* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x)
    if (!keep || keep[e]) out[keep ? off[e] : e] = keys[e];
}

// basis_C (basis.cpp:110-118): smallest n in [1, C) with translate(id, n) == id, else C.
__global__ void k_mono_period(const uint64_t* __restrict__ ids, int64_t dim, int nphi, int nel, int C,
                              uint8_t* __restrict__ period) {
  const int q = nphi / C;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x) {
    int D = C;
    for (int n = 1; n < C; n++) {
      int par;
      if (mrot(ids[i], q * n, nphi, nel, 0, &par) == ids[i]) {
        D = n;
        break;
      }
    }
    period[i] = (uint8_t)D;
  }
}

// ---- Hamiltonian ---------------------------------------------------------------
struct MonoGen {
  const uint64_t* id;
  const uint8_t* period;
  int64_t dim;
  int nphi, nel, C, q, K, T, npairs;
  int cap;              // table slots per warp (power of two, >= npairs * T + 1)
  double diag;          // E_cl * nel
  int imag;             // K > 0: the phase factors have imaginary parts
  const double* V2;     // [nphi][nphi]: 2 V[s][|t|]
  const double2* F;     // [C][C][2 C - 1]: (cos, sin)(2 pi K d / C) / sqrt(Cl Cr) at [Cl-1][Cr-1][d + C - 1]
  int* err;             // set when a table insert finds no free slot (never, by the sizing)
  int compact;          // 1: per-(k1, pair) hop masks, only hops with empty targets become items
  const uint64_t* mkey; // orbit-member table: keys (~0 = empty)
  const uint32_t* mval; //   (representative index << 5) | translations from the representative
  uint64_t mmask;       //   slots - 1
};

constexpr uint64_t MEMBER_EMPTY = ~0ULL;

// 64-bit mixing (the finalizer of MurmurHash3) for the member table's slots.
__device__ __forceinline__ uint64_t mix64(uint64_t x) {
  x ^= x >> 33;
  x *= 0xff51afd7ed558ccdULL;
  x ^= x >> 33;
  x *= 0xc4ceb9fe1a85ec53ULL;
  x ^= x >> 33;
  return x;
}

// Every member translate(id_i, k), k in [0, period_i) (k = 0 only without
// translation symmetry), keyed to (i << 5) | k. Open addressing with linear
// probing in at least twice as many slots as members.
__global__ void k_member_insert(const uint64_t* __restrict__ id, const uint8_t* __restrict__ period, int64_t dim,
                                int nphi, int nel, int q, int orbits, uint64_t* __restrict__ key,
                                uint32_t* __restrict__ val, uint64_t mask, int* err) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x) {
    const int P = orbits ? period[i] : 1;
    for (int k = 0; k < P; k++) {
      int par;
      const uint64_t m = k == 0 ? id[i] : mrot(id[i], k * q, nphi, nel, 0, &par);
      uint64_t h = mix64(m) & mask;
      bool done = false;
      for (uint64_t probe = 0; probe <= mask; probe++) {
        const unsigned long long prev = atomicCAS(reinterpret_cast<unsigned long long*>(key + h),
                                                  (unsigned long long)MEMBER_EMPTY, (unsigned long long)m);
        if (prev == MEMBER_EMPTY || prev == m) {
          val[h] = (uint32_t)(i << 5) | (uint32_t)k;
          done = true;
          break;
        }
        h = (h + 1) & mask;
      }
      if (!done) atomicExch(err, 1);
    }
  }
}

__device__ __forceinline__ bool member_find(const uint64_t* __restrict__ key, const uint32_t* __restrict__ val,
                                            uint64_t mask, uint64_t m, uint32_t* out) {
  uint64_t h = mix64(m) & mask;
  for (uint64_t probe = 0; probe <= mask; probe++) {
    const uint64_t k = key[h];
    if (k == m) {
      *out = val[h];
      return true;
    }
    if (k == MEMBER_EMPTY) return false;
    h = (h + 1) & mask;
  }
  return false;
}

constexpr int EMPTY = -1;

// Electrons of b strictly between a and c (either order), as a parity.
__device__ __forceinline__ int occupied_between(uint64_t b, int a, int c) {
  const int lo = a < c ? a : c, hi = a < c ? c : a;
  if (hi - lo <= 1) return 0;
  return pc64(b & (((1ULL << (hi - lo - 1)) - 1) << (lo + 1))) & 1;
}

// Bit position of the k-th (0-based) set bit of x.
__device__ __forceinline__ int nth_bit(uint64_t x, int k) {
  for (int i = 0; i < k; i++) x &= x - 1;
  return __ffsll((long long)x) - 1;
}

// Slot of `col` in a per-warp table (inserted if absent; *fresh = 1 then).
__device__ __forceinline__ int table_slot(int* __restrict__ key, int cap, int col, int* err, int* fresh) {
  int h = (int)(((uint32_t)col * 2654435761u) & (uint32_t)(cap - 1));
  for (int probe = 0; probe < cap; probe++) {
    const int k = atomicCAS(&key[h], EMPTY, col);
    if (k == EMPTY || k == col) {
      *fresh = k == EMPTY;
      return h;
    }
    h = (h + 1) & (cap - 1);
  }
  atomicExch(err, 1);
  *fresh = 0;
  return -1;
}

// Per-warp shared memory: the table (cap slots: 16-byte value, 4-byte column, 8-byte sort key),
// 32 round terms and a counter, and with compaction (cq > 0) a hop mask and a prefix count per
// (k1, occupied pair).
__host__ __device__ inline size_t mono_warp_bytes(int cap, int cq) {
  return (size_t)cap * (16 + 4 + 8) + 640 + (size_t)((cq + 1) & ~1) * 8;  // a multiple of 16 bytes
}

// Pair p (0-based, ascending (a, b) with a < b) of the occupied orbitals: the a-th and b-th set bits.
__device__ __forceinline__ void pair_orbitals(uint64_t lb, int p, int nel, int* n, int* m) {
  int a = 0, rr = p;
  while (rr >= nel - 1 - a) {
    rr -= nel - 1 - a;
    a++;
  }
  *n = nth_bit(lb, a);
  *m = nth_bit(lb, a + 1 + rr);
}

// Bit ti (t = ti - nphi/2) set when orbitals (n + t) mod nphi and (m - t) mod nphi are both
// empty in lb without n and m: the hops the reference does not skip for occupied targets.
__device__ __forceinline__ uint32_t hop_mask(uint64_t lb, int n, int m, int nphi, int T) {
  const uint64_t nmask = (1ULL << nphi) - 1, tmask = (1ULL << T) - 1;
  const int half = nphi / 2;
  const uint64_t E = ~(lb ^ ((1ULL << n) | (1ULL << m))) & nmask;
  const uint64_t R = __brevll(E) >> (64 - nphi);  // bit y = bit nphi - 1 - y of E
  auto rotr = [&](uint64_t x, int sh) { return sh ? (((x >> sh) | (x << (nphi - sh))) & nmask) : x; };
  const uint64_t xa = rotr(E, ((n - half) % nphi + nphi) % nphi);            // bit ti: orbital n + t
  const uint64_t xb = rotr(R, ((nphi - 1 - m - half) % nphi + nphi) % nphi);  // bit ti: orbital m - t
  return (uint32_t)(((xa | (xa << nphi)) & (xb | (xb << nphi))) & tmask);
}

// Launch shape of one row pass. The first launch covers every row with a small
// table (`cap` slots) and gives up on a row once `limit` columns are in its
// table (marking it in ovf and appending it to ovf_list); the second covers the
// rows of ovf_list with a table that holds any row (limit = cap). Pass 1 of the
// first launch skips the marked rows.
struct RowPass {
  int cap, limit;
  const int32_t* rows;  // null: rows 0..nrows-1
  int64_t nrows;
  int64_t stride;       // pass 2: row i is written at i * stride (a staging buffer) with its length
  uint8_t* ovf;         // [dim] 1: the row is built by the second launch
  int32_t* ovf_list;
  int* ovf_count;
};

template <int CPLX>
__global__ void __launch_bounds__(256) k_mono_rows(MonoGen G, RowPass R, int pass, int64_t* __restrict__ row_nnz,
                                                   const int64_t* __restrict__ row_ptr, int32_t* __restrict__ col,
                                                   double* __restrict__ val) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5, wpb = blockDim.x >> 5;
  const int cap = R.cap;
  const int cq = G.compact ? G.C * G.npairs : 0;
  unsigned char* base = smem + (size_t)wib * mono_warp_bytes(cap, cq);
  double2* tv = reinterpret_cast<double2*>(base);                       // [cap] accumulators
  uint64_t* sb = reinterpret_cast<uint64_t*>(base + (size_t)cap * 16);  // [cap] (col << 32 | slot), sorted
  int* tk = reinterpret_cast<int*>(base + (size_t)cap * 24);            // [cap] column or EMPTY
  double2* sval = reinterpret_cast<double2*>(base + (size_t)cap * 28);  // [32] round terms
  int* used = reinterpret_cast<int*>(base + (size_t)cap * 28 + 512);    // columns in the table
  uint32_t* pm = reinterpret_cast<uint32_t*>(base + (size_t)cap * 28 + 640);  // [cq] hop masks
  int* pp = reinterpret_cast<int*>(pm + cq);                                    // [cq] prefix counts
  const int nphi = G.nphi, half = nphi / 2;
  const uint64_t nmask = (1ULL << nphi) - 1;
  const int per_k1 = G.npairs * G.T;
  for (int64_t r_ = (int64_t)blockIdx.x * wpb + wib; r_ < R.nrows; r_ += (int64_t)gridDim.x * wpb) {
    const int64_t i = R.rows ? R.rows[r_] : r_;
    if (pass == 1 && !R.rows && R.ovf[i]) continue;
    for (int s = lane; s < cap; s += 32) {
      tk[s] = EMPTY;
      tv[s] = make_double2(0.0, 0.0);
    }
    if (lane == 0) *used = 0;
    __syncwarp();
    bool full = false;
    const uint64_t idi = G.id[i];
    const int Cl = G.K < 0 ? 1 : G.period[i];
    const int nq = Cl * G.npairs;
    int nitems = Cl * per_k1;
    if (G.compact) {
      // only the hops with both targets empty, in the same (k1, pair, t) order
      for (int qq = lane; qq < nq; qq += 32) {
        const int k1 = qq / G.npairs, p = qq - k1 * G.npairs;
        int par, n, m;
        const uint64_t lb = k1 == 0 ? idi : mrot(idi, k1 * G.q, nphi, G.nel, 0, &par);
        pair_orbitals(lb, p, G.nel, &n, &m);
        pm[qq] = hop_mask(lb, n, m, nphi, G.T);
      }
      __syncwarp();
      int run = 0;
      for (int q0 = 0; q0 < nq; q0 += 32) {
        const int qq = q0 + lane;
        const int c = qq < nq ? __popc(pm[qq]) : 0;
        int incl = c;
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, incl, o);
          if (lane >= o) incl += y;
        }
        if (qq < nq) pp[qq] = run + incl - c;
        run += __shfl_sync(0xffffffffu, incl, 31);
      }
      __syncwarp();
      nitems = run;
    }
    for (int base_w = 0; base_w < nitems; base_w += 32) {
      const int w = base_w + lane;
      int hit_col = -1;
      double2 term = make_double2(0.0, 0.0);
      if (w < nitems) {
        int k1, p, t;
        if (G.compact) {
          int lo = 0, hi = nq - 1;  // the last (k1, pair) whose prefix count is <= w
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (pp[mid] <= w) lo = mid;
            else hi = mid - 1;
          }
          uint32_t x = pm[lo];
          for (int k = w - pp[lo]; k > 0; k--) x &= x - 1;
          k1 = lo / G.npairs;
          p = lo - k1 * G.npairs;
          t = __ffs(x) - 1 - half;
        } else {
          k1 = w / per_k1;
          const int r = w - k1 * per_k1;
          p = r / G.T;
          t = r - p * G.T - half;
        }
        int parl = 0;
        const uint64_t lb = k1 == 0 ? idi : mrot(idi, k1 * G.q, nphi, G.nel, 0, &parl);
        int n, m;
        pair_orbitals(lb, p, G.nel, &n, &m);
        const uint64_t b = lb ^ ((1ULL << n) | (1ULL << m));
        int nt = n + t, mt = m - t;
        if (nt >= nphi) nt -= nphi;
        else if (nt < 0) nt += nphi;
        if (mt < 0) mt += nphi;
        else if (mt >= nphi) mt -= nphi;
        // nt == mt: the reference's two masks carry into one bit and the target,
        // with nel - 1 electrons, is never in the basis
        const uint64_t mt_mask = (1ULL << nt) | (1ULL << mt);
        if (nt != mt && (mt_mask & b) == 0) {
          const uint64_t rb0 = (b | mt_mask) & nmask;
          // The reference tries inv_translate(rb0, k2) for k2 in [0, Cr), Cr the period of
          // rb0, and adds the one that is a representative (lanczos_hamiltonian.cpp:160-184);
          // the member table gives that representative and k2 in one lookup, and Cr is
          // the representative's period.
          uint32_t mv;
          if (member_find(G.mkey, G.mval, G.mmask, rb0, &mv)) {
            const int j = (int)(mv >> 5), k2 = (int)(mv & 31);
            const int Cr = G.K < 0 ? 1 : G.period[j];
            int parr = 0;
            if (k2) {
              const int nc = pc64(rb0 & ((1ULL << (k2 * G.q)) - 1));
              parr = (nc * (G.nel - nc)) & 1;
            }
            // get_sign (basis.cpp:152-174): electrons of b between n and nt and between m and mt,
            // plus one when nt > mt (the pair crosses; n < m here)
            const int par = occupied_between(b, n, nt) + occupied_between(b, m, mt) + (nt > mt ? 1 : 0) + parl + parr;
            // 2 V sign FT / sqrt(Cl Cr) (lanczos_hamiltonian.cpp:180-181): the factor is
            // tabulated on the host from the reference's expression, sign flips are exact
            const double v2 = G.V2[(mt > n ? mt - n : n - mt) * nphi + (t < 0 ? -t : t)];
            const double x = (par & 1) ? -v2 : v2;
            const double2 f = G.F[((Cl - 1) * G.C + (Cr - 1)) * (2 * G.C - 1) + (k1 - k2 + G.C - 1)];
            term = make_double2(x * f.x, G.imag ? x * f.y : 0.0);
            hit_col = j;
          }
        }
      }
      sval[lane] = term;
      __syncwarp();
      const unsigned grp = __match_any_sync(0xffffffffu, hit_col >= 0 ? hit_col : -1 - lane);
      if (hit_col >= 0 && lane == __ffs(grp) - 1) {
        int fresh;
        const int s = table_slot(tk, cap, hit_col, G.err, &fresh);
        if (fresh) atomicAdd(used, 1);
        if (s >= 0) {
          double2 acc = tv[s];
          if (G.imag) {
            for (unsigned g = grp; g; g &= g - 1) {
              const double2 v = sval[__ffs(g) - 1];
              acc.x += v.x;
              acc.y += v.y;
            }
          } else {
            for (unsigned g = grp; g; g &= g - 1) acc.x += sval[__ffs(g) - 1].x;
          }
          tv[s] = acc;
        }
      }
      __syncwarp();
      if (*used > R.limit) {
        full = true;
        break;
      }
    }
    if (full) {
      // too many columns for this table: the row goes to the second launch (pass 1
      // regenerates the same columns, so a row that fitted in pass 0 fits again)
      if (lane == 0) {
        if (pass != 1) {
          R.ovf[i] = 1;
          R.ovf_list[atomicAdd(R.ovf_count, 1)] = (int32_t)i;
          row_nnz[i] = 0;
        } else {
          atomicExch(G.err, 1);
        }
      }
      __syncwarp();
      continue;
    }
    if (lane == 0) {
      int fresh;
      const int s = table_slot(tk, cap, (int)i, G.err, &fresh);
      if (s >= 0) tv[s].x += G.diag;
    }
    __syncwarp();
    // kept entries (|value| > 1e-10, lanczos_hamiltonian.cpp:188-194)
    int kept = 0;
    for (int s0 = 0; s0 < cap; s0 += 32) {
      const int s = s0 + lane;
      bool keep = tk[s] != EMPTY;
      if (keep) {
        // |value| > 1e-10 as std::abs (hypot) decides it; the squared norm settles all
        // but values within 1e-7 of the threshold
        const double re = tv[s].x, im = tv[s].y, q = re * re + im * im;
        keep = q > 1.0000001e-20 ? true : (q < 0.9999999e-20 ? false : hypot(re, im) > 1e-10);
      }
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (pass && keep) sb[kept + __popc(bal & ((1u << lane) - 1))] = ((uint64_t)(uint32_t)tk[s] << 32) | (uint32_t)s;
      kept += __popc(bal);
    }
    if (!pass) {
      if (lane == 0) row_nnz[i] = kept;
      __syncwarp();
      continue;
    }
    int n2 = 1;
    while (n2 < kept) n2 <<= 1;
    for (int s = kept + lane; s < n2; s += 32) sb[s] = ~0ULL;
    __syncwarp();
    for (int k = 2; k <= n2; k <<= 1)
      for (int j = k >> 1; j > 0; j >>= 1) {
        for (int x = lane; x < n2; x += 32) {
          const int l = x ^ j;
          if (l > x) {
            const uint64_t u = sb[x], v = sb[l];
            if ((u > v) == ((x & k) == 0)) {
              sb[x] = v;
              sb[l] = u;
            }
          }
        }
        __syncwarp();
      }
    const int64_t o = pass == 2 ? i * R.stride : row_ptr[i];
    if (pass == 2 && lane == 0) row_nnz[i] = kept;
    for (int r = lane; r < kept; r += 32) {
      const uint64_t e = sb[r];
      const double2 v = tv[(uint32_t)e];
      col[o + r] = (int32_t)(e >> 32);
      if (CPLX) {
        val[2 * (o + r)] = v.x;
        val[2 * (o + r) + 1] = v.y;
      } else {
        val[o + r] = v.x;
      }
    }
    __syncwarp();
  }
}

// Staged rows (pass 2) into the CSR: one warp per row, rows of the second launch skipped.
__global__ void k_mono_unstage(const int32_t* __restrict__ scol, const double* __restrict__ sval, int64_t stride,
                               int vw, const int64_t* __restrict__ row_ptr, const uint8_t* __restrict__ ovf,
                               int64_t dim, int32_t* __restrict__ col, double* __restrict__ val) {
  const int lane = threadIdx.x & 31;
  const int64_t warps = (int64_t)gridDim.x * (blockDim.x >> 5);
  for (int64_t i = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < dim; i += warps) {
    if (ovf[i]) continue;
    const int64_t o = row_ptr[i], n = row_ptr[i + 1] - o, src = i * stride;
    for (int64_t k = lane; k < n; k += 32) col[o + k] = scol[src + k];
    for (int64_t k = lane; k < n * vw; k += 32) val[o * vw + k] = sval[src * vw + k];
  }
}

// lanczos_hamiltonian.cpp:53-67: V[s][ky] = sum over kx in [-nphi/2, nphi/2], (kx, ky) != 0, of
// V(kx, ky) cos(2 pi s kx / nphi) / (2 lx ly), V(q) = 2 pi / q e^{-q^2/2} (1 - e^{-q^2/2})^{2 nLL}.
void mono_coulomb_table(int nphi, double lx, double ly, int nLL, std::vector<double>& V) {
  V.assign((size_t)nphi * nphi, 0.0);
  for (int s = 0; s < nphi; s++)
    for (int ky = 0; ky < nphi; ky++) {
      double v = 0;
      for (int kx = -nphi / 2; kx <= nphi / 2; kx++) {
        if (ky == 0 && kx == 0) continue;
        const double q = std::sqrt(kx * kx / (lx * lx) + ky * ky / (ly * ly)) * 2.0 * M_PI;
        const double vq = 2.0 * M_PI / (q + 1e-30) * std::exp(-q * q / 2.0) * std::pow(1.0 - std::exp(-q * q / 2.0), nLL * 2);
        v += vq * std::cos(2.0 * M_PI * s * kx / nphi) / (2.0 * lx * ly);
      }
      V[(size_t)s * nphi + ky] = v;
    }
}

double mono_classical_energy(int nphi, double lx, double ly) {
  double E = -2.0;
  for (int i = 0; i < nphi; i++)
    for (int j = 0; j < nphi; j++)
      if (!(i == 0 && j == 0)) {
        const double z = (i * i * lx / ly + j * j * ly / lx) * M_PI;
        E += std::sqrt(M_PI / z) * std::erfc(std::sqrt(z));
      }
  return E / std::sqrt(lx * ly);
}

int gcd_int(int a, int b) {
  while (b) {
    const int t = a % b;
    a = b;
    b = t;
  }
  return a;
}

void build_mono_basis(blqh_ctx* ctx, blqh_basis* B) {
  const blqh_sector_mono& s = B->msector;
  const int nphi = s.nphi, nel = s.nel, C = gcd_int(nel, nphi);
  TimerScope ts(ctx, TM_BASIS);
  DevBufs G;
  std::vector<uint64_t> binom(32 * 32, 0);
  for (int n = 0; n < 32; n++) {
    binom[n * 32] = 1;
    for (int k = 1; k <= n; k++) binom[n * 32 + k] = binom[(n - 1) * 32 + k - 1] + (k <= n - 1 ? binom[(n - 1) * 32 + k] : 0);
  }
  const int64_t total = (int64_t)binom[nphi * 32 + nel];
  uint64_t* dbin = G.add(dalloc<uint64_t>(ctx, binom.size()));
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(dbin, binom.data(), binom.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  uint32_t* ok = G.add(dalloc<uint32_t>(ctx, total));
  int64_t* off = G.add(dalloc<int64_t>(ctx, total));
  const int BLK = 256;
  k_mono_enum<<<grid_for(ctx, total, BLK), BLK, 0, ctx->stream>>>(total, nphi, nel, s.J, dbin, ok);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  int64_t N = 0;
  scan_exclusive_u32_to_i64(ctx, ok, off, total, &N);
  B->dim = 0;
  if (N == 0) return;
  uint64_t* keys = G.add(dalloc<uint64_t>(ctx, N));
  k_mono_scatter<<<grid_for(ctx, total, BLK), BLK, 0, ctx->stream>>>(total, nphi, nel, dbin, ok, off, keys);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  const uint32_t* keep = nullptr;
  int64_t* koff = nullptr;
  int64_t dim = N;
  if (s.K >= 0 && C > 1) {
    int64_t n2 = 1;
    while (n2 < N) n2 <<= 1;
    uint64_t* skey = G.add(dalloc<uint64_t>(ctx, n2));
    uint32_t* sidx = G.add(dalloc<uint32_t>(ctx, n2));
    sorted_copy_u64(ctx, keys, N, skey, sidx, n2);
    uint32_t* pos = s.rep_mode == BLQH_REP_REFERENCE ? G.add(iteration_positions(ctx, keys, N)) : nullptr;
    uint32_t* kp = G.add(dalloc<uint32_t>(ctx, N));
    koff = G.add(dalloc<int64_t>(ctx, N));
    k_mono_survive<<<grid_for(ctx, N, BLK), BLK, 0, ctx->stream>>>(keys, N, skey, sidx, pos, nphi, nel, C,
                                                                   s.rep_mode, kp);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    scan_exclusive_u32_to_i64(ctx, kp, koff, N, &dim);
    keep = kp;
  }
  B->dim = dim;
  if (dim == 0) return;
  int64_t d2 = 1;
  while (d2 < dim) d2 <<= 1;
  uint64_t* ids = dalloc<uint64_t>(ctx, d2);
  B->d_id = ids;
  k_mono_compact<<<grid_for(ctx, N, BLK), BLK, 0, ctx->stream>>>(keys, keep, koff, N, ids);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  pad_keys_u64(ctx, ids, dim, d2);
  sort_keys_u64(ctx, ids, nullptr, d2);
  B->d_period = dalloc<uint8_t>(ctx, dim);
  k_mono_period<<<grid_for(ctx, dim, BLK), BLK, 0, ctx->stream>>>(ids, dim, nphi, nel, C, B->d_period);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_BASIS, 6);
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
}

int mono_table_cap(int nphi, int nel) {
  const int npairs = nel * (nel - 1) / 2, T = 2 * (nphi / 2) + 1;
  int cap = 32;
  while (cap < npairs * T + 1) cap <<= 1;
  return cap;
}

void build_mono_hamil(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_mono& p, blqh_csr* M) {
  const blqh_sector_mono& s = B->msector;
  const int nphi = s.nphi, nel = s.nel, C = gcd_int(nel, nphi);
  std::vector<double> V;
  mono_coulomb_table(nphi, p.lx, p.ly, p.nLL, V);
  for (double& v : V) v = 2.0 * v;  // the reference's 2.0 * Coulomb_matrix[...], exact
  // complex<double>(cos(a), sin(a)) / sqrt(Cl * Cr), a = 2 pi K (k1 - k2) / C, evaluated as the
  // reference writes it (lanczos_hamiltonian.cpp:180) for every Cl, Cr in [1, C] and k1 - k2
  const int nd = 2 * C - 1;
  std::vector<double> F((size_t)2 * C * C * nd, 0.0);
  for (int Cl = 1; Cl <= C; Cl++)
    for (int Cr = 1; Cr <= C; Cr++)
      for (int d = -(C - 1); d <= C - 1; d++) {
        const long kx = s.K < 0 ? 0 : s.K, dd = d, Cc = C, CC = (long)Cl * Cr;
        const double ang = 2.0 * M_PI * kx * dd / Cc, sq = std::sqrt((double)CC);
        const size_t o = 2 * (((size_t)(Cl - 1) * C + (Cr - 1)) * nd + (d + C - 1));
        F[o] = std::cos(ang) / sq;
        F[o + 1] = std::sin(ang) / sq;
      }
  DevBufs G;
  double* dV = G.add(dalloc<double>(ctx, V.size()));
  double* dF = G.add(dalloc<double>(ctx, F.size()));
  int* derr = G.add(dalloc<int>(ctx, 1));
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(dV, V.data(), V.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(dF, F.data(), F.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(derr, 0, 4, ctx->stream));
  const bool cplx = !(s.K <= 0 || 2 * s.K == C);
  MonoGen g{};
  g.id = B->d_id;
  g.period = B->d_period;
  g.dim = B->dim;
  g.nphi = nphi;
  g.nel = nel;
  g.C = C;
  g.q = nphi / C;
  g.K = s.K;
  g.T = 2 * (nphi / 2) + 1;
  g.npairs = nel * (nel - 1) / 2;
  g.cap = mono_table_cap(nphi, nel);
  g.diag = mono_classical_energy(nphi, p.lx, p.ly) * nel;
  g.imag = s.K > 0;
  g.V2 = dV;
  g.F = reinterpret_cast<const double2*>(dF);
  g.err = derr;
  {
    // orbit-member table: at most dim * C members (dim without translation symmetry)
    const int64_t members = s.K >= 0 ? B->dim * C : B->dim;
    uint64_t slots = 1024;
    while (slots < (uint64_t)(2 * members)) slots <<= 1;
    uint64_t* mkey = G.add(dalloc<uint64_t>(ctx, slots));
    uint32_t* mval = G.add(dalloc<uint32_t>(ctx, slots));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(mkey, 0xFF, slots * 8, ctx->stream));
    TimerScope tb(ctx, TM_BUILD);
    k_member_insert<<<grid_for(ctx, B->dim, 256), 256, 0, ctx->stream>>>(B->d_id, B->d_period, B->dim, nphi, nel,
                                                                         nphi / C, s.K >= 0, mkey, mval, slots - 1,
                                                                         derr);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_BUILD, 1);
    g.mkey = mkey;
    g.mval = mval;
    g.mmask = slots - 1;
  }
  const int64_t dim = B->dim;
  M->dim = dim;
  M->is_complex = cplx;
  M->precision = BLQH_VAL_FP64;
  M->d_row_ptr = dalloc<int64_t>(ctx, dim + 1);
  auto kern = cplx ? k_mono_rows<1> : k_mono_rows<0>;
  // first launch: a 512-slot table per warp (about 15 KB, so that 12-14 warps share an SM);
  // rows with more than 3/4 of it in use go to a second launch with a table that holds any row
  // (BLQH_MONO_FIRST_CAP, a power of two >= 64, sets the first table's size: tests use it to send rows
  // through the second launch)
  int cap_env = 512;
  if (const char* e = getenv("BLQH_MONO_FIRST_CAP")) {
    const int v = atoi(e);
    if (v >= 64 && (v & (v - 1)) == 0) cap_env = v;
  }
  const int cap_full = g.cap, cap_first = std::min(cap_full, cap_env);
  uint8_t* ovf = G.add(dalloc<uint8_t>(ctx, dim));
  int32_t* ovf_list = G.add(dalloc<int32_t>(ctx, dim));
  int* ovf_count = G.add(dalloc<int>(ctx, 1));
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(ovf, 0, dim, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(ovf_count, 0, 4, ctx->stream));
  g.compact = C * g.npairs <= 1024 && g.T <= 32;
  const int cq = g.compact ? C * g.npairs : 0;
  auto launch = [&](const RowPass& R, int pass, int32_t* dcol, double* dval) {
    const size_t per_warp = mono_warp_bytes(R.cap, cq);
    const int wpb = (int)std::max<size_t>(1, std::min<size_t>(8, (110 * 1024) / per_warp));
    const size_t sm = per_warp * wpb;
    BLQH_TRY_CUDA(ctx, smem_attr_at_least(kern, (int)sm));
    const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((R.nrows + wpb - 1) / wpb, (int64_t)ctx->num_sms * 16));
    kern<<<grid, 32 * wpb, sm, ctx->stream>>>(g, R, pass, M->d_row_ptr, M->d_row_ptr, dcol, dval);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_BUILD, 1);
  };
  const int limit = cap_first < cap_full ? cap_first * 3 / 4 : cap_first;
  // a row that fits the first table has at most limit + 1 entries (the diagonal joins last); the
  // first launch writes each row once into a staging buffer of that stride when it fits in 8 GB,
  // else it counts (pass 0) and generates the rows again to write them (pass 1)
  const int64_t stride = cap_first < cap_full ? limit + 1 : cap_first;
  const int vw = cplx ? 2 : 1;
  const bool staged = (double)dim * stride * (4 + 8 * vw) <= 8.0 * (1ULL << 30);
  int32_t* scol = staged ? G.add(dalloc<int32_t>(ctx, (size_t)dim * stride)) : nullptr;
  double* sval = staged ? G.add(dalloc<double>(ctx, (size_t)dim * stride * vw)) : nullptr;
  RowPass first{cap_first, limit, nullptr, dim, stride, ovf, ovf_list, ovf_count};
  TimerScope ts(ctx, TM_BUILD);
  launch(first, staged ? 2 : 0, scol, sval);
  int nover = 0;
  if (cap_first < cap_full) {
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(&nover, ovf_count, 4, cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  }
  RowPass second{cap_full, cap_full, ovf_list, nover, 0, ovf, ovf_list, ovf_count};
  if (nover) launch(second, 0, nullptr, nullptr);
  int64_t nnz = 0;
  scan_exclusive_i64(ctx, M->d_row_ptr, M->d_row_ptr, dim, &nnz);
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(M->d_row_ptr + dim, &nnz, 8, cudaMemcpyHostToDevice, ctx->stream));
  M->nnz = nnz;
  M->mean_row = dim ? (double)nnz / dim : 0;
  M->d_col = dalloc<int32_t>(ctx, std::max<int64_t>(1, nnz));
  M->d_val = dev_alloc(ctx, std::max<int64_t>(1, nnz) * (cplx ? 16 : 8) + 16);
  if (staged) {
    k_mono_unstage<<<grid_for(ctx, dim * 32, 256), 256, 0, ctx->stream>>>(
        scol, sval, stride, vw, M->d_row_ptr, ovf, dim, M->d_col, reinterpret_cast<double*>(M->d_val));
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_BUILD, 1);
  } else {
    launch(first, 1, M->d_col, reinterpret_cast<double*>(M->d_val));
  }
  if (nover) launch(second, 1, M->d_col, reinterpret_cast<double*>(M->d_val));
  int herr = 0;
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(&herr, derr, 4, cudaMemcpyDeviceToHost, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (herr) {
    set_error(ctx, BLQH_ERR_CAPACITY, "blqh_hamil_build_mono: a row table overflowed");
    throw BlqhError{BLQH_ERR_CAPACITY, "row table overflow"};
  }
}

}  // namespace

void mono_hamil_build_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_mono& p, blqh_csr* M) {
  build_mono_hamil(ctx, B, p, M);
}

extern "C" {

int blqh_mono_classical_energy(int nphi, double lx, double ly, double* e_cl) {
  if (!e_cl || nphi < 1 || !(lx > 0) || !(ly > 0)) return BLQH_ERR_ARG;
  *e_cl = mono_classical_energy(nphi, lx, ly);
  return BLQH_OK;
}

int blqh_mono_coulomb_table(int nphi, double lx, double ly, int nLL, double* V) {
  if (!V || nphi < 1 || !(lx > 0) || !(ly > 0) || nLL < 0) return BLQH_ERR_ARG;
  std::vector<double> t;
  mono_coulomb_table(nphi, lx, ly, nLL, t);
  std::copy(t.begin(), t.end(), V);
  return BLQH_OK;
}

int blqh_basis_build_mono(blqh_ctx* ctx, const blqh_sector_mono* s, blqh_basis** out) {
  if (!ctx || !s || !out) return BLQH_ERR_ARG;
  *out = nullptr;
  if (s->nphi < 2 || s->nphi > 31 || s->nel < 1 || s->nel > s->nphi || s->J >= s->nphi ||
      s->K >= gcd_int(s->nel, s->nphi) || (s->rep_mode != BLQH_REP_REFERENCE && s->rep_mode != BLQH_REP_MIN)) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_basis_build_mono: sector outside 2 <= nphi <= 31, 0 < nel <= nphi, "
                                         "J < nphi, K < gcd(nel, nphi)");
    return BLQH_ERR_UNSUPPORTED;
  }
  double cand = 1;
  for (int i = 1; i <= s->nel; i++) cand = cand * (s->nphi - s->nel + i) / i;
  if (cand > (double)(1 << 28)) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_basis_build_mono: more than 2^28 candidate states");
    return BLQH_ERR_UNSUPPORTED;
  }
  blqh_basis* B = new blqh_basis;
  B->ctx = ctx;
  B->model = BLQH_MODEL_MONOLAYER;
  B->msector = *s;
  B->sector.nphi = s->nphi;
  B->sector.nel = s->nel;
  B->sector.nel_up = s->nel;
  B->sector.J = s->J;
  B->sector.K = s->K;
  B->sector.rep_mode = s->rep_mode;
  try {
    cudaSetDevice(ctx->device);
    build_mono_basis(ctx, B);
  } catch (const BlqhError& e) {
    blqh_basis_destroy(B);
    return e.code;
  }
  *out = B;
  return BLQH_OK;
}

int blqh_hamil_build_mono(blqh_ctx* ctx, const blqh_basis* b, const blqh_params_mono* p, blqh_csr** out) {
  if (!ctx || !b || !p || !out) return BLQH_ERR_ARG;
  *out = nullptr;
  if (b->model != BLQH_MODEL_MONOLAYER) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_hamil_build_mono: the basis is not a monolayer basis");
    return BLQH_ERR_ARG;
  }
  if (b->dim == 0) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_hamil_build_mono: empty sector");
    return BLQH_ERR_ARG;
  }
  if (b->dim >= (1LL << 27)) {  // the member table packs (row << 5) | translations into 32 bits
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_hamil_build_mono: more than 2^27 rows");
    return BLQH_ERR_UNSUPPORTED;
  }
  if (!(p->lx > 0) || !(p->ly > 0) || p->nLL < 0) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_hamil_build_mono: lx, ly > 0 and nLL >= 0 required");
    return BLQH_ERR_ARG;
  }
  if (mono_warp_bytes(mono_table_cap(b->msector.nphi, b->msector.nel), 1024) > 200 * 1024) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_hamil_build_mono: row table larger than shared memory");
    return BLQH_ERR_UNSUPPORTED;
  }
  blqh_csr* M = new blqh_csr;
  M->ctx = ctx;
  try {
    cudaSetDevice(ctx->device);
    build_mono_hamil(ctx, b, *p, M);
  } catch (const BlqhError& e) {
    free_csr(M);
    return e.code;
  }
  *out = M;
  return BLQH_OK;
}

}  // extern "C"
