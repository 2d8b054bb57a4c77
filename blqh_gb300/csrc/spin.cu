// The spinful bilayer (BLQH_with_spin): basis and Hamiltonian on the device.
//
// States are 4 * nphi bits in four blocks of nphi orbitals: block 0 = upper
// layer spin up, 1 = upper spin down, 2 = lower spin up, 3 = lower spin down
// (BLQH_with_spin/basis.cpp:262-300 fills bits [0, 2 nphi) with the upper
// layer, basis.cpp:98-108 counts spin up as blocks 0 and 2).
//
// Basis (replaces basis::init, generate_fixed_density, generate_all_density,
// basis.cpp:74-141, 240-300): the reference inserts every state of momentum J
// into a std::unordered_map in depth-first order (the lexicographic order of
// the sorted orbital tuple), erases while iterating each state whose orbit has
// another member still present, then erases states with the wrong spin count
// and sorts the survivors. Here: candidates are enumerated in that order, the
// momentum filter and a scan give each inserted state its insertion index, the
// container's iteration order comes from the same libstdc++ emulation as the
// spinless basis (iteration_positions), lookups use a sorted copy (bitonic
// sort), a state survives when it is last in iteration order among its orbit
// members present, and the spin filter and sort follow.
//
// Hamiltonian (replaces lhamil::peer_set_hamil, lanczos_hamiltonian.cpp:86-927):
// one thread block per row accumulates the row densely in shared memory, as
// the reference accumulates it in a dense vector: ten two-body families
// (same-spin and opposite-spin pairs in each layer with the intralayer table,
// four interlayer pairs with the interlayer table, the two opposite-spin ones
// with the twist phase), layer tunnelling with the parallel-field phase and
// spin-flip tunnelling (both only for Delta_SAS > 0), the charging, bias and
// Zeeman diagonal; entries with |value| > 1e-10 are kept. Sector sizes are
// modest in this model (474 states at nphi = 6): the dense row limits a
// sector to BLQH_SPIN_MAX_DIM states. Values are FP64 (the accumulation order
// differs from the reference's by the threads' atomics: values agree to
// rounding).
#include <algorithm>
#include <cmath>
#include <vector>

#include "blqh_internal.h"

namespace {

constexpr uint64_t KEY_PAD = ~0ULL;

__device__ __forceinline__ int pc64(uint64_t x) { return __popcll(x); }

// Translate (inv = 0: rotate every block left by `bits`) or inverse translate
// (rotate right), with the reference's fermion parity (basis.cpp:401-477).
__device__ __forceinline__ uint64_t rot4(uint64_t c, int bits, int nphi, int inv, int* par) {
  const uint64_t mask = (1ULL << nphi) - 1;
  const uint64_t msign = inv ? ((1ULL << bits) - 1) : (((1ULL << bits) - 1) << (nphi - bits));
  uint64_t out = 0;
  int nsign = 0;
  for (int b = 0; b < 4; b++) {
    const uint64_t x = (c >> (b * nphi)) & mask;
    const int ncross = pc64(x & msign), nb = pc64(x);
    nsign += (nb - ncross) * ncross;
    const uint64_t y = inv ? (((x >> bits) | (x << (nphi - bits))) & mask) : (((x << bits) | (x >> (nphi - bits))) & mask);
    out |= y << (b * nphi);
  }
  *par = nsign & 1;
  return out;
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

// Candidate g in depth-first order. Fixed split: g = upper index * n_lower + lower index
// over the lexicographic pattern lists; free split: the lexicographic list of nel-subsets.
__global__ void k_spin_enum(const uint64_t* __restrict__ pu, int64_t nu, const uint64_t* __restrict__ pl, int64_t nl,
                            int nphi, int J, uint32_t* __restrict__ ok, int64_t total) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t c = pl ? (pu[g / nl] | pl[g % nl]) : pu[g];
    int k = 0;
    for (uint64_t x = c; x; x &= x - 1) k += (__ffsll((long long)x) - 1) % nphi;
    ok[g] = (J < 0 || k % nphi == J) ? 1u : 0u;
  }
}

__global__ void k_spin_scatter(const uint64_t* __restrict__ pu, int64_t nu, const uint64_t* __restrict__ pl, int64_t nl,
                               const uint32_t* __restrict__ ok, const int64_t* __restrict__ off, int64_t total,
                               uint64_t* __restrict__ keys) {
  for (int64_t g = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; g < total; g += (int64_t)gridDim.x * blockDim.x)
    if (ok[g]) keys[off[g]] = pl ? (pu[g / nl] | pl[g % nl]) : pu[g];
}

// One stage of a bitonic sort of (key, value) pairs, n a power of two.
__global__ void k_bitonic(uint64_t* __restrict__ key, uint32_t* __restrict__ val, int64_t n, int64_t k, int64_t j) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t l = i ^ j;
    if (l <= i) continue;
    const bool up = (i & k) == 0;
    const uint64_t a = key[i], b = key[l];
    if ((a > b) == up) {
      key[i] = b;
      key[l] = a;
      if (val) {
        const uint32_t t = val[i];
        val[i] = val[l];
        val[l] = t;
      }
    }
  }
}

// keep[e]: the state survives the orbit filter (last in iteration order among
// its present orbit members, or smallest for BLQH_REP_MIN) and has nel_su spin-up electrons.
__global__ void k_spin_survive(const uint64_t* __restrict__ keys, int64_t N, const uint64_t* __restrict__ skey,
                               const uint32_t* __restrict__ sidx, const uint32_t* __restrict__ pos, int nphi, int K,
                               int rep_mode, int nel_su, uint32_t* __restrict__ keep) {
  const uint64_t mask = (1ULL << nphi) - 1;
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x) {
    const uint64_t c = keys[e];
    bool live = true;
    if (K >= 0)
      for (int n = 1; n < nphi && live; n++) {
        int par;
        const uint64_t m = rot4(c, n, nphi, 1, &par);
        if (m == c) continue;
        const int64_t s = find_key(skey, N, m);
        if (s < 0) continue;
        if (rep_mode == BLQH_REP_MIN) live = !(m < c);
        else live = !(pos[sidx[s]] > pos[e]);
      }
    if (live && nel_su >= 0) live = (pc64(c & mask) + pc64((c >> (2 * nphi)) & mask)) == nel_su;
    keep[e] = live ? 1u : 0u;
  }
}

__global__ void k_spin_compact(const uint64_t* __restrict__ keys, const uint32_t* __restrict__ keep,
                               const int64_t* __restrict__ off, int64_t N, uint64_t* __restrict__ out) {
  for (int64_t e = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; e < N; e += (int64_t)gridDim.x * blockDim.x)
    if (keep[e]) out[off[e]] = keys[e];
}

__global__ void k_spin_period(const uint64_t* __restrict__ ids, int64_t dim, int nphi, uint8_t* __restrict__ period) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x) {
    int D = nphi;
    for (int n = 1; n < nphi; n++) {
      int par;
      if (rot4(ids[i], n, nphi, 1, &par) == ids[i]) {
        D = n;
        break;
      }
    }
    period[i] = (uint8_t)D;
  }
}

// ---- Hamiltonian --------------------------------------------------------------
struct SpinGen {
  const uint64_t* id;
  const uint8_t* period;
  int64_t dim;
  int nphi, nel, K;
  double Ec, d, dsas, dv, dz, theta_b, theta_y;
  const double* V;  // [2][nphi][nphi]
};

// Parity of the empty orbitals of c strictly between a and b (a < b): get_sign(c, n, nt), basis.cpp:187-197.
__device__ __forceinline__ int empties_between(uint64_t c, int a, int b) {
  if (b - a <= 1) return 0;
  const uint64_t span = ((1ULL << (b - a - 1)) - 1) << (a + 1);
  return ((b - a - 1) - pc64(c & span)) & 1;
}

// get_sign(c, n, m, nt, mt, t) of basis.cpp:158-185 as a parity.
__device__ __forceinline__ int pair_parity(uint64_t c, int n, int m, int nt, int mt) {
  const uint64_t b = c ^ ((1ULL << n) | (1ULL << m));
  int ns = 0;
  int kl = nt < n ? nt : n, kr = nt < n ? n : nt;
  ns += empties_between(b, kl, kr);
  kl = mt < m ? mt : m;
  kr = mt < m ? m : mt;
  ns += empties_between(b, kl, kr);
  if ((nt > mt && m > n) || (mt > nt && m < n)) ns++;
  return ns & 1;
}

// The ten two-body families in the reference's order: block of n, block of m,
// n < m within one block, interlayer table, twist phase.
__constant__ int c_fam[10][5] = {{0, 0, 1, 0, 0}, {1, 1, 1, 0, 0}, {0, 1, 0, 0, 0}, {2, 2, 1, 0, 0}, {3, 3, 1, 0, 0},
                                 {2, 3, 0, 0, 0}, {0, 2, 0, 1, 0}, {1, 3, 0, 1, 0}, {0, 3, 0, 1, 1}, {1, 2, 0, 1, 1}};

__device__ __forceinline__ void cadd(double* acc, int64_t j, double re, double im) {
  atomicAdd(acc + 2 * j, re);
  atomicAdd(acc + 2 * j + 1, im);
}

// Adds the contribution of target rbasis_0 (before the right-hand translations) to the row.
__device__ void add_target(const SpinGen& G, double* acc, uint64_t rb0, int ql, int Dl, int parl, int parh,
                           double amp_re, double amp_im) {
  int Dr = G.nphi;
  for (int D = 1; D < G.nphi; D++) {
    int p;
    if (rot4(rb0, D, G.nphi, 0, &p) == rb0) {
      Dr = D;
      break;
    }
  }
  if (G.K < 0) Dr = 1;
  for (int qr = 0; qr < Dr; qr++) {
    int parr = 0;
    const uint64_t rb = qr == 0 ? rb0 : rot4(rb0, qr, G.nphi, 1, &parr);
    const int64_t j = find_key(G.id, G.dim, rb);
    if (j < 0) continue;
    const double sign = ((parh + parl + parr) & 1) ? -1.0 : 1.0;
    // FT[ql][qr] = exp(2 pi i (ql - qr) K / nphi)
    double fr = 1.0, fi = 0.0;
    if (G.K > 0) {
      const double ang = 2.0 * M_PI * (ql - qr) * G.K / G.nphi;
      fr = cos(ang);
      fi = sin(ang);
    }
    const double f = sign / sqrt((double)(Dl * Dr));
    cadd(acc, j, (amp_re * fr - amp_im * fi) * f, (amp_re * fi + amp_im * fr) * f);
  }
}

// Per row: all candidates, dense accumulation in shared memory; pass 0 counts
// kept entries, pass 1 writes them at row_ptr (ascending columns).
__global__ void __launch_bounds__(256) k_spin_rows(SpinGen G, int pass, int64_t* __restrict__ row_nnz,
                                                   const int64_t* __restrict__ row_ptr, int32_t* __restrict__ col,
                                                   double* __restrict__ val, int cplx) {
  extern __shared__ double acc[];  // [2 * dim]
  const int nphi = G.nphi;
  for (int64_t i = blockIdx.x; i < G.dim; i += gridDim.x) {
    for (int64_t k = threadIdx.x; k < 2 * G.dim; k += blockDim.x) acc[k] = 0.0;
    __syncthreads();
    const uint64_t idi = G.id[i];
    const int Dl = G.K < 0 ? 1 : G.period[i];
    const int npair_same = nphi * (nphi - 1) / 2, npair_cross = nphi * nphi, nt_range = 2 * nphi - 1;
    const int hop_items = (4 * npair_same + 6 * npair_cross) * nt_range;
    const int tun_items = G.dsas > 0 ? 6 * nphi : 0;
    const int per_ql = hop_items + tun_items;
    for (int it = threadIdx.x; it < Dl * per_ql; it += blockDim.x) {
      const int ql = it / per_ql;
      int w = it - ql * per_ql;
      int parl = 0;
      const uint64_t lb = ql == 0 ? idi : rot4(idi, ql, nphi, 0, &parl);
      if (w < hop_items) {
        // family, pair, t
        int f = 0;
        for (; f < 10; f++) {
          const int np = (c_fam[f][2] ? npair_same : npair_cross) * nt_range;
          if (w < np) break;
          w -= np;
        }
        const int ti = w % nt_range, pi = w / nt_range;
        const int t = ti - (nphi - 1);
        const int ba = c_fam[f][0], bb = c_fam[f][1];
        int n, m;
        if (c_fam[f][2]) {
          // pi-th pair (a < b) of one block, in the reference's loop order
          int a = 0, r = pi;
          while (r >= nphi - 1 - a) {
            r -= nphi - 1 - a;
            a++;
          }
          n = ba * nphi + a;
          m = ba * nphi + a + 1 + r;
        } else {
          n = ba * nphi + pi / nphi;
          m = bb * nphi + pi % nphi;
        }
        const uint64_t mask = (1ULL << n) | (1ULL << m);
        if ((lb & mask) != mask) continue;
        const uint64_t b = lb ^ mask;
        const int offa = ba * nphi, offb = bb * nphi;
        int nt = n + t, mt = m - t;
        if (nt >= offa + nphi) nt -= nphi;
        else if (nt < offa) nt += nphi;
        if (mt < offb) mt += nphi;
        else if (mt >= offb + nphi) mt -= nphi;
        const int s = abs((mt - offb) - (n - offa));
        const uint64_t mt_mask = (1ULL << nt) | (1ULL << mt);
        if ((mt_mask & b) != 0) continue;
        if (!c_fam[f][3] && nt == mt) continue;
        const double v = G.V[c_fam[f][3] * nphi * nphi + s * nphi + abs(t)];
        double are = v, aim = 0.0;
        if (c_fam[f][4] && G.theta_y != 0.0) {
          are = v * cos(G.theta_y * t / nphi);
          aim = v * sin(G.theta_y * t / nphi);
        }
        add_target(G, acc, mt_mask + b, ql, Dl, parl, pair_parity(lb, n, m, nt, mt), are, aim);
      } else {
        w -= hop_items;
        const int kind = w / nphi, r = w % nphi;
        // 0..3: layer tunnelling (-Delta_SAS / 4, parallel-field phase); 4, 5: spin flip (-Delta_SAS / 2)
        int n, nt, lo, hi;
        double amp = -0.25 * G.dsas, ph = 0.0;
        switch (kind) {
          case 0: n = r; nt = n + 2 * nphi; lo = n; hi = nt; ph = G.theta_b * r * G.d; break;
          case 1: n = 2 * nphi + r; nt = n - 2 * nphi; lo = nt; hi = n; ph = -G.theta_b * nt * G.d; break;
          case 2: n = nphi + r; nt = n + 2 * nphi; lo = n; hi = nt; ph = G.theta_b * (n % nphi) * G.d; break;
          case 3: n = 3 * nphi + r; nt = n - 2 * nphi; lo = nt; hi = n; ph = -G.theta_b * (n % nphi) * G.d; break;
          case 4: n = r; nt = n + 3 * nphi; lo = n; hi = nt; amp = -0.5 * G.dsas; break;
          default: n = nphi + r; nt = n + nphi; lo = n; hi = nt; amp = -0.5 * G.dsas; break;
        }
        const uint64_t mask = (1ULL << n) | (1ULL << nt);
        const uint64_t kn = mask & lb;
        if (kn == mask || kn == 0) continue;
        const uint64_t rb0 = lb - kn + (kn ^ mask);
        add_target(G, acc, rb0, ql, Dl, parl, empties_between(lb, lo, hi), amp * cos(ph), amp * sin(ph));
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const uint64_t mk = (1ULL << nphi) - 1;
      const int n0 = pc64(idi & mk), n1 = pc64((idi >> nphi) & mk), n2 = pc64((idi >> (2 * nphi)) & mk),
                n3 = pc64((idi >> (3 * nphi)) & mk);
      double a = acc[2 * i];
      a += G.Ec * G.nel;
      a += -G.d * (n0 + n1) * (n2 + n3) / nphi;
      a += -0.5 * G.dv * (n0 + n1 - n2 - n3);
      a += -0.5 * G.dz * (n0 + n2 - n1 - n3);
      acc[2 * i] = a;
    }
    __syncthreads();
    // kept entries in ascending column order: count (warp ballots) or write
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < 32) {
      int64_t out = pass ? row_ptr[i] : 0;
      for (int64_t k0 = 0; k0 < G.dim; k0 += 32) {
        const int64_t k = k0 + lane;
        bool keep = false;
        double re = 0.0, im = 0.0;
        if (k < G.dim) {
          re = acc[2 * k];
          im = acc[2 * k + 1];
          keep = sqrt(re * re + im * im) > 1e-10;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (pass && keep) {
          const int64_t o = out + __popc(bal & ((1u << lane) - 1));
          col[o] = (int32_t)k;
          if (cplx) {
            val[2 * o] = re;
            val[2 * o + 1] = im;
          } else {
            val[o] = re;
          }
        }
        out += __popc(bal);
      }
      if (!pass && lane == 0) row_nnz[i] = out;
    }
    __syncthreads();
  }
}

std::vector<uint64_t> lex_subsets(int n, int k, int shift) {
  // k-subsets of [0, n) as bit patterns (shifted), lexicographic in the sorted tuple
  std::vector<uint64_t> out;
  if (k < 0 || k > n) return out;
  std::vector<int> a(k);
  for (int i = 0; i < k; i++) a[i] = i;
  while (true) {
    uint64_t c = 0;
    for (int i = 0; i < k; i++) c |= 1ULL << (a[i] + shift);
    out.push_back(c);
    int i = k - 1;
    while (i >= 0 && a[i] == n - k + i) i--;
    if (i < 0) break;
    a[i]++;
    for (int j = i + 1; j < k; j++) a[j] = a[j - 1] + 1;
  }
  return out;
}

template <class T>
T* upload_vec(blqh_ctx* ctx, const std::vector<T>& v) {
  T* p = dalloc<T>(ctx, std::max<size_t>(1, v.size()));
  if (!v.empty()) BLQH_TRY_CUDA(ctx, cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice));
  return p;
}

void sort_keys(blqh_ctx* ctx, uint64_t* key, uint32_t* val, int64_t n) {
  for (int64_t k = 2; k <= n; k <<= 1)
    for (int64_t j = k >> 1; j > 0; j >>= 1)
      k_bitonic<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(key, val, n, k, j);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
}

__global__ void k_iota(uint32_t* v, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    v[i] = (uint32_t)i;
}

__global__ void k_fill_key(uint64_t* k, int64_t a, int64_t b) {
  for (int64_t i = a + (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < b; i += (int64_t)gridDim.x * blockDim.x)
    k[i] = KEY_PAD;
}

void build_spin_basis(blqh_ctx* ctx, blqh_basis* B) {
  const blqh_sector_spin& s = B->ssector;
  const int nphi = s.nphi;
  TimerScope ts(ctx, TM_BASIS);
  DevBufs G;
  std::vector<uint64_t> up, lo;
  if (s.nel_up >= 0) {
    up = lex_subsets(2 * nphi, s.nel_up, 0);
    lo = lex_subsets(2 * nphi, s.nel - s.nel_up, 2 * nphi);
  } else {
    up = lex_subsets(4 * nphi, s.nel, 0);
  }
  const int64_t nu = (int64_t)up.size(), nl = s.nel_up >= 0 ? (int64_t)lo.size() : 1;
  const int64_t total = nu * nl;
  if (total == 0) {
    B->dim = 0;
    return;
  }
  const uint64_t* dpu = G.add(upload_vec(ctx, up));
  const uint64_t* dpl = s.nel_up >= 0 ? G.add(upload_vec(ctx, lo)) : nullptr;
  uint32_t* ok = G.add(dalloc<uint32_t>(ctx, total));
  int64_t* off = G.add(dalloc<int64_t>(ctx, total));
  const int BLK = 256;
  k_spin_enum<<<grid_for(ctx, total, BLK), BLK, 0, ctx->stream>>>(dpu, nu, dpl, nl, nphi, s.J, ok, total);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  int64_t N = 0;
  scan_exclusive_u32_to_i64(ctx, ok, off, total, &N);
  if (N == 0) {
    B->dim = 0;
    return;
  }
  uint64_t* keys = G.add(dalloc<uint64_t>(ctx, N));
  k_spin_scatter<<<grid_for(ctx, total, BLK), BLK, 0, ctx->stream>>>(dpu, nu, dpl, nl, ok, off, total, keys);
  // sorted copy for lookups, with the insertion index of each key
  int64_t n2 = 1;
  while (n2 < N) n2 <<= 1;
  uint64_t* skey = G.add(dalloc<uint64_t>(ctx, n2));
  uint32_t* sidx = G.add(dalloc<uint32_t>(ctx, n2));
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(skey, keys, N * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  k_fill_key<<<grid_for(ctx, n2 - N + 1, BLK), BLK, 0, ctx->stream>>>(skey, N, n2);
  k_iota<<<grid_for(ctx, n2, BLK), BLK, 0, ctx->stream>>>(sidx, n2);
  sort_keys(ctx, skey, sidx, n2);
  const bool emulate = s.rep_mode == BLQH_REP_REFERENCE && s.K >= 0;
  uint32_t* pos = emulate ? G.add(iteration_positions(ctx, keys, N)) : nullptr;
  uint32_t* keep = G.add(dalloc<uint32_t>(ctx, N));
  int64_t* koff = G.add(dalloc<int64_t>(ctx, N));
  k_spin_survive<<<grid_for(ctx, N, BLK), BLK, 0, ctx->stream>>>(keys, N, skey, sidx, pos, nphi, s.K, s.rep_mode,
                                                                 s.nel_su, keep);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  int64_t dim = 0;
  scan_exclusive_u32_to_i64(ctx, keep, koff, N, &dim);
  B->dim = dim;
  if (dim == 0) return;
  int64_t d2 = 1;
  while (d2 < dim) d2 <<= 1;
  uint64_t* ids = dalloc<uint64_t>(ctx, d2);
  B->d_id = ids;
  k_spin_compact<<<grid_for(ctx, N, BLK), BLK, 0, ctx->stream>>>(keys, keep, koff, N, ids);
  k_fill_key<<<grid_for(ctx, d2 - dim + 1, BLK), BLK, 0, ctx->stream>>>(ids, dim, d2);
  sort_keys(ctx, ids, nullptr, d2);
  B->d_period = dalloc<uint8_t>(ctx, dim);
  k_spin_period<<<grid_for(ctx, dim, BLK), BLK, 0, ctx->stream>>>(ids, dim, nphi, B->d_period);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_BASIS, 8);
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
}

void build_spin_hamil(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_spin& p, blqh_csr* M) {
  const blqh_sector_spin& s = B->ssector;
  const int nphi = s.nphi;
  // interaction tables: the spinful table has cos((2 pi s - theta_x) q_x / nphi)
  // (BLQH_with_spin/lanczos_hamiltonian.cpp:45-85), the spinless one
  // cos((2 pi s + 2 theta_x) q_x / nphi): the same routine with theta_x -> -theta_x / 2
  blqh_params q{};
  q.lx = p.lx;
  q.ly = p.ly;
  q.d = p.d;
  q.nLL = p.nLL;
  q.theta_x = -0.5 * p.theta_x;
  double Ec = 0;
  std::vector<double> V;
  coulomb_tables_host(nphi, s.K, q, &Ec, V);
  DevBufs G;
  double* dV = G.add(upload_vec(ctx, V));
  const bool cplx = !((s.K <= 0 || 2 * s.K == nphi) && p.theta_y == 0.0 && p.theta_b == 0.0);
  SpinGen g{};
  g.id = B->d_id;
  g.period = B->d_period;
  g.dim = B->dim;
  g.nphi = nphi;
  g.nel = s.nel;
  g.K = s.K;
  g.Ec = Ec;
  g.d = p.d;
  g.dsas = p.delta_sas;
  g.dv = p.delta_v;
  g.dz = p.delta_z;
  g.theta_b = p.theta_b;
  g.theta_y = p.theta_y;
  g.V = dV;
  const int64_t dim = B->dim;
  M->dim = dim;
  M->is_complex = cplx;
  M->precision = BLQH_VAL_FP64;
  M->d_row_ptr = dalloc<int64_t>(ctx, dim + 1);
  const size_t sm = (size_t)dim * 16;
  BLQH_TRY_CUDA(ctx, cudaFuncSetAttribute(k_spin_rows, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  const int grid = (int)std::min<int64_t>(dim, (int64_t)ctx->num_sms * 8);
  TimerScope ts(ctx, TM_BUILD);
  k_spin_rows<<<grid, 256, sm, ctx->stream>>>(g, 0, M->d_row_ptr, nullptr, nullptr, nullptr, cplx);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  int64_t nnz = 0;
  scan_exclusive_i64(ctx, M->d_row_ptr, M->d_row_ptr, dim, &nnz);
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(M->d_row_ptr + dim, &nnz, 8, cudaMemcpyHostToDevice, ctx->stream));
  M->nnz = nnz;
  M->mean_row = dim ? (double)nnz / dim : 0;
  M->d_col = dalloc<int32_t>(ctx, std::max<int64_t>(1, nnz));
  M->d_val = dev_alloc(ctx, std::max<int64_t>(1, nnz) * (cplx ? 16 : 8) + 16);
  k_spin_rows<<<grid, 256, sm, ctx->stream>>>(g, 1, nullptr, M->d_row_ptr, M->d_col,
                                              reinterpret_cast<double*>(M->d_val), cplx);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_BUILD, 2);
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
}

}  // namespace

void sort_keys_u64(blqh_ctx* ctx, uint64_t* key, uint32_t* val, int64_t n_pow2) { sort_keys(ctx, key, val, n_pow2); }

void pad_keys_u64(blqh_ctx* ctx, uint64_t* key, int64_t from, int64_t to) {
  if (to > from) k_fill_key<<<grid_for(ctx, to - from, 256), 256, 0, ctx->stream>>>(key, from, to);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
}

void sorted_copy_u64(blqh_ctx* ctx, const uint64_t* keys, int64_t N, uint64_t* skey, uint32_t* sidx, int64_t n2) {
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(skey, keys, N * 8, cudaMemcpyDeviceToDevice, ctx->stream));
  pad_keys_u64(ctx, skey, N, n2);
  k_iota<<<grid_for(ctx, n2, 256), 256, 0, ctx->stream>>>(sidx, n2);
  sort_keys(ctx, skey, sidx, n2);
}

void spin_hamil_build_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_spin& p, blqh_csr* M) {
  build_spin_hamil(ctx, B, p, M);
}

extern "C" {

int blqh_basis_build_spin(blqh_ctx* ctx, const blqh_sector_spin* s, blqh_basis** out) {
  if (!ctx || !s || !out) return BLQH_ERR_ARG;
  *out = nullptr;
  const int nel_dn = s->nel_up >= 0 ? s->nel - s->nel_up : 0;
  if (s->nphi < 2 || 4 * s->nphi > 60 || s->nel < 1 || s->nel > 4 * s->nphi || s->nel_up > s->nel ||
      (s->nel_up >= 0 && (s->nel_up > 2 * s->nphi || nel_dn > 2 * s->nphi)) || s->K >= s->nphi ||
      s->J >= s->nphi || (s->rep_mode != BLQH_REP_REFERENCE && s->rep_mode != BLQH_REP_MIN)) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_basis_build_spin: sector outside 2 <= nphi <= 15, 0 < nel <= 4 nphi, "
                                         "0 <= nel_up <= nel (or < 0), J, K < nphi");
    return BLQH_ERR_UNSUPPORTED;
  }
  {
    // candidate count: C(2 nphi, nel_up) C(2 nphi, nel_dn) or C(4 nphi, nel), bounded to 2^26
    auto binom = [](int n, int k) {
      double r = 1;
      for (int i = 1; i <= k; i++) r = r * (n - k + i) / i;
      return r;
    };
    const double cand = s->nel_up >= 0 ? binom(2 * s->nphi, s->nel_up) * binom(2 * s->nphi, nel_dn)
                                       : binom(4 * s->nphi, s->nel);
    if (cand > (double)(1 << 26)) {
      set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_basis_build_spin: more than 2^26 candidate states");
      return BLQH_ERR_UNSUPPORTED;
    }
  }
  blqh_basis* B = new blqh_basis;
  B->ctx = ctx;
  B->model = BLQH_MODEL_SPINFUL;
  B->ssector = *s;
  B->sector.nphi = s->nphi;
  B->sector.nel = s->nel;
  B->sector.nel_up = s->nel_up;
  B->sector.J = s->J;
  B->sector.K = s->K;
  B->sector.rep_mode = s->rep_mode;
  try {
    cudaSetDevice(ctx->device);
    build_spin_basis(ctx, B);
  } catch (const BlqhError& e) {
    blqh_basis_destroy(B);
    return e.code;
  }
  *out = B;
  return BLQH_OK;
}

int blqh_hamil_build_spin(blqh_ctx* ctx, const blqh_basis* b, const blqh_params_spin* p, blqh_csr** out) {
  if (!ctx || !b || !p || !out) return BLQH_ERR_ARG;
  *out = nullptr;
  if (b->model != BLQH_MODEL_SPINFUL) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_hamil_build_spin: the basis is not a spinful basis");
    return BLQH_ERR_ARG;
  }
  if (b->dim == 0) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_hamil_build_spin: empty sector");
    return BLQH_ERR_ARG;
  }
  if (b->dim > BLQH_SPIN_MAX_DIM) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_hamil_build_spin: sector larger than BLQH_SPIN_MAX_DIM");
    return BLQH_ERR_UNSUPPORTED;
  }
  blqh_csr* M = new blqh_csr;
  M->ctx = ctx;
  try {
    cudaSetDevice(ctx->device);
    build_spin_hamil(ctx, b, *p, M);
  } catch (const BlqhError& e) {
    free_csr(M);
    return e.code;
  }
  *out = M;
  return BLQH_OK;
}

}  // extern "C"
