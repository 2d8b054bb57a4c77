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
// one thread block per row accumulates the row in shared memory (the reference
// accumulates it in a dense vector of dim entries): ten two-body families
// (same-spin and opposite-spin pairs in each layer with the intralayer table,
// four interlayer pairs with the interlayer table, the two opposite-spin ones
// with the twist phase), layer tunnelling with the parallel-field phase and
// spin-flip tunnelling (both only for Delta_SAS > 0), the charging, bias and
// Zeeman diagonal; entries with |value| > 1e-10 are kept. The row lives in an
// open-addressing table (column -> value) sized by the number of moves from
// the row's state, C(Ne, 2) (2 nphi - 1) + 6 nphi + 1, which bounds its
// distinct columns (translating the row state permutes its moves, so every
// translate reaches the same target orbits); its occupied slots are then
// sorted by column. No sector-size limit. Values are FP64 (the accumulation
// order differs from the reference's by the threads' atomics: values agree to
// rounding); FP32 values are the FP64 sums rounded once.
#include <algorithm>
#include <cmath>
#include <string>
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

// A row under construction: open-addressing table in shared memory.
struct RowTable {
  int* keys;     // [slots] column, -1 empty
  double* acc;   // [2 slots] (re, im)
  int slots;     // power of two
  int* overflow; // set when a row has more distinct columns than the table holds
};

// Slot of column j (claimed if new), -1 if the table is full.
__device__ __forceinline__ int table_slot(const RowTable& T, int j) {
  uint32_t h = ((uint32_t)j * 2654435761u) & (uint32_t)(T.slots - 1);
  for (int probe = 0; probe < T.slots; probe++) {
    const int k = T.keys[h];
    if (k == j) return (int)h;
    if (k == -1) {
      const int prev = atomicCAS(T.keys + h, -1, j);
      if (prev == -1 || prev == j) return (int)h;
    }
    h = (h + 1) & (uint32_t)(T.slots - 1);
  }
  atomicOr(T.overflow, 1);
  return -1;
}

__device__ __forceinline__ void cadd(const RowTable& T, int64_t j, double re, double im) {
  const int h = table_slot(T, (int)j);
  if (h < 0) return;
  atomicAdd(T.acc + 2 * h, re);
  atomicAdd(T.acc + 2 * h + 1, im);
}

// Adds the contribution of target rbasis_0 (before the right-hand translations) to the row.
__device__ void add_target(const SpinGen& G, const RowTable& acc, uint64_t rb0, int ql, int Dl, int parl, int parh,
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

// Per row: all candidates accumulate into the row's table; its occupied slots
// are sorted by column (bitonic, in shared memory); pass 0 counts kept entries,
// pass 1 writes them at row_ptr (ascending columns); pass 2 (regenerated
// Rayleigh quotient) writes rq_part[i] = Re(conj(psi_i) sum_k H_ik psi_k) over
// the row's kept entries in column order, FP64, nothing stored.
__global__ void __launch_bounds__(256) k_spin_rows(SpinGen G, int pass, int slots, int64_t* __restrict__ row_nnz,
                                                   const int64_t* __restrict__ row_ptr, int32_t* __restrict__ col,
                                                   double* __restrict__ val, int cplx, int* overflow,
                                                   const double* __restrict__ psi, double* __restrict__ rq_part) {
  extern __shared__ __align__(16) unsigned char sm_raw[];
  RowTable acc{reinterpret_cast<int*>(sm_raw + (size_t)slots * 16), reinterpret_cast<double*>(sm_raw), slots,
               overflow};
  int2* order = reinterpret_cast<int2*>(sm_raw + (size_t)slots * 20);  // [slots] (column, slot)
  __shared__ int n_occ;
  const int nphi = G.nphi;
  for (int64_t i = blockIdx.x; i < G.dim; i += gridDim.x) {
    for (int k = threadIdx.x; k < slots; k += blockDim.x) {
      acc.keys[k] = -1;
      acc.acc[2 * k] = acc.acc[2 * k + 1] = 0.0;
    }
    if (threadIdx.x == 0) n_occ = 0;
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
      const int h = table_slot(acc, (int)i);
      if (h >= 0) {
        double a = acc.acc[2 * h];
        a += G.Ec * G.nel;
        a += -G.d * (n0 + n1) * (n2 + n3) / nphi;
        a += -0.5 * G.dv * (n0 + n1 - n2 - n3);
        a += -0.5 * G.dz * (n0 + n2 - n1 - n3);
        acc.acc[2 * h] = a;
      }
    }
    __syncthreads();
    // occupied slots, sorted by column
    for (int k = threadIdx.x; k < slots; k += blockDim.x)
      if (acc.keys[k] >= 0) order[atomicAdd(&n_occ, 1)] = make_int2(acc.keys[k], k);
    __syncthreads();
    const int n = n_occ;
    int P = 1;
    while (P < n) P <<= 1;
    for (int k = n + threadIdx.x; k < P; k += blockDim.x) order[k] = make_int2(0x7FFFFFFF, -1);
    __syncthreads();
    for (int k = 2; k <= P; k <<= 1)
      for (int jj = k >> 1; jj > 0; jj >>= 1) {
        for (int t = threadIdx.x; t < P; t += blockDim.x) {
          const int u = t ^ jj;
          if (u > t) {
            const int2 a = order[t], b = order[u];
            if ((a.x > b.x) == ((t & k) == 0)) {
              order[t] = b;
              order[u] = a;
            }
          }
        }
        __syncthreads();
      }
    const int lane = threadIdx.x & 31;
    if (threadIdx.x < 32 && pass == 2) {
      double sr = 0.0, si = 0.0;
      for (int k0 = 0; k0 < n; k0 += 32) {
        const int k = k0 + lane;
        if (k < n) {
          const int c = order[k].x;
          const double re = acc.acc[2 * order[k].y], im = acc.acc[2 * order[k].y + 1];
          if (sqrt(re * re + im * im) > 1e-10) {
            const double xr = cplx ? psi[2 * (int64_t)c] : psi[c], xi = cplx ? psi[2 * (int64_t)c + 1] : 0.0;
            sr += re * xr - im * xi;
            si += re * xi + im * xr;
          }
        }
      }
      for (int o = 16; o > 0; o >>= 1) {
        sr += __shfl_xor_sync(0xffffffffu, sr, o);
        si += __shfl_xor_sync(0xffffffffu, si, o);
      }
      if (lane == 0) {
        const double pr = cplx ? psi[2 * i] : psi[i], pim = cplx ? psi[2 * i + 1] : 0.0;
        rq_part[i] = pr * sr + pim * si;  // Re(conj(psi_i) s)
      }
    } else if (threadIdx.x < 32) {
      // kept entries in ascending column order: count (warp ballots) or write
      int64_t out = pass ? row_ptr[i] : 0;
      for (int k0 = 0; k0 < n; k0 += 32) {
        const int k = k0 + lane;
        bool keep = false;
        double re = 0.0, im = 0.0;
        int c = 0;
        if (k < n) {
          c = order[k].x;
          re = acc.acc[2 * order[k].y];
          im = acc.acc[2 * order[k].y + 1];
          keep = sqrt(re * re + im * im) > 1e-10;
        }
        const unsigned bal = __ballot_sync(0xffffffffu, keep);
        if (pass && keep) {
          const int64_t o = out + __popc(bal & ((1u << lane) - 1));
          col[o] = (int32_t)c;
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

// ---- ground-state observables ----------------------------------------------------
// The reference evaluates them from psir_0 (BLQH_with_spin/lanczos_hamiltonian.cpp:
// 1217-1593), the complex conjugate of the ground state psi (its reconstruction
// conjugates the Krylov vectors); here from psi directly:
//   pseudospin_Sz = (2 <N_0 + N_1> - Ne) / (2 Ne), Sz = (2 <N_0 + N_2> - Ne) / (2 Ne)  (:1239-1251)
//   upper_Sz = <(2 N_0 - N_u) / (2 N_u + 1e-8)>, N_u = N_0 + N_1; down_Sz likewise with
//       blocks 2, 3                                                                   (:1253-1271)
//   occupation(alpha, j) = sum_i |psi_i|^2 (1/D_i) sum_{q < D_i} [orbital j of block
//       alpha (0 or, for any other alpha, 1) occupied in translate(id_i, q)]           (:1217-1237)
//   M(a, b) = sum_i sum_{ql < Dl} sum_o psi_i conj(psi_j) FT[ql][qr] sign / sqrt(Dl Dr)
//       over the moves of one electron between block a and block b at orbital o
//       (whichever of the two is occupied moves), j the target's representative  (:1273-1593)
//   pseudospin_Sx = |sum of the eight interlayer M, each 1/4| / Ne; spinflip_tunneling =
//       |(M(0, 3) + M(1, 2)) / 2| / Ne.
// Block partials: [0] <N_0 + N_1>, [1] <N_0 + N_2>, [2] upper_Sz, [3] down_Sz,
// [4 + 2 p .. 5 + 2 p] M of move pair p (re, im), [20 ..] occupations (block 0, then 1).
__constant__ int c_move_pairs[8][2] = {{0, 2}, {2, 0}, {1, 3}, {3, 1}, {0, 3}, {3, 0}, {1, 2}, {2, 1}};

__global__ void __launch_bounds__(256) k_spin_observables(const uint64_t* __restrict__ id,
                                                          const uint8_t* __restrict__ period, int64_t dim, int nphi,
                                                          int K, const double* __restrict__ psi, int cplx,
                                                          double* __restrict__ part) {
  __shared__ double acc[20 + 2 * 15];
  const int nv = 20 + 2 * nphi;
  for (int k = threadIdx.x; k < nv; k += blockDim.x) acc[k] = 0.0;
  __syncthreads();
  const uint64_t mk = (1ULL << nphi) - 1;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < dim; i += (int64_t)gridDim.x * blockDim.x) {
    const double pr = cplx ? psi[2 * i] : psi[i], pim = cplx ? psi[2 * i + 1] : 0.0;
    const double w = pr * pr + pim * pim;
    const uint64_t idi = id[i];
    const int n0 = pc64(idi & mk), n1 = pc64((idi >> nphi) & mk), n2 = pc64((idi >> (2 * nphi)) & mk),
              n3 = pc64((idi >> (3 * nphi)) & mk);
    atomicAdd(acc + 0, (n0 + n1) * w);
    atomicAdd(acc + 1, (n0 + n2) * w);
    atomicAdd(acc + 2, (2.0 * n0 - (n0 + n1)) / (2.0 * (n0 + n1) + 1e-8) * w);
    atomicAdd(acc + 3, (2.0 * n2 - (n2 + n3)) / (2.0 * (n2 + n3) + 1e-8) * w);
    const int Dl = K < 0 ? 1 : period[i];
    double mr[8], mi[8];
    for (int p = 0; p < 8; p++) mr[p] = mi[p] = 0.0;
    for (int ql = 0; ql < Dl; ql++) {
      int parl = 0;
      const uint64_t lb = ql == 0 ? idi : rot4(idi, ql, nphi, 0, &parl);
      for (int j = 0; j < nphi; j++) {
        if ((lb >> j) & 1) atomicAdd(acc + 20 + j, w / Dl);
        if ((lb >> (j + nphi)) & 1) atomicAdd(acc + 20 + nphi + j, w / Dl);
      }
      for (int p = 0; p < 8; p++) {
        for (int o = 0; o < nphi; o++) {
          const int n = c_move_pairs[p][0] * nphi + o, nt = c_move_pairs[p][1] * nphi + o;
          const uint64_t mask = (1ULL << n) | (1ULL << nt);
          const uint64_t kn = lb & mask;
          if (kn == mask || kn == 0) continue;
          const uint64_t rb0 = lb ^ mask;
          int Dr = nphi;
          for (int D = 1; D < nphi; D++) {
            int q;
            if (rot4(rb0, D, nphi, 0, &q) == rb0) {
              Dr = D;
              break;
            }
          }
          if (K < 0) Dr = 1;
          const int hpar = empties_between(lb, n < nt ? n : nt, n < nt ? nt : n);
          for (int qr = 0; qr < Dr; qr++) {
            int parr = 0;
            const uint64_t rb = qr == 0 ? rb0 : rot4(rb0, qr, nphi, 1, &parr);
            const int64_t jj = find_key(id, dim, rb);
            if (jj < 0) continue;
            const double qr_ = cplx ? psi[2 * jj] : psi[jj], qi_ = cplx ? -psi[2 * jj + 1] : 0.0;  // conj(psi_j)
            const double cr = pr * qr_ - pim * qi_, ci = pr * qi_ + pim * qr_;                      // psi_i conj(psi_j)
            double fr = 1.0, fi = 0.0;
            if (K > 0) {
              const double ang = 2.0 * M_PI * (ql - qr) * K / nphi;
              fr = cos(ang);
              fi = sin(ang);
            }
            const double f = (((hpar + parl + parr) & 1) ? -1.0 : 1.0) / sqrt((double)(Dl * Dr));
            mr[p] += (cr * fr - ci * fi) * f;
            mi[p] += (cr * fi + ci * fr) * f;
          }
        }
      }
    }
    for (int p = 0; p < 8; p++) {
      if (mr[p] != 0.0) atomicAdd(acc + 4 + 2 * p, mr[p]);
      if (mi[p] != 0.0) atomicAdd(acc + 5 + 2 * p, mi[p]);
    }
  }
  __syncthreads();
  for (int k = threadIdx.x; k < nv; k += blockDim.x) part[(int64_t)blockIdx.x * nv + k] = acc[k];
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

// Row generator set-up shared by the build and the regenerated Rayleigh quotient.
struct SpinSetup {
  SpinGen g{};
  bool cplx = false;
  int slots = 0;
  size_t smem = 0;
  int grid = 0;
};

SpinSetup spin_setup(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_spin& p, DevBufs& G) {
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
  double* dV = G.add(upload_vec(ctx, V));
  SpinSetup S;
  S.cplx = !((s.K <= 0 || 2 * s.K == nphi) && p.theta_y == 0.0 && p.theta_b == 0.0);
  SpinGen& g = S.g;
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
  // table slots: a power of two >= twice the distinct columns a row can have
  const int64_t moves = (int64_t)s.nel * (s.nel - 1) / 2 * (2 * nphi - 1) + 6 * nphi + 1;
  S.slots = 64;
  while (S.slots < 2 * moves) S.slots <<= 1;
  S.smem = (size_t)S.slots * 28;  // (re, im) + column + sort pair per slot
  int smem_max = 0;
  cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  if (S.smem > (size_t)smem_max - 1024) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_hamil_build_spin: a row's table (" + std::to_string(S.slots) +
                                             " slots) exceeds shared memory (too many electrons)");
    throw BlqhError{BLQH_ERR_UNSUPPORTED, "spin row table"};
  }
  BLQH_TRY_CUDA(ctx, smem_attr_at_least(k_spin_rows, (int)S.smem));
  S.grid = (int)std::min<int64_t>(B->dim, (int64_t)ctx->num_sms * 8);
  return S;
}

void check_overflow(blqh_ctx* ctx, const int* over) {
  int ov = 0;
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(&ov, over, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (ov) {
    set_error(ctx, BLQH_ERR_CAPACITY, "spinful row generator: a row had more distinct columns than its table");
    throw BlqhError{BLQH_ERR_CAPACITY, "spin row table"};
  }
}

__global__ void k_f64_to_f32(const double* __restrict__ a, float* __restrict__ b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = (float)a[i];
}

void build_spin_hamil(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_spin& p, int prec, blqh_csr* M) {
  DevBufs G;
  const SpinSetup S = spin_setup(ctx, B, p, G);
  const int64_t dim = B->dim;
  const bool cplx = S.cplx;
  M->dim = dim;
  M->is_complex = cplx;
  M->precision = BLQH_VAL_FP64;
  M->d_row_ptr = dalloc<int64_t>(ctx, dim + 1);
  int* over = G.add(dalloc<int>(ctx, 1));
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(over, 0, sizeof(int), ctx->stream));
  TimerScope ts(ctx, TM_BUILD);
  k_spin_rows<<<S.grid, 256, S.smem, ctx->stream>>>(S.g, 0, S.slots, M->d_row_ptr, nullptr, nullptr, nullptr, cplx,
                                                    over, nullptr, nullptr);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  int64_t nnz = 0;
  scan_exclusive_i64(ctx, M->d_row_ptr, M->d_row_ptr, dim, &nnz);
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(M->d_row_ptr + dim, &nnz, 8, cudaMemcpyHostToDevice, ctx->stream));
  M->nnz = nnz;
  M->mean_row = dim ? (double)nnz / dim : 0;
  M->d_col = dalloc<int32_t>(ctx, std::max<int64_t>(1, nnz));
  M->d_val = dev_alloc(ctx, std::max<int64_t>(1, nnz) * (cplx ? 16 : 8) + 16);
  k_spin_rows<<<S.grid, 256, S.smem, ctx->stream>>>(S.g, 1, S.slots, nullptr, M->d_row_ptr, M->d_col,
                                                    reinterpret_cast<double*>(M->d_val), cplx, over, nullptr, nullptr);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_BUILD, 2);
  check_overflow(ctx, over);
  if (prec == BLQH_VAL_FP32) {  // FP32 values, rounded from the FP64 sums
    const int64_t n = std::max<int64_t>(1, nnz) * (cplx ? 2 : 1);
    float* f = static_cast<float*>(dev_alloc(ctx, n * 4 + 16));
    k_f64_to_f32<<<grid_for(ctx, n, 256, 8), 256, 0, ctx->stream>>>(reinterpret_cast<const double*>(M->d_val), f, n);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_BUILD);
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    dev_free(M->d_val);
    M->d_val = f;
    M->precision = BLQH_VAL_FP32;
  }
}

}  // namespace

// out[0..5] = Sz, pseudospin_Sz, upper_Sz, down_Sz, pseudospin_Sx, spinflip_tunneling
// (the reference's order), out[6 .. 6 + 2 nphi) = occupations (alpha 0, then 1).
void spin_observables_impl(blqh_ctx* ctx, const blqh_basis* B, const double* psi, int cplx, double* out) {
  const int nphi = B->ssector.nphi, nel = B->ssector.nel, nv = 20 + 2 * nphi;
  const int grid = grid_for(ctx, B->dim, 256, 4);
  double* part = dalloc<double>(ctx, (size_t)grid * nv);
  std::vector<double> h((size_t)grid * nv);
  try {
    TimerScope tm(ctx, TM_MISC);
    k_spin_observables<<<grid, 256, 0, ctx->stream>>>(B->d_id, B->d_period, B->dim, nphi, B->ssector.K, psi, cplx,
                                                      part);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_MISC);
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(h.data(), part, h.size() * 8, cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } catch (...) {
    dev_free(part);
    throw;
  }
  dev_free(part);
  std::vector<double> t(nv, 0.0);
  for (int g = 0; g < grid; g++)
    for (int k = 0; k < nv; k++) t[k] += h[(size_t)g * nv + k];
  double sxr = 0, sxi = 0;
  for (int p = 0; p < 8; p++) {
    sxr += 0.25 * t[4 + 2 * p];
    sxi += 0.25 * t[5 + 2 * p];
  }
  const double sfr = 0.5 * (t[4 + 2 * 4] + t[4 + 2 * 6]), sfi = 0.5 * (t[5 + 2 * 4] + t[5 + 2 * 6]);
  out[0] = (2.0 * t[1] - nel) / (2.0 * nel);
  out[1] = (2.0 * t[0] - nel) / (2.0 * nel);
  out[2] = t[2];
  out[3] = t[3];
  out[4] = std::sqrt(sxr * sxr + sxi * sxi) / nel;
  out[5] = std::sqrt(sfr * sfr + sfi * sfi) / nel;
  for (int k = 0; k < 2 * nphi; k++) out[6 + k] = t[20 + k];
}

// <x|H|x> with the spinful matrix elements regenerated in FP64 (x on the device, normalized):
// per-row partials written by k_spin_rows (pass 2), summed in row order on the host.
double spin_rayleigh_regen_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params_spin& p, const double* x) {
  DevBufs G;
  const SpinSetup S = spin_setup(ctx, B, p, G);
  double* part = G.add(dalloc<double>(ctx, B->dim));
  int* over = G.add(dalloc<int>(ctx, 1));
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(over, 0, sizeof(int), ctx->stream));
  {
    TimerScope ts(ctx, TM_BUILD);
    k_spin_rows<<<S.grid, 256, S.smem, ctx->stream>>>(S.g, 2, S.slots, nullptr, nullptr, nullptr, nullptr, S.cplx,
                                                      over, x, part);
    BLQH_TRY_CUDA(ctx, cudaGetLastError());
    count_launch(ctx, TM_BUILD);
  }
  check_overflow(ctx, over);
  std::vector<double> h(B->dim);
  BLQH_TRY_CUDA(ctx, cudaMemcpy(h.data(), part, B->dim * 8, cudaMemcpyDeviceToHost));
  double e = 0;
  for (double v : h) e += v;
  return e;
}

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
  build_spin_hamil(ctx, B, p, BLQH_VAL_FP64, M);
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

int blqh_hamil_build_spin_prec(blqh_ctx* ctx, const blqh_basis* b, const blqh_params_spin* p, int value_precision,
                               blqh_csr** out) {
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
  if (value_precision != BLQH_VAL_FP64 && value_precision != BLQH_VAL_FP32) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_hamil_build_spin_prec: value_precision is BLQH_VAL_FP64 or BLQH_VAL_FP32");
    return BLQH_ERR_ARG;
  }
  blqh_csr* M = new blqh_csr;
  M->ctx = ctx;
  try {
    cudaSetDevice(ctx->device);
    build_spin_hamil(ctx, b, *p, value_precision, M);
  } catch (const BlqhError& e) {
    free_csr(M);
    return e.code;
  }
  *out = M;
  return BLQH_OK;
}

int blqh_hamil_build_spin(blqh_ctx* ctx, const blqh_basis* b, const blqh_params_spin* p, blqh_csr** out) {
  return blqh_hamil_build_spin_prec(ctx, b, p, BLQH_VAL_FP64, out);
}

}  // extern "C"
