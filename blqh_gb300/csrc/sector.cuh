// Bit-level operations on bilayer Fock states, usable on host and device.
//
// A spinless bilayer state is a 2*nphi-bit word: bits [0, nphi) are the upper
// layer's orbitals, bits [nphi, 2 nphi) the lower layer's. These helpers
// restate the reference's basis::translate / inv_translate / get_sign
// (BLQH_without_spin/basis.cpp:158-197, 292-341) with popcounts and rotates.
#pragma once

#include <stdint.h>

#include "blqh_internal.h"

#if defined(__CUDACC__)
#define HD __host__ __device__ __forceinline__
#else
#define HD inline
#endif

HD int popc64(uint64_t x) {
#if defined(__CUDA_ARCH__)
  return __popcll(x);
#else
  return __builtin_popcountll(x);
#endif
}
HD int popc32(uint32_t x) {
#if defined(__CUDA_ARCH__)
  return __popc(x);
#else
  return __builtin_popcount(x);
#endif
}

// floor(n / d) for 0 <= n < 2^32 and a divisor fixed at set-up, by a multiply
// and shifts (division by invariant integers, Granlund & Montgomery 1994).
struct FastDiv {
  uint32_t d = 1, m = 0, s = 0;
  FastDiv() = default;
  explicit FastDiv(uint32_t div) : d(div) {
    if (d <= 1) return;
    uint32_t l = 0;
    while ((1ULL << l) < d) l++;
    s = l;
    m = (uint32_t)((((1ULL << 32) * ((1ULL << l) - d)) / d) + 1);
  }
  HD uint32_t div(uint32_t n) const {
    if (d <= 1) return n;
#if defined(__CUDA_ARCH__)
    const uint32_t t = __umulhi(n, m);
#else
    const uint32_t t = (uint32_t)(((uint64_t)n * m) >> 32);
#endif
    return (t + ((n - t) >> 1)) >> (s - 1);
  }
};

// Bits strictly between lo and hi (lo < hi), as a mask.
HD uint64_t open_range(int lo, int hi) {
  if (hi - lo <= 1) return 0;
  uint64_t upto_hi = (hi >= 64) ? ~0ULL : ((1ULL << hi) - 1);
  return upto_hi & ~((1ULL << (lo + 1)) - 1);
}

// translate(c, k): every layer rotated left by k orbitals (basis.cpp:292-317).
// Returns the sign parity (0 even, 1 odd) of (-1)^{sum (n_b - x_b) x_b}, x_b the
// electrons of layer b that wrap around (its k top orbitals).
HD uint64_t translate_bits(uint64_t c, int k, int nphi, int* parity) {
  const uint64_t m = (1ULL << nphi) - 1;
  uint64_t u = c & m, d = (c >> nphi) & m;
  int p = 0;
  if (k != 0) {
    const uint64_t top = ((1ULL << k) - 1) << (nphi - k);
    int xu = popc64(u & top), xd = popc64(d & top);
    int nu = popc64(u), nd = popc64(d);
    p = ((nu - xu) * xu + (nd - xd) * xd) & 1;
    u = ((u << k) | (u >> (nphi - k))) & m;
    d = ((d << k) | (d >> (nphi - k))) & m;
  }
  *parity = p;
  return (d << nphi) | u;
}

// inv_translate(c, k): rotate right by k (basis.cpp:318-341); x_b = electrons in
// the k bottom orbitals of layer b.
HD uint64_t inv_translate_bits(uint64_t c, int k, int nphi, int* parity) {
  const uint64_t m = (1ULL << nphi) - 1;
  uint64_t u = c & m, d = (c >> nphi) & m;
  int p = 0;
  if (k != 0) {
    const uint64_t bot = (1ULL << k) - 1;
    int xu = popc64(u & bot), xd = popc64(d & bot);
    int nu = popc64(u), nd = popc64(d);
    p = ((nu - xu) * xu + (nd - xd) * xd) & 1;
    u = ((u >> k) | (u << (nphi - k))) & m;
    d = ((d >> k) | (d << (nphi - k))) & m;
  }
  *parity = p;
  return (d << nphi) | u;
}

// Two-body hop parity (basis.cpp:158-185): empty orbitals of b = c^{n,m}
// strictly between n and nt and strictly between m and mt, plus one when the
// two electrons cross.
HD int hop2_parity(uint64_t c, int n, int m, int nt, int mt) {
  const uint64_t b = c ^ ((1ULL << n) | (1ULL << m));
  int lo = nt < n ? nt : n, hi = nt < n ? n : nt;
  int e = (hi - lo > 1) ? (hi - lo - 1) - popc64(b & open_range(lo, hi)) : 0;
  lo = mt < m ? mt : m;
  hi = mt < m ? m : mt;
  e += (hi - lo > 1) ? (hi - lo - 1) - popc64(b & open_range(lo, hi)) : 0;
  if ((nt > mt && m > n) || (mt > nt && m < n)) e++;
  return e & 1;
}

// Tunnelling parity (basis.cpp:187-197): empty orbitals of c strictly in (n, nt), n < nt.
HD int hop1_parity(uint64_t c, int n, int nt) {
  return ((nt - n - 1) - popc64(c & open_range(n, nt))) & 1;
}

// Smallest k in [1, nphi) with inv_translate(c, k) == c, else nphi (basis.cpp:111-118).
HD int orbit_period(uint64_t c, int nphi) {
  int par;
  for (int k = 1; k < nphi; k++)
    if (inv_translate_bits(c, k, nphi, &par) == c) return k;
  return nphi;
}

// Dense index of a state among those kept by the reference's depth-first
// enumeration (= its insertion order into basis_set), or -1 when the state is
// not one of them (wrong electron counts or wrong total momentum).
HD int64_t sector_index(const SectorIdx& S, uint64_t c) {
  const int nphi = S.nphi;
  if (c >> (2 * nphi)) return -1;
  if (!S.all_density) {
    const uint32_t cu = (uint32_t)(c & S.lmask), cd = (uint32_t)((c >> nphi) & S.lmask);
    if (popc32(cu) != S.nel_up || popc32(cd) != S.nel_dn) return -1;
    int need = 0;
    if (S.J >= 0) {
      // residues are in [0, nphi): wrap sums with one conditional subtraction
      const int ru = S.resid[cu], rd = S.resid[cd];
      int tot = ru + rd;
      tot -= (tot >= nphi) ? nphi : 0;
      if (tot != S.J) return -1;
      need = S.J - ru;
      need += (need < 0) ? nphi : 0;
    }
    return (int64_t)S.upA[cu] + (int64_t)S.loB[(int64_t)cd * nphi + need];
  }
  // free layer split: lexicographic rank of the sorted orbital tuple among the
  // tuples with the right momentum, from prefix-summed completion counts.
  if (popc64(c) != S.nel) return -1;
  const int L = 2 * nphi;
  int need;
  if (S.J >= 0) {
    int r = 0;
    for (uint64_t t = c; t; t &= t - 1) {
#if defined(__CUDA_ARCH__)
      r += (__ffsll((long long)t) - 1) % nphi;
#else
      r += __builtin_ctzll(t) % nphi;
#endif
    }
    if (r % nphi != S.J) return -1;
    need = S.J;
  } else {
    need = 0;
  }
  int64_t rank = 0;
  int lo = 0, i = 0;
  for (uint64_t t = c; t; t &= t - 1, i++) {
#if defined(__CUDA_ARCH__)
    const int o = __ffsll((long long)t) - 1;
#else
    const int o = __builtin_ctzll(t);
#endif
    const int k = S.nel - 1 - i;  // electrons still to place after this one
    const int64_t* row = S.PE + ((int64_t)k * (L + 1)) * nphi;
    rank += row[(int64_t)o * nphi + need] - row[(int64_t)lo * nphi + need];
    if (S.J >= 0) need = (need - o % nphi + nphi) % nphi;
    lo = o + 1;
  }
  return rank;
}
