// K2 — Hamiltonian rows on the device (CSR build), and K8 — the FP64
// Rayleigh quotient with matrix elements regenerated on the fly.
//
// Replaces lhamil::init_Coulomb_matrix, peer_set_hamil and set_hamil
// (BLQH_without_spin/lanczos_hamiltonian.cpp:37-85, 87-358, 361-385).
//
// The reference builds row i of the momentum-K Hamiltonian by translating the
// representative id[i] by every ql < Dl (its orbit period), applying every
// two-body hop c+c+cc and tunnelling term to each translate, and, for each
// target, searching qr < Dr for the translate that is a basis representative,
// accumulating V * sign * FT[ql][qr] / sqrt(Dl Dr) into a dense scratch row.
//
// This kernel computes the same numbers with less work, one warp per row:
//   * hops are enumerated once per unordered target pair; the reference's
//     two labelings (direct, exchange) and its two momentum transfers t and
//     t -/+ nphi for one target are summed into one coefficient, with the two
//     transfers pre-summed in a table W[s][t] = V[s][t] + V[s][nphi - t];
//   * the target's representative row j and translation q come from one load
//     of a dense map indexed by the target's depth-first rank (built with the
//     basis) instead of a hash probe per qr;
//   * for even nphi the reference's hop operator commutes with translations,
//     so the sum over the Dl translates of the row state collapses to the
//     untranslated hops times a phase factor G: G = Dl * sign * FT[0][q] when
//     the target orbit carries momentum K coherently, and an explicit sum over
//     ql of the translation signs and phases otherwise (short, null orbits);
//   * for odd nphi (where the reference's empty-site sign convention is not
//     translation covariant) every translate is enumerated, exactly as the
//     reference does ("literal" mode);
//   * candidates of a row are sorted by column in shared memory and merged,
//     thresholded at |H_ij| > 1e-10 like the reference
//     (lanczos_hamiltonian.cpp:342-347);
//   * one generation pass writes each row to a staging area (stride = the
//     candidate capacity); rows whose candidates overflow the capacity are
//     recorded and regenerated with a larger buffer; a scan and a copy then
//     form the CSR. The Rayleigh pass contracts the same rows with a vector.
//
// Arithmetic. GB300's FP64 pipe runs at a small fraction of its integer and
// FP32 rates, and an FP64 instruction issued by a partly active warp costs as
// much as a full one. In real sectors (every phase is +-1) a candidate is an
// integer combination of interaction-table entries, so the tables are held as
// 64-bit fixed point (scaled by 2^52) and candidates, merges and the diagonal
// are exact integer sums; each kept entry is converted to FP64 once, with all
// lanes busy, times its factor Dl / sqrt(Dl Dr) (or 1 / sqrt(Dl Dr)).
// Integer sums are associative, so real rows are bit-reproducible in any
// order. Complex sectors accumulate in FP64 in generation order.
#include <cmath>
#include <cstring>
#include <algorithm>
#include <map>
#include <mutex>
#include <set>

#include "sector.cuh"

namespace {

constexpr uint32_t NONE = 0xFFFFFFFFu;
constexpr int ROW_WARPS = 4;  // warps per block
// electron pairs of a row state (C(nel, 2) + 1 with the tunnelling entry)
// fill a per-warp array of pair_cap masks and prefix counts (RowGen::pair_cap)
constexpr int FIXED_BITS = 52;  // fixed-point scale of the real-sector tables

struct RowGen {
  SectorIdx S;
  HamilTables T;
  const double* W;     // [2][nphi][nphi] pre-summed transfers (FP64, complex sectors)
  const long long* Wq; // the same in fixed point (real sectors)
  long long tun_q;     // -Delta_SAS / 2 in fixed point
  const double* DLF;   // [16][16] Dl / sqrt(Dl Dr)
  const double* FQC;   // [16][16] Dl / sqrt(Dl Dr) * 2^-52 (coherent, real)
  const double* FQI;   // [16][16] 1 / sqrt(Dl Dr) * 2^-52 (literal or incoherent, real)
  uint64_t ft_neg;     // bit m + nphi set when the real phase FT(m) is -1
  const uint64_t* id;
  const uint8_t* period;
  const uint8_t* compat;
  const uint32_t* map;
  int64_t dim;
  int K;
  int cap;             // candidate buffer per warp (power of two)
  int pair_cap;        // electron-pair slots per warp (C(nel, 2) + 2, a multiple of 2)
  int key32;           // sort keys fit 32 bits: (row j) << slot_bits | slot
  int slot_bits;
};

// What a pass does with each merged row.
struct Sink {
  int phase;                 // PH_STAGE or PH_RQ
  const int32_t* rows;       // optional row list (overflow re-run); null = all rows
  int64_t nrows;
  int32_t* row_nnz;          // [dim] entries kept per row (-1: overflowed this capacity)
  int32_t* st_col;           // staging [slot_row * cap]
  void* st_val;              // staging values (double or Cx)
  int32_t* overflow_rows;    // rows that overflowed, appended
  int* overflow_count;
  int* bad_value;            // a merged real entry decoded out of range (fixed-point overflow)
  const double* psi;         // RQ vector
  double* rq_partial;        // [2 * gridDim.x]
};

struct Cx {
  double re, im;
};

__constant__ uint8_t c_pair_lo[120];
__constant__ uint8_t c_pair_hi[120];

enum { PH_STAGE = 0, PH_RQ = 1 };

// buffer element while a row is assembled / staged element
template <bool CPLX>
struct BufT;
template <>
struct BufT<false> {
  using T = long long;
};
template <>
struct BufT<true> {
  using T = Cx;
};
template <bool CPLX>
struct StageT;
template <>
struct StageT<false> {
  using T = double;
};
template <>
struct StageT<true> {
  using T = Cx;
};

__device__ __forceinline__ double sgn(int parity) { return parity ? -1.0 : 1.0; }

// e^{2 pi i m K / nphi}, m in (-nphi, nphi), as the reference's FT table.
__device__ __forceinline__ Cx ftc(const HamilTables& T, int m) { return Cx{T.FTc[m + T.nphi], T.FTs[m + T.nphi]}; }

__device__ __forceinline__ int ftneg(const RowGen& R, int m, int nphi) { return (int)((R.ft_neg >> (m + nphi)) & 1); }

// Real sectors: integer multiplier g of a candidate (signs and +-1 phases of
// the translates summed); the FP64 factor is applied after merging.
__device__ __forceinline__ int real_multiplier(const RowGen& R, uint64_t x, int q, int Dl, int Dr, int ql,
                                               int signl_par, bool coherent, int nphi) {
  int p;
  if (R.T.literal) {
    inv_translate_bits(x, q, nphi, &p);
    return (p ^ signl_par ^ ftneg(R, ql - q, nphi)) ? -1 : 1;
  }
  if (coherent) {
    inv_translate_bits(x, q, nphi, &p);
    return (p ^ ftneg(R, -q, nphi)) ? -1 : 1;
  }
  int g = 0;
  for (int qq = 0; qq < Dl; qq++) {
    int p1, p2;
    const uint64_t y = translate_bits(x, qq, nphi, &p1);
    int qr = q + qq;
    while (qr >= Dr) qr -= Dr;
    inv_translate_bits(y, qr, nphi, &p2);
    g += (p1 ^ p2 ^ ftneg(R, qq - qr, nphi)) ? -1 : 1;
  }
  return g;
}

// Complex sectors: value coef * G / sqrt(Dl Dr) in FP64 (see the file comment).
__device__ __forceinline__ Cx complex_value(const RowGen& R, Cx coef, uint64_t x, int q, int Dl, int Dr, int ql,
                                            int signl_par, bool coherent, int nphi) {
  Cx v;
  int p;
  if (!R.T.literal && coherent) {
    inv_translate_bits(x, q, nphi, &p);
    const double f = __ldg(&R.DLF[(Dl - 1) * 16 + (Dr - 1)]);
    const Cx ph = ftc(R.T, -q);
    const double s = p ? -f : f;
    const double gr = s * ph.re, gi = s * ph.im;
    v.re = coef.re * gr - coef.im * gi;
    v.im = coef.re * gi + coef.im * gr;
    return v;
  }
  Cx G{0.0, 0.0};
  if (R.T.literal) {
    inv_translate_bits(x, q, nphi, &p);
    const Cx f = ftc(R.T, ql - q);
    const double s = sgn(p ^ signl_par);
    G.re = s * f.re;
    G.im = s * f.im;
  } else {
    for (int qq = 0; qq < Dl; qq++) {
      int p1, p2;
      const uint64_t y = translate_bits(x, qq, nphi, &p1);
      int qr = q + qq;
      while (qr >= Dr) qr -= Dr;
      inv_translate_bits(y, qr, nphi, &p2);
      const Cx f = ftc(R.T, qq - qr);
      const double s = sgn(p1 ^ p2);
      G.re += s * f.re;
      G.im += s * f.im;
    }
  }
  const double inv = __ldg(&R.T.isq[(Dl - 1) * 16 + (Dr - 1)]);
  v.re = (coef.re * G.re - coef.im * G.im) * inv;
  v.im = (coef.re * G.im + coef.im * G.re) * inv;
  return v;
}

// One row per warp; candidates are appended to a per-warp buffer, sorted by
// (column, generation slot), merged, thresholded and handed to the sink.
// NPHI > 0 fixes nphi at compile time (divisions by constants); 0 reads it at run time.
// DIR (the Rayleigh quotient <psi|H|psi>): every candidate is multiplied by
// psi at its column and summed at once, without staging, sorting or merging
// (the sum is linear in the candidates; elements that merge to |H_ij| <= 1e-10,
// which the stored matrix drops, are included, a change far below 1e-12 in E).
template <bool CPLX, class KeyT, int NPHI, bool DIR>
__global__ void __launch_bounds__(ROW_WARPS * 32) k_rows(RowGen R, Sink sk) {
  using BT = typename BufT<CPLX>::T;
  using ST = typename StageT<CPLX>::T;
  extern __shared__ __align__(16) unsigned char smem[];
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  const int cap = DIR ? 0 : R.cap;
  const size_t per_warp = (size_t)cap * (sizeof(BT) + sizeof(KeyT)) + 64 + (size_t)R.pair_cap * 8;
  unsigned char* base = smem + per_warp * wib;
  BT* vals = reinterpret_cast<BT*>(base);
  KeyT* keys = reinterpret_cast<KeyT*>(base + (size_t)cap * sizeof(BT));
  uint8_t* occ = base + (size_t)cap * (sizeof(BT) + sizeof(KeyT));  // upper [0,16), lower [16,32)
  uint32_t* pmask = reinterpret_cast<uint32_t*>(occ + 64);             // per pair: allowed targets
  int* ppre = reinterpret_cast<int*>(occ + 64 + R.pair_cap * 4);      // per pair: first candidate
  const int nphi = NPHI ? NPHI : R.T.nphi;
  const uint64_t lmask = (1ULL << nphi) - 1;
  const double* W0 = R.W;
  const double* W1 = R.W + nphi * nphi;
  const long long* W0q = R.Wq;
  const long long* W1q = R.Wq + nphi * nphi;
  const double* V1 = R.T.V + nphi * nphi;
  const int sb = R.slot_bits;
  const KeyT slot_mask = (KeyT)((1ULL << sb) - 1);
  Cx rq_acc{0.0, 0.0};

  const int64_t nrows = sk.rows ? sk.nrows : R.dim;
  const int64_t warps_total = (int64_t)gridDim.x * ROW_WARPS;
  for (int64_t t = (int64_t)blockIdx.x * ROW_WARPS + wib; t < nrows; t += warps_total) {
    const int64_t i = sk.rows ? sk.rows[t] : t;
    const uint64_t c0 = R.id[i];
    const int Dl = (R.K < 0) ? 1 : R.period[i];
    const int nql = R.T.literal ? Dl : 1;
    int cnt = 0;
    Cx drow{0.0, 0.0};   // DIR: this lane's sum of H_ij psi_j over its candidates
    Cx diag{0.0, 0.0};   // complex sectors
    long long diag_q = 0;  // real sectors (fixed point, factor applied at merge)
    for (int ql = 0; ql < nql; ql++) {
      int pl = 0;
      const uint64_t lb = ql ? translate_bits(c0, ql, nphi, &pl) : c0;
      const uint32_t u = (uint32_t)(lb & lmask), d = (uint32_t)((lb >> nphi) & lmask);
      const int nu = popc32(u), nd = popc32(d);
      __syncwarp();
      if (lane == 0) {
        int k = 0;
        for (uint32_t s = u; s; s &= s - 1) occ[k++] = (uint8_t)(__ffs(s) - 1);
        k = 16;
        for (uint32_t s = d; s; s &= s - 1) occ[k++] = (uint8_t)(__ffs(s) - 1);
      }
      __syncwarp();
      // Candidates, compacted: for every electron pair (upper, lower, inter-layer,
      // then one entry for the tunnelling moves) the mask of target orbitals a
      // whose move is allowed (both targets empty, and for same-layer pairs
      // a < the partner's orbital, one of the two labelings) is built from the
      // empty-orbital masks by a bit reversal and a rotation; lanes then take
      // only allowed candidates, in the same (pair, a) order as a walk over all
      // pair x orbital slots would visit them.
      const int PU = nu * (nu - 1) / 2, PL = nd * (nd - 1) / 2, PX = nu * nd;
      const int PT = (R.T.dsas > 0) ? 1 : 0;
      const int P = PU + PL + PX + PT;
      const uint32_t lm32 = (uint32_t)lmask;
      auto rev = [&](uint32_t e) { return __brev(e) >> (32 - nphi); };           // bit i <- bit nphi-1-i
      auto rotl = [&](uint32_t v, int k) {                                      // bit a <- bit (a - k) mod nphi
        return k ? (((v << k) | (v >> (nphi - k))) & lm32) : v;
      };
      auto bits = [&](int lo_, int hi_) {  // bits [lo_, hi_) of a 32-bit word
        return hi_ > lo_ ? (((hi_ >= 32) ? 0xffffffffu : ((1u << hi_) - 1u)) & ~((1u << lo_) - 1u)) : 0u;
      };
      int total = 0;
      for (int p0 = 0; p0 < P; p0 += 32) {
        const int pp = p0 + lane;
        uint32_t M = 0;
        if (pp < PU + PL) {
          const bool lower = pp >= PU;
          const int q = lower ? pp - PU : pp;
          const uint8_t* oc = occ + (lower ? 16 : 0);
          const int nl = oc[c_pair_lo[q]], ml = oc[c_pair_hi[q]];
          const uint32_t lay = lower ? d : u;
          const uint32_t E = ~(lay ^ (1u << nl) ^ (1u << ml)) & lm32;
          int t = nl + ml;
          t -= (t >= nphi) ? nphi : 0;
          const int k = (t + 1 == nphi) ? 0 : t + 1;
          // a < (t - a) mod nphi: a < (t + 1) / 2, or t < a < (t + nphi + 1) / 2
          const uint32_t LT = bits(0, (t + 1) / 2) | bits(t + 1, (t + nphi + 1) / 2);
          M = E & rotl(rev(E), k) & LT;
        } else if (pp < PU + PL + PX) {
          const int q = pp - PU - PL;
          const int pu = q / nd, pd = q - pu * nd;
          const int n = occ[pu], ml = occ[16 + pd];
          const uint32_t Eu = ~(u ^ (1u << n)) & lm32, Ed = ~(d ^ (1u << ml)) & lm32;
          int t = n + ml;
          t -= (t >= nphi) ? nphi : 0;
          const int k = (t + 1 == nphi) ? 0 : t + 1;
          M = Eu & rotl(rev(Ed), k);
        } else if (pp < P) {
          M = (u ^ d) & lm32;  // exactly one of (n, n + nphi) occupied
        }
        const int cp = __popc(M);
        int inc = cp;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
          const int y = __shfl_up_sync(0xffffffffu, inc, o);
          if (lane >= o) inc += y;
        }
        if (pp < P) {
          pmask[pp] = M;
          ppre[pp] = total + inc - cp;
        }
        total += __shfl_sync(0xffffffffu, inc, 31);
      }
      __syncwarp();
      for (int c0 = 0; c0 < total; c0 += 32) {
        const int cidx = c0 + lane;
        bool valid = false;
        uint64_t x = 0;
        Cx coef{0.0, 0.0};
        long long coef_q = 0;
        if (cidx < total) {
          // the pair: the last one whose candidates start at or before cidx
          int plo = 0, phi = P;
          while (phi - plo > 1) {
            const int mid = (plo + phi) >> 1;
            if (ppre[mid] <= cidx) plo = mid;
            else phi = mid;
          }
          const int pp = plo;
          uint32_t mk = pmask[pp];
          for (int r = cidx - ppre[pp]; r > 0; r--) mk &= mk - 1;
          const int a = __ffs(mk) - 1;
          valid = true;
          if (pp < PU + PL) {
            // same-layer pair (lanczos_hamiltonian.cpp:109-230)
            const bool lower = pp >= PU;
            const int q = lower ? pp - PU : pp;
            const int lo = lower ? nphi : 0;
            const uint8_t* oc = occ + (lower ? 16 : 0);
            const int nl = oc[c_pair_lo[q]], ml = oc[c_pair_hi[q]];
            int bl = nl + ml - a;  // in (-nphi, 2 nphi)
            bl += (bl < 0) ? nphi : 0;
            bl -= (bl >= nphi) ? nphi : 0;
            const int n = lo + nl, m = lo + ml;
            const uint64_t rest = lb ^ ((1ULL << n) | (1ULL << m));
            const int A = lo + a, Bt = lo + bl;
            x = rest | (1ULL << A) | (1ULL << Bt);
            // labeling (nt, mt) = (A, Bt) and the exchange (Bt, A)
            int t1 = a - nl, t2 = bl - nl;
            t1 += (t1 < 0) ? nphi : 0;
            t2 += (t2 < 0) ? nphi : 0;
            const int i1 = abs(Bt - n) * nphi + t1, i2 = abs(A - n) * nphi + t2;
            const int p1 = hop2_parity(lb, n, m, A, Bt), p2 = hop2_parity(lb, n, m, Bt, A);
            if constexpr (CPLX) {
              coef.re = sgn(p1) * __ldg(&W0[i1]) + sgn(p2) * __ldg(&W0[i2]);
            } else {
              const long long w1 = __ldg(&W0q[i1]), w2 = __ldg(&W0q[i2]);
              coef_q = (p1 ? -w1 : w1) + (p2 ? -w2 : w2);
            }
          } else if (pp < PU + PL + PX) {
            // inter-layer pair (lanczos_hamiltonian.cpp:232-292)
            const int q = pp - PU - PL;
            const int pu = q / nd, pd = q - pu * nd;
            const int n = occ[pu], ml = occ[16 + pd], m = nphi + ml;
            int bl = n + ml - a;  // in (-nphi, 2 nphi)
            bl += (bl < 0) ? nphi : 0;
            bl -= (bl >= nphi) ? nphi : 0;
            const int mt = nphi + bl;
            const uint64_t rest = lb ^ ((1ULL << n) | (1ULL << m));
            x = rest | (1ULL << a) | (1ULL << mt);
            int t1 = a - n;
            t1 += (t1 < 0) ? nphi : 0;
            const int sidx = abs(bl - n);
            const int par = hop2_parity(lb, n, m, a, mt);
            if constexpr (CPLX) {
              const double sg = sgn(par);
              if (R.T.theta_y != 0.0) {
                // twist phase e^{2 i theta_y t / nphi} per momentum transfer t
                const double v1 = V1[sidx * nphi + t1];
                coef.re = sg * v1 * R.T.TWc[t1 + nphi];
                coef.im = sg * v1 * R.T.TWs[t1 + nphi];
                if (t1 > 0) {
                  const double v2 = V1[sidx * nphi + (nphi - t1)];
                  coef.re += sg * v2 * R.T.TWc[t1];
                  coef.im += sg * v2 * R.T.TWs[t1];
                }
              } else {
                coef.re = sg * __ldg(&W1[sidx * nphi + t1]);
              }
            } else {
              const long long w = __ldg(&W1q[sidx * nphi + t1]);
              coef_q = par ? -w : w;
            }
          } else {
            // tunnelling (lanczos_hamiltonian.cpp:294-322)
            const int n = a, nt = n + nphi;
            x = lb ^ ((1ULL << n) | (1ULL << nt));
            const int par = hop1_parity(lb, n, nt);
            if constexpr (CPLX) coef.re = -0.5 * R.T.dsas * sgn(par);
            else coef_q = par ? -R.tun_q : R.tun_q;
          }
        }
        int64_t j = -1;
        BT v{};
        if (valid) {
          // A translate of the row state lies in momentum sector J + ql*nel, and
          // so do its targets: look up the target translated back by ql, whose
          // representative is reached from x itself by ql + q translations.
          int pq;
          const uint64_t xs = (ql == 0) ? x : inv_translate_bits(x, ql, nphi, &pq);
          const int64_t e = sector_index(R.S, xs);
          const uint32_t ent = (e >= 0) ? __ldg(&R.map[e]) : NONE;
          if (ent == NONE) {
            valid = false;
          } else {
            j = ent >> 5;
            const int Dr = (R.K < 0) ? 1 : R.period[j];
            int q = (int)(ent & 31);
            if (ql) {
              q += ql;
              while (q >= Dr) q -= Dr;
            }
            const bool coh = R.compat[j] != 0;
            if constexpr (CPLX) {
              v = complex_value(R, coef, x, q, Dl, Dr, ql, pl, coh, nphi);
              if (j == i) {
                diag.re += v.re;
                diag.im += v.im;
                valid = false;
              }
            } else {
              const int g = real_multiplier(R, x, q, Dl, Dr, ql, pl, coh, nphi);
              v = coef_q * (long long)g;
              if (j == i) {
                diag_q += v;
                valid = false;
              }
            }
          }
        }
        if constexpr (DIR) {
          if (valid) {
            double vr, vi = 0.0;
            if constexpr (CPLX) {
              vr = v.re;
              vi = v.im;
            } else {
              const int Dr = (R.K < 0) ? 1 : R.period[j];
              const bool ff = R.T.literal || !R.compat[j];
              vr = (double)v * __ldg(&(ff ? R.FQI : R.FQC)[(Dl - 1) * 16 + (Dr - 1)]);
            }
            const double xr = CPLX ? sk.psi[2 * j] : sk.psi[j];
            const double xi = CPLX ? sk.psi[2 * j + 1] : 0.0;
            drow.re += vr * xr - vi * xi;
            drow.im += vr * xi + vi * xr;
          }
        } else {
          const unsigned bal = __ballot_sync(0xffffffffu, valid);
          const int slot = cnt + __popc(bal & ((1u << lane) - 1));
          if (valid && slot < cap) {
            keys[slot] = (KeyT)(((KeyT)j << sb) | (KeyT)slot);
            vals[slot] = v;
          }
          cnt += __popc(bal);
        }
      }
    }
    if constexpr (DIR) {
      // the diagonal: this lane's two-body part, and on lane 0 the one-body terms
      Cx dd{0.0, 0.0};
      if constexpr (CPLX) {
        dd = diag;
      } else {
        const bool ff = R.T.literal || !R.compat[i];
        dd.re = (double)diag_q * __ldg(&(ff ? R.FQI : R.FQC)[(Dl - 1) * 16 + (Dl - 1)]);
      }
      if (lane == 0) {
        const int nu0 = popc64(c0 & lmask), nd0 = R.S.nel - nu0;
        dd.re += R.T.Ec * R.S.nel - R.T.d * nu0 * nd0 / nphi;
        if (R.T.dv > 0) dd.re += 0.5 * R.T.dv * nu0 - 0.5 * R.T.dv * nd0;
      }
      const double pr = CPLX ? sk.psi[2 * i] : sk.psi[i];
      const double pim = CPLX ? sk.psi[2 * i + 1] : 0.0;
      drow.re += dd.re * pr - dd.im * pim;
      drow.im += dd.re * pim + dd.im * pr;
      // conj(psi_i) (H psi)_i, this lane's part
      rq_acc.re += pr * drow.re + pim * drow.im;
      rq_acc.im += pr * drow.im - pim * drow.re;
      continue;
    }
    // diagonal: the two-body part reduced over the warp (in a fixed order for
    // complex sectors, exactly for real ones); one-body terms are added at merge
    if constexpr (CPLX) {
      for (int o = 16; o > 0; o >>= 1) {
        diag.re += __shfl_xor_sync(0xffffffffu, diag.re, o);
        diag.im += __shfl_xor_sync(0xffffffffu, diag.im, o);
      }
    } else {
      for (int o = 16; o > 0; o >>= 1) diag_q += __shfl_xor_sync(0xffffffffu, diag_q, o);
    }
    if (cnt + 1 > cap) {
      // this row does not fit: record it for a run with a larger buffer
      if (lane == 0 && sk.phase == PH_STAGE) {
        sk.row_nnz[i] = -1;
        const int k = atomicAdd(sk.overflow_count, 1);
        sk.overflow_rows[k] = (int32_t)i;
      }
      if (lane == 0 && sk.phase == PH_RQ) atomicAdd(sk.overflow_count, 1);
      continue;
    }
    if (lane == 0) {
      keys[cnt] = (KeyT)(((KeyT)i << sb) | (KeyT)cnt);
      if constexpr (CPLX) vals[cnt] = diag;
      else vals[cnt] = diag_q;
    }
    cnt += 1;
    // bitonic sort of keys[0, npad)
    int npad = 32;
    while (npad < cnt) npad <<= 1;
    for (int k = cnt + lane; k < npad; k += 32) keys[k] = (KeyT)~(KeyT)0;
    __syncwarp();
    for (int k = 2; k <= npad; k <<= 1) {
      for (int jj = k >> 1; jj > 0; jj >>= 1) {
        for (int tt = lane; tt < (npad >> 1); tt += 32) {
          const int a = ((tt & ~(jj - 1)) << 1) | (tt & (jj - 1));
          const int b = a + jj;
          const KeyT ka = keys[a], kb = keys[b];
          const bool up = (a & k) == 0;
          if ((ka > kb) == up) {
            keys[a] = kb;
            keys[b] = ka;
          }
        }
        __syncwarp();
      }
    }
    // one-body diagonal terms (lanczos_hamiltonian.cpp:324-339), FP64
    const int nu0 = popc64(c0 & lmask), nd0 = R.S.nel - nu0;
    double one_body = R.T.Ec * R.S.nel;
    one_body += -R.T.d * nu0 * nd0 / nphi;
    if (R.T.dv > 0) one_body += 0.5 * R.T.dv * nu0 - 0.5 * R.T.dv * nd0;
    // merge runs of equal column, convert, threshold, emit
    int nout = 0;
    const int64_t sbase = (sk.phase == PH_STAGE) ? (sk.rows ? t : i) * (int64_t)cap : 0;
    Cx psi_i{0.0, 0.0};
    if (sk.phase == PH_RQ) {
      psi_i.re = CPLX ? sk.psi[2 * i] : sk.psi[i];
      psi_i.im = CPLX ? sk.psi[2 * i + 1] : 0.0;
    }
    Cx row_dot{0.0, 0.0};
    for (int b0 = 0; b0 < cnt; b0 += 32) {
      const int idx = b0 + lane;
      bool keep = false;
      uint32_t jcol = 0;
      Cx sum{0.0, 0.0};
      if (idx < cnt) {
        const uint64_t jc = (uint64_t)(keys[idx] >> sb);
        const bool head = (idx == 0) || ((uint64_t)(keys[idx - 1] >> sb) != jc);
        if (head) {
          jcol = (uint32_t)jc;
          if constexpr (CPLX) {
            for (int k = idx; k < cnt && (uint64_t)(keys[k] >> sb) == jc; k++) {
              const Cx tv = vals[(int)(keys[k] & slot_mask)];
              sum.re += tv.re;
              sum.im += tv.im;
            }
          } else {
            long long acc = 0;
            for (int k = idx; k < cnt && (uint64_t)(keys[k] >> sb) == jc; k++) acc += vals[(int)(keys[k] & slot_mask)];
            const int Dr = (R.K < 0) ? 1 : R.period[jcol];
            const bool ff = R.T.literal || !R.compat[jcol];
            const double fac = __ldg(&(ff ? R.FQI : R.FQC)[(Dl - 1) * 16 + (Dr - 1)]);
            sum.re = (double)acc * fac;
            if (acc > (1LL << 62) || acc < -(1LL << 62)) atomicOr(sk.bad_value, 1);  // |acc| * 2^-52 > 1024
          }
          if (jcol == (uint32_t)i) sum.re += one_body;
          keep = sum.re * sum.re + sum.im * sum.im > 1e-20;  // |H_ij| > 1e-10
        }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, keep);
      if (keep) {
        const int o = nout + __popc(bal & ((1u << lane) - 1));
        if (sk.phase == PH_STAGE) {
          sk.st_col[sbase + o] = (int32_t)jcol;
          if constexpr (CPLX) reinterpret_cast<ST*>(sk.st_val)[sbase + o] = sum;
          else reinterpret_cast<ST*>(sk.st_val)[sbase + o] = sum.re;
        } else {
          const double xr = CPLX ? sk.psi[2 * (int64_t)jcol] : sk.psi[jcol];
          const double xi = CPLX ? sk.psi[2 * (int64_t)jcol + 1] : 0.0;
          row_dot.re += sum.re * xr - sum.im * xi;
          row_dot.im += sum.re * xi + sum.im * xr;
        }
      }
      nout += __popc(bal);
    }
    if (sk.phase == PH_STAGE && lane == 0) sk.row_nnz[i] = nout;
    if (sk.phase == PH_RQ) {
      // conj(psi_i) * (H psi)_i
      rq_acc.re += psi_i.re * row_dot.re + psi_i.im * row_dot.im;
      rq_acc.im += psi_i.re * row_dot.im - psi_i.im * row_dot.re;
    }
    __syncwarp();
  }
  if (sk.phase == PH_RQ) {
    __shared__ double red[ROW_WARPS][2];
    for (int o = 16; o > 0; o >>= 1) {
      rq_acc.re += __shfl_xor_sync(0xffffffffu, rq_acc.re, o);
      rq_acc.im += __shfl_xor_sync(0xffffffffu, rq_acc.im, o);
    }
    if (lane == 0) {
      red[wib][0] = rq_acc.re;
      red[wib][1] = rq_acc.im;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      double a = 0, b = 0;
      for (int w = 0; w < ROW_WARPS; w++) {
        a += red[w][0];
        b += red[w][1];
      }
      sk.rq_partial[2 * blockIdx.x] = a;
      sk.rq_partial[2 * blockIdx.x + 1] = b;
    }
  }
}

// Staging -> CSR (one warp per row). Rows regenerated after an overflow come
// from the second staging area, at their position in the overflow list.
template <bool CPLX>
__global__ void k_compact(int64_t dim, const int64_t* row_ptr, const int32_t* st_col, const void* st_val, int cap,
                          const int32_t* ov_pos, const int32_t* ov_col, const void* ov_val, int ov_cap,
                          int32_t* col, void* val64, void* val32, void* res) {
  using VT = typename StageT<CPLX>::T;
  const int lane = threadIdx.x & 31;
  const int64_t w = ((int64_t)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int64_t nw = ((int64_t)gridDim.x * blockDim.x) >> 5;
  for (int64_t i = w; i < dim; i += nw) {
    const int64_t o = row_ptr[i], n = row_ptr[i + 1] - o;
    const int32_t op = ov_pos ? ov_pos[i] : -1;
    const int32_t* sc = (op >= 0) ? ov_col + (int64_t)op * ov_cap : st_col + i * (int64_t)cap;
    const VT* sv = (op >= 0) ? reinterpret_cast<const VT*>(ov_val) + (int64_t)op * ov_cap
                             : reinterpret_cast<const VT*>(st_val) + i * (int64_t)cap;
    for (int64_t k = lane; k < n; k += 32) {
      col[o + k] = sc[k];
      Cx v;
      if constexpr (CPLX) v = sv[k];
      else v = Cx{sv[k], 0.0};
      if (val64) {
        if (CPLX) reinterpret_cast<double2*>(val64)[o + k] = make_double2(v.re, v.im);
        else reinterpret_cast<double*>(val64)[o + k] = v.re;
      }
      if (val32) {
        const float re = (float)v.re, im = (float)v.im;
        if (CPLX) reinterpret_cast<float2*>(val32)[o + k] = make_float2(re, im);
        else reinterpret_cast<float*>(val32)[o + k] = re;
        if (res) {
          if (CPLX)
            reinterpret_cast<float2*>(res)[o + k] =
                make_float2((float)(v.re - (double)re), (float)(v.im - (double)im));
          else reinterpret_cast<float*>(res)[o + k] = (float)(v.re - (double)re);
        }
      }
    }
  }
}

__global__ void k_mark_overflow(const int32_t* rows, int n, int32_t* ov_pos) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) ov_pos[rows[t]] = t;
}

__global__ void k_i32_to_i64(const int32_t* a, int64_t* b, int64_t n) {
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    b[i] = a[i];
}

// Upper bound of candidates (plus the diagonal entry) in one row.
int row_bound(const blqh_sector& s, int literal) {
  const int nphi = s.nphi;
  auto intra = [&](int k) { return k * (k - 1) / 2 * ((nphi - k + 2) / 2 + 1); };
  int bound;
  if (s.nel_up >= 0) {
    const int nu = s.nel_up, nd = s.nel - s.nel_up;
    bound = intra(nu) + intra(nd) + nu * nd * (nphi - (nu < nd ? nu : nd) + 1) + nphi + 1;
  } else {
    int best = 0;
    for (int nu = 0; nu <= s.nel; nu++) {
      const int nd = s.nel - nu;
      if (nu > nphi || nd > nphi) continue;
      int b = intra(nu) + intra(nd) + nu * nd * (nphi + 1) + nphi + 1;
      if (b > best) best = b;
    }
    bound = best;
  }
  if (literal) bound *= nphi;
  return bound;
}

int pow2_at_least(int x) {
  int c = 32;
  while (c < x) c <<= 1;
  return c;
}

std::set<int> g_pair_ready;
std::mutex g_pair_mu;  // contexts on several host threads
void init_pair_tables(int device) {
  std::lock_guard<std::mutex> lk(g_pair_mu);
  if (g_pair_ready.count(device)) return;
  uint8_t lo[120], hi[120];
  int p = 0;
  for (int h = 1; h < 16; h++)
    for (int l = 0; l < h; l++) {
      lo[p] = (uint8_t)l;
      hi[p] = (uint8_t)h;
      p++;
    }
  cudaMemcpyToSymbol(c_pair_lo, lo, sizeof(lo));
  cudaMemcpyToSymbol(c_pair_hi, hi, sizeof(hi));
  g_pair_ready.insert(device);
}

struct TablesDev {
  double* buf = nullptr;
  ~TablesDev() { dev_free(buf); }
};

// Interaction tables on the device plus the generator description.
RowGen make_rowgen(blqh_ctx* ctx, const blqh_basis* B, const blqh_params& p, TablesDev& td, bool* is_complex) {
  const int nphi = B->sector.nphi, K = B->sector.K;
  double Ec;
  std::vector<double> V;
  coulomb_tables_host(nphi, K, p, &Ec, V);
  // layout (8-byte slots): V [2n^2] | W [2n^2] | FTc FTs TWc TWs [4 * 2n] |
  //                        isq, DLF, FQC, FQI [4 * 256] | Wq [2n^2] (int64)
  const size_t nV = 2 * nphi * nphi;
  std::vector<double> t(3 * nV + 8 * nphi + 1024, 0.0);
  double* tV = t.data();
  double* tW = tV + nV;
  double* tF = tW + nV;
  double* tI = tF + 8 * nphi;
  double* tD = tI + 256;
  double* tC = tD + 256;
  double* tJ = tC + 256;
  long long* tQ = reinterpret_cast<long long*>(tJ + 256);
  const double scale = std::ldexp(1.0, FIXED_BITS);
  for (size_t k = 0; k < nV; k++) tV[k] = V[k];
  for (int a = 0; a < 2; a++)
    for (int s = 0; s < nphi; s++)
      for (int q = 0; q < nphi; q++) {
        const double* row = &V[a * nphi * nphi + s * nphi];
        const double w = row[q] + (q > 0 ? row[nphi - q] : 0.0);
        tW[a * nphi * nphi + s * nphi + q] = w;
        tQ[a * nphi * nphi + s * nphi + q] = std::llrint(w * scale);
      }
  for (int m = -nphi; m < nphi; m++) {
    tF[m + nphi] = cos(2.0 * M_PI * m * K / nphi);  // K < 0 only ever reads m = 0
    tF[2 * nphi + m + nphi] = sin(2.0 * M_PI * m * K / nphi);
    tF[4 * nphi + m + nphi] = cos(2 * p.theta_y * m / nphi);
    tF[6 * nphi + m + nphi] = sin(2 * p.theta_y * m / nphi);
  }
  // Real arithmetic when every phase is +-1: K in {0, nphi/2} (or no
  // translation symmetry) and no twist.
  const bool real = (K <= 0 || 2 * K == nphi) && p.theta_y == 0.0;
  uint64_t ftneg = 0;
  if (real)
    for (int m = -nphi; m < nphi; m++) {
      tF[m + nphi] = (tF[m + nphi] > 0) ? 1.0 : -1.0;
      if (tF[m + nphi] < 0) ftneg |= 1ULL << (m + nphi);
    }
  for (int dl = 1; dl <= 16; dl++)
    for (int dr = 1; dr <= 16; dr++) {
      const int k = (dl - 1) * 16 + (dr - 1);
      tI[k] = 1.0 / sqrt((double)(dl * dr));
      tD[k] = dl / sqrt((double)(dl * dr));
      tC[k] = tD[k] / scale;
      tJ[k] = tI[k] / scale;
    }
  *is_complex = !real;
  td.buf = dalloc<double>(ctx, t.size());
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(td.buf, t.data(), t.size() * 8, cudaMemcpyHostToDevice, ctx->stream));
  RowGen R{};
  R.S = B->sx;
  R.T.nphi = nphi;
  R.T.is_complex = !real;
  R.T.literal = (nphi % 2 == 1) && K >= 0;
  R.T.Ec = Ec;
  R.T.d = p.d;
  R.T.dsas = p.delta_sas;
  R.T.dv = p.delta_v;
  R.T.theta_y = p.theta_y;
  R.T.V = td.buf;
  R.W = td.buf + nV;
  R.T.FTc = td.buf + 2 * nV;
  R.T.FTs = R.T.FTc + 2 * nphi;
  R.T.TWc = R.T.FTc + 4 * nphi;
  R.T.TWs = R.T.FTc + 6 * nphi;
  R.T.isq = R.T.FTc + 8 * nphi;
  R.DLF = R.T.isq + 256;
  R.FQC = R.DLF + 256;
  R.FQI = R.FQC + 256;
  R.Wq = reinterpret_cast<const long long*>(R.FQI + 256);
  R.tun_q = std::llrint(-0.5 * p.delta_sas * scale);
  R.ft_neg = ftneg;
  R.id = B->d_id;
  R.period = B->d_period;
  R.compat = B->d_compat;
  R.map = B->d_map;
  R.dim = B->dim;
  R.K = K;
  const int nel = B->sector.nel;
  R.pair_cap = (nel * (nel - 1) / 2 + 2 + 1) & ~1;  // C(nel, 2) + 1 pairs, rounded up to even
  return R;
}

void set_capacity(RowGen& R, int cap) {
  R.cap = cap;
  int sb = 0;
  while ((1 << sb) < cap) sb++;
  R.slot_bits = sb;
  int jb = 0;
  while ((1LL << jb) < R.dim) jb++;
  R.key32 = (jb + sb) <= 31;
}

size_t rows_smem(const RowGen& R, bool cplx, bool direct = false) {
  const size_t pairs = (size_t)R.pair_cap * 8;
  if (direct) return (size_t)ROW_WARPS * (64 + pairs);
  return (size_t)ROW_WARPS * ((size_t)R.cap * ((cplx ? 16 : 8) + (R.key32 ? 4 : 8)) + 64 + pairs);
}

template <bool CPLX, class KeyT, int NPHI>
void launch_n(blqh_ctx* ctx, const RowGen& R, const Sink& sk, int grid, size_t sm) {
  if (sk.phase == PH_RQ) {
    k_rows<CPLX, uint32_t, NPHI, true><<<grid, ROW_WARPS * 32, rows_smem(R, CPLX, true), ctx->stream>>>(R, sk);
    return;
  }
  smem_attr_at_least(k_rows<CPLX, KeyT, NPHI, false>, (int)sm);
  k_rows<CPLX, KeyT, NPHI, false><<<grid, ROW_WARPS * 32, sm, ctx->stream>>>(R, sk);
}

template <bool CPLX, class KeyT>
void launch_t(blqh_ctx* ctx, const RowGen& R, const Sink& sk, int grid, size_t sm) {
  switch (R.T.nphi) {
    case 8: launch_n<CPLX, KeyT, 8>(ctx, R, sk, grid, sm); break;
    case 10: launch_n<CPLX, KeyT, 10>(ctx, R, sk, grid, sm); break;
    case 12: launch_n<CPLX, KeyT, 12>(ctx, R, sk, grid, sm); break;
    case 14: launch_n<CPLX, KeyT, 14>(ctx, R, sk, grid, sm); break;
    case 16: launch_n<CPLX, KeyT, 16>(ctx, R, sk, grid, sm); break;
    default: launch_n<CPLX, KeyT, 0>(ctx, R, sk, grid, sm); break;
  }
}

int rows_grid(blqh_ctx* ctx, const RowGen& R, bool cplx, int64_t nrows, bool direct = false) {
  const size_t sm = rows_smem(R, cplx, direct);
  int per_sm = (int)(220 * 1024 / (sm ? sm : 1));
  if (per_sm < 1) per_sm = 1;
  if (per_sm > 8) per_sm = 8;
  int64_t need = (nrows + ROW_WARPS - 1) / ROW_WARPS;
  int64_t g = (int64_t)ctx->num_sms * per_sm;
  if (g > need) g = need;
  return (int)(g < 1 ? 1 : g);
}

void launch_rows(blqh_ctx* ctx, const RowGen& R, bool cplx, const Sink& sk, int grid) {
  const size_t sm = rows_smem(R, cplx, sk.phase == PH_RQ);
  int limit = 0;
  cudaDeviceGetAttribute(&limit, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
  if (sm > (size_t)limit) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED,
              "hamil_build: the per-row candidate buffer (" + std::to_string(sm) + " bytes per block) exceeds shared "
              "memory; sectors this large with odd nphi are not supported");
    throw BlqhError{BLQH_ERR_UNSUPPORTED, "smem"};
  }
  if (cplx) {
    if (R.key32) launch_t<true, uint32_t>(ctx, R, sk, grid, sm);
    else launch_t<true, uint64_t>(ctx, R, sk, grid, sm);
  } else {
    if (R.key32) launch_t<false, uint32_t>(ctx, R, sk, grid, sm);
    else launch_t<false, uint64_t>(ctx, R, sk, grid, sm);
  }
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_BUILD);
}

template <class T>
struct DevBuf {
  T* p = nullptr;
  DevBuf() = default;
  DevBuf(blqh_ctx* c, size_t n) { p = dalloc<T>(c, n); }
  ~DevBuf() { dev_free(p); }
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
};

// First buffer capacity: the bound when it is small, else 512 (rows beyond
// that are rare and are regenerated with the full bound).
// First staging capacity: up to 512 candidates; a row that does not fit is
// regenerated in a second pass with the full bound. At Nphi = 16, 8 + 8 rows
// have 493-576 candidates (about one in six overflows); a capacity of 1024,
// which fits all of them, measured slower (lower occupancy).
int first_capacity(int bound) { return bound <= 512 ? pow2_at_least(bound) : 512; }

}  // namespace

// lanczos_hamiltonian.cpp:37-85: background energy and interaction tables.
// V[a][s][qy] = sum over qx (ascending, the reference's order) of
// 2 V_a(qx, qy) cos(2 pi s qx / nphi [+ 2 theta_x]) / (2 lx ly). The potential
// is evaluated once per (qx, qy) for all s, each V[a][s][qy] still summed in
// the same qx order, so the values are those of the per-s loop. The tables
// depend on (nphi, lx, ly, d, nLL, theta_x) only and are memoized: a sweep
// over sectors and Delta_SAS at one layer distance computes them once (at
// d = 0 the interlayer sum runs over ~2000 nphi terms).
void coulomb_tables_host(int nphi, int K, const blqh_params& p, double* Ec_out, std::vector<double>& V) {
  (void)K;
  static std::mutex mu;
  static std::map<std::vector<double>, std::pair<double, std::vector<double>>> memo;
  const std::vector<double> key = {(double)nphi, p.lx, p.ly, p.d, (double)p.nLL, p.theta_x};
  {
    std::lock_guard<std::mutex> lk(mu);
    auto it = memo.find(key);
    if (it != memo.end()) {
      *Ec_out = it->second.first;
      V = it->second.second;
      return;
    }
  }
  const double lx = p.lx, ly = p.ly;
  auto vq = [&](int alpha, int qx, int qy) {
    const double q = sqrt(qx * qx / (lx * lx) + qy * qy / (ly * ly)) * 2.0 * M_PI;
    const double ff = pow(1.0 - exp(-q * q / 2.0), p.nLL * 2);
    if (alpha == 1) return 2.0 * M_PI / q * exp(-q * q / 2.0 - q * p.d) * ff;
    return 2.0 * M_PI / q * exp(-q * q / 2.0) * ff;
  };
  double Ec = -2.0;
  for (int i = 0; i < nphi; i++)
    for (int j = 0; j < nphi; j++)
      if (!(i == 0 && j == 0)) Ec += erfc(sqrt(M_PI * (i * i * lx / ly + j * j * ly / lx)));
  Ec /= sqrt(lx * ly);
  *Ec_out = Ec;
  V.assign(2 * nphi * nphi, 0.0);
  std::vector<double> acc(nphi);
  for (int qy = 0; qy < nphi; qy++) {
    std::fill(acc.begin(), acc.end(), 0.0);
    for (int qx = -nphi; qx <= nphi; qx++) {
      if (qx == 0 && qy == 0) continue;
      const double f = vq(0, qx, qy);
      for (int s = 0; s < nphi; s++) acc[s] += 2.0 * f * cos(2.0 * M_PI * s * qx / nphi) / (2.0 * lx * ly);
    }
    for (int s = 0; s < nphi; s++) V[s * nphi + qy] = acc[s];
    std::fill(acc.begin(), acc.end(), 0.0);
    for (int qx = (int)(-10 * nphi / (p.d + 0.01)); qx < 10 * nphi / (p.d + 0.01); qx++) {
      if (qx == 0 && qy == 0) continue;
      const double f = vq(1, qx, qy);
      for (int s = 0; s < nphi; s++)
        acc[s] += 2.0 * f * cos((2.0 * M_PI * s + 2 * p.theta_x) * qx / nphi) / (2.0 * lx * ly);
    }
    for (int s = 0; s < nphi; s++) V[nphi * nphi + s * nphi + qy] = acc[s];
  }
  std::lock_guard<std::mutex> lk(mu);
  if (memo.size() > 4096) memo.clear();
  memo[key] = {Ec, V};
}

// Build the CSR: one generation pass into staging (plus a pass for the rows
// that overflowed), scan, copy. Values stored in FP64 or FP32.
int hamil_build_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params& p, int prec, blqh_csr* M) {
  init_pair_tables(ctx->device);
  TablesDev td;
  bool cplx = false;
  RowGen R = make_rowgen(ctx, B, p, td, &cplx);
  const int bound = row_bound(B->sector, R.T.literal);
  set_capacity(R, first_capacity(bound));
  const int64_t dim = B->dim;
  const size_t vsz = cplx ? 16 : 8;
  M->dim = dim;
  M->is_complex = cplx;
  M->precision = prec;
  M->d_row_ptr = dalloc<int64_t>(ctx, dim + 1);
  DevBuf<int32_t> row_nnz(ctx, dim);
  DevBuf<int32_t> st_col(ctx, (size_t)dim * R.cap);
  DevBuf<unsigned char> st_val(ctx, (size_t)dim * R.cap * vsz);
  DevBuf<int32_t> ov_rows(ctx, dim);
  DevBuf<int> ov_count(ctx, 2);  // [0] overflowing rows, [1] fixed-point range flag
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(ov_count.p, 0, 2 * sizeof(int), ctx->stream));
  Sink sk{};
  sk.phase = PH_STAGE;
  sk.row_nnz = row_nnz.p;
  sk.st_col = st_col.p;
  sk.st_val = st_val.p;
  sk.overflow_rows = ov_rows.p;
  sk.overflow_count = ov_count.p;
  sk.bad_value = ov_count.p + 1;
  {
    TimerScope ts(ctx, TM_BUILD);
    launch_rows(ctx, R, cplx, sk, rows_grid(ctx, R, cplx, dim));
  }
  int flags[2] = {0, 0};
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(flags, ov_count.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  const int nov = flags[0];
  // rows that did not fit: regenerate them with the full bound into a second staging area
  DevBuf<int32_t> ov_pos, ov_col;
  DevBuf<unsigned char> ov_val;
  RowGen R2 = R;
  if (nov > 0) {
    set_capacity(R2, pow2_at_least(bound));
    ov_pos.p = dalloc<int32_t>(ctx, dim);
    ov_col.p = dalloc<int32_t>(ctx, (size_t)nov * R2.cap);
    ov_val.p = dalloc<unsigned char>(ctx, (size_t)nov * R2.cap * vsz);
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(ov_pos.p, 0xFF, dim * 4, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(ov_count.p, 0, sizeof(int), ctx->stream));
    k_mark_overflow<<<grid_for(ctx, nov, 256, 4), 256, 0, ctx->stream>>>(ov_rows.p, nov, ov_pos.p);
    Sink s2 = sk;
    s2.rows = ov_rows.p;
    s2.nrows = nov;
    s2.st_col = ov_col.p;
    s2.st_val = ov_val.p;
    DevBuf<int32_t> junk(ctx, dim);
    s2.overflow_rows = junk.p;
    {
      TimerScope ts(ctx, TM_BUILD);
      launch_rows(ctx, R2, cplx, s2, rows_grid(ctx, R2, cplx, nov));
    }
    int nov2 = 0;
    BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(&nov2, ov_count.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    if (nov2 > 0) {
      set_error(ctx, BLQH_ERR_CAPACITY, "hamil_build: row candidates exceed the computed bound");
      throw BlqhError{BLQH_ERR_CAPACITY, "capacity"};
    }
  }
  int bad = 0;
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(&bad, ov_count.p + 1, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (bad) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "hamil_build: a matrix element exceeds the fixed-point range");
    throw BlqhError{BLQH_ERR_UNSUPPORTED, "range"};
  }
  k_i32_to_i64<<<grid_for(ctx, dim, 256, 8), 256, 0, ctx->stream>>>(row_nnz.p, M->d_row_ptr, dim);
  int64_t nnz = 0;
  scan_exclusive_i64(ctx, M->d_row_ptr, M->d_row_ptr, dim, &nnz);
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(M->d_row_ptr + dim, &nnz, 8, cudaMemcpyHostToDevice, ctx->stream));
  M->nnz = nnz;
  M->mean_row = dim ? (double)nnz / dim : 0;
  M->d_col = dalloc<int32_t>(ctx, nnz);
  const size_t vs = (prec == BLQH_VAL_FP64 ? 8 : 4) * (cplx ? 2 : 1);
  M->d_val = dev_alloc(ctx, nnz * vs + 16);
  void* v64 = prec == BLQH_VAL_FP64 ? M->d_val : nullptr;
  void* v32 = prec == BLQH_VAL_FP32 ? M->d_val : nullptr;
  if (prec == BLQH_VAL_FP32) {  // the FP32 rests (4 bytes per value); without room, the finisher regenerates
    try {
      M->d_res = dev_alloc(ctx, nnz * vs + 16);
    } catch (const BlqhError& e) {
      if (e.code != BLQH_ERR_NOMEM) throw;
      M->d_res = nullptr;
      ctx->last_error.clear();
    }
  }
  const int cg = grid_for(ctx, dim * 32, 256, 16);
  if (cplx)
    k_compact<true><<<cg, 256, 0, ctx->stream>>>(dim, M->d_row_ptr, st_col.p, st_val.p, R.cap, ov_pos.p, ov_col.p,
                                                 ov_val.p, R2.cap, M->d_col, v64, v32, M->d_res);
  else
    k_compact<false><<<cg, 256, 0, ctx->stream>>>(dim, M->d_row_ptr, st_col.p, st_val.p, R.cap, ov_pos.p, ov_col.p,
                                                  ov_val.p, R2.cap, M->d_col, v64, v32, M->d_res);
  BLQH_TRY_CUDA(ctx, cudaGetLastError());
  count_launch(ctx, TM_BUILD, 2 + (nov > 0 ? 1 : 0));
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  return BLQH_OK;
}

// <psi|H|psi> with regenerated FP64 elements (psi on the device, FP64).
double rayleigh_regen_impl(blqh_ctx* ctx, const blqh_basis* B, const blqh_params& p, const double* d_psi,
                           bool want_complex) {
  init_pair_tables(ctx->device);
  TablesDev td;
  bool cplx = false;
  RowGen R = make_rowgen(ctx, B, p, td, &cplx);
  if (cplx != want_complex) {
    set_error(ctx, BLQH_ERR_ARG, "rayleigh_fp64: vector type does not match the sector");
    throw BlqhError{BLQH_ERR_ARG, "type"};
  }
  // full bound: every row must fit (no staging to defer overflows to)
  set_capacity(R, pow2_at_least(row_bound(B->sector, R.T.literal)));
  DevBuf<int> ov_count(ctx, 2);  // [0] overflowing rows, [1] fixed-point range flag
  BLQH_TRY_CUDA(ctx, cudaMemsetAsync(ov_count.p, 0, 2 * sizeof(int), ctx->stream));
  const int grid = rows_grid(ctx, R, cplx, B->dim, true);
  DevBuf<double> part(ctx, 2 * grid);
  Sink sk{};
  sk.phase = PH_RQ;
  sk.overflow_count = ov_count.p;
  sk.bad_value = ov_count.p + 1;
  sk.psi = d_psi;
  sk.rq_partial = part.p;
  {
    TimerScope ts(ctx, TM_BUILD);
    launch_rows(ctx, R, cplx, sk, grid);
  }
  std::vector<double> h(2 * grid);
  int fl[2] = {0, 0};
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(h.data(), part.p, 16 * grid, cudaMemcpyDeviceToHost, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(fl, ov_count.p, 2 * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  if (fl[1]) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "rayleigh_fp64: a matrix element exceeds the fixed-point range");
    throw BlqhError{BLQH_ERR_UNSUPPORTED, "range"};
  }
  if (fl[0]) {
    set_error(ctx, BLQH_ERR_CAPACITY, "rayleigh_fp64: row candidates exceed the computed bound");
    throw BlqhError{BLQH_ERR_CAPACITY, "capacity"};
  }
  double e = 0;
  for (int b = 0; b < grid; b++) e += h[2 * b];
  return e;
}

// Regenerated FP64 Rayleigh quotients for many vectors without host round
// trips (the batched sweep): tables built once per instance, launches
// enqueued on the context stream (graph-capturable), block partials left on
// the device; flags read once at the end.
struct RqPlan {
  RowGen R{};
  TablesDev td;
  bool cplx = false;
  int grid = 0;
  int* d_flags = nullptr;  // [0] overflowing rows, [1] fixed-point range
  ~RqPlan() { dev_free(d_flags); }
};

RqPlan* rq_plan_create(blqh_ctx* ctx, const blqh_basis* B, const blqh_params& p) {
  init_pair_tables(ctx->device);
  RqPlan* P = new RqPlan;
  try {
    P->R = make_rowgen(ctx, B, p, P->td, &P->cplx);
    set_capacity(P->R, pow2_at_least(row_bound(B->sector, P->R.T.literal)));
    P->grid = rows_grid(ctx, P->R, P->cplx, B->dim, true);
    P->d_flags = dalloc<int>(ctx, 2);
    BLQH_TRY_CUDA(ctx, cudaMemsetAsync(P->d_flags, 0, 2 * sizeof(int), ctx->stream));
  } catch (...) {
    delete P;
    throw;
  }
  return P;
}

int rq_plan_grid(const RqPlan* P) { return P->grid; }
bool rq_plan_complex(const RqPlan* P) { return P->cplx; }

void rq_plan_launch(blqh_ctx* ctx, RqPlan* P, const double* d_psi, double* d_partial) {
  Sink sk{};
  sk.phase = PH_RQ;
  sk.overflow_count = P->d_flags;
  sk.bad_value = P->d_flags + 1;
  sk.psi = d_psi;
  sk.rq_partial = d_partial;
  launch_rows(ctx, P->R, P->cplx, sk, P->grid);
}

// 0, or the error code after recording it (reads the device flags: synchronizes).
int rq_plan_check(blqh_ctx* ctx, RqPlan* P) {
  int fl[2] = {0, 0};
  cudaMemcpy(fl, P->d_flags, sizeof(fl), cudaMemcpyDeviceToHost);
  if (fl[1]) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "rayleigh_fp64: a matrix element exceeds the fixed-point range");
    return BLQH_ERR_UNSUPPORTED;
  }
  if (fl[0]) {
    set_error(ctx, BLQH_ERR_CAPACITY, "rayleigh_fp64: row candidates exceed the computed bound");
    return BLQH_ERR_CAPACITY;
  }
  return 0;
}

void rq_plan_destroy(RqPlan* P) { delete P; }

void free_csr(blqh_csr* m) {
  if (!m) return;
  dev_free(m->d_row_ptr);
  dev_free(m->d_col);
  dev_free(m->d_val);
  dev_free(m->d_res);
  blocked_release(m);
  delete m;
}

extern "C" {

int blqh_hamil_build(blqh_ctx* ctx, const blqh_basis* b, const blqh_params* p, int prec, blqh_csr** out) {
  if (!ctx || !b || !p || !out) return BLQH_ERR_ARG;
  if (prec != BLQH_VAL_FP64 && prec != BLQH_VAL_FP32) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_hamil_build: unknown value precision");
    return BLQH_ERR_ARG;
  }
  *out = nullptr;
  if (b->model != BLQH_MODEL_SPINLESS) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_hamil_build: not a spinless basis (use the spinful or monolayer builder)");
    return BLQH_ERR_ARG;
  }
  if (b->dim == 0) {
    set_error(ctx, BLQH_ERR_ARG, "blqh_hamil_build: empty basis");
    return BLQH_ERR_ARG;
  }
  if (b->dim >= (1LL << 27)) {
    set_error(ctx, BLQH_ERR_UNSUPPORTED, "blqh_hamil_build: more than 2^27 rows");
    return BLQH_ERR_UNSUPPORTED;
  }
  blqh_csr* M = new blqh_csr();
  M->ctx = ctx;
  try {
    cudaSetDevice(ctx->device);
    hamil_build_impl(ctx, b, *p, prec, M);
  } catch (const BlqhError& e) {
    free_csr(M);
    return e.code;
  }
  *out = M;
  return BLQH_OK;
}

int blqh_csr_info(const blqh_csr* m, int64_t* dim, int64_t* nnz, int* is_complex, int* prec) {
  if (!m) return BLQH_ERR_ARG;
  if (dim) *dim = m->dim;
  if (nnz) *nnz = m->nnz;
  if (is_complex) *is_complex = m->is_complex;
  if (prec) *prec = m->precision;
  return BLQH_OK;
}

int blqh_csr_get(blqh_ctx* ctx, const blqh_csr* m, int64_t* row_ptr, int32_t* col, double* val) {
  if (!ctx || !m) return BLQH_ERR_ARG;
  try {
    if (row_ptr)
      BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(row_ptr, m->d_row_ptr, (m->dim + 1) * 8, cudaMemcpyDeviceToHost, ctx->stream));
    if (col) BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(col, m->d_col, m->nnz * 4, cudaMemcpyDeviceToHost, ctx->stream));
    if (val) {
      const int64_t n = m->nnz * (m->is_complex ? 2 : 1);
      if (m->precision == BLQH_VAL_FP64) {
        BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(val, m->d_val, n * 8, cudaMemcpyDeviceToHost, ctx->stream));
      } else {
        std::vector<float> f(n);
        BLQH_TRY_CUDA(ctx, cudaMemcpyAsync(f.data(), m->d_val, n * 4, cudaMemcpyDeviceToHost, ctx->stream));
        BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        for (int64_t i = 0; i < n; i++) val[i] = f[i];
      }
    }
    BLQH_TRY_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
  } catch (const BlqhError& e) {
    return e.code;
  }
  return BLQH_OK;
}

int blqh_csr_destroy(blqh_csr* m) {
  free_csr(m);
  return BLQH_OK;
}

}  // extern "C"
