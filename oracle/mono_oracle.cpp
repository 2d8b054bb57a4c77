// CPU oracle for the monolayer exact-diagonalization path.
//
// TEST INFRASTRUCTURE ONLY. This file restates, in plain C++, the monolayer
// model of the reference (qiongz/BLQH, directory Monolayer) so that the tests
// and the smoke check can check the CUDA library against it. Nothing in the
// product (blqh_gb300/) links, loads or calls this code.
//
// The reference's Monolayer directory does not compile as shipped (basis.h:42-43
// declares translate / inv_translate with three parameters, basis.cpp:263 and
// :277 define them with four; the build also wants icpc, MKL and GSL), so this
// restatement is pinned to the reference's own recorded outputs instead
// (Monolayer/check: ek_nphi_18_nel_6 and gs_energy_nel{4,5,6}, turned into
// fixtures by tests/golden/make_golden_mono.py, checked by
// tests/test_mono_oracle.py).
//
// Conventions shared with the reference:
//   state bit n = orbital n, n in [0, nphi). C = gcd(nel, nphi) translations,
//   each by q = nphi / C orbitals. The sector basis keeps one member per
//   translation orbit; which member survives follows the iteration order of a
//   libstdc++ std::unordered_map filled in depth-first order
//   (Monolayer/basis.cpp:59-119). The oracle uses the same container the same way.
#include <algorithm>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <unordered_map>
#include <vector>

using cplx = std::complex<double>;

namespace {

struct MBasis {
  int nphi = 0, nel = 0, J = -1, K = -1, C = 1, q = 0;
  int rep_mode = 0;  // 0: reference survivor, 1: numerically smallest orbit member
  std::vector<uint64_t> id;
  std::vector<int16_t> period;
  std::unordered_map<uint64_t, int64_t> index;
};

inline int popc(uint64_t x) { return __builtin_popcountll(x); }

// basis.cpp:41-47 — the largest common divisor of nel and nphi.
int common_divisor(int n, int m) {
  int N = 1;
  for (int i = 1; i <= n; i++)
    if (n % i == 0 && m % i == 0) N = i;
  return N;
}

// basis.cpp:263-275 — rotate left by k q orbitals; sign (-1)^{c (nel - c)},
// c = electrons in the k q top orbitals.
uint64_t translate(const MBasis& B, uint64_t c, int k, int& sign) {
  const int bits = k * B.nphi / B.C, rev = B.nphi - bits;
  const uint64_t mask = (1ULL << B.nphi) - 1, msign = (1ULL << bits) - 1;
  c &= mask;
  const int ncross = popc((msign << rev) & c);
  sign = ((ncross * (B.nel - ncross)) % 2 == 0) ? 1 : -1;
  return ((c << bits) | (c >> rev)) & mask;
}

// basis.cpp:277-289 — rotate right by k q orbitals; c = electrons in the k q bottom orbitals.
uint64_t inv_translate(const MBasis& B, uint64_t c, int k, int& sign) {
  const int bits = k * B.nphi / B.C, rev = B.nphi - bits;
  const uint64_t mask = (1ULL << B.nphi) - 1, msign = (1ULL << bits) - 1;
  c &= mask;
  const int ncross = popc(msign & c);
  sign = ((ncross * (B.nel - ncross)) % 2 == 0) ? 1 : -1;
  return ((c >> bits) | (c << rev)) & mask;
}

// basis.cpp:152-174 — fermion sign of moving n -> nt and m -> mt: the
// electrons of c ^ {n, m} strictly between n and nt and strictly between m and
// mt, plus one when the pair crosses.
int get_sign(uint64_t c, int n, int m, int nt, int mt) {
  const uint64_t b = c ^ ((1ULL << n) | (1ULL << m));
  int ns = 0;
  for (int k = std::min(n, nt) + 1; k < std::max(n, nt); k++) ns += (b >> k) & 1;
  for (int k = std::min(m, mt) + 1; k < std::max(m, mt); k++) ns += (b >> k) & 1;
  if ((nt > mt && m > n) || (mt > nt && m < n)) ns++;
  return (ns % 2 == 0) ? 1 : -1;
}

// basis.cpp:216-235 — depth-first enumeration of the nel-subsets of [0, nphi),
// inserting those of momentum J (sum of orbitals mod nphi).
void dfs(MBasis& B, int count, int j, long Ji, uint64_t config, std::unordered_map<uint64_t, int64_t>& set) {
  count++;
  config = (count == 1 ? 0 : config);
  j = (count == 1 ? 0 : j + 1);
  for (int i = j; i < B.nphi - (B.nel - count); i++) {
    const long k = Ji + i;
    const uint64_t c = config + (1ULL << i);
    if (count < B.nel) dfs(B, count, i, k, c, set);
    else if (B.J < 0 || k % B.nphi == B.J) set[c] = (int64_t)c;
  }
}

// basis.cpp:59-119 — build the sector basis.
void basis_init(MBasis& B) {
  B.C = common_divisor(B.nel, B.nphi);
  B.q = B.nphi / B.C;
  std::unordered_map<uint64_t, int64_t> set;
  dfs(B, 0, 0, 0, 0, set);
  const uint64_t mask = (1ULL << B.nphi) - 1;
  if (B.K >= 0) {
    if (B.rep_mode == 0) {
      // basis.cpp:70-89: erase while iterating every state with another orbit member still present.
      for (auto it = set.begin(); it != set.end();) {
        const uint64_t c = it->first & mask;
        bool drop = false;
        for (int n = 1; n < B.C; n++) {
          const int sh = B.q * n;
          const uint64_t cf = ((c >> sh) | (c << (B.nphi - sh))) & mask;
          if (set.find(cf) != set.end() && cf != c) { drop = true; break; }
        }
        if (drop) it = set.erase(it);
        else ++it;
      }
    } else {
      std::vector<uint64_t> keep;
      for (auto& kv : set) {
        const uint64_t c = kv.first;
        bool drop = false;
        for (int n = 1; n < B.C; n++) {
          const int sh = B.q * n;
          const uint64_t cf = ((c >> sh) | (c << (B.nphi - sh))) & mask;
          if (cf < c && set.find(cf) != set.end()) { drop = true; break; }
        }
        if (!drop) keep.push_back(c);
      }
      set.clear();
      for (uint64_t c : keep) set[c] = (int64_t)c;
    }
  }
  for (auto& kv : set) B.id.push_back(kv.second);
  std::sort(B.id.begin(), B.id.end());
  for (size_t i = 0; i < B.id.size(); i++) B.index[B.id[i]] = (int64_t)i;
  // basis.cpp:110-118: basis_C = smallest n in [1, C) with translate(id, n) == id, else C.
  int sign;
  B.period.assign(B.id.size(), (int16_t)B.C);
  for (size_t i = 0; i < B.id.size(); i++)
    for (int n = 1; n < B.C; n++)
      if (translate(B, B.id[i], n, sign) == B.id[i]) { B.period[i] = (int16_t)n; break; }
}

// lanczos_hamiltonian.cpp:53-56 — Fourier transform of the Coulomb interaction.
double coulomb_q(int kx, int ky, double lx, double ly, int nLL) {
  const double q = std::sqrt(kx * kx / (lx * lx) + ky * ky / (ly * ly)) * 2.0 * M_PI;
  return 2.0 * M_PI / (q + 1e-30) * std::exp(-q * q / 2.0) * std::pow(1.0 - std::exp(-q * q / 2.0), nLL * 2);
}

// lanczos_hamiltonian.cpp:58-67 — V[s][ky] = sum over kx in [-nphi/2, nphi/2], (kx, ky) != 0,
// of V(kx, ky) cos(2 pi s kx / nphi) / (2 lx ly).
void coulomb_table(int nphi, double lx, double ly, int nLL, std::vector<double>& V) {
  V.assign((size_t)nphi * nphi, 0.0);
  for (int s = 0; s < nphi; s++)
    for (int ky = 0; ky < nphi; ky++) {
      double v = 0;
      for (int kx = -nphi / 2; kx <= nphi / 2; kx++)
        if (!(ky == 0 && kx == 0)) v += coulomb_q(kx, ky, lx, ly, nLL) * std::cos(2.0 * M_PI * s * kx / nphi) / (2.0 * lx * ly);
      V[(size_t)s * nphi + ky] = v;
    }
}

// lanczos_hamiltonian.cpp:68-74 with matrix.cpp:320-336 — classical energy
// E_cl = (-2 + sum_{(i, j) != 0} I(z_ij)) / sqrt(lx ly), z_ij = pi (i^2 lx / ly + j^2 ly / lx),
// I(z) = integral_1^inf t^{-1/2} e^{-z t} dt. The reference evaluates I by GSL's
// adaptive quadrature (gsl_integration_qagiu, tolerance 1e-6); substituting
// u = z t gives I(z) = z^{-1/2} Gamma(1/2, z) = sqrt(pi / z) erfc(sqrt(z)),
// evaluated here in closed form.
double classical_energy(int nphi, double lx, double ly) {
  double E = -2.0;
  for (int i = 0; i < nphi; i++)
    for (int j = 0; j < nphi; j++)
      if (!(i == 0 && j == 0)) {
        const double z = (i * i * lx / ly + j * j * ly / lx) * M_PI;
        E += std::sqrt(M_PI / z) * std::erfc(std::sqrt(z));
      }
  return E / std::sqrt(lx * ly);
}

struct MHamil {
  std::vector<int64_t> row_ptr;
  std::vector<int64_t> col;
  std::vector<cplx> val;
  double E_cl = 0;
};

// lanczos_hamiltonian.cpp:77-198 — one row. acc is a dense scratch row (zero on
// entry and on exit); the += sequence per column is the reference's.
void build_row(const MBasis& B, const std::vector<double>& V, double E_cl, int64_t i, std::vector<cplx>& acc,
               std::vector<int64_t>& touched, std::vector<char>& mark, std::vector<std::pair<int64_t, cplx>>& out) {
  const int nphi = B.nphi, kx = B.K;
  auto add = [&](int64_t j, cplx v) {
    if (!mark[j]) { mark[j] = 1; touched.push_back(j); }
    acc[j] += v;
  };
  const int Cl = kx < 0 ? 1 : B.period[i];
  for (int k1 = 0; k1 < Cl; k1++) {
    int signl = 1, sg;
    const uint64_t lb = (k1 == 0) ? B.id[i] : translate(B, B.id[i], k1, signl);
    for (int n = 0; n < nphi - 1; n++)
      for (int m = n + 1; m < nphi; m++) {
        const uint64_t mask = (1ULL << n) + (1ULL << m);
        if ((lb & mask) != mask) continue;
        const uint64_t b = lb ^ mask;
        for (int t = -nphi / 2; t <= nphi / 2; t++) {
          const int nt = n + t >= nphi ? n + t - nphi : (n + t < 0 ? n + t + nphi : n + t);
          const int mt = m - t < 0 ? m - t + nphi : (m - t >= nphi ? m - t - nphi : m - t);
          const int s = std::abs(n - mt);
          // nt == mt gives a target with nel - 1 electrons (the two masks carry
          // into one bit), which is never in the basis: no contribution.
          if (nt == mt) continue;
          const uint64_t mask_t = (1ULL << nt) + (1ULL << mt);
          if ((mask_t & b) != 0) continue;
          const uint64_t rb0 = mask_t + b;
          int Cr = B.C;
          for (int k2 = 1; k2 <= B.C; k2++)
            if (translate(B, rb0, k2, sg) == rb0) { Cr = k2; break; }
          if (kx < 0) Cr = 1;
          for (int k2 = 0; k2 < Cr; k2++) {
            int signr = 1;
            const uint64_t rb = (k2 == 0) ? rb0 : inv_translate(B, rb0, k2, signr);
            auto f = B.index.find(rb);
            if (f == B.index.end()) continue;
            const int sign = get_sign(lb, n, m, nt, mt) * signl * signr;
            const double ang = 2.0 * M_PI * kx * (k1 - k2) / B.C;
            const cplx FT = cplx(std::cos(ang), std::sin(ang)) / std::sqrt((double)(Cl * Cr));
            add(f->second, 2.0 * V[(size_t)s * nphi + std::abs(t)] * sign * FT);
          }
        }
      }
  }
  add(i, cplx(E_cl * B.nel, 0.0));
  std::sort(touched.begin(), touched.end());
  out.clear();
  for (int64_t j : touched) {
    if (std::abs(acc[j]) > 1e-10) out.emplace_back(j, acc[j]);
    acc[j] = 0;
    mark[j] = 0;
  }
  touched.clear();
}

}  // namespace

extern "C" {

void* orc_mono_basis_new(int nphi, int nel, int J, int K, int rep_mode) {
  MBasis* B = new MBasis();
  B->nphi = nphi;
  B->nel = nel;
  B->J = J;
  B->K = K;
  B->rep_mode = rep_mode;
  basis_init(*B);
  return B;
}
void orc_mono_basis_free(void* h) { delete static_cast<MBasis*>(h); }
int64_t orc_mono_basis_size(void* h) { return (int64_t) static_cast<MBasis*>(h)->id.size(); }
void orc_mono_basis_ids(void* h, uint64_t* out) {
  auto* B = static_cast<MBasis*>(h);
  std::memcpy(out, B->id.data(), B->id.size() * 8);
}
void orc_mono_basis_periods(void* h, int16_t* out) {
  auto* B = static_cast<MBasis*>(h);
  std::memcpy(out, B->period.data(), B->period.size() * 2);
}
uint64_t orc_mono_translate(void* h, uint64_t c, int k, int inverse, int* sign) {
  auto* B = static_cast<MBasis*>(h);
  return inverse ? inv_translate(*B, c, k, *sign) : translate(*B, c, k, *sign);
}
double orc_mono_classical_energy(int nphi, double lx, double ly) { return classical_energy(nphi, lx, ly); }
void orc_mono_coulomb_table(int nphi, double lx, double ly, int nLL, double* out) {
  std::vector<double> V;
  coulomb_table(nphi, lx, ly, nLL, V);
  std::memcpy(out, V.data(), V.size() * 8);
}

// Rows [row_begin, row_end) of the Hamiltonian (row_end < 0: to the last row).
void* orc_mono_hamil_new(void* basis, double lx, double ly, int nLL, int nthreads, int64_t row_begin,
                         int64_t row_end) {
  auto* B = static_cast<MBasis*>(basis);
  MHamil* H = new MHamil();
  std::vector<double> V;
  coulomb_table(B->nphi, lx, ly, nLL, V);
  H->E_cl = classical_energy(B->nphi, lx, ly);
  const int64_t dim = (int64_t)B->id.size();
  if (row_end < 0 || row_end > dim) row_end = dim;
  if (row_begin < 0) row_begin = 0;
  const int64_t nrows = row_end > row_begin ? row_end - row_begin : 0;
  std::vector<std::vector<std::pair<int64_t, cplx>>> rows(nrows);
  if (nthreads < 1) nthreads = 1;
#pragma omp parallel num_threads(nthreads)
  {
    std::vector<cplx> acc(dim, 0.0);
    std::vector<char> mark(dim, 0);
    std::vector<int64_t> touched;
#pragma omp for schedule(dynamic, 16)
    for (int64_t r = 0; r < nrows; r++) build_row(*B, V, H->E_cl, row_begin + r, acc, touched, mark, rows[r]);
  }
  H->row_ptr.assign(nrows + 1, 0);
  for (int64_t r = 0; r < nrows; r++) H->row_ptr[r + 1] = H->row_ptr[r] + (int64_t)rows[r].size();
  H->col.resize(H->row_ptr[nrows]);
  H->val.resize(H->row_ptr[nrows]);
  for (int64_t r = 0; r < nrows; r++) {
    int64_t o = H->row_ptr[r];
    for (auto& e : rows[r]) { H->col[o] = e.first; H->val[o] = e.second; o++; }
  }
  return H;
}
void orc_mono_hamil_free(void* h) { delete static_cast<MHamil*>(h); }
int64_t orc_mono_hamil_nnz(void* h) { return (int64_t) static_cast<MHamil*>(h)->col.size(); }
int64_t orc_mono_hamil_rows(void* h) { return (int64_t) static_cast<MHamil*>(h)->row_ptr.size() - 1; }

// y = H x over the rows the handle holds (Mat::operator*, matrix.cpp), complex.
void orc_mono_spmv(void* h, const double* x, double* y, int nthreads) {
  auto* H = static_cast<MHamil*>(h);
  const cplx* xc = reinterpret_cast<const cplx*>(x);
  cplx* yc = reinterpret_cast<cplx*>(y);
  const int64_t n = (int64_t)H->row_ptr.size() - 1;
#pragma omp parallel for schedule(static) num_threads(nthreads < 1 ? 1 : nthreads)
  for (int64_t i = 0; i < n; i++) {
    cplx s = 0;
    for (int64_t k = H->row_ptr[i]; k < H->row_ptr[i + 1]; k++) s += H->val[k] * xc[H->col[k]];
    yc[i] = s;
  }
}

void orc_mono_hamil_csr(void* h, int64_t* row_ptr, int64_t* col, double* val) {
  auto* H = static_cast<MHamil*>(h);
  std::memcpy(row_ptr, H->row_ptr.data(), H->row_ptr.size() * 8);
  std::memcpy(col, H->col.data(), H->col.size() * 8);
  std::memcpy(val, H->val.data(), H->val.size() * 16);
}

}  // extern "C"
