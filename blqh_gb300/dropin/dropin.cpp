// Implementation of the drop-in classes over the C ABI of libblqh_gpu.so.
// Errors of the library are raised as std::runtime_error (the reference has no
// error path; on success the behaviour of its main() is unchanged).
#include <cstdio>
#include <stdexcept>
#include <string>

#include "../../include/blqh_gpu.h"
#include "basis.h"
#include "hamiltonian.h"
#include "lanczos_hamiltonian.h"
#include "saveload.h"
#include "tridiag.h"
#include "matrix.h"

namespace {

blqh_ctx* ctx() {
  static blqh_ctx* c = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    const char* dev = getenv("BLQH_DEVICE");
    if (blqh_ctx_create(dev ? atoi(dev) : 0, &c) != BLQH_OK)
      throw std::runtime_error(std::string("libblqh_gpu: ") + blqh_last_error(nullptr));
  });
  return c;
}

void check(int rc, const char* what) {
  if (rc != BLQH_OK) throw std::runtime_error(std::string(what) + ": " + blqh_last_error(ctx()));
}

int popc(unsigned long x) { return __builtin_popcountl(x); }

int env_precision() {
  const char* p = getenv("BLQH_PRECISION");
  return (p && std::string(p) == "fp32") ? BLQH_VAL_FP32 : BLQH_VAL_FP64;
}

double env_tol() {
  const char* t = getenv("BLQH_TOL");
  return t ? atof(t) : 1e-12;
}

}  // namespace

// ---------------------------------------------------------------------------
// basis
basis::basis() {}
basis::basis(int _nphi, int _nel) : nphi(_nphi), nel(_nel) {}
basis::basis(int _nphi, int _nel, int _nel_up) : nphi(_nphi), nel(_nel), nel_up(_nel_up), nel_down(_nel - _nel_up) {}
basis::basis(int _nphi, int _nel, int _nel_up, int _J, int _K)
    : nphi(_nphi), nel(_nel), nel_up(_nel_up), nel_down(_nel - _nel_up), K(_K), J(_J) {}
basis::~basis() {}

const basis& basis::operator=(const basis& o) {
  if (this != &o) {
    nphi = o.nphi;
    nel = o.nel;
    nel_up = o.nel_up;
    nel_down = o.nel_down;
    nbasis = o.nbasis;
    K = o.K;
    J = o.J;
    popcount_table = o.popcount_table;
    basis_set = o.basis_set;
    id = o.id;
    basis_C = o.basis_C;
    device = o.device;
  }
  return *this;
}

unsigned long basis::factorial(int N, int m) {
  unsigned long num = 1, den = 1;
  for (long i = N - m + 1; i <= N; i++) num *= i;
  for (long i = 1; i <= m; i++) den *= i;
  return num / den;
}

long basis::common_divisor(int n, int m) {
  long g = 1;
  for (int i = 1; i <= n; i++)
    if (n % i == 0 && m % i == 0) g = i;
  return g;
}

void basis::init() {
  blqh_sector s = {nphi, nel, nel_up, J, K, BLQH_REP_REFERENCE};
  blqh_basis* b = nullptr;
  check(blqh_basis_build(ctx(), &s, &b), "basis::init");
  device = std::shared_ptr<blqh_basis>(b, [](blqh_basis* p) { blqh_basis_destroy(p); });
  int64_t dim = 0;
  blqh_basis_size(b, &dim);
  nbasis = dim;
  id.assign(dim, 0);
  basis_C.assign(dim, 0);
  if (dim) {
    std::vector<uint64_t> ids(dim);
    std::vector<int16_t> per(dim);
    check(blqh_basis_get(ctx(), b, ids.data(), per.data()), "basis::init");
    for (int64_t i = 0; i < dim; i++) {
      id[i] = ids[i];
      basis_C[i] = per[i];
    }
  }
  basis_set.clear();
  basis_set.reserve(dim);
  for (int64_t i = 0; i < dim; i++) basis_set.emplace(id[i], i);
  popcount_table.assign(1UL << nphi, 0);
  for (unsigned long p = 0; p < (1UL << nphi); p++) popcount_table[p] = popc(p);
}

void basis::init(int _nphi, int _nel) {
  nphi = _nphi;
  nel = _nel;
  nel_up = nel_down = -1;
  K = J = -1;
  init();
}

void basis::init(int _nphi, int _nel, int _nel_up) {
  nphi = _nphi;
  nel = _nel;
  nel_up = _nel_up;
  nel_down = _nel - _nel_up;
  K = J = -1;
  init();
}

void basis::init(int _nphi, int _nel, int _nel_up, int _J, int _K) {
  nphi = _nphi;
  nel = _nel;
  nel_up = _nel_up;
  nel_down = _nel - _nel_up;
  J = _J;
  K = _K;
  init();
}

void basis::clear() {
  basis_set.clear();
  id.clear();
  basis_C.clear();
  popcount_table.clear();
  device.reset();
}

int basis::get_nel_upper(long i) { return popc(id[i] & ((1UL << nphi) - 1)); }

// basis.cpp:158-185: empty orbitals of c^{n,m} strictly between n and nt and
// between m and mt, plus one for a crossing.
int basis::get_sign(unsigned long c, int n, int m, int nt, int mt, int) {
  const unsigned long b = c ^ ((1UL << n) | (1UL << m));
  int ns = 0;
  for (int k = std::min(n, nt) + 1; k < std::max(n, nt); k++) ns += ((b >> k) & 1) == 0;
  for (int k = std::min(m, mt) + 1; k < std::max(m, mt); k++) ns += ((b >> k) & 1) == 0;
  if ((nt > mt && m > n) || (mt > nt && m < n)) ns++;
  return ns % 2 == 0 ? 1 : -1;
}

int basis::get_sign(unsigned long c, int n, int nt) {
  int ns = 0;
  for (int i = n + 1; i < nt; i++) ns += ((c >> i) & 1) == 0;
  return ns % 2 == 0 ? 1 : -1;
}

// basis.cpp:292-341: each layer rotated by k; sign from the electrons that wrap.
unsigned long basis::translate(unsigned long c, int k, int& sign) {
  const unsigned long m = (1UL << nphi) - 1;
  unsigned long u = c & m, d = (c >> nphi) & m;
  const unsigned long top = k ? ((1UL << k) - 1) << (nphi - k) : 0;
  const int xu = popc(u & top), xd = popc(d & top), nu = popc(u), nd = popc(d);
  sign = (((nu - xu) * xu + (nd - xd) * xd) % 2 == 0) ? 1 : -1;
  if (k) {
    u = ((u << k) | (u >> (nphi - k))) & m;
    d = ((d << k) | (d >> (nphi - k))) & m;
  }
  return (d << nphi) | u;
}

unsigned long basis::inv_translate(unsigned long c, int k, int& sign) {
  const unsigned long m = (1UL << nphi) - 1;
  unsigned long u = c & m, d = (c >> nphi) & m;
  const unsigned long bot = (1UL << k) - 1;
  const int xu = popc(u & bot), xd = popc(d & bot), nu = popc(u), nd = popc(d);
  sign = (((nu - xu) * xu + (nd - xd) * xd) % 2 == 0) ? 1 : -1;
  if (k) {
    u = ((u >> k) | (u << (nphi - k))) & m;
    d = ((d >> k) | (d << (nphi - k))) & m;
  }
  return (d << nphi) | u;
}

void basis::prlong() {
  cout << "---------------------------------------" << endl;
  for (long i = 0; i < nbasis; i++) {
    cout << " | ";
    for (int n = 0; n < nphi; n++)
      if ((id[i] >> n) & 1) cout << n << " ";
    cout << ">| ";
    for (int n = nphi; n < 2 * nphi; n++)
      if ((id[i] >> n) & 1) cout << n - nphi << " ";
    cout << "> " << setw(6) << id[i] << " " << i << " " << basis_C[i] << endl;
  }
  cout << "---------------------------------------" << endl;
  cout << "No. basis: " << setw(6) << nbasis << endl;
}

// ---------------------------------------------------------------------------
// lhamil
lhamil::lhamil() {}
lhamil::lhamil(const Mat& _H, long _nHilbert, long _lambda, unsigned _seed)
    : seed(_seed), nHilbert(_nHilbert), lambda(_lambda), H(_H) {}
lhamil::lhamil(long _lambda, unsigned _seed) : seed(_seed), lambda(_lambda) {}
lhamil::~lhamil() {}

const lhamil& lhamil::operator=(const lhamil& o) {
  if (this != &o) {
    nHilbert = o.nHilbert;
    H = o.H;
    seed = o.seed;
    lambda = o.lambda;
    E0 = o.E0;
    sector = o.sector;
    norm = o.norm;
    overlap = o.overlap;
    psir_0 = o.psir_0;
    psi_0 = o.psi_0;
    psi_n0 = o.psi_n0;
    eigenvalues = o.eigenvalues;
    csr_ = o.csr_;
    lz_ = o.lz_;
    precision_ = o.precision_;
    for (int i = 0; i < 7; i++) params_[i] = o.params_[i];
  }
  return *this;
}

void lhamil::set_hamil(double _lx, double _ly, long _nphi, long _nLL, double _d, double dsas, double dv,
                       double theta_x, double theta_y, int) {
  lx = _lx;
  ly = _ly;
  nphi = _nphi;
  nLL = _nLL;
  d = _d;
  if (!sector.device) sector.init();
  nHilbert = sector.nbasis;
  params_[0] = lx;
  params_[1] = ly;
  params_[2] = d;
  params_[3] = dsas;
  params_[4] = dv;
  params_[5] = theta_x;
  params_[6] = theta_y;
  precision_ = env_precision();
  blqh_params p = {lx, ly, d, dsas, dv, theta_x, theta_y, (int)nLL};
  blqh_csr* m = nullptr;
  check(blqh_hamil_build(ctx(), sector.device.get(), &p, precision_, &m), "lhamil::set_hamil");
  csr_ = std::shared_ptr<blqh_csr>(m, [](blqh_csr* q) { blqh_csr_destroy(q); });
  lz_.reset();
}

void lhamil::coeff_update() { coeff_explicit_update(); }

void lhamil::coeff_explicit_update() {
  if (!csr_) throw std::runtime_error("lhamil::coeff_explicit_update: call set_hamil first");
  blqh_lanczos_opts o = {(int)lambda, 1, tol_ >= 0 ? tol_ : env_tol(), 10, seed, 0, 0};
  blqh_lanczos* l = nullptr;
  check(blqh_lanczos_create(ctx(), csr_.get(), &o, &l), "lhamil::coeff_explicit_update");
  lz_ = std::shared_ptr<blqh_lanczos>(l, [](blqh_lanczos* q) { blqh_lanczos_destroy(q); });
  int steps = 0;
  check(blqh_lanczos_iterate(l, &steps), "lhamil::coeff_explicit_update");
  overlap.assign(steps, 0.0);
  norm.assign(steps + 1, 0.0);
  check(blqh_lanczos_coeffs(l, overlap.data(), norm.data()), "lhamil::coeff_explicit_update");
}

void lhamil::diag() {
  if (!lz_) coeff_explicit_update();
  const size_t m = overlap.size();
  eigenvalues.assign(m, 0.0);
  psi_0.assign(m, 0.0);
  check(blqh_lanczos_eig(lz_.get(), eigenvalues.data(), psi_0.data()), "lhamil::diag");
  // first components of the Ritz vectors in the Krylov basis (the reference's psi_n0)
  std::vector<double> ev;
  if (!tridiag_first_row(overlap.data(), norm.data(), (int)m, ev, psi_n0)) psi_n0.assign(m, 0.0);
}

void lhamil::eigenstates_reconstruction() {
  if (eigenvalues.empty()) diag();
  E0 = eigenvalues[0];
  int64_t dim = 0, nnz = 0;
  int cplx = 0, prec = 0;
  blqh_csr_info(csr_.get(), &dim, &nnz, &cplx, &prec);
  std::vector<double> v(dim * (cplx ? 2 : 1));
  check(blqh_lanczos_ritz_vector(lz_.get(), v.data()), "lhamil::eigenstates_reconstruction");
  psir_0.assign(dim, 0.0);
  for (int64_t i = 0; i < dim; i++) psir_0[i] = cplx ? complex<double>(v[2 * i], v[2 * i + 1]) : complex<double>(v[i], 0);
}

double lhamil::ground_state_energy() {
  if (psir_0.empty()) return 0;
  double e = 0;
  const char* compat = getenv("BLQH_COMPAT_CONJ");
  if (compat && compat[0] == '1') {
    // the value the reference prints: <conj(psi)|H|conj(psi)> (lanczos_hamiltonian.cpp:610-656)
    blqh_params p = {params_[0], params_[1], params_[2], params_[3], params_[4], params_[5], params_[6], (int)nLL};
    const bool regen = precision_ != BLQH_VAL_FP64;
    check(blqh_lanczos_rayleigh_conj(lz_.get(), regen ? sector.device.get() : nullptr, regen ? &p : nullptr, &e),
          "lhamil::ground_state_energy");
    return e;
  }
  if (precision_ == BLQH_VAL_FP64) {
    check(blqh_lanczos_rayleigh(lz_.get(), &e), "lhamil::ground_state_energy");
  } else {
    blqh_params p = {params_[0], params_[1], params_[2], params_[3], params_[4], params_[5], params_[6], (int)nLL};
    check(blqh_lanczos_rayleigh_fp64(lz_.get(), sector.device.get(), &p, &e), "lhamil::ground_state_energy");
  }
  return e;
}

// lanczos_hamiltonian.cpp:658-678: <n_j> of one layer in the ground state; the
// translates of a representative share its weight equally.
double lhamil::occupatation_number(int alpha, int j) {
  const unsigned long mask = 1UL << (alpha == 0 ? j : j + nphi);
  double occ = 0;
  for (long i = 0; i < nHilbert; i++) {
    const int D = sector.K < 0 ? 1 : sector.basis_C[i];
    int hits = 0, s;
    for (int q = 0; q < D; q++) hits += (sector.translate(sector.id[i], q, s) & mask) == mask;
    occ += std::norm(psir_0[i]) * hits / D;
  }
  return occ;
}

// lanczos_hamiltonian.cpp:680-690: pseudospin S_z = (2 <N_upper> - Ne) / (2 Ne).
double lhamil::pseudospin_Sz() {
  double up = 0;
  for (long i = 0; i < nHilbert; i++) up += sector.get_nel_upper(i) * std::norm(psir_0[i]);
  return (2.0 * up - sector.nel) / (2.0 * sector.nel);
}

void lhamil::save_to_file(const char* filename) { lanczos_save(*this, filename); }
void lhamil::read_from_file(const char* filename) { lanczos_read(*this, filename); }

void lhamil::print_eigen(int range) {
  if (range >= (int)eigenvalues.size()) range = eigenvalues.size();
  cout << "Eigenvalues:= [";
  for (int i = 0; i < range; i++) cout << eigenvalues[i] << ", ";
  cout << ",...]" << endl;
}

void lhamil::print_lhamil(int range) {
  if (range >= (int)overlap.size()) range = overlap.size();
  for (int i = 0; i < range; i++) {
    cout << (i == 0 ? "[[" : " [");
    for (int j = 0; j < range; j++) {
      if (j == i + 1) cout << norm[j] << ",";
      else if (j == i - 1) cout << norm[i] << ",";
      else if (j == i) cout << overlap[i] << ",";
      else cout << 0 << ",";
    }
    cout << (i == range - 1 ? "]]" : "]") << endl;
  }
}

void lhamil::fetch_hamil() {
  int64_t dim = 0, nnz = 0;
  int cplx = 0, prec = 0;
  blqh_csr_info(csr_.get(), &dim, &nnz, &cplx, &prec);
  std::vector<int64_t> rp(dim + 1);
  std::vector<int32_t> col(nnz);
  std::vector<double> val(nnz * (cplx ? 2 : 1));
  check(blqh_csr_get(ctx(), csr_.get(), rp.data(), col.data(), val.data()), "lhamil::fetch_hamil");
  H.clear();
  H.outer_starts.resize(dim);
  H.outer_size.resize(dim);
  H.inner_indices.resize(nnz);
  H.value.resize(nnz);
  for (int64_t i = 0; i < dim; i++) {
    H.outer_starts[i] = rp[i];
    H.outer_size[i] = rp[i + 1] - rp[i];
  }
  for (int64_t k = 0; k < nnz; k++) {
    H.inner_indices[k] = col[k];
    H.value[k] = cplx ? complex<double>(val[2 * k], val[2 * k + 1]) : complex<double>(val[k], 0);
  }
}

// ---------------------------------------------------------------------------
// hamil (dense ED replaced by a Lanczos run to the end of its Krylov space)
hamil::hamil() {}
hamil::~hamil() {}

const hamil& hamil::operator=(const hamil& o) {
  if (this != &o) {
    nHilbert = o.nHilbert;
    d = o.d;
    nphi = o.nphi;
    sector = o.sector;
    eigenvalues = o.eigenvalues;
    psi_0 = o.psi_0;
    lz_ = o.lz_;
  }
  return *this;
}

void hamil::set_hamil(double _lx, double _ly, long _nphi, long _nLL, double _d, double dsas, double dv,
                      double theta_x, double theta_y, int nthread) {
  lx = _lx;
  ly = _ly;
  nphi = _nphi;
  nLL = _nLL;
  d = _d;
  if (!sector.device) sector.init();
  lz_.sector = sector;
  lz_.seed = seed;
  nHilbert = sector.nbasis;
  lz_.lambda = nHilbert < 4096 ? nHilbert : 4096;
  lz_.tol_ = 0;  // every level the Krylov space holds, converged
  lz_.set_hamil(lx, ly, nphi, nLL, d, dsas, dv, theta_x, theta_y, nthread);
}

void hamil::diag() {
  lz_.coeff_explicit_update();
  lz_.diag();
  lz_.eigenstates_reconstruction();
  eigenvalues = lz_.eigenvalues;
  psi_0 = lz_.psir_0;
}

double hamil::ground_state_energy() {
  if (psi_0.empty()) return 0;
  return lz_.ground_state_energy();
}

double hamil::pseudospin_Sz() { return lz_.pseudospin_Sz(); }

void hamil::print_eigen(int range) { lz_.print_eigen(range); }
