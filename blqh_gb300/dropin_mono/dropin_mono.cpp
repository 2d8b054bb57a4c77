// Implementation of the monolayer drop-in classes over the C ABI of libblqh_gpu.so.
// Errors of the library are raised as std::runtime_error.
#include <cstdio>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/blqh_gpu.h"
#include "../dropin/saveload.h"
#include "../dropin/tridiag.h"
#include "basis.h"
#include "hamiltonian.h"
#include "lanczos_hamiltonian.h"

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

double env_tol() {
  const char* t = getenv("BLQH_TOL");
  return t ? atof(t) : 1e-12;
}

// lanczos_hamiltonian.cpp:53-56
double coulomb_q(int kx, int ky, double lx, double ly, long nLL) {
  const double q = std::sqrt(kx * kx / (lx * lx) + ky * ky / (ly * ly)) * 2.0 * M_PI;
  return 2.0 * M_PI / (q + 1e-30) * std::exp(-q * q / 2.0) * std::pow(1.0 - std::exp(-q * q / 2.0), nLL * 2);
}

void tables(long nphi, double lx, double ly, long nLL, vector<double>& V, double& E_cl) {
  V.assign(nphi * nphi, 0.0);
  check(blqh_mono_coulomb_table((int)nphi, lx, ly, (int)nLL, V.data()), "init_Coulomb_matrix");
  check(blqh_mono_classical_energy((int)nphi, lx, ly, &E_cl), "init_Coulomb_matrix");
}

}  // namespace

// ---------------------------------------------------------------------------
// basis
basis::basis() {}
basis::basis(long _nphi, long _nel) : nphi(_nphi), nel(_nel), J(-1), K(-1) {}
basis::basis(long _nphi, long _nel, long _J, long _K) : nphi(_nphi), nel(_nel), J(_J), K(_K) {}
basis::~basis() {}

const basis& basis::operator=(const basis& o) {
  if (this != &o) {
    nphi = o.nphi;
    nel = o.nel;
    C = o.C;
    J = o.J;
    K = o.K;
    nbasis = o.nbasis;
    basis_set = o.basis_set;
    id = o.id;
    popcount_table = o.popcount_table;
    basis_C = o.basis_C;
    device = o.device;
  }
  return *this;
}

unsigned long basis::factorial(long N, long m) {
  unsigned long num = 1, den = 1;
  for (long i = N - m + 1; i <= N; i++) num *= i;
  for (long i = 1; i <= m; i++) den *= i;
  return num / den;
}

long basis::common_divisor(long n, long m) {
  long r = 1;
  for (long i = 1; i <= n; i++)
    if (n % i == 0 && m % i == 0) r = i;
  return r;
}

void basis::init() {
  C = common_divisor(nel, nphi);
  blqh_sector_mono s = {(int)nphi, (int)nel, (int)J, (int)K, BLQH_REP_REFERENCE};
  blqh_basis* b = nullptr;
  check(blqh_basis_build_mono(ctx(), &s, &b), "basis::init");
  device = std::shared_ptr<blqh_basis>(b, [](blqh_basis* q) { blqh_basis_destroy(q); });
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
  for (long i = 0; i < nbasis; i++) basis_set[id[i]] = i;
  popcount_table.assign(1UL << nphi, 0);
  for (unsigned long i = 0; i < (1UL << nphi); i++) popcount_table[i] = __builtin_popcountl(i);
}

void basis::init(long _nphi, long _nel) {
  nphi = _nphi;
  nel = _nel;
  J = K = -1;
  init();
}

void basis::init(long _nphi, long _nel, long _J, long _K) {
  nphi = _nphi;
  nel = _nel;
  J = _J;
  K = _K;
  init();
}

long basis::onsite_potential(long i, long n) { return (id[i] >> n) & 1UL; }

long basis::creation(long s, long n) { return (s >> n) & 1L ? s : s + (1L << n); }

long basis::annihilation(long s, long n) { return (s >> n) & 1L ? s - (1L << n) : s; }

// basis.cpp:152-174: electrons of c ^ {n, m} strictly between n and nt and
// between m and mt, plus one for a crossing.
int basis::get_sign(long c, long n, long m, long nt, long mt) {
  const unsigned long b = (unsigned long)c ^ ((1UL << n) | (1UL << m));
  int ns = 0;
  for (long k = std::min(n, nt) + 1; k < std::max(n, nt); k++) ns += (b >> k) & 1;
  for (long k = std::min(m, mt) + 1; k < std::max(m, mt); k++) ns += (b >> k) & 1;
  if ((nt > mt && m > n) || (mt > nt && m < n)) ns++;
  return ns % 2 ? -1 : 1;
}

// basis.cpp:263-289: rotation by k nphi / C orbitals; ncross electrons wrap and
// the sign is (-1)^{ncross (nel - ncross)}.
unsigned long basis::translate(unsigned long c, int k, int& sign, int& ncross) {
  const int bits = (int)(k * nphi / C), rev = (int)nphi - bits;
  const unsigned long mask = (1UL << nphi) - 1, ms = (1UL << bits) - 1;
  c &= mask;
  ncross = __builtin_popcountl((ms << rev) & c);
  sign = (ncross * (nel - ncross)) % 2 == 0 ? 1 : -1;
  return ((c << bits) | (c >> rev)) & mask;
}

unsigned long basis::inv_translate(unsigned long c, int k, int& sign, int& ncross) {
  const int bits = (int)(k * nphi / C), rev = (int)nphi - bits;
  const unsigned long mask = (1UL << nphi) - 1, ms = (1UL << bits) - 1;
  c &= mask;
  ncross = __builtin_popcountl(ms & c);
  sign = (ncross * (nel - ncross)) % 2 == 0 ? 1 : -1;
  return ((c >> bits) | (c << rev)) & mask;
}

void basis::prlong() {
  cout << "---------------------------------------" << endl;
  for (long i = 0; i < nbasis; i++) {
    for (long n = 0; n < nphi; n++)
      if ((id[i] >> n) & 1) cout << n << " ";
    cout << "   " << bitset<20>(id[i]).to_string() << " " << setw(6) << id[i] << " " << i << endl;
  }
  cout << "---------------------------------------" << endl;
  cout << "No. basis: " << setw(6) << nbasis << endl;
}

void basis::clear() {
  basis_set.clear();
  id.clear();
  basis_C.clear();
  popcount_table.clear();
  device.reset();
  nbasis = 0;
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
    norm = o.norm;
    overlap = o.overlap;
    psir_0 = o.psir_0;
    psi_0 = o.psi_0;
    psi_n0 = o.psi_n0;
    eigenvalues = o.eigenvalues;
    csr_ = o.csr_;
    lz_ = o.lz_;
  }
  return *this;
}

void lhamil::clear() {
  H.clear();
  psir_0.clear();
  psi_n0.clear();
  psi_0.clear();
  eigenvalues.clear();
  Coulomb_matrix.clear();
  norm.clear();
  overlap.clear();
  csr_.reset();
  lz_.reset();
}

double lhamil::Coulomb_interaction(int q_x, int q_y) { return coulomb_q(q_x, q_y, lx, ly, nLL); }

void lhamil::init_Coulomb_matrix() { tables(nphi, lx, ly, nLL, Coulomb_matrix, E_cl); }

void lhamil::set_hamil(basis& sector, double _lx, double _ly, long _nphi, long _nLL) {
  lx = _lx;
  ly = _ly;
  nphi = _nphi;
  nLL = _nLL;
  init_Coulomb_matrix();
  if (!sector.device) sector.init();
  nHilbert = sector.nbasis;
  blqh_params_mono p = {lx, ly, (int)nLL};
  blqh_csr* m = nullptr;
  check(blqh_hamil_build_mono(ctx(), sector.device.get(), &p, &m), "lhamil::set_hamil");
  csr_ = std::shared_ptr<blqh_csr>(m, [](blqh_csr* q) { blqh_csr_destroy(q); });
  lz_.reset();
  psir_0.clear();
  eigenvalues.clear();
  norm.clear();
  overlap.clear();
}

void lhamil::coeff_update() { coeff_explicit_update(); }

void lhamil::coeff_explicit_update() {
  if (!csr_) throw std::runtime_error("lhamil::coeff_explicit_update: call set_hamil first");
  const long steps_max = lambda < nHilbert ? lambda : nHilbert;
  blqh_lanczos_opts o = {(int)steps_max, 1, tol_ >= 0 ? tol_ : env_tol(), 10, seed, 0, 0};
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
  std::vector<double> ev;
  if (!tridiag_first_row(overlap.data(), norm.data(), (int)m, ev, psi_n0)) psi_n0.assign(m, 0.0);
}

// lanczos_hamiltonian.cpp:362-385 with l: the leading l x l block of the tridiagonal.
void lhamil::diag(int l) {
  if (overlap.empty()) coeff_explicit_update();
  const int m = std::min<int>(l, (int)overlap.size());
  std::vector<double> ev, first;
  if (!tridiag_first_row(overlap.data(), norm.data(), m, ev, first)) throw std::runtime_error("lhamil::diag");
  eigenvalues = ev;
  psi_n0 = first;
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
  for (int64_t i = 0; i < dim; i++)
    psir_0[i] = cplx ? complex<double>(v[2 * i], v[2 * i + 1]) : complex<double>(v[i], 0);
}

double lhamil::ground_state_energy() {
  if (psir_0.empty() || !lz_) return 0;
  double e = 0;
  check(blqh_lanczos_rayleigh(lz_.get(), &e), "lhamil::ground_state_energy");
  return e;
}

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

void lhamil::save_to_file(const char* filename) { lanczos_save(*this, filename); }
void lhamil::read_from_file(const char* filename) { lanczos_read(*this, filename); }

// ---------------------------------------------------------------------------
// hamil (dense ED replaced by a Lanczos run to the end of its Krylov space)
hamil::hamil() {}
hamil::~hamil() { delete[] hamiltonian; }

const hamil& hamil::operator=(const hamil& o) {
  if (this != &o) {
    nHilbert = o.nHilbert;
    nLL = o.nLL;
    nphi = o.nphi;
    lx = o.lx;
    ly = o.ly;
    E_cl = o.E_cl;
    Coulomb_matrix = o.Coulomb_matrix;
    eigenvalues = o.eigenvalues;
    psi_0 = o.psi_0;
    psi_n0 = o.psi_n0;
    delete[] hamiltonian;
    hamiltonian = nullptr;
    if (o.hamiltonian) {
      hamiltonian = new complex<double>[nHilbert * nHilbert];
      std::copy(o.hamiltonian, o.hamiltonian + nHilbert * nHilbert, hamiltonian);
    }
    lz_ = o.lz_;
  }
  return *this;
}

double hamil::Coulomb_interaction(int q_x, int q_y) { return coulomb_q(q_x, q_y, lx, ly, nLL); }

void hamil::init_Coulomb_matrix() { tables(nphi, lx, ly, nLL, Coulomb_matrix, E_cl); }

void hamil::set_hamil(basis sector, double _lx, double _ly, int _nphi, int _nLL) {
  lx = _lx;
  ly = _ly;
  nphi = _nphi;
  nLL = _nLL;
  init_Coulomb_matrix();
  if (!sector.device) sector.init();
  nHilbert = sector.nbasis;
  lz_.seed = 1;
  lz_.lambda = nHilbert < 4096 ? nHilbert : 4096;
  lz_.tol_ = 0;  // every level the Krylov space holds, converged
  lz_.set_hamil(sector, lx, ly, nphi, nLL);
  // the dense array of the reference (row-major nHilbert x nHilbert), from the GPU CSR
  delete[] hamiltonian;
  hamiltonian = nullptr;
  int64_t dim = 0, nnz = 0;
  int cplx = 0, prec = 0;
  const blqh_csr* m = lz_.device_hamiltonian().get();
  blqh_csr_info(m, &dim, &nnz, &cplx, &prec);
  std::vector<int64_t> rp(dim + 1);
  std::vector<int32_t> col(nnz);
  std::vector<double> val(nnz * (cplx ? 2 : 1));
  check(blqh_csr_get(ctx(), m, rp.data(), col.data(), val.data()), "hamil::set_hamil");
  hamiltonian = new complex<double>[dim * dim]();
  for (int64_t i = 0; i < dim; i++)
    for (int64_t k = rp[i]; k < rp[i + 1]; k++)
      hamiltonian[i * dim + col[k]] = cplx ? complex<double>(val[2 * k], val[2 * k + 1]) : complex<double>(val[k], 0);
}

void hamil::diag() {
  lz_.coeff_explicit_update();
  lz_.diag();
  lz_.eigenstates_reconstruction();
  eigenvalues = lz_.eigenvalues;
  psi_0 = lz_.psir_0;
  psi_n0.assign(lz_.psi_n0.begin(), lz_.psi_n0.end());
}

double hamil::ground_state_energy() {
  if (psi_0.empty()) return 0;
  return lz_.ground_state_energy();
}

void hamil::print_hamil(int range) {
  if (range > nHilbert) range = nHilbert;
  for (int i = 0; i < range; i++) {
    cout << (i == 0 ? "[[" : " [");
    for (int j = 0; j < range; j++) cout << (hamiltonian ? hamiltonian[i * nHilbert + j] : complex<double>(0)) << ",";
    cout << (i == range - 1 ? "]]" : "]") << endl;
  }
}

void hamil::print_eigen(int range) { lz_.print_eigen(range); }
