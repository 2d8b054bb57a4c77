// Implementation of the spinful drop-in classes over the C ABI of libblqh_gpu.so.
// Errors of the library are raised as std::runtime_error.
#include <cstdio>
#include <mutex>
#include <stdexcept>
#include <string>

#include "../../include/blqh_gpu.h"
#include "basis.h"
#include "hamiltonian.h"
#include "lanczos_hamiltonian.h"
#include "../dropin/saveload.h"
#include "../dropin/tridiag.h"

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

double env_tol() {
  const char* t = getenv("BLQH_TOL");
  return t ? atof(t) : 1e-12;
}

}  // namespace

// ---------------------------------------------------------------------------
// basis
basis::basis() {}
basis::basis(const int& _nphi, const int& _nel) : nphi(_nphi), nel(_nel) {}
basis::basis(const int& _nphi, const int& _nel, const int& _J, const int& _K) : nphi(_nphi), nel(_nel), K(_K), J(_J) {}
basis::basis(const int& _nphi, const int& _nel, const int& _nel_up, const int& _J, const int& _K)
    : nphi(_nphi), nel(_nel), nel_up(_nel_up), nel_down(_nel - _nel_up), K(_K), J(_J) {}
basis::~basis() {}

const basis& basis::operator=(const basis& o) {
  if (this != &o) {
    nphi = o.nphi;
    nel = o.nel;
    nel_up = o.nel_up;
    nel_down = o.nel_down;
    nel_su = o.nel_su;
    nel_sd = o.nel_sd;
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

unsigned long basis::factorial(const int& N, const int& m) const {
  unsigned long num = 1, den = 1;
  for (long i = N - m + 1; i <= N; i++) num *= i;
  for (long i = 1; i <= m; i++) den *= i;
  return num / den;
}

long basis::common_divisor(const int& n, const int& m) const {
  long r = 1;
  for (int i = 1; i <= n; i++)
    if (n % i == 0 && m % i == 0) r = i;
  return r;
}

void basis::init() {
  blqh_sector_spin s = {nphi, nel, nel_up, nel_su, J, K, BLQH_REP_REFERENCE};
  blqh_basis* b = nullptr;
  check(blqh_basis_build_spin(ctx(), &s, &b), "basis::init");
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
  for (unsigned long i = 0; i < (1UL << nphi); i++) popcount_table[i] = popc(i);
}

void basis::init(const int& _nphi, const int& _nel) {
  nphi = _nphi;
  nel = _nel;
  nel_up = nel_down = nel_su = nel_sd = -1;
  J = K = -1;
  init();
}

void basis::init(const int& _nphi, const int& _nel, const int& _J, const int& _K) {
  nphi = _nphi;
  nel = _nel;
  nel_up = nel_down = nel_su = nel_sd = -1;
  J = _J;
  K = _K;
  init();
}

void basis::init(const int& _nphi, const int& _nel, const int& _nel_up, const int& _J, const int& _K) {
  nphi = _nphi;
  nel = _nel;
  nel_up = _nel_up;
  nel_down = nel - nel_up;
  nel_su = nel_sd = -1;
  J = _J;
  K = _K;
  init();
}

void basis::init(const int& _nphi, const int& _nel, const int& _nel_up, const int& _nel_su, const int& _J,
                 const int& _K) {
  nphi = _nphi;
  nel = _nel;
  nel_up = _nel_up;
  nel_down = nel - nel_up;
  nel_su = _nel_su;
  nel_sd = nel - nel_su;
  J = _J;
  K = _K;
  init();
}

void basis::clear() {
  basis_set.clear();
  id.clear();
  popcount_table.clear();
  basis_C.clear();
  device.reset();
  nbasis = 0;
}

// basis.cpp:200-231: empty orbitals of c^{n,m} strictly between n and nt and
// between m and mt, plus one for a crossing.
int basis::get_sign(const unsigned long& c, const int& n, const int& m, const int& nt, const int& mt,
                    const int&) const {
  const unsigned long b = c ^ ((1UL << n) | (1UL << m));
  int ns = 0;
  for (int k = std::min(n, nt) + 1; k < std::max(n, nt); k++) ns += !((b >> k) & 1);
  for (int k = std::min(m, mt) + 1; k < std::max(m, mt); k++) ns += !((b >> k) & 1);
  if ((nt > mt && m > n) || (mt > nt && m < n)) ns++;
  return ns % 2 ? -1 : 1;
}

// basis.cpp:233-243: empty orbitals of c strictly between n and nt.
int basis::get_sign(const unsigned long& c, const int& n, const int& nt) const {
  int ns = 0;
  for (int i = n + 1; i < nt; i++) ns += !((c >> i) & 1);
  return ns % 2 ? -1 : 1;
}

int basis::get_nel(const int& a, const unsigned long& c) const {
  if (a < 0 || a > 3) return 0;
  return popc((c >> (a * nphi)) & ((1UL << nphi) - 1));
}

int basis::get_nel(const int& a, const long& i) const { return get_nel(a, (unsigned long)id[i]); }

// basis.cpp:401-477: every block rotated by k; the sign counts, per block,
// (electrons that do not wrap) x (electrons that wrap).
unsigned long basis::translate(const unsigned long& c, const int& k, int& sign) const {
  const unsigned long m = (1UL << nphi) - 1, ms = ((1UL << k) - 1) << (nphi - k);
  unsigned long out = 0;
  int ns = 0;
  for (int b = 0; b < 4; b++) {
    const unsigned long x = (c >> (b * nphi)) & m;
    const int cr = popc(x & ms);
    ns += (popc(x) - cr) * cr;
    out |= (((x << k) | (x >> (nphi - k))) & m) << (b * nphi);
  }
  sign = ns % 2 ? -1 : 1;
  return out;
}

unsigned long basis::inv_translate(const unsigned long& c, const int& k, int& sign) const {
  const unsigned long m = (1UL << nphi) - 1, ms = (1UL << k) - 1;
  unsigned long out = 0;
  int ns = 0;
  for (int b = 0; b < 4; b++) {
    const unsigned long x = (c >> (b * nphi)) & m;
    const int cr = popc(x & ms);
    ns += (popc(x) - cr) * cr;
    out |= (((x >> k) | (x << (nphi - k))) & m) << (b * nphi);
  }
  sign = ns % 2 ? -1 : 1;
  return out;
}

void basis::prlong() const {
  cout << "---------------------------------------" << endl;
  for (long i = 0; i < nbasis; i++) {
    cout << " | ";
    for (int blk = 0; blk < 4; blk++) {
      for (int n = 0; n < nphi; n++)
        if ((id[i] >> (blk * nphi + n)) & 1) cout << n << " ";
      cout << ">| ";
    }
    cout << setw(10) << id[i] << " " << i << " " << basis_C[i] << endl;
  }
  cout << "No. basis: " << setw(6) << nbasis << endl;
}

// ---------------------------------------------------------------------------
// lhamil
lhamil::lhamil() {}
lhamil::lhamil(const Mat& _H, const long& _nHilbert, const long& _lambda, const unsigned& _seed)
    : seed(_seed), nHilbert(_nHilbert), lambda(_lambda), H(_H) {}
lhamil::lhamil(const long& _lambda, const unsigned& _seed) : seed(_seed), lambda(_lambda) {}
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
    eigenvalues = o.eigenvalues;
    csr_ = o.csr_;
    lz_ = o.lz_;
    obs_ = o.obs_;
  }
  return *this;
}

void lhamil::set_hamil(const double& _lx, const double& _ly, const long& _nphi, const long& _nLL, const double& _d,
                       const double& dsas, const double& dv, const double& dz, const double& theta_b,
                       const double& theta_x, const double& theta_y, const int&) {
  lx = _lx;
  ly = _ly;
  nphi = _nphi;
  nLL = _nLL;
  d = _d;
  if (!sector.device) sector.init();
  nHilbert = sector.nbasis;
  blqh_params_spin p = {lx, ly, d, dsas, dv, dz, theta_b, theta_x, theta_y, (int)nLL};
  blqh_csr* m = nullptr;
  check(blqh_hamil_build_spin(ctx(), sector.device.get(), &p, &m), "lhamil::set_hamil");
  csr_ = std::shared_ptr<blqh_csr>(m, [](blqh_csr* q) { blqh_csr_destroy(q); });
  lz_.reset();
  psir_0.clear();
  eigenvalues.clear();
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
  obs_.clear();
  psir_0.assign(dim, 0.0);
  for (int64_t i = 0; i < dim; i++) psir_0[i] = cplx ? complex<double>(v[2 * i], v[2 * i + 1]) : complex<double>(v[i], 0);
}

double lhamil::ground_state_energy() const {
  if (psir_0.empty()) return 0;
  double e = 0;
  check(blqh_lanczos_rayleigh(lz_.get(), &e), "lhamil::ground_state_energy");
  return e;
}

double lhamil::first_excited_state_energy() const {
  return eigenvalues.size() > 1 ? eigenvalues[1] : 0;
}

// The ground-state observables (BLQH_with_spin/lanczos_hamiltonian.cpp:1217-1593)
// are evaluated on the device from the library's ground state, all at once on
// first use after eigenstates_reconstruction (blqh_lanczos_observables_spin):
// [Sz, pseudospin_Sz, upper_Sz, down_Sz, pseudospin_Sx, spinflip_tunneling,
// occupations of block 0, then block 1].
const std::vector<double>& lhamil::observables() const {
  if (obs_.empty()) {
    if (!lz_) throw std::runtime_error("lhamil: observables before eigenstates_reconstruction");
    std::vector<double> o(6 + 2 * nphi);
    check(blqh_lanczos_observables_spin(lz_.get(), sector.device.get(), o.data()), "lhamil observables");
    obs_ = o;
  }
  return obs_;
}

// :1217-1237: alpha 0 counts orbital j of block 0, any other alpha orbital j of block 1.
double lhamil::occupatation_number(const int& alpha, const int& j) const {
  return observables()[6 + (alpha == 0 ? 0 : nphi) + j];
}
double lhamil::pseudospin_Sz() const { return observables()[1]; }  // :1239-1244
double lhamil::Sz() const { return observables()[0]; }             // :1246-1251
double lhamil::upper_Sz() const { return observables()[2]; }       // :1253-1262
double lhamil::down_Sz() const { return observables()[3]; }        // :1263-1271
double lhamil::pseudospin_Sx() const { return observables()[4]; }  // :1273-1517
double lhamil::spinflip_tunneling() const { return observables()[5]; }  // :1519-1593

void lhamil::save_to_file(const char* filename) { lanczos_save(*this, filename); }
void lhamil::read_from_file(const char* filename) { lanczos_read(*this, filename); }

void lhamil::print_eigen(int range) const {
  if (range >= (int)eigenvalues.size()) range = eigenvalues.size();
  cout << "Eigenvalues:= [";
  for (int i = 0; i < range; i++) cout << eigenvalues[i] << ", ";
  cout << ",...]" << endl;
}

void lhamil::print_lhamil(int range) const {
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

// ---------------------------------------------------------------------------
// hamil (dense ED replaced by a Lanczos run to the end of its Krylov space)
hamil::hamil() {}
hamil::~hamil() {}

void hamil::set_hamil(const double& _lx, const double& _ly, const long& _nphi, const long& _nLL, const double& _d,
                      const double& dsas, const double& dv, const double& dz, const int& nthread) {
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
  lz_.set_hamil(lx, ly, nphi, nLL, d, dsas, dv, dz, 0, 0, 0, nthread);
}

void hamil::diag() {
  lz_.coeff_explicit_update();
  lz_.diag();
  lz_.eigenstates_reconstruction();
  eigenvalues = lz_.eigenvalues;
  psi_0 = lz_.psir_0;
}

double hamil::ground_state_energy() const {
  if (psi_0.empty()) return 0;
  return lz_.ground_state_energy();
}

double hamil::Sz() const { return lz_.Sz(); }
double hamil::pseudospin_Sz() const { return lz_.pseudospin_Sz(); }
void hamil::print_eigen(int range) const { lz_.print_eigen(range); }
