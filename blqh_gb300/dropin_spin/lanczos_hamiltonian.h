// Drop-in lanczos_hamiltonian.h for the spinful model: the reference's Lanczos
// Hamiltonian class (BLQH_with_spin/lanczos_hamiltonian.h:12-79) computed by
// libblqh_gpu.so: set_hamil builds the spinful CSR on the GPU
// (blqh_hamil_build_spin, FP64 values; nthread is ignored), the Lanczos pass,
// tridiagonal solve, ground state and energy run on the GPU as in the spinless
// drop-in. Sz, pseudospin_Sz, upper_Sz, down_Sz, pseudospin_Sx,
// spinflip_tunneling and occupatation_number are evaluated on the GPU from the
// ground state (blqh_lanczos_observables_spin); pseudospin_Chi and
// spectral_function are not provided.
// Environment: BLQH_DEVICE (default 0), BLQH_TOL (default 1e-12).
#ifndef BLQH_DROPIN_SPIN_LANCZOS_HAMILTONIAN_H
#define BLQH_DROPIN_SPIN_LANCZOS_HAMILTONIAN_H
#include <memory>
#include <mutex>
#include <thread>

#include "basis.h"
#include "matrix.h"

void swap(Vec* a, Vec* b, Vec* c);

struct blqh_csr;
struct blqh_lanczos;

class lhamil {
 public:
  unsigned seed = 0;
  long nHilbert = 0;
  long lambda = 200;
  long nLL = 0, nphi = 0;
  double lx = 0, ly = 0, d = 0;
  double E0 = 0, Ec = 0;
  vector<double> Coulomb_matrix;
  vector<complex<double> > FT;
  basis sector;
  Mat H;
  std::vector<double> norm;
  std::vector<double> overlap;
  std::vector<complex<double> > psir_0;
  std::vector<complex<double> > psir_1;
  std::vector<double> psi_0;
  std::vector<double> psi_1;
  std::vector<double> psi_n0;
  std::vector<double> eigenvalues;

  lhamil();
  lhamil(const Mat& _H, const long& _nHilbert, const long& _lambda, const unsigned& _seed);
  lhamil(const long& _lambda, const unsigned& _seed);
  ~lhamil();
  const lhamil& operator=(const lhamil&);
  void set_hamil(const double& _lx, const double& _ly, const long& _nphi, const long& _nLL, const double& _d,
                 const double& _Delta_SAS, const double& _Delta_V, const double& _Delta_Z, const double& _theta_B,
                 const double& theta_x, const double& theta_y, const int& nthread);
  void coeff_update();
  void coeff_explicit_update();
  void diag();
  void eigenstates_reconstruction();
  double ground_state_energy() const;
  double first_excited_state_energy() const;
  double occupatation_number(const int& alpha, const int& j) const;
  double pseudospin_Sz() const;
  double Sz() const;
  double upper_Sz() const;
  double down_Sz() const;
  double pseudospin_Sx() const;
  double spinflip_tunneling() const;
  void save_to_file(const char* filename);  //!< the reference's checkpoint text format
  void read_from_file(const char* filename);
  void print_eigen(int n) const;
  void print_lhamil(int n) const;

 private:
  friend class hamil;
  double tol_ = -1;  // >= 0: convergence tolerance instead of BLQH_TOL (0: run to lambda or breakdown)
  const std::vector<double>& observables() const;
  mutable std::vector<double> obs_;
  std::shared_ptr<blqh_csr> csr_;
  std::shared_ptr<blqh_lanczos> lz_;
};

#endif
