// Drop-in lanczos_hamiltonian.h for the monolayer: the reference's Lanczos
// Hamiltonian class (Monolayer/lanczos_hamiltonian.h:6-63) computed by
// libblqh_gpu.so. set_hamil builds the monolayer CSR on the GPU
// (blqh_hamil_build_mono, FP64 values) and fills Coulomb_matrix and E_cl;
// coeff_update / coeff_explicit_update run the Lanczos recurrence on the GPU
// with full FP64 reorthogonalization (stopping when the lowest Ritz value moves
// less than BLQH_TOL, default 1e-12, between checks, or after lambda steps, or
// when the Krylov space is exhausted); diag, eigenstates_reconstruction and
// ground_state_energy follow as in the bilayer drop-ins. psir_0 holds the ground
// state itself. Gram_Schmidt_orthogonalization, coeff_update_wopt and
// spectral_function are not provided.
// Environment: BLQH_DEVICE (default 0), BLQH_TOL (default 1e-12).
#ifndef BLQH_DROPIN_MONO_LANCZOS_HAMILTONIAN_H
#define BLQH_DROPIN_MONO_LANCZOS_HAMILTONIAN_H
#include <memory>

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
  long nphi = 0, nLL = 0;
  long off_head = 0;
  double lx = 0, ly = 0, E0 = 0, E_cl = 0;
  vector<double> Coulomb_matrix;  // [s * nphi + q_y]
  Mat H;
  std::vector<double> norm;
  std::vector<double> overlap;
  std::vector<complex<double> > psir_0;
  std::vector<double> psi_0;
  std::vector<double> psi_n0;
  std::vector<double> eigenvalues;

  lhamil();
  lhamil(const Mat& _H, long _nHilbert, long _lambda, unsigned _seed);
  lhamil(long _lambda, unsigned _seed);
  ~lhamil();
  const lhamil& operator=(const lhamil&);
  void clear();
  void set_hamil(basis& _sector, double _lx, double _ly, long _nphi, long nLL);
  void coeff_update();
  void coeff_explicit_update();
  void diag();
  void diag(int l);  // eigenvalues of the leading l x l block of the tridiagonal
  void eigenstates_reconstruction();
  double Coulomb_interaction(int q_x, int q_y);
  double ground_state_energy();
  void init_Coulomb_matrix();
  void print_lhamil(int n);
  void print_eigen(int n);
  void save_to_file(const char* filename);  //!< the reference's checkpoint text format
  void read_from_file(const char* filename);
  std::shared_ptr<blqh_csr> device_hamiltonian() const { return csr_; }  //!< the GPU CSR (null before set_hamil)

 private:
  friend class hamil;
  double tol_ = -1;  // >= 0: convergence tolerance instead of BLQH_TOL (0: run to lambda or breakdown)
  std::shared_ptr<blqh_csr> csr_;
  std::shared_ptr<blqh_lanczos> lz_;
};

#endif
