// Drop-in lanczos_hamiltonian.h: the reference's Lanczos Hamiltonian class
// (BLQH_without_spin/lanczos_hamiltonian.h:11-75) with the same public members
// and methods, computed by libblqh_gpu.so:
//   set_hamil              -> CSR built on the GPU (blqh_hamil_build); nthread is ignored
//   coeff_explicit_update  -> Lanczos pass 1 on the GPU with full FP64 reorthogonalization,
//                             stopping at convergence or an invariant subspace (<= lambda steps)
//   diag                   -> tridiagonal eigensolve on the GPU
//   eigenstates_reconstruction -> ground state from the stored Krylov basis (not conjugated)
//   ground_state_energy    -> <psi|H|psi>
// Environment: BLQH_DEVICE (default 0), BLQH_PRECISION=fp32 for FP32 CSR values with the
// FP64 regenerated Rayleigh quotient, BLQH_TOL (default 1e-12).
#ifndef BLQH_DROPIN_LANCZOS_HAMILTONIAN_H
#define BLQH_DROPIN_LANCZOS_HAMILTONIAN_H
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
  unsigned seed = 0;   //!< Seed for RNGs
  long nHilbert = 0;   //!< Hilbert space size
  long lambda = 200;   //!< Lanczos update steps (upper bound)
  long nLL = 0, nphi = 0;
  double lx = 0, ly = 0, d = 0;
  double E0 = 0, Ec = 0;
  vector<double> Coulomb_matrix;
  vector<complex<double> > FT;
  basis sector;
  Mat H;  //!< host copy of the CSR, filled only by fetch_hamil()
  std::vector<double> norm;
  std::vector<double> overlap;
  std::vector<complex<double> > psir_0;
  std::vector<complex<double> > psir_1;
  std::vector<double> psi_0;
  std::vector<double> psi_1;
  std::vector<double> psi_n0;
  std::vector<double> eigenvalues;

  lhamil();
  lhamil(const Mat& _H, long _nHilbert, long _lambda, unsigned _seed);
  lhamil(long _lambda, unsigned _seed);
  ~lhamil();
  const lhamil& operator=(const lhamil&);
  void set_hamil(double _lx, double _ly, long _nphi, long _nLL, double _d, double _Delta_SAS, double _Delta_V,
                 double theta_x, double theta_y, int nthread);
  void coeff_update();
  void coeff_explicit_update();
  void diag();
  void eigenstates_reconstruction();
  double ground_state_energy();
  double occupatation_number(int alpha, int j);
  double pseudospin_Sz();
  void save_to_file(const char* filename);  //!< the reference's checkpoint text format
  void read_from_file(const char* filename);
  void print_eigen(int n);
  void print_lhamil(int n);
  void fetch_hamil();  //!< copy the device CSR into H (host memory: 24 B per nonzero)

 private:
  friend class hamil;
  double tol_ = -1;  // >= 0: convergence tolerance instead of BLQH_TOL (0: run to lambda or breakdown)
  std::shared_ptr<blqh_csr> csr_;
  std::shared_ptr<blqh_lanczos> lz_;
  double params_[7] = {0, 0, 0, 0, 0, 0, 0};
  int precision_ = 0;
};

#endif
