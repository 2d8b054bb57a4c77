// Drop-in hamiltonian.h for the spinful model: the reference's dense
// exact-diagonalization class (BLQH_with_spin/hamiltonian.h:7-58). As in the
// spinless drop-in, the Hamiltonian is built as a CSR on the GPU and diag()
// runs the reorthogonalized Lanczos, without a convergence stop, to the end of
// its Krylov space (at most min(nHilbert, 4096) steps), which yields the exact
// ground state and the distinct levels it can reach.
#ifndef BLQH_DROPIN_SPIN_HAMILTONIAN_H
#define BLQH_DROPIN_SPIN_HAMILTONIAN_H
#include "basis.h"
#include "lanczos_hamiltonian.h"
#include "matrix.h"

class hamil {
 public:
  long nHilbert = 0;
  unsigned seed = 1;
  long nphi = 0, nLL = 0;
  double lx = 0, ly = 0, d = 0;
  double Ec = 0;
  basis sector;
  std::vector<double> eigenvalues;
  std::vector<complex<double> > psi_0;

  hamil();
  ~hamil();
  void set_hamil(const double& _lx, const double& _ly, const long& _nphi, const long& _nLL, const double& _d,
                 const double& _Delta_SAS, const double& _Delta_V, const double& _Delta_Z, const int& nthread);
  double ground_state_energy() const;
  double Sz() const;
  double pseudospin_Sz() const;
  void diag();
  void print_eigen(int range) const;

 private:
  lhamil lz_;
};

#endif
