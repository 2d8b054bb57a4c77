// Drop-in hamiltonian.h: the reference's dense exact-diagonalization class
// (BLQH_without_spin/hamiltonian.h:7-57). The reference stores the full
// nHilbert^2 complex matrix and calls zheevd; here the same Hamiltonian is built
// as a CSR on the GPU and diag() runs the reorthogonalized Lanczos, without a
// convergence stop, to the end of its Krylov space (at most min(nHilbert, 4096)
// steps), which yields the exact
// ground state and the distinct eigenvalues it can reach. `hamiltonian` stays
// empty; `psi_0` is the ground state in the sector basis.
#ifndef BLQH_DROPIN_HAMILTONIAN_H
#define BLQH_DROPIN_HAMILTONIAN_H
#include <mutex>
#include <thread>

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
  std::vector<double> Coulomb_matrix;
  vector<complex<double> > FT;
  std::vector<complex<double> > hamiltonian;
  std::vector<double> eigenvalues;
  std::vector<complex<double> > psi_0;
  std::vector<complex<double> > psi_1;
  std::vector<complex<double> > psi_n0;

  hamil();
  ~hamil();
  void set_hamil(double _lx, double _ly, long _nphi, long _nLL, double _d, double _Delta_SAS, double _Delta_V,
                 double theta_x, double theta_y, int nthread);
  const hamil& operator=(const hamil&);
  double ground_state_energy();
  double pseudospin_Sz();
  void diag();
  void print_eigen(int range);

 private:
  lhamil lz_;
};

#endif
