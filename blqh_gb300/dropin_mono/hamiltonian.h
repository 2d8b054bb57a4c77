// Drop-in hamiltonian.h for the monolayer: the reference's dense
// exact-diagonalization class (Monolayer/hamiltonian.h:6-45). set_hamil builds
// the Hamiltonian as a CSR on the GPU (the same elements as the reference's
// dense array) and expands it into `hamiltonian` (nHilbert^2, row-major) for
// code that reads it. diag() runs the reorthogonalized Lanczos, without a
// convergence stop, to the end of its Krylov space (at most min(nHilbert, 4096)
// steps): eigenvalues are the distinct levels of the sector, each once (a dense
// solver lists a degenerate level once per state), and psi_0 is the ground state.
#ifndef BLQH_DROPIN_MONO_HAMILTONIAN_H
#define BLQH_DROPIN_MONO_HAMILTONIAN_H
#include "basis.h"
#include "lanczos_hamiltonian.h"
#include "matrix.h"

class hamil {
 public:
  long nHilbert = 0;
  long nLL = 0, nphi = 0, off_head = 0;
  double lx = 0, ly = 0, E_cl = 0;
  vector<double> Coulomb_matrix;
  complex<double>* hamiltonian = nullptr;
  std::vector<double> eigenvalues;
  std::vector<complex<double> > psi_0;
  std::vector<complex<double> > psi_n0;

  hamil();
  ~hamil();
  hamil(const hamil&) = delete;
  void set_hamil(basis sector, double _lx, double _ly, int nphi, int _nLL);
  const hamil& operator=(const hamil&);
  double ground_state_energy();
  void init_Coulomb_matrix();
  double Coulomb_interaction(int q_x, int q_y);
  void diag();
  void print_hamil(int range);
  void print_eigen(int range);

 private:
  lhamil lz_;
};

#endif
