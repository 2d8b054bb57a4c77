// Uses the drop-in classes the way the reference's main() does (dense check,
// then the three-pass Lanczos), and prints the numbers the tests compare.
// usage: dropin_driver nphi nel nel_up J K d
#include <cstdio>
#include <cstdlib>

#include "basis.h"
#include "hamiltonian.h"
#include "lanczos_hamiltonian.h"

int main(int argc, char** argv) {
  if (argc < 7) return 2;
  const int nphi = atoi(argv[1]), nel = atoi(argv[2]), nel_up = atoi(argv[3]), J = atoi(argv[4]), K = atoi(argv[5]);
  const double d = atof(argv[6]);
  const double ly = sqrt(nphi * 2.0 * M_PI), lx = ly;
  hamil config;
  config.sector.init(nphi, nel, nel_up, J, K);
  config.set_hamil(lx, ly, nphi, 0, d, 0.0, 0.0, 0, 0, 4);
  config.diag();
  printf("nHilbert %ld\nE_dense %.12f\n", config.sector.nbasis, config.ground_state_energy() / nel);
  lhamil lconfig(200, 1);
  lconfig.sector.init(nphi, nel, nel_up, J, K);
  lconfig.set_hamil(lx, ly, nphi, 0, d, 0.0, 0.0, 0, 0, 4);
  lconfig.coeff_explicit_update();
  lconfig.diag();
  lconfig.eigenstates_reconstruction();
  printf("E_lanczos %.12f\n", lconfig.ground_state_energy() / nel);
  printf("steps %zu\n", lconfig.overlap.size());
  printf("id0 %lu\n", (unsigned long)lconfig.sector.id[0]);
  double amax = 0;
  for (long i = 0; i < lconfig.nHilbert; i++) amax = std::max(amax, std::abs(lconfig.psir_0[i]));
  printf("amax %.10f\nSz %.12f\n", amax, lconfig.pseudospin_Sz());
  return 0;
}
