// Uses the spinful drop-in classes the way the reference's BLQH_with_spin main()
// does (dense check, then the three-pass Lanczos) and prints the numbers the
// tests compare.
// usage: dropin_spin_driver nphi nel nel_up nel_su J K d dsas dv dz
#include <cstdio>
#include <cstdlib>

#include "basis.h"
#include "hamiltonian.h"
#include "lanczos_hamiltonian.h"

int main(int argc, char** argv) {
  if (argc < 11) return 2;
  const int nphi = atoi(argv[1]), nel = atoi(argv[2]), nel_up = atoi(argv[3]), nel_su = atoi(argv[4]);
  const int J = atoi(argv[5]), K = atoi(argv[6]);
  const double d = atof(argv[7]), dsas = atof(argv[8]), dv = atof(argv[9]), dz = atof(argv[10]);
  const double ly = sqrt(nphi * 2.0 * M_PI), lx = ly;
  hamil config;
  config.sector.init(nphi, nel, nel_up, nel_su, J, K);
  config.set_hamil(lx, ly, nphi, 0, d, dsas, dv, dz, 4);
  config.diag();
  printf("nHilbert %ld\nE_dense %.14f\n", config.sector.nbasis, config.ground_state_energy());
  lhamil lconfig(200, 1);
  lconfig.sector.init(nphi, nel, nel_up, nel_su, J, K);
  lconfig.set_hamil(lx, ly, nphi, 0, d, dsas, dv, dz, 0, 0, 0, 4);
  lconfig.coeff_explicit_update();
  lconfig.diag();
  lconfig.eigenstates_reconstruction();
  printf("E_lanczos %.14f\n", lconfig.ground_state_energy());
  printf("eig0 %.14f\n", lconfig.eigenvalues[0]);
  printf("id0 %lu\nidlast %lu\n", (unsigned long)lconfig.sector.id[0],
         (unsigned long)lconfig.sector.id[lconfig.nHilbert - 1]);
  printf("pseudospin_Sz %.14f\nSz %.14f\nupper_Sz %.14f\ndown_Sz %.14f\nSx %.14f\nspinflip %.14f\n",
         lconfig.pseudospin_Sz(), lconfig.Sz(), lconfig.upper_Sz(), lconfig.down_Sz(), lconfig.pseudospin_Sx(),
         lconfig.spinflip_tunneling());
  for (int a = 0; a < 2; a++)
    for (int j = 0; j < nphi; j++) printf("occ_%d_%d %.14f\n", a, j, lconfig.occupatation_number(a, j));
  return 0;
}
