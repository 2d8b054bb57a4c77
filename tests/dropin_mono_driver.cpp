// Uses the monolayer drop-in classes the way the reference's Monolayer main()
// does (the three-pass Lanczos of a sector, then the dense class) and prints the
// numbers the tests compare; also round-trips the Lanczos checkpoint file.
// usage: dropin_mono_driver nphi nel J K gamma checkpoint_path
#include <cstdio>
#include <cstdlib>

#include "basis.h"
#include "hamiltonian.h"
#include "lanczos_hamiltonian.h"

int main(int argc, char** argv) {
  if (argc < 7) return 2;
  const int nphi = atoi(argv[1]), nel = atoi(argv[2]), J = atoi(argv[3]), K = atoi(argv[4]);
  const double gamma = atof(argv[5]);
  const double ly = sqrt(2.0 * M_PI * nphi / gamma), lx = ly * gamma;
  basis sector(nphi, nel, J, K);
  sector.init();
  printf("nHilbert %ld\nC %ld\n", sector.nbasis, sector.C);
  lhamil lconfig(400, 1);
  lconfig.set_hamil(sector, lx, ly, nphi, 0);
  lconfig.coeff_update();
  lconfig.diag();
  lconfig.eigenstates_reconstruction();
  printf("E_lanczos %.14f\neig0 %.14f\nE_cl %.14f\n", lconfig.ground_state_energy(), lconfig.eigenvalues[0],
         lconfig.E_cl);
  printf("V01 %.14f\n", lconfig.Coulomb_matrix[0 * nphi + 1]);
  lconfig.save_to_file(argv[6]);
  lhamil back;
  back.read_from_file(argv[6]);
  printf("read_lambda %ld\nread_eig0 %.14f\n", back.lambda, back.eigenvalues[0]);
  hamil config;
  config.set_hamil(sector, lx, ly, nphi, 0);
  config.diag();
  printf("E_dense %.14f\n", config.ground_state_energy());
  for (size_t i = 0; i < config.eigenvalues.size() && i < 10; i++) printf("level %.14f\n", config.eigenvalues[i]);
  double herm = 0;
  for (long i = 0; i < config.nHilbert; i++)
    for (long j = 0; j < config.nHilbert; j++)
      herm = std::max(herm, std::abs(config.hamiltonian[i * config.nHilbert + j] -
                                     std::conj(config.hamiltonian[j * config.nHilbert + i])));
  printf("herm %.3e\n", herm);
  return 0;
}
