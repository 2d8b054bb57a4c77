// Probe driver for the reference's spinful model (test infrastructure).
//
// Links BLQH_with_spin's own basis / lhamil / hamil / matrix objects, compiled
// unmodified from their sources by oracle/build_ref.sh into oracle/_ref/spin,
// and drives lhamil directly with a fixed seed. Writes the basis, the CSR (rows
// in index order), the Lanczos coefficients, Ritz values, reconstructed ground
// state and Rayleigh quotient as raw little-endian arrays into an output
// folder; optionally the dense ED eigenvalues.
//
// usage: ref_probe_spin nphi nel nel_up nel_su J K d dsas dv dz lambda seed outdir [dense 0|1]
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "basis.h"
#include "hamiltonian.h"
#include "lanczos_hamiltonian.h"

template <class T>
static void dump(const std::string& dir, const char* name, const T* p, size_t n) {
  std::string f = dir + "/" + name + ".bin";
  FILE* fp = fopen(f.c_str(), "wb");
  if (!fp) { perror(f.c_str()); exit(1); }
  if (n) fwrite(p, sizeof(T), n, fp);
  fclose(fp);
}

int main(int argc, char** argv) {
  if (argc < 14) {
    fprintf(stderr, "usage: %s nphi nel nel_up nel_su J K d dsas dv dz lambda seed outdir [dense]\n", argv[0]);
    return 2;
  }
  int nphi = atoi(argv[1]), nel = atoi(argv[2]), nel_up = atoi(argv[3]), nel_su = atoi(argv[4]);
  int J = atoi(argv[5]), K = atoi(argv[6]);
  double d = atof(argv[7]), dsas = atof(argv[8]), dv = atof(argv[9]), dz = atof(argv[10]);
  int lambda = atoi(argv[11]);
  unsigned seed = (unsigned)strtoul(argv[12], 0, 10);
  std::string out = argv[13];
  int dense = argc > 14 ? atoi(argv[14]) : 0;
  double ly = sqrt(nphi * 2.0 * M_PI), lx = ly;

  FILE* meta = fopen((out + "/meta.txt").c_str(), "w");
  lhamil L(lambda, seed);
  L.sector.init(nphi, nel, nel_up, nel_su, J, K);
  long dim = L.sector.nbasis;
  fprintf(meta, "dim %ld\n", dim);
  dump(out, "id", L.sector.id.data(), L.sector.id.size());
  dump(out, "period", L.sector.basis_C.data(), L.sector.basis_C.size());
  if (dim == 0) { fclose(meta); return 0; }
  L.set_hamil(lx, ly, nphi, 0, d, dsas, dv, dz, 0, 0, 0, 1);
  std::vector<long> row_ptr(dim + 1, 0), col;
  std::vector<std::complex<double>> val;
  for (long i = 0; i < dim; i++) {
    row_ptr[i + 1] = row_ptr[i] + L.H.outer_size[i];
    for (long k = 0; k < L.H.outer_size[i]; k++) {
      col.push_back(L.H.inner_indices[L.H.outer_starts[i] + k]);
      val.push_back(L.H.value[L.H.outer_starts[i] + k]);
    }
  }
  fprintf(meta, "nnz %ld\nEc %.17g\n", (long)col.size(), L.Ec);
  dump(out, "row_ptr", row_ptr.data(), row_ptr.size());
  dump(out, "col", col.data(), col.size());
  dump(out, "val", val.data(), val.size());
  L.coeff_explicit_update();
  L.diag();
  L.eigenstates_reconstruction();
  double E = L.ground_state_energy();
  fprintf(meta, "E_rq %.17g\n", E);
  dump(out, "alpha", L.overlap.data(), L.overlap.size());
  dump(out, "beta", L.norm.data(), L.norm.size());
  dump(out, "eigenvalues", L.eigenvalues.data(), L.eigenvalues.size());
  dump(out, "psir0", L.psir_0.data(), L.psir_0.size());
  // the reference's ground-state observables (BLQH_with_spin/lanczos_hamiltonian.cpp:1217-1593):
  // Sz, pseudospin_Sz, upper_Sz, down_Sz, pseudospin_Sx, spinflip_tunneling, then
  // occupatation_number(0, j) and (1, j) for j < nphi
  std::vector<double> obs = {L.Sz(), L.pseudospin_Sz(), L.upper_Sz(), L.down_Sz(), L.pseudospin_Sx(),
                             L.spinflip_tunneling()};
  for (int a = 0; a < 2; a++)
    for (int j = 0; j < nphi; j++) obs.push_back(L.occupatation_number(a, j));
  dump(out, "obs", obs.data(), obs.size());
  if (dense) {
    hamil Hd;
    Hd.sector.init(nphi, nel, nel_up, nel_su, J, K);
    Hd.set_hamil(lx, ly, nphi, 0, d, dsas, dv, dz, 1);
    Hd.diag();
    fprintf(meta, "E_dense_printed %.17g\n", Hd.ground_state_energy());
    dump(out, "dense_eigenvalues", Hd.eigenvalues, (size_t)Hd.nHilbert);
  }
  fclose(meta);
  return 0;
}
