// Probe driver for the reference build in oracle/_ref (test infrastructure).
//
// It links the reference's own basis / lhamil / hamil / matrix objects,
// compiled unmodified from their sources by oracle/build_ref.sh, and drives
// lhamil directly with a fixed seed (the reference main() runs dense ED first
// and reads an uninitialised seed). It writes the sector basis, the CSR matrix
// (rows in index order), the Lanczos coefficients, the Ritz values, the
// reconstructed ground state and the Rayleigh quotient as raw little-endian
// arrays into an output folder, plus per-stage wall times in meta.txt.
//
// usage: ref_probe nphi nel nel_up J K d dsas dv lambda seed nthread outdir [dense 0|1] [gamma] [obs 0|1]
// (obs = 1: also the reference's observables, pseudospin_Sz, pseudospin_Sx and
// occupatation_number for every orbital, into obs.bin)
#include <chrono>
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

static double now() {
  return std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
}

int main(int argc, char** argv) {
  if (argc < 13) {
    fprintf(stderr, "usage: %s nphi nel nel_up J K d dsas dv lambda seed nthread outdir [dense] [gamma]\n", argv[0]);
    return 2;
  }
  int nphi = atoi(argv[1]), nel = atoi(argv[2]), nel_up = atoi(argv[3]), J = atoi(argv[4]), K = atoi(argv[5]);
  double d = atof(argv[6]), dsas = atof(argv[7]), dv = atof(argv[8]);
  int lambda = atoi(argv[9]);
  unsigned seed = (unsigned)strtoul(argv[10], 0, 10);
  int nthread = atoi(argv[11]);
  std::string out = argv[12];
  int dense = argc > 13 ? atoi(argv[13]) : 0;
  double gamma = argc > 14 ? atof(argv[14]) : 1.0;
  int obs = argc > 15 ? atoi(argv[15]) : 0;
  double ly = sqrt(nphi * 2.0 * M_PI / gamma), lx = ly * gamma;

  FILE* meta = fopen((out + "/meta.txt").c_str(), "w");
  double t0 = now();
  lhamil L(lambda, seed);
  L.sector.init(nphi, nel, nel_up, J, K);
  double t1 = now();
  long dim = L.sector.nbasis;
  fprintf(meta, "dim %ld\nt_basis %.6f\n", dim, t1 - t0);
  dump(out, "id", L.sector.id.data(), L.sector.id.size());
  dump(out, "period", L.sector.basis_C.data(), L.sector.basis_C.size());
  if (dim == 0) { fclose(meta); return 0; }

  L.set_hamil(lx, ly, nphi, 0, d, dsas, dv, 0, 0, nthread);
  double t2 = now();
  // rows in index order
  std::vector<long> row_ptr(dim + 1, 0), col;
  std::vector<std::complex<double>> val;
  for (long i = 0; i < dim; i++) {
    row_ptr[i + 1] = row_ptr[i] + L.H.outer_size[i];
    for (long k = 0; k < L.H.outer_size[i]; k++) {
      col.push_back(L.H.inner_indices[L.H.outer_starts[i] + k]);
      val.push_back(L.H.value[L.H.outer_starts[i] + k]);
    }
  }
  fprintf(meta, "nnz %ld\nt_build %.6f\nEc %.17g\n", (long)col.size(), t2 - t1, L.Ec);
  dump(out, "row_ptr", row_ptr.data(), row_ptr.size());
  dump(out, "col", col.data(), col.size());
  dump(out, "val", val.data(), val.size());
  dump(out, "V", L.Coulomb_matrix.data(), L.Coulomb_matrix.size());

  L.coeff_explicit_update();
  double t3 = now();
  L.diag();
  double t4 = now();
  L.eigenstates_reconstruction();
  double t5 = now();
  double E = L.ground_state_energy();
  double t6 = now();
  fprintf(meta, "t_lanczos %.6f\nt_diag %.6f\nt_recon %.6f\nt_rq %.6f\nE_rq %.17g\n", t3 - t2, t4 - t3, t5 - t4,
          t6 - t5, E);
  dump(out, "alpha", L.overlap.data(), L.overlap.size());
  dump(out, "beta", L.norm.data(), L.norm.size());
  dump(out, "eigenvalues", L.eigenvalues.data(), L.eigenvalues.size());
  dump(out, "psir0", L.psir_0.data(), L.psir_0.size());
  if (obs) {
    std::vector<double> o;
    o.push_back(L.pseudospin_Sz());
    o.push_back(L.pseudospin_Sx());
    for (int a = 0; a < 2; a++)
      for (int j = 0; j < nphi; j++) o.push_back(L.occupatation_number(a, j));
    dump(out, "obs", o.data(), o.size());
  }

  if (dense) {
    hamil Hd;
    Hd.sector.init(nphi, nel, nel_up, J, K);
    Hd.set_hamil(lx, ly, nphi, 0, d, dsas, dv, 0, 0, nthread);
    Hd.diag();
    double Ed = Hd.ground_state_energy();
    fprintf(meta, "E_dense_printed %.17g\n", Ed);
    dump(out, "dense_eigenvalues", Hd.eigenvalues.data(), Hd.eigenvalues.size());
  }
  fclose(meta);
  return 0;
}
