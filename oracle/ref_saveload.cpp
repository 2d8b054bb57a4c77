// Probe of the Lanczos checkpoint format (lhamil::save_to_file / read_from_file,
// BLQH_without_spin/lanczos_hamiltonian.cpp:738-819). Test infrastructure: it is
// compiled against the reference's own sources (oracle/build_ref.sh ->
// oracle/_ref/ref_saveload) and, by tests/test_saveload.py, against the drop-in
// classes, so that each side's writer can be read by the other's reader.
//
// usage: ref_saveload write OUT IN   (IN: nHilbert lambda seed, then lambda
//                                     eigenvalues, lambda+1 norm, lambda overlap,
//                                     lambda psi_0, lambda psi_n0)
//        ref_saveload read FILE      (prints the same layout with 17 digits)
#include <cstdio>
#include <cstring>
#include <vector>

#include "lanczos_hamiltonian.h"

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  lhamil L(200, 1);
  if (!strcmp(argv[1], "write")) {
    if (argc < 4) return 2;
    FILE* f = fopen(argv[3], "r");
    if (!f) return 3;
    long nh = 0, n = 0;
    unsigned seed = 0;
    if (fscanf(f, "%ld %ld %u", &nh, &n, &seed) != 3) return 4;
    L.nHilbert = nh;
    L.lambda = n;
    L.seed = seed;
    auto rd = [&](std::vector<double>& v, long k) {
      v.assign(k, 0.0);
      for (auto& x : v)
        if (fscanf(f, "%lf", &x) != 1) x = 0.0;
    };
    rd(L.eigenvalues, n);
    rd(L.norm, n + 1);
    rd(L.overlap, n);
    rd(L.psi_0, n);
    rd(L.psi_n0, n);
    fclose(f);
    L.save_to_file(argv[2]);
    return 0;
  }
  L.read_from_file(argv[2]);
  printf("%ld %ld %u\n", L.nHilbert, L.lambda, L.seed);
  const std::vector<double>* lists[] = {&L.eigenvalues, &L.norm, &L.overlap, &L.psi_0, &L.psi_n0};
  for (auto* v : lists) {
    for (double x : *v) printf("%.17g ", x);
    printf("\n");
  }
  return 0;
}
