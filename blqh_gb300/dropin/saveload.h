// The reference's Lanczos checkpoint text format (BLQH_without_spin/
// lanczos_hamiltonian.cpp:738-819, the same in BLQH_with_spin): a line each for
// nHilbert, lambda and seed, then eigenvalues, norm (one more entry), overlap,
// psi_0 and psi_n0 as "name:=  [ v , v , ... ,  ] " with 8 significant digits.
// Shared by the spinless and spinful drop-in lhamil classes. The lambda written
// is the number of Lanczos steps taken (overlap.size()): the reference's reader
// takes that many entries per list, and the drop-in may stop before lambda.
#ifndef BLQH_DROPIN_SAVELOAD_H
#define BLQH_DROPIN_SAVELOAD_H
#include <fstream>
#include <iomanip>
#include <stdexcept>
#include <string>
#include <vector>

template <class LH>
void lanczos_save(const LH& L, const char* filename) {
  if (L.eigenvalues.empty()) return;  // as the reference: nothing before diag()
  const size_t n = L.overlap.size();
  std::ofstream f(filename);
  if (!f) throw std::runtime_error(std::string("save_to_file: cannot open ") + filename);
  auto list = [&](const char* name, const std::vector<double>& v, size_t count) {
    f << name << std::setw(10) << std::setprecision(8) << " [ ";
    for (size_t i = 0; i < count; i++) f << (i < v.size() ? v[i] : 0.0) << " , ";
    f << " ] " << std::endl;
  };
  f << "nHilbert:=" << std::setw(10) << " " << L.nHilbert << std::endl;
  f << "lambda:=" << std::setw(10) << " " << (long)n << std::endl;
  f << "seed:=" << std::setw(10) << " " << L.seed << std::endl;
  list("eigenvalues:=", L.eigenvalues, n);
  list("norm:=", L.norm, n + 1);
  list("overlap:=", L.overlap, n);
  list("psi_0:=", L.psi_0, n);
  list("psi_n0:=", L.psi_n0, n);
}

template <class LH>
void lanczos_read(LH& L, const char* filename) {
  std::ifstream f(filename);
  if (!f) throw std::runtime_error(std::string("read_from_file: cannot open ") + filename);
  std::string tok;
  auto number = [&](const char* what) {
    f >> tok;  // the "name:=" label
    long v = 0;
    if (!(f >> v)) throw std::runtime_error(std::string("read_from_file: bad ") + what);
    return v;
  };
  L.nHilbert = number("nHilbert");
  L.lambda = number("lambda");
  L.seed = (unsigned)number("seed");
  auto list = [&](const char* what, std::vector<double>& v, long count) {
    f >> tok >> tok;  // "name:=" "["
    v.clear();
    for (long i = 0; i < count; i++) {
      double x = 0;
      if (!(f >> x)) throw std::runtime_error(std::string("read_from_file: bad ") + what);
      f >> tok;  // ","
      v.push_back(x);
    }
    f >> tok;  // "]"
  };
  list("eigenvalues", L.eigenvalues, L.lambda);
  list("norm", L.norm, L.lambda + 1);
  list("overlap", L.overlap, L.lambda);
  list("psi_0", L.psi_0, L.lambda);
  list("psi_n0", L.psi_n0, L.lambda);
}

#endif
