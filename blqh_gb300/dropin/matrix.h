// Drop-in matrix.h: the reference's Vec and Mat containers (BLQH_without_spin/
// matrix.h:37-88) for code that names them. On the GPU path the Hamiltonian
// lives in device memory; lhamil::H stays empty unless filled by
// lhamil::fetch_hamil(). Vec keeps the reference's complex<double> storage.
#ifndef BLQH_DROPIN_MATRIX_H
#define BLQH_DROPIN_MATRIX_H
#include <cmath>
#include <complex>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <vector>

using namespace std;

class Vec {
 public:
  std::vector<complex<double> > value;
  long size = 0;

  Vec() {}
  explicit Vec(long n) : size(n) { value.reserve(n); }
  Vec(long n, const complex<double> init) : value(n, init), size(n) {}
  void assign(long n, const complex<double> init) {
    size = n;
    value.assign(n, init);
  }
  void clear() {
    value.clear();
    size = 0;
  }
  double normed();  // normalizes, returns the former norm
  complex<double> operator*(const Vec& rhs) const;  // <this | rhs>
};

class Mat {
 public:
  // CSR with per-row start and length, as the reference stores it (matrix.h:75-76)
  std::vector<long> outer_starts, outer_size, inner_indices;
  std::vector<complex<double> > value;
  void clear() {
    outer_starts.clear();
    outer_size.clear();
    inner_indices.clear();
    value.clear();
  }
  Vec operator*(const Vec& x) const;
  vector<complex<double> > operator*(const vector<complex<double> >& x) const;
};

#endif
