// Host containers Vec / Mat of the drop-in libraries (spinless and spinful):
// the reference's matrix.cpp:84-267 operations that user code calls.
#include "matrix.h"

double Vec::normed() {
  double n = 0;
  for (auto& v : value) n += std::norm(v);
  n = sqrt(n);
  for (auto& v : value) v /= n;
  return n;
}

complex<double> Vec::operator*(const Vec& rhs) const {
  complex<double> s = 0;
  for (long i = 0; i < size && i < rhs.size; i++) s += conj(value[i]) * rhs.value[i];
  return s;
}

Vec Mat::operator*(const Vec& x) const {
  Vec y(x.size, 0.0);
  for (size_t i = 0; i < outer_starts.size(); i++)
    for (long k = outer_starts[i]; k < outer_starts[i] + outer_size[i]; k++) y.value[i] += value[k] * x.value[inner_indices[k]];
  return y;
}

vector<complex<double> > Mat::operator*(const vector<complex<double> >& x) const {
  vector<complex<double> > y(x.size(), 0.0);
  for (size_t i = 0; i < outer_starts.size(); i++)
    for (long k = outer_starts[i]; k < outer_starts[i] + outer_size[i]; k++) y[i] += value[k] * x[inner_indices[k]];
  return y;
}

void swap(Vec* a, Vec* b, Vec* c) {
  *a = *b;
  *b = *c;
}

