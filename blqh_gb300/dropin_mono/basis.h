// Drop-in basis.h for the monolayer: the reference's sector basis
// (Monolayer/basis.h:21-53) with the same public members and methods. init()
// builds the basis on the GPU (blqh_basis_build_mono) with the reference's own
// representatives and fills id, basis_C, nbasis, C and basis_set. translate and
// inv_translate take the four parameters of their definitions
// (Monolayer/basis.cpp:263, 277); the reference's header declares three.
#ifndef BLQH_DROPIN_MONO_BASIS_H
#define BLQH_DROPIN_MONO_BASIS_H
#include <algorithm>
#include <bitset>
#include <cmath>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <memory>
#include <string.h>
#include <unordered_map>
#include <vector>

using namespace std;

struct blqh_basis;

class basis {
 public:
  long nphi = 0, nel = 0, C = 1, J = -1, K = -1;
  long nbasis = 0;
  std::unordered_map<unsigned long, long> basis_set;  // representative -> index
  vector<unsigned long> id;                           // index -> representative, ascending
  vector<int> popcount_table;
  vector<short> basis_C;                              // orbit period of each representative

  explicit basis();
  basis(long _nphi, long _nel);
  basis(long _nphi, long _nel, long _J, long _K);
  const basis& operator=(const basis&);
  ~basis();
  long onsite_potential(long i, long n);
  unsigned long factorial(long, long);
  long common_divisor(long, long);
  void init();
  void init(long, long);
  void init(long, long, long, long);
  unsigned long translate(unsigned long c, int k, int& sign, int& ncross);
  unsigned long inv_translate(unsigned long c, int k, int& sign, int& ncross);
  long creation(long s, long n);
  long annihilation(long s, long n);
  int get_sign(long c, long n, long m, long nt, long mt);
  void prlong();
  void clear();

  std::shared_ptr<blqh_basis> device;  // GPU handle (shared by copies); null before init()
};

#endif
