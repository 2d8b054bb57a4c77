// Drop-in basis.h for the spinful model: the reference's sector basis
// (BLQH_with_spin/basis.h:16-49) with the same public members and methods.
// init() builds the basis on the GPU (blqh_basis_build_spin) with the
// reference's own representatives and fills id, basis_C, nbasis and basis_set.
// States have 4 nphi bits: upper layer spin up, upper spin down, lower spin up,
// lower spin down.
#ifndef BLQH_DROPIN_SPIN_BASIS_H
#define BLQH_DROPIN_SPIN_BASIS_H
#include <algorithm>
#include <bitset>
#include <climits>
#include <cmath>
#include <cstdlib>
#include <iomanip>
#include <iostream>
#include <map>
#include <memory>
#include <string.h>
#include <unordered_map>
#include <vector>

using namespace std;

struct blqh_basis;

class basis {
 public:
  int nphi = 0, nel = 0, nel_up = -1, nel_down = -1, nel_su = -1, nel_sd = -1;
  long nbasis = 0;
  int K = -1, J = -1;
  vector<int> popcount_table;
  std::unordered_map<unsigned long, long> basis_set;  // representative -> index
  vector<unsigned long> id;                           // index -> representative, ascending
  vector<short> basis_C;                              // orbit period of each representative

  explicit basis();
  basis(const int& _nphi, const int& _nel);
  basis(const int& _nphi, const int& _nel, const int& _J, const int& _K);
  basis(const int& _nphi, const int& _nel, const int& _nel_up, const int& _J, const int& _K);
  const basis& operator=(const basis&);
  ~basis();
  void init();
  void init(const int& _nphi, const int& _nel);
  void init(const int& _nphi, const int& _nel, const int& _J, const int& _K);
  void init(const int& _nphi, const int& _nel, const int& _nel_up, const int& _J, const int& _K);
  void init(const int& _nphi, const int& _nel, const int& _nel_up, const int& _nel_su, const int& _J,
            const int& _K);
  int get_sign(const unsigned long& c, const int& n, const int& m, const int& nt, const int& mt, const int& t) const;
  int get_sign(const unsigned long& c, const int& n, const int& nt) const;
  int get_nel(const int& a, const long& i) const;
  int get_nel(const int& a, const unsigned long& c) const;
  unsigned long translate(const unsigned long& c, const int& k, int& sign) const;
  unsigned long inv_translate(const unsigned long& c, const int& k, int& sign) const;
  unsigned long factorial(const int&, const int&) const;
  long common_divisor(const int&, const int&) const;
  void prlong() const;
  void clear();

  std::shared_ptr<blqh_basis> device;  // GPU handle (shared by copies); null before init()
};

#endif
