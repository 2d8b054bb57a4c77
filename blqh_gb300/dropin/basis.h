// Drop-in basis.h: the reference's sector basis (BLQH_without_spin/basis.h:25-56)
// with the same public members and methods; init() builds the basis on the
// GPU (blqh_basis_build) and fills id, basis_C, nbasis and the index map
// basis_set on the host. The representatives are the reference's own
// (BLQH_REP_REFERENCE), so id[] matches the reference element for element.
#ifndef BLQH_DROPIN_BASIS_H
#define BLQH_DROPIN_BASIS_H
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
  int nphi = 0, nel = 0, nel_up = -1, nel_down = -1;  // orbitals per layer, electrons, upper-layer electrons
  long nbasis = 0;                                    // sector dimension
  int K = -1, J = -1;                                 // translation sector, total momentum
  vector<int> popcount_table;                         // popcount of every nphi-bit pattern
  vector<int> nel_up_table;
  std::unordered_map<unsigned long, long> basis_set;  // representative -> index
  vector<unsigned long> id;                           // index -> representative, ascending
  vector<short> basis_C;                              // orbit period of each representative

  explicit basis();
  basis(int _nphi, int _nel);
  basis(int _nphi, int _nel, int _nel_up);
  basis(int _nphi, int _nel, int _nel_up, int _J, int _K);
  const basis& operator=(const basis&);
  ~basis();
  unsigned long factorial(int, int);
  long common_divisor(int, int);
  void init();
  void init(int _nphi, int _nel);
  void init(int _nphi, int _nel, int _nel_up);
  void init(int _nphi, int _nel, int _nel_up, int _J, int _K);
  int get_nel_upper(long);
  int get_sign(unsigned long c, int n, int m, int nt, int mt, int t);
  int get_sign(unsigned long c, int n, int nt);
  unsigned long translate(unsigned long c, int k, int& sign);
  unsigned long inv_translate(unsigned long c, int k, int& sign);
  void clear();
  void prlong();

  // GPU handle of the basis (shared by copies); null before init().
  std::shared_ptr<blqh_basis> device;
};

#endif
