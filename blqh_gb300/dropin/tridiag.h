// Host eigen-solve of a small symmetric tridiagonal (the Lanczos matrix) that
// returns the eigenvalues and the FIRST component of every eigenvector: the
// weights of the start vector on the Ritz vectors, which the reference keeps
// as psi_n0 (BLQH_without_spin/lanczos_hamiltonian.cpp:597-603, from LAPACK
// dsyevd). Implicit QL with Wilkinson-type shifts (the EISPACK tql2 scheme);
// only the first row of the rotation product is accumulated (Golub-Welsch),
// so the cost is O(m^2). Eigenvector signs are arbitrary, as with LAPACK.
#ifndef BLQH_DROPIN_TRIDIAG_H
#define BLQH_DROPIN_TRIDIAG_H
#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

// diag[0..m), off[1..m) couples i-1 and i (the Lanczos norm[] layout).
// evals ascending; first[i] = first component of the eigenvector of evals[i].
// Returns false if an eigenvalue did not converge in 60 sweeps.
inline bool tridiag_first_row(const double* diag, const double* off, int m, std::vector<double>& evals,
                              std::vector<double>& first) {
  std::vector<double> d(diag, diag + m), e(m, 0.0), z(m, 0.0);
  for (int i = 0; i + 1 < m; i++) e[i] = off[i + 1];  // e[i] couples i and i+1
  if (m > 0) z[0] = 1.0;
  for (int l = 0; l < m; l++) {
    for (int iter = 0;; iter++) {
      int mm = l;
      for (; mm + 1 < m; mm++) {
        const double dd = std::fabs(d[mm]) + std::fabs(d[mm + 1]);
        if (std::fabs(e[mm]) <= 2.2e-16 * dd) break;
      }
      if (mm == l) break;
      if (iter == 60) return false;
      double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
      double r = std::hypot(g, 1.0);
      g = d[mm] - d[l] + e[l] / (g + (g >= 0 ? r : -r));
      double s = 1.0, c = 1.0, p = 0.0;
      int i = mm - 1;
      bool deflated = false;
      for (; i >= l; i--) {
        double f = s * e[i];
        const double b = c * e[i];
        r = std::hypot(f, g);
        e[i + 1] = r;
        if (r == 0.0) {  // underflow: split here and restart
          d[i + 1] -= p;
          e[mm] = 0.0;
          deflated = true;
          break;
        }
        s = f / r;
        c = g / r;
        g = d[i + 1] - p;
        r = (d[i] - g) * s + 2.0 * c * b;
        p = s * r;
        d[i + 1] = g + p;
        g = c * r - b;
        f = z[i + 1];
        z[i + 1] = s * z[i] + c * f;
        z[i] = c * z[i] - s * f;
      }
      if (deflated) continue;
      d[l] -= p;
      e[l] = g;
      e[mm] = 0.0;
    }
  }
  std::vector<int> ord(m);
  std::iota(ord.begin(), ord.end(), 0);
  std::stable_sort(ord.begin(), ord.end(), [&](int a, int b) { return d[a] < d[b]; });
  evals.resize(m);
  first.resize(m);
  for (int i = 0; i < m; i++) {
    evals[i] = d[ord[i]];
    first[i] = z[ord[i]];
  }
  return true;
}

#endif
