/* Bodies for the GSL stand-ins: never reached on the exact-diagonalization
 * path (the reference's callers of these integrators are commented out). */
#include <stdio.h>
#include <stdlib.h>
#include "gsl/gsl_integration.h"
#include "gsl/gsl_sf_bessel.h"
static void unreachable(const char* what) {
  fprintf(stderr, "oracle/_ref: GSL routine %s was called; the stub cannot serve it\n", what);
  abort();
}
gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n) { (void)n; unreachable("workspace_alloc"); return 0; }
int gsl_integration_qagiu(gsl_function* f, double a, double ea, double er, size_t l, gsl_integration_workspace* w,
                          double* r, double* e) {
  (void)f; (void)a; (void)ea; (void)er; (void)l; (void)w; (void)r; (void)e;
  unreachable("qagiu");
  return 0;
}
double gsl_sf_bessel_J0(double x) { (void)x; unreachable("bessel_J0"); return 0; }
