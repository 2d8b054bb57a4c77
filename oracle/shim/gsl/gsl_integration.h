/* Minimal stand-in for the GSL integration header, used only to compile the
 * reference sources into the oracle under oracle/_ref. The reference declares
 * GSL integrators it never calls on the exact-diagonalization path; the stub
 * bodies in oracle/shim/gsl_stub.c abort if that ever changes. */
#ifndef BLQH_SHIM_GSL_INTEGRATION_H
#define BLQH_SHIM_GSL_INTEGRATION_H
#include <stddef.h>
#ifdef __cplusplus
extern "C" {
#endif
typedef struct { double (*function)(double x, void* params); void* params; } gsl_function;
typedef struct gsl_integration_workspace gsl_integration_workspace;
gsl_integration_workspace* gsl_integration_workspace_alloc(size_t n);
int gsl_integration_qagiu(gsl_function* f, double a, double epsabs, double epsrel, size_t limit,
                          gsl_integration_workspace* w, double* result, double* abserr);
#ifdef __cplusplus
}
#endif
#endif
