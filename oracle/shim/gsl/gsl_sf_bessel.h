/* Stand-in for the GSL Bessel header (see gsl_integration.h in this folder). */
#ifndef BLQH_SHIM_GSL_SF_BESSEL_H
#define BLQH_SHIM_GSL_SF_BESSEL_H
#ifdef __cplusplus
extern "C" {
#endif
double gsl_sf_bessel_J0(double x);
#ifdef __cplusplus
}
#endif
#endif
