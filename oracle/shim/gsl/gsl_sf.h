/* Stand-in for the GSL special-function umbrella header. */
#ifndef BLQH_SHIM_GSL_SF_H
#define BLQH_SHIM_GSL_SF_H
#include "gsl_sf_bessel.h"
#endif
