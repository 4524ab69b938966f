/* Stand-in for GSL's gsl_sf_gamma.h (oracle/_ref only): Gamma through the C library, factorial by exact product. */
#ifndef ORACLE_REF_SHIM_GSL_SF_GAMMA_H
#define ORACLE_REF_SHIM_GSL_SF_GAMMA_H
#include "gsl_errno.h"
double gsl_sf_gamma(double x);
double gsl_sf_fact(unsigned int n);
#endif
