/* Stand-in for GSL's gsl_poly.h (oracle/_ref only). */
#ifndef ORACLE_REF_SHIM_GSL_POLY_H
#define ORACLE_REF_SHIM_GSL_POLY_H
#include <stddef.h>
int gsl_poly_eval_derivs(const double c[], size_t lenc, double x, double res[], size_t lenres);
#endif
