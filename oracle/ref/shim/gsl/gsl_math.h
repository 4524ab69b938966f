/* Stand-in for GSL's gsl_math.h (oracle/_ref only): the macros the reference uses. */
#ifndef ORACLE_REF_SHIM_GSL_MATH_H
#define ORACLE_REF_SHIM_GSL_MATH_H
#include <math.h>
#define GSL_MAX(a, b) ((a) > (b) ? (a) : (b))
#define GSL_MIN(a, b) ((a) < (b) ? (a) : (b))
#define GSL_DBL_EPSILON 2.2204460492503131e-16
static inline double gsl_pow_2(const double x) { return x*x; }
#include "gsl_errno.h"
#endif
