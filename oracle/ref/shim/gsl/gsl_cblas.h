/* Stand-in for GSL's gsl_cblas.h (oracle/_ref only): the CBLAS enums and calls, as declared for MKL. */
#ifndef ORACLE_REF_SHIM_GSL_CBLAS_H
#define ORACLE_REF_SHIM_GSL_CBLAS_H
#include "mkl.h"
#endif
