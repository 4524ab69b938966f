/* Stand-in for GSL's gsl_errno.h (oracle/_ref only). */
#ifndef ORACLE_REF_SHIM_GSL_ERRNO_H
#define ORACLE_REF_SHIM_GSL_ERRNO_H
enum { GSL_SUCCESS = 0, GSL_FAILURE = -1, GSL_CONTINUE = -2, GSL_EDOM = 1, GSL_EINVAL = 4, GSL_ENOMEM = 8 };
void gsl_error(const char* reason, const char* file, int line, int gsl_errno);
#define GSL_ERROR(reason, gsl_errno) do { gsl_error(reason, __FILE__, __LINE__, gsl_errno); return gsl_errno; } while (0)
#define GSL_ERROR_NULL(reason, gsl_errno) do { gsl_error(reason, __FILE__, __LINE__, gsl_errno); return 0; } while (0)
typedef struct { double val; double err; } gsl_sf_result;
#endif
