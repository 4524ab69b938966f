/* Stand-in for gsl_sf_result.h (oracle/_ref only). */
#include "gsl_errno.h"
