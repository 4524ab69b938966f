/* Stand-in for GSL's complex matrix permutation (oracle/_ref only); declared with the real one. */
#include "gsl_permute_matrix_double.h"
