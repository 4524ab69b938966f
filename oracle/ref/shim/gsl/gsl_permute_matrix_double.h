/* Stand-in for GSL's permutation and matrix views (oracle/_ref only). gsl_permute_matrix follows GSL's documented
 * meaning: every row is permuted from the right, A'(i, j) = A(i, p[j]). */
#ifndef ORACLE_REF_SHIM_GSL_PERMUTE_MATRIX_DOUBLE_H
#define ORACLE_REF_SHIM_GSL_PERMUTE_MATRIX_DOUBLE_H
#include <stddef.h>
typedef struct { size_t size; size_t* data; } gsl_permutation;
typedef struct { size_t size1, size2, tda; double* data; void* block; int owner; } gsl_matrix;
typedef struct { size_t size1, size2, tda; double* data; void* block; int owner; } gsl_matrix_complex;
int gsl_permute_matrix(const gsl_permutation* p, gsl_matrix* A);
int gsl_permute_matrix_complex(const gsl_permutation* p, gsl_matrix_complex* A);
#endif
