/* Stand-in for Intel MKL's mkl.h, used only to compile the reference's own sources into oracle/_ref (test
 * infrastructure). The BLAS/LAPACK calls forward to the ILP64 OpenBLAS bundled with numpy (see shims.c); the
 * in-place transposes are plain loops. MKL_INT is int as in the reference's LP64 MKL build. */
#ifndef ORACLE_REF_SHIM_MKL_H
#define ORACLE_REF_SHIM_MKL_H
#include <stddef.h>
#include <complex.h>

typedef int MKL_INT;
typedef MKL_INT lapack_int;
#ifndef MKL_Complex16
#define MKL_Complex16 double _Complex
#endif

typedef enum { CblasRowMajor = 101, CblasColMajor = 102 } CBLAS_LAYOUT;
typedef CBLAS_LAYOUT CBLAS_ORDER;
typedef enum { CblasNoTrans = 111, CblasTrans = 112, CblasConjTrans = 113 } CBLAS_TRANSPOSE;
typedef enum { CblasUpper = 121, CblasLower = 122 } CBLAS_UPLO;

#define LAPACK_ROW_MAJOR 101
#define LAPACK_COL_MAJOR 102

void cblas_dgemm(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, MKL_INT m, MKL_INT n, MKL_INT k, double alpha,
                 const double* a, MKL_INT lda, const double* b, MKL_INT ldb, double beta, double* c, MKL_INT ldc);
void cblas_zgemm(CBLAS_LAYOUT, CBLAS_TRANSPOSE, CBLAS_TRANSPOSE, MKL_INT m, MKL_INT n, MKL_INT k,
                 const void* alpha, const void* a, MKL_INT lda, const void* b, MKL_INT ldb, const void* beta,
                 void* c, MKL_INT ldc);
void cblas_dgemv(CBLAS_LAYOUT, CBLAS_TRANSPOSE, MKL_INT m, MKL_INT n, double alpha, const double* a, MKL_INT lda,
                 const double* x, MKL_INT incx, double beta, double* y, MKL_INT incy);
void cblas_zgemv(CBLAS_LAYOUT, CBLAS_TRANSPOSE, MKL_INT m, MKL_INT n, const void* alpha, const void* a,
                 MKL_INT lda, const void* x, MKL_INT incx, const void* beta, void* y, MKL_INT incy);

double cblas_ddot(MKL_INT n, const double* x, MKL_INT incx, const double* y, MKL_INT incy);

void mkl_dimatcopy(char ordering, char trans, size_t rows, size_t cols, double alpha, double* ab, size_t lda,
                   size_t ldb);
void mkl_zimatcopy(char ordering, char trans, size_t rows, size_t cols, MKL_Complex16 alpha, MKL_Complex16* ab,
                   size_t lda, size_t ldb);

MKL_INT LAPACKE_dsgesv(int layout, MKL_INT n, MKL_INT nrhs, double* a, MKL_INT lda, MKL_INT* ipiv, double* b,
                       MKL_INT ldb, double* x, MKL_INT ldx, MKL_INT* iter);
MKL_INT LAPACKE_zcgesv(int layout, MKL_INT n, MKL_INT nrhs, MKL_Complex16* a, MKL_INT lda, MKL_INT* ipiv,
                       MKL_Complex16* b, MKL_INT ldb, MKL_Complex16* x, MKL_INT ldx, MKL_INT* iter);
MKL_INT LAPACKE_dsysv(int layout, char uplo, MKL_INT n, MKL_INT nrhs, double* a, MKL_INT lda, MKL_INT* ipiv,
                      double* b, MKL_INT ldb);
MKL_INT LAPACKE_zsysv(int layout, char uplo, MKL_INT n, MKL_INT nrhs, MKL_Complex16* a, MKL_INT lda,
                      MKL_INT* ipiv, MKL_Complex16* b, MKL_INT ldb);
#endif
