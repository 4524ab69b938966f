/* Implementations behind the stand-in headers of shim/ (oracle/_ref only: TEST INFRASTRUCTURE).
 *
 * - BLAS/LAPACK: the reference's LP64 MKL calls forward to the ILP64 OpenBLAS that numpy bundles
 *   (scipy_cblas_*64_, scipy_LAPACKE_*64_), widening the integer arguments. The ILP64 LAPACKE routines take
 *   64-bit pivot and iteration arrays, so those are copied back into the caller's int arrays.
 * - mkl_?imatcopy (in-place transpose with scaling, the only use the reference makes of it): a copy through a
 *   temporary buffer, following MKL's documented meaning of ordering / rows / cols / lda / ldb.
 * - GSL: gsl_sf_gamma is the C library's tgamma; gsl_sf_fact an exact product (exact in double up to 22!, then
 *   correctly rounded products as GSL's table); gsl_permute_matrix applies p to every row from the right,
 *   A'(i, j) = A(i, p[j]), as GSL documents; gsl_poly_eval_derivs is Horner's scheme with derivatives.
 * - PETSc / SLEPc: every function aborts. The explicit residual path never calls them.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "mkl.h"
#include "gsl/gsl_errno.h"
#include "gsl/gsl_sf_gamma.h"
#include "gsl/gsl_poly.h"
#include "gsl/gsl_permute_matrix_double.h"

typedef int64_t i64;

/* numpy's OpenBLAS (ILP64, symbol suffix 64_). */
void scipy_cblas_dgemm64_(int, int, int, i64, i64, i64, double, const double*, i64, const double*, i64, double,
                          double*, i64);
void scipy_cblas_zgemm64_(int, int, int, i64, i64, i64, const void*, const void*, i64, const void*, i64,
                          const void*, void*, i64);
void scipy_cblas_dgemv64_(int, int, i64, i64, double, const double*, i64, const double*, i64, double, double*,
                          i64);
void scipy_cblas_zgemv64_(int, int, i64, i64, const void*, const void*, i64, const void*, i64, const void*,
                          void*, i64);
i64 scipy_LAPACKE_dsgesv64_(int, i64, i64, double*, i64, i64*, double*, i64, double*, i64, i64*);
i64 scipy_LAPACKE_zcgesv64_(int, i64, i64, double _Complex*, i64, i64*, double _Complex*, i64, double _Complex*,
                            i64, i64*);
i64 scipy_LAPACKE_dsysv64_(int, char, i64, i64, double*, i64, i64*, double*, i64);
i64 scipy_LAPACKE_zsysv64_(int, char, i64, i64, double _Complex*, i64, i64*, double _Complex*, i64);
void scipy_openblas_set_num_threads64_(int);
double scipy_cblas_ddot64_(i64, const double*, i64, const double*, i64);

__attribute__((constructor)) static void single_threaded_blas(void)
{
	/* The reference is a serial code: one BLAS thread. */
	scipy_openblas_set_num_threads64_(1);
}

void cblas_dgemm(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, MKL_INT m, MKL_INT n, MKL_INT k,
                 double alpha, const double* a, MKL_INT lda, const double* b, MKL_INT ldb, double beta, double* c,
                 MKL_INT ldc)
{
	scipy_cblas_dgemm64_(l, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

void cblas_zgemm(CBLAS_LAYOUT l, CBLAS_TRANSPOSE ta, CBLAS_TRANSPOSE tb, MKL_INT m, MKL_INT n, MKL_INT k,
                 const void* alpha, const void* a, MKL_INT lda, const void* b, MKL_INT ldb, const void* beta,
                 void* c, MKL_INT ldc)
{
	scipy_cblas_zgemm64_(l, ta, tb, m, n, k, alpha, a, lda, b, ldb, beta, c, ldc);
}

void cblas_dgemv(CBLAS_LAYOUT l, CBLAS_TRANSPOSE t, MKL_INT m, MKL_INT n, double alpha, const double* a,
                 MKL_INT lda, const double* x, MKL_INT incx, double beta, double* y, MKL_INT incy)
{
	scipy_cblas_dgemv64_(l, t, m, n, alpha, a, lda, x, incx, beta, y, incy);
}

void cblas_zgemv(CBLAS_LAYOUT l, CBLAS_TRANSPOSE t, MKL_INT m, MKL_INT n, const void* alpha, const void* a,
                 MKL_INT lda, const void* x, MKL_INT incx, const void* beta, void* y, MKL_INT incy)
{
	scipy_cblas_zgemv64_(l, t, m, n, alpha, a, lda, x, incx, beta, y, incy);
}

double cblas_ddot(MKL_INT n, const double* x, MKL_INT incx, const double* y, MKL_INT incy)
{
	return scipy_cblas_ddot64_(n, x, incx, y, incy);
}

/* In-place B = alpha * op(A). 'R': A is rows x cols with row stride lda, B is cols x rows with row stride ldb;
 * 'C': the same with columns. Only trans = 'T' and 'N' are meaningful for the reference. */
#define DEFINE_IMATCOPY(NAME, T)                                                                                \
void NAME(char ordering, char trans, size_t rows, size_t cols, T alpha, T* ab, size_t lda, size_t ldb)         \
{                                                                                                              \
	const int row_major = (ordering == 'R' || ordering == 'r');                                            \
	const int tr = (trans == 'T' || trans == 't' || trans == 'C' || trans == 'c');                         \
	const size_t n_out = tr ? cols : rows, m_out = tr ? rows : cols; /* outer x inner extents of B */      \
	const size_t n_in = row_major ? rows : cols, m_in = row_major ? cols : rows;                           \
	T* tmp = malloc(sizeof(T) * (n_in * m_in ? n_in * m_in : 1));                                          \
	if (!tmp) abort();                                                                                     \
	for (size_t i = 0; i < n_in; ++i)                                                                      \
		for (size_t j = 0; j < m_in; ++j)                                                              \
			tmp[i * m_in + j] = ab[i * lda + j];                                                   \
	(void)n_out; (void)m_out;                                                                              \
	for (size_t i = 0; i < n_in; ++i)                                                                      \
		for (size_t j = 0; j < m_in; ++j) {                                                            \
			const T v = alpha * tmp[i * m_in + j];                                                 \
			if (tr) ab[j * ldb + i] = v; else ab[i * ldb + j] = v;                                 \
		}                                                                                              \
	free(tmp);                                                                                             \
}
DEFINE_IMATCOPY(mkl_dimatcopy, double)
DEFINE_IMATCOPY(mkl_zimatcopy, double _Complex)

static void copy_ipiv(MKL_INT* dst, const i64* src, i64 n)
{
	for (i64 i = 0; i < n; ++i)
		dst[i] = (MKL_INT)src[i];
}

MKL_INT LAPACKE_dsgesv(int layout, MKL_INT n, MKL_INT nrhs, double* a, MKL_INT lda, MKL_INT* ipiv, double* b,
                       MKL_INT ldb, double* x, MKL_INT ldx, MKL_INT* iter)
{
	i64* piv = malloc(sizeof(i64) * (size_t)(n > 0 ? n : 1));
	i64 it = 0;
	const i64 info = scipy_LAPACKE_dsgesv64_(layout, n, nrhs, a, lda, piv, b, ldb, x, ldx, &it);
	copy_ipiv(ipiv, piv, n);
	*iter = (MKL_INT)it;
	free(piv);
	return (MKL_INT)info;
}

MKL_INT LAPACKE_zcgesv(int layout, MKL_INT n, MKL_INT nrhs, MKL_Complex16* a, MKL_INT lda, MKL_INT* ipiv,
                       MKL_Complex16* b, MKL_INT ldb, MKL_Complex16* x, MKL_INT ldx, MKL_INT* iter)
{
	i64* piv = malloc(sizeof(i64) * (size_t)(n > 0 ? n : 1));
	i64 it = 0;
	const i64 info = scipy_LAPACKE_zcgesv64_(layout, n, nrhs, a, lda, piv, b, ldb, x, ldx, &it);
	copy_ipiv(ipiv, piv, n);
	*iter = (MKL_INT)it;
	free(piv);
	return (MKL_INT)info;
}

MKL_INT LAPACKE_dsysv(int layout, char uplo, MKL_INT n, MKL_INT nrhs, double* a, MKL_INT lda, MKL_INT* ipiv,
                      double* b, MKL_INT ldb)
{
	i64* piv = malloc(sizeof(i64) * (size_t)(n > 0 ? n : 1));
	const i64 info = scipy_LAPACKE_dsysv64_(layout, uplo, n, nrhs, a, lda, piv, b, ldb);
	copy_ipiv(ipiv, piv, n);
	free(piv);
	return (MKL_INT)info;
}

MKL_INT LAPACKE_zsysv(int layout, char uplo, MKL_INT n, MKL_INT nrhs, MKL_Complex16* a, MKL_INT lda,
                      MKL_INT* ipiv, MKL_Complex16* b, MKL_INT ldb)
{
	i64* piv = malloc(sizeof(i64) * (size_t)(n > 0 ? n : 1));
	const i64 info = scipy_LAPACKE_zsysv64_(layout, uplo, n, nrhs, a, lda, piv, b, ldb);
	copy_ipiv(ipiv, piv, n);
	free(piv);
	return (MKL_INT)info;
}

void gsl_error(const char* reason, const char* file, int line, int gsl_errno)
{
	fprintf(stderr, "gsl error %d at %s:%d: %s\n", gsl_errno, file, line, reason);
	abort();
}

double gsl_sf_gamma(double x)
{
	return tgamma(x);
}

double gsl_sf_fact(unsigned int n)
{
	double f = 1.0;
	for (unsigned int i = 2; i <= n; ++i)
		f *= (double)i;
	return f;
}

int gsl_poly_eval_derivs(const double c[], size_t lenc, double x, double res[], size_t lenres)
{
	for (size_t k = 0; k < lenres; ++k)
		res[k] = 0.0;
	for (size_t i = lenc; i-- > 0;) {
		for (size_t k = lenres - 1; k > 0; --k)
			res[k] = res[k] * x + res[k - 1];
		res[0] = res[0] * x + c[i];
	}
	double fact = 1.0;
	for (size_t k = 2; k < lenres; ++k) {
		fact *= (double)k;
		res[k] *= fact;
	}
	return GSL_SUCCESS;
}

int gsl_permute_matrix(const gsl_permutation* p, gsl_matrix* A)
{
	const size_t n = p->size;
	double* row = malloc(sizeof(double) * (n ? n : 1));
	for (size_t i = 0; i < A->size1; ++i) {
		double* r = A->data + i * A->tda;
		for (size_t j = 0; j < n; ++j)
			row[j] = r[p->data[j]];
		memcpy(r, row, sizeof(double) * n);
	}
	free(row);
	return GSL_SUCCESS;
}

int gsl_permute_matrix_complex(const gsl_permutation* p, gsl_matrix_complex* A)
{
	const size_t n = p->size;
	double* row = malloc(sizeof(double) * 2 * (n ? n : 1));
	for (size_t i = 0; i < A->size1; ++i) {
		double* r = A->data + 2 * i * A->tda;
		for (size_t j = 0; j < n; ++j) {
			row[2 * j] = r[2 * p->data[j]];
			row[2 * j + 1] = r[2 * p->data[j] + 1];
		}
		memcpy(r, row, sizeof(double) * 2 * n);
	}
	free(row);
	return GSL_SUCCESS;
}

#define PETSC_STUB(name) \
	int name() { fprintf(stderr, "oracle/_ref: PETSc/SLEPc call %s reached; the explicit path never calls it\n", #name); abort(); }
PETSC_STUB(PetscInitialize) PETSC_STUB(PetscFinalize) PETSC_STUB(PetscPrintf)
PETSC_STUB(SlepcInitialize) PETSC_STUB(SlepcFinalize)
PETSC_STUB(MatCreateSeqAIJ) PETSC_STUB(MatSetValues) PETSC_STUB(MatAssemblyBegin) PETSC_STUB(MatAssemblyEnd)
PETSC_STUB(MatDestroy) PETSC_STUB(MatMatMult) PETSC_STUB(MatView) PETSC_STUB(MatSetUp) PETSC_STUB(MatSetFromOptions)
PETSC_STUB(MatRestoreRow) PETSC_STUB(MatGetRow) PETSC_STUB(MatMultAdd) PETSC_STUB(MatMult) PETSC_STUB(MatGetSize)
PETSC_STUB(MatTransposeMatMult) PETSC_STUB(MatNorm) PETSC_STUB(MatMatTransposeMult) PETSC_STUB(MatMatSolve)
PETSC_STUB(MatIsSymmetric) PETSC_STUB(MatDestroySubMatrices) PETSC_STUB(MatCreateSubMatrices) PETSC_STUB(MatAXPY)
PETSC_STUB(ISCreateGeneral) PETSC_STUB(ISDestroy)
PETSC_STUB(VecDestroy) PETSC_STUB(VecCreateSeq) PETSC_STUB(VecSetValues) PETSC_STUB(VecScale) PETSC_STUB(VecNorm)
PETSC_STUB(VecSetUp) PETSC_STUB(VecSetFromOptions) PETSC_STUB(VecRestoreSubVector) PETSC_STUB(VecGetValues)
PETSC_STUB(VecGetSubVector) PETSC_STUB(VecAssemblyEnd) PETSC_STUB(VecAssemblyBegin) PETSC_STUB(VecView)
PETSC_STUB(VecSetValue) PETSC_STUB(VecGetSize) PETSC_STUB(VecCopy)
PETSC_STUB(PetscViewerPushFormat) PETSC_STUB(PetscViewerASCIIOpen) PETSC_STUB(PetscViewerDestroy)
PETSC_STUB(KSPSolve) PETSC_STUB(KSPSetUp) PETSC_STUB(KSPSetType) PETSC_STUB(KSPSetTolerances)
PETSC_STUB(KSPSetOperators) PETSC_STUB(KSPSetInitialGuessNonzero) PETSC_STUB(KSPSetFromOptions)
PETSC_STUB(KSPSetComputeSingularValues) PETSC_STUB(KSPGetPC) PETSC_STUB(KSPGetIterationNumber)
PETSC_STUB(KSPGetConvergedReason) PETSC_STUB(KSPDestroy) PETSC_STUB(KSPCreate)
PETSC_STUB(KSPComputeExtremeSingularValues) PETSC_STUB(PCSetType) PETSC_STUB(PCSetUp)
PETSC_STUB(EPSSolve) PETSC_STUB(EPSSetWhichEigenpairs) PETSC_STUB(EPSSetTolerances) PETSC_STUB(EPSSetProblemType)
PETSC_STUB(EPSSetOperators) PETSC_STUB(EPSSetFromOptions) PETSC_STUB(EPSGetIterationNumber)
PETSC_STUB(EPSGetEigenpair) PETSC_STUB(EPSGetConverged) PETSC_STUB(EPSDestroy) PETSC_STUB(EPSCreate)
PETSC_STUB(EPSComputeError)
