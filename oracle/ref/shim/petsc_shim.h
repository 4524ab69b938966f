/* Stand-in for the PETSc and SLEPc headers (oracle/_ref only). The explicit DG path never touches PETSc: the types
 * exist so that the reference's implicit-solver files compile, and every function aborts if it is ever called
 * (shims.c). The declarations are unprototyped so that one declaration fits every call site. */
#ifndef ORACLE_REF_SHIM_PETSC_H
#define ORACLE_REF_SHIM_PETSC_H
#include <stdio.h>
#include "mpi.h"
typedef int PetscInt;
typedef int PetscErrorCode;
typedef int PetscMPIInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef struct oracle_ref_petsc_obj* Mat;
typedef struct oracle_ref_petsc_obj* Vec;
typedef struct oracle_ref_petsc_obj* KSP;
typedef struct oracle_ref_petsc_obj* PC;
typedef struct oracle_ref_petsc_obj* SlepcEPS_t;
typedef struct oracle_ref_petsc_obj* PetscViewer;
typedef struct oracle_ref_petsc_obj* IS;
typedef const char* KSPType;
typedef const char* PCType;
typedef int KSPConvergedReason;
typedef int InsertMode;
typedef int MatAssemblyType;
typedef int MatReuse;
typedef int NormType;
typedef int PetscViewerFormat;
typedef int PetscCopyMode;
typedef int EPSProblemType;
typedef int EPSWhich;
#define PETSC_NULL NULL
#define PETSC_DEFAULT (-2)
#define PETSC_DECIDE (-1)
#define PETSC_COMM_WORLD 0
#define PETSC_COMM_SELF 0
#define PETSC_USE_POINTER 2
#define INSERT_VALUES 1
#define ADD_VALUES 2
#define MAT_FINAL_ASSEMBLY 0
#define MAT_FLUSH_ASSEMBLY 1
#define MAT_INITIAL_MATRIX 0
#define SAME_NONZERO_PATTERN 0
#define DIFFERENT_NONZERO_PATTERN 1
#define MAT_REUSE_MATRIX 1
#define PETSC_VIEWER_ASCII_MATLAB 1
#define NORM_1 0
#define NORM_2 1
#define NORM_FROBENIUS 2
#define NORM_INFINITY 3
#define KSP_DIVERGED_ITS (-3)
#define KSPPREONLY "preonly"
#define KSPGMRES "gmres"
#define PCLU "lu"
#define PCCHOLESKY "cholesky"
#define PCILU "ilu"
#define PCNONE "none"
#define EPS_HEP 1
#define EPS_NHEP 2
#define EPS_GHEP 3
#define EPS_LARGEST_MAGNITUDE 1
#define EPS_SMALLEST_MAGNITUDE 2
#define EPS_LARGEST_REAL 3
#define EPS_SMALLEST_REAL 4
#define EPS_ERROR_RELATIVE 1
#define CHKERRQ(e) (void)(e)
#define PetscFunctionBegin
#define PetscFunctionReturn(x) return (x)

int PetscInitialize(); int PetscFinalize(); int PetscPrintf();
int SlepcInitialize(); int SlepcFinalize();
int MatCreateSeqAIJ(); int MatSetValues(); int MatAssemblyBegin(); int MatAssemblyEnd(); int MatDestroy();
int MatMatMult(); int MatView(); int MatSetUp(); int MatSetFromOptions(); int MatRestoreRow(); int MatGetRow();
int MatMultAdd(); int MatMult(); int MatGetSize(); int MatTransposeMatMult(); int MatNorm();
int MatMatTransposeMult(); int MatMatSolve(); int MatIsSymmetric(); int MatDestroySubMatrices();
int MatCreateSubMatrices(); int MatAXPY(); int ISCreateGeneral(); int ISDestroy();
int VecDestroy(); int VecCreateSeq(); int VecSetValues(); int VecScale(); int VecNorm(); int VecSetUp();
int VecSetFromOptions(); int VecRestoreSubVector(); int VecGetValues(); int VecGetSubVector();
int VecAssemblyEnd(); int VecAssemblyBegin(); int VecView(); int VecSetValue(); int VecGetSize(); int VecCopy();
int PetscViewerPushFormat(); int PetscViewerASCIIOpen(); int PetscViewerDestroy();
int KSPSolve(); int KSPSetUp(); int KSPSetType(); int KSPSetTolerances(); int KSPSetOperators();
int KSPSetInitialGuessNonzero(); int KSPSetFromOptions(); int KSPSetComputeSingularValues(); int KSPGetPC();
int KSPGetIterationNumber(); int KSPGetConvergedReason(); int KSPDestroy(); int KSPCreate();
int KSPComputeExtremeSingularValues(); int PCSetType(); int PCSetUp();
int EPSSolve(); int EPSSetWhichEigenpairs(); int EPSSetTolerances(); int EPSSetProblemType();
int EPSSetOperators(); int EPSSetFromOptions(); int EPSGetIterationNumber(); int EPSGetEigenpair();
int EPSGetConverged(); int EPSDestroy(); int EPSCreate(); int EPSComputeError();
#endif
