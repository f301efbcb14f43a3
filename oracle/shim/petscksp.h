// oracle/shim/petscksp.h -- TEST INFRASTRUCTURE ONLY.
//
// The subset of PETSc's KSP API that the reference's CPU inner solve calls
// (src/StaticBTESolver.cpp:31, :272-307, :833), implemented in
// oracle/shim/petsc_shim.cpp on top of oracle/krylov.h: a sequential AIJ
// matrix that wraps the caller's CSR arrays without copying, sequential
// vectors, and a KSP that runs PETSc's defaults for such a matrix, GMRES(30)
// with left ILU(0).  PETSc itself is not installed and cannot be.
//
// Environment knobs (test use only):
//   BTE_SHIM_KSP_RTOL   overrides the relative tolerance given to KSPSetTolerances
//                       (e.g. 1e-13 for an "exact" inner solve).
#pragma once
#include <cstddef>

typedef int PetscErrorCode;
typedef int PetscInt;
typedef double PetscScalar;
typedef double PetscReal;
typedef int MPI_Comm_petsc_shim;
#define PETSC_COMM_SELF 0
#define PETSC_DEFAULT -2
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES } InsertMode;

typedef struct _p_Mat* Mat;
typedef struct _p_Vec* Vec;
typedef struct _p_KSP* KSP;
typedef struct _p_PC* PC;

PetscErrorCode PetscInitialize(int*, char***, const char*, const char*);
PetscErrorCode PetscFinalize(void);
PetscErrorCode MatCreateSeqAIJWithArrays(int comm, PetscInt m, PetscInt n, PetscInt* i, PetscInt* j,
                                         PetscScalar* a, Mat* A);
PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType);
PetscErrorCode MatAssemblyEnd(Mat, MatAssemblyType);
PetscErrorCode MatDestroy(Mat*);
PetscErrorCode VecCreateSeq(int comm, PetscInt n, Vec* v);
PetscErrorCode VecDuplicate(Vec, Vec*);
PetscErrorCode VecSetValues(Vec, PetscInt n, const PetscInt* idx, const PetscScalar* y, InsertMode);
PetscErrorCode VecGetValues(Vec, PetscInt n, const PetscInt* idx, PetscScalar* y);
PetscErrorCode VecAssemblyBegin(Vec);
PetscErrorCode VecAssemblyEnd(Vec);
PetscErrorCode VecDestroy(Vec*);
PetscErrorCode KSPCreate(int comm, KSP*);
PetscErrorCode KSPSetOperators(KSP, Mat, Mat);
PetscErrorCode KSPGetPC(KSP, PC*);
PetscErrorCode KSPSetTolerances(KSP, PetscReal rtol, PetscReal abstol, PetscReal dtol, PetscInt maxits);
PetscErrorCode KSPSolve(KSP, Vec b, Vec x);
PetscErrorCode KSPDestroy(KSP*);
