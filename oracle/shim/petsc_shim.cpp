// oracle/shim/petsc_shim.cpp -- TEST INFRASTRUCTURE ONLY.
// Implements oracle/shim/petscksp.h with the GMRES(30)+ILU(0) restatement in
// oracle/krylov.h.  Statistics of the last solves are exposed through
// petsc_shim_stats() so the reference harness can report inner iterations.
#include "petscksp.h"
#include "../krylov.h"
#include <cstdlib>
#include <vector>

struct _p_Mat { int n; int* rowptr; int* col; double* val; };
struct _p_Vec { std::vector<double> v; };
struct _p_PC { int dummy; };
struct _p_KSP {
    Mat A = nullptr;
    double rtol = 1e-5, abstol = 1e-50, dtol = 1e5;
    int maxit = 10000;
    _p_PC pc{};
};

static long long g_solves = 0, g_iters = 0, g_unconverged = 0;

extern "C" void petsc_shim_stats(long long* solves, long long* iters, long long* unconverged) {
    *solves = g_solves; *iters = g_iters; *unconverged = g_unconverged;
}
extern "C" void petsc_shim_reset_stats() { g_solves = g_iters = g_unconverged = 0; }

PetscErrorCode PetscInitialize(int*, char***, const char*, const char*) { return 0; }
PetscErrorCode PetscFinalize(void) { return 0; }
PetscErrorCode MatCreateSeqAIJWithArrays(int, PetscInt m, PetscInt, PetscInt* i, PetscInt* j,
                                         PetscScalar* a, Mat* A) {
    *A = new _p_Mat{m, i, j, a};
    return 0;
}
PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType) { return 0; }
PetscErrorCode MatAssemblyEnd(Mat, MatAssemblyType) { return 0; }
PetscErrorCode MatDestroy(Mat* A) { delete *A; *A = nullptr; return 0; }
PetscErrorCode VecCreateSeq(int, PetscInt n, Vec* v) {
    *v = new _p_Vec;
    (*v)->v.assign(n, 0.0);
    return 0;
}
PetscErrorCode VecDuplicate(Vec a, Vec* b) {
    *b = new _p_Vec;
    (*b)->v.assign(a->v.size(), 0.0);
    return 0;
}
PetscErrorCode VecSetValues(Vec x, PetscInt n, const PetscInt* idx, const PetscScalar* y, InsertMode mode) {
    for (int k = 0; k < n; ++k) {
        if (mode == ADD_VALUES) x->v[idx[k]] += y[k];
        else x->v[idx[k]] = y[k];
    }
    return 0;
}
PetscErrorCode VecGetValues(Vec x, PetscInt n, const PetscInt* idx, PetscScalar* y) {
    for (int k = 0; k < n; ++k) y[k] = x->v[idx[k]];
    return 0;
}
PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
PetscErrorCode VecAssemblyEnd(Vec) { return 0; }
PetscErrorCode VecDestroy(Vec* v) { delete *v; *v = nullptr; return 0; }
PetscErrorCode KSPCreate(int, KSP* k) { *k = new _p_KSP; return 0; }
PetscErrorCode KSPSetOperators(KSP k, Mat A, Mat) { k->A = A; return 0; }
PetscErrorCode KSPGetPC(KSP k, PC* pc) { *pc = &k->pc; return 0; }
PetscErrorCode KSPSetTolerances(KSP k, PetscReal rtol, PetscReal abstol, PetscReal dtol, PetscInt maxits) {
    if (rtol != PETSC_DEFAULT) k->rtol = rtol;
    if (abstol != PETSC_DEFAULT) k->abstol = abstol;
    if (dtol != PETSC_DEFAULT) k->dtol = dtol;
    if (maxits != PETSC_DEFAULT) k->maxit = maxits;
    if (const char* e = std::getenv("BTE_SHIM_KSP_RTOL")) k->rtol = std::atof(e);
    return 0;
}
PetscErrorCode KSPSolve(KSP k, Vec b, Vec x) {
    oracle::Csr A;
    A.n = k->A->n;
    A.rowptr.assign(k->A->rowptr, k->A->rowptr + A.n + 1);
    A.col.assign(k->A->col, k->A->col + A.rowptr[A.n]);
    A.val.assign(k->A->val, k->A->val + A.rowptr[A.n]);
    oracle::KrylovResult r = oracle::gmres_ilu0(A, b->v.data(), x->v.data(), k->rtol, k->abstol,
                                                k->dtol, k->maxit);
    ++g_solves;
    g_iters += r.iterations;
    if (!r.converged) ++g_unconverged;
    return 0;
}
PetscErrorCode KSPDestroy(KSP* k) { delete *k; *k = nullptr; return 0; }
