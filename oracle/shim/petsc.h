/* Minimal, functional stand-in for the part of PETSc the reference aMat
 * headers call, used only to compile them into the CPU oracle library
 * (oracle/_ref). Test infrastructure, not product code.
 *
 * Vec is a dense array. Mat is either a row-wise sparse map (for the
 * reference's assembled operator, include/aMatBased.hpp:148-165, 214-258,
 * 294-352, 458-460) or a shell whose MULT / GET_DIAGONAL callbacks are the
 * reference's own trampolines (include/aMatFree.hpp:358-401, 536-570).
 * INSERT_VALUES overwrites and ADD_VALUES accumulates immediately, which is
 * what PETSc yields after assembly for the call orders the reference uses.
 * KSP/PC are declared so the headers compile; the oracle's CG is its own
 * restatement (oracle/afm_oracle.c). */
#ifndef ORACLE_SHIM_PETSC_H
#define ORACLE_SHIM_PETSC_H

#include "mpi.h"
#include <map>
#include <vector>
#include <cstdio>
#include <cstdlib>
#include <cmath>

typedef int PetscErrorCode;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef double PetscScalar;
typedef double PetscReal;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES } InsertMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { MAT_NEW_NONZERO_ALLOCATION_ERR, MAT_KEEP_NONZERO_PATTERN, MAT_OTHER_OPTION } MatOption;
typedef enum { MATOP_MULT, MATOP_GET_DIAGONAL, MATOP_GET_DIAGONAL_BLOCK } MatOperation;
typedef enum { NORM_1, NORM_2, NORM_INFINITY } NormType;
typedef const char* MatType;
typedef const char* VecType;
typedef const char* KSPType;
typedef const char* PCType;
typedef int PetscViewerFormat;

#define PETSC_DECIDE (-1)
#define PETSC_DETERMINE (-1)
#define PETSC_DEFAULT (-2)
#define PETSC_NULL nullptr
#define PETSC_COMM_SELF MPI_COMM_SELF
#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define MATSEQAIJ "seqaij"
#define MATMPIAIJ "mpiaij"
#define MATSHELL "shell"
#define VECSTANDARD "standard"
#define VECMPI "mpi"
#define VECSEQ "seq"
#define KSPCG "cg"
#define PCJACOBI "jacobi"
#define PCNONE "none"
#define PETSC_VIEWER_ASCII_MATLAB 1

struct _p_Vec { std::vector<double> a; PetscInt n = 0; };
typedef _p_Vec* Vec;

struct _p_Mat {
    PetscInt m = 0, n = 0;
    bool shell = false, assembled = false;
    void* ctx = nullptr;
    void (*mult)(void) = nullptr;
    void (*getdiag)(void) = nullptr;
    std::vector<std::map<PetscInt, double>> rows;
};
typedef _p_Mat* Mat;
typedef struct _p_KSP { int dummy; }* KSP;
typedef struct _p_PC { int dummy; }* PC;
typedef struct _p_Viewer { int dummy; }* PetscViewer;
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)

/* ---- Vec ---- */
static inline PetscErrorCode VecCreate(MPI_Comm, Vec* v) { *v = new _p_Vec(); return 0; }
static inline PetscErrorCode VecSetSizes(Vec v, PetscInt n, PetscInt N) {
    v->n = (n >= 0) ? n : N; v->a.assign((size_t)v->n, 0.0); return 0;
}
static inline PetscErrorCode VecSetType(Vec, VecType) { return 0; }
static inline PetscErrorCode VecSetFromOptions(Vec) { return 0; }
static inline PetscErrorCode VecSet(Vec v, PetscScalar a) { for (auto& x : v->a) x = a; return 0; }
static inline PetscErrorCode VecZeroEntries(Vec v) { return VecSet(v, 0.0); }
static inline PetscErrorCode VecSetValue(Vec v, PetscInt i, PetscScalar a, InsertMode m) {
    if (m == ADD_VALUES) v->a[(size_t)i] += a; else v->a[(size_t)i] = a; return 0;
}
static inline PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt* ix, const PetscScalar* y, InsertMode m) {
    for (PetscInt k = 0; k < n; k++) VecSetValue(v, ix[k], y[k], m); return 0;
}
static inline PetscErrorCode VecGetValues(Vec v, PetscInt n, const PetscInt* ix, PetscScalar* y) {
    for (PetscInt k = 0; k < n; k++) y[k] = v->a[(size_t)ix[k]]; return 0;
}
static inline PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
static inline PetscErrorCode VecAssemblyEnd(Vec) { return 0; }
static inline PetscErrorCode VecGetArray(Vec v, PetscScalar** p) { *p = v->a.data(); return 0; }
static inline PetscErrorCode VecGetArrayRead(Vec v, const PetscScalar** p) { *p = v->a.data(); return 0; }
static inline PetscErrorCode VecRestoreArray(Vec, PetscScalar**) { return 0; }
static inline PetscErrorCode VecRestoreArrayRead(Vec, const PetscScalar**) { return 0; }
static inline PetscErrorCode VecGetSize(Vec v, PetscInt* n) { *n = v->n; return 0; }
static inline PetscErrorCode VecGetLocalSize(Vec v, PetscInt* n) { *n = v->n; return 0; }
static inline PetscErrorCode VecDestroy(Vec* v) { delete *v; *v = nullptr; return 0; }
static inline PetscErrorCode VecView(Vec, PetscViewer) { return 0; }
static inline PetscErrorCode VecSwap(Vec x, Vec y) { x->a.swap(y->a); return 0; }
static inline PetscErrorCode VecAXPY(Vec y, PetscScalar a, Vec x) {
    for (size_t i = 0; i < y->a.size(); i++) y->a[i] += a * x->a[i]; return 0;
}
static inline PetscErrorCode VecDuplicate(Vec x, Vec* y) { *y = new _p_Vec(*x); return 0; }
static inline PetscErrorCode VecCopy(Vec x, Vec y) { y->a = x->a; return 0; }
static inline PetscErrorCode VecNorm(Vec x, NormType, PetscReal* r) {
    double s = 0; for (double t : x->a) s += t * t; *r = std::sqrt(s); return 0;
}

/* ---- Mat ---- */
static inline PetscErrorCode MatCreate(MPI_Comm, Mat* A) { *A = new _p_Mat(); return 0; }
static inline PetscErrorCode MatSetSizes(Mat A, PetscInt m, PetscInt n, PetscInt M, PetscInt N) {
    A->m = (m >= 0) ? m : M; A->n = (n >= 0) ? n : N; A->rows.assign((size_t)A->m, {}); return 0;
}
static inline PetscErrorCode MatCreateSeqAIJ(MPI_Comm c, PetscInt m, PetscInt n, PetscInt, const PetscInt*, Mat* A) {
    MatCreate(c, A); return MatSetSizes(*A, m, n, m, n);
}
static inline PetscErrorCode MatSetType(Mat, MatType) { return 0; }
static inline PetscErrorCode MatSetFromOptions(Mat) { return 0; }
static inline PetscErrorCode MatSeqAIJSetPreallocation(Mat, PetscInt, const PetscInt*) { return 0; }
static inline PetscErrorCode MatMPIAIJSetPreallocation(Mat, PetscInt, const PetscInt*, PetscInt, const PetscInt*) { return 0; }
static inline PetscErrorCode MatSetOption(Mat, MatOption, PetscBool) { return 0; }
static inline PetscErrorCode MatSetValue(Mat A, PetscInt i, PetscInt j, PetscScalar a, InsertMode m) {
    double& s = A->rows[(size_t)i][j];
    if (m == ADD_VALUES) s += a; else s = a; return 0;
}
static inline PetscErrorCode MatSetValues(Mat A, PetscInt nr, const PetscInt* ir, PetscInt nc, const PetscInt* ic,
                                          const PetscScalar* v, InsertMode m) {
    for (PetscInt r = 0; r < nr; r++)
        for (PetscInt c = 0; c < nc; c++) MatSetValue(A, ir[r], ic[c], v[(size_t)r * nc + c], m);
    return 0;
}
static inline PetscErrorCode MatAssemblyBegin(Mat, MatAssemblyType) { return 0; }
static inline PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType) { A->assembled = true; return 0; }
static inline PetscErrorCode MatAssembled(Mat A, PetscBool* f) { *f = A->assembled ? PETSC_TRUE : PETSC_FALSE; return 0; }
static inline PetscErrorCode MatZeroEntries(Mat A) { for (auto& r : A->rows) for (auto& kv : r) kv.second = 0; return 0; }
static inline PetscErrorCode MatView(Mat, PetscViewer) { return 0; }
static inline PetscErrorCode MatDestroy(Mat* A) { delete *A; *A = nullptr; return 0; }
/* include/aMatFree.hpp:523 passes a Mat where PETSc takes a Mat*: accept both */
static inline PetscErrorCode MatDestroy(Mat A) { delete A; return 0; }
static inline PetscErrorCode MatCreateShell(MPI_Comm, PetscInt m, PetscInt n, PetscInt, PetscInt, void* ctx, Mat* A) {
    *A = new _p_Mat(); (*A)->m = m; (*A)->n = n; (*A)->shell = true; (*A)->ctx = ctx; return 0;
}
static inline PetscErrorCode MatShellSetOperation(Mat A, MatOperation op, void (*f)(void)) {
    if (op == MATOP_MULT) A->mult = f; else if (op == MATOP_GET_DIAGONAL) A->getdiag = f; return 0;
}
template <typename T> static inline PetscErrorCode MatShellGetContext(Mat A, T* ctx) {
    *reinterpret_cast<void**>(ctx) = A->ctx; return 0;
}
static inline PetscErrorCode MatMult(Mat A, Vec x, Vec y) {
    if (A->shell) return ((PetscErrorCode(*)(Mat, Vec, Vec))A->mult)(A, x, y);
    for (PetscInt i = 0; i < A->m; i++) {
        double s = 0; for (auto& kv : A->rows[(size_t)i]) s += kv.second * x->a[(size_t)kv.first];
        y->a[(size_t)i] = s;
    }
    return 0;
}
static inline PetscErrorCode MatGetDiagonal(Mat A, Vec d) {
    if (A->shell) return ((PetscErrorCode(*)(Mat, Vec))A->getdiag)(A, d);
    for (PetscInt i = 0; i < A->m; i++) {
        auto it = A->rows[(size_t)i].find(i); d->a[(size_t)i] = (it == A->rows[(size_t)i].end()) ? 0.0 : it->second;
    }
    return 0;
}
static inline PetscErrorCode MatGetDiagonalBlock(Mat A, Mat* a) { *a = A; return 0; }

/* ---- viewers, KSP, PC: declared so the headers compile ---- */
static inline PetscErrorCode PetscViewerASCIIOpen(MPI_Comm, const char*, PetscViewer* v) { *v = nullptr; return 0; }
static inline PetscErrorCode PetscViewerPushFormat(PetscViewer, PetscViewerFormat) { return 0; }
static inline PetscErrorCode PetscViewerDestroy(PetscViewer*) { return 0; }
static inline PetscErrorCode KSPCreate(MPI_Comm, KSP*) { fprintf(stderr, "oracle petsc shim: KSP not provided\n"); abort(); }
static inline PetscErrorCode KSPSetType(KSP, KSPType) { return 0; }
static inline PetscErrorCode KSPSetFromOptions(KSP) { return 0; }
static inline PetscErrorCode KSPSetTolerances(KSP, PetscReal, PetscReal, PetscReal, PetscInt) { return 0; }
static inline PetscErrorCode KSPSetOperators(KSP, Mat, Mat) { return 0; }
static inline PetscErrorCode KSPGetPC(KSP, PC*) { return 0; }
static inline PetscErrorCode KSPSolve(KSP, Vec, Vec) { return 0; }
static inline PetscErrorCode KSPDestroy(KSP*) { return 0; }
static inline PetscErrorCode PCSetType(PC, PCType) { return 0; }
static inline PetscErrorCode PCSetFromOptions(PC) { return 0; }
static inline PetscErrorCode PetscInitialize(int*, char***, const char*, const char*) { return 0; }
static inline PetscErrorCode PetscFinalize() { return 0; }

#endif
