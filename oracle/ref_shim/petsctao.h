// Minimal single-rank stand-in for <petsctao.h> (test infrastructure only).
// It provides just the Vec and Tao calls that minimizer.cpp makes, backed by
// plain arrays.  TaoSolve does not minimise: it records the objective
// callback so the harness can call the reference's formFunctionAndGradient.
#ifndef A2C_REF_SHIM_PETSCTAO_H
#define A2C_REF_SHIM_PETSCTAO_H
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <vector>
#include "mpi.h"
typedef int PetscErrorCode;
typedef int PetscMPIInt;
typedef int PetscInt;
typedef double PetscReal;
typedef double PetscScalar;
typedef int InsertMode;
typedef int TaoConvergedReason;
typedef const char *TaoType;
struct ShimVec { std::vector<double> a; };
typedef ShimVec *Vec;
struct ShimTao;
typedef ShimTao *Tao;
typedef PetscErrorCode (*ShimObjGrad)(Tao, Vec, PetscReal *, Vec, void *);
typedef PetscErrorCode (*ShimBounds)(Tao, Vec, Vec, void *);
struct ShimTao {
  ShimObjGrad objgrad = nullptr;
  void *objctx = nullptr;
  ShimBounds bounds = nullptr;
  void *bctx = nullptr;
  Vec x = nullptr;
  double f = 0.0;
};
extern Tao shim_last_tao;
#define PETSC_COMM_WORLD MPI_COMM_WORLD
#define PETSC_DECIDE (-1)
#define PETSC_INFINITY (HUGE_VAL)
#define PETSC_NINFINITY (-HUGE_VAL)
#define MPIU_REAL MPI_DOUBLE
#define MPIU_SUM MPI_SUM
#define INSERT_VALUES 1
#define TAOBLMVM "blmvm"
#define CHKERRQ(e) do { if (e) return (e); } while (0)
#define PetscFunctionReturn(x) return (x)
static inline PetscErrorCode PetscInitialize(int *, char ***, const char *, const char *) { return 0; }
static inline PetscErrorCode PetscPrintf(MPI_Comm, const char *fmt, ...) {
  va_list ap; va_start(ap, fmt); vfprintf(stdout, fmt, ap); va_end(ap); return 0;
}
static inline PetscErrorCode PetscSplitOwnership(MPI_Comm, PetscInt *n, PetscInt *N) {
  if (*n == PETSC_DECIDE) *n = *N; else if (*N == PETSC_DECIDE) *N = *n; return 0;
}
static inline PetscErrorCode VecCreateMPI(MPI_Comm, PetscInt, PetscInt N, Vec *v) {
  *v = new ShimVec; (*v)->a.assign((size_t)N, 0.0); return 0;
}
static inline PetscErrorCode VecSet(Vec v, PetscScalar s) { for (auto &e : v->a) e = s; return 0; }
static inline PetscErrorCode VecDuplicate(Vec v, Vec *w) { *w = new ShimVec; (*w)->a.assign(v->a.size(), 0.0); return 0; }
static inline PetscErrorCode VecGetOwnershipRange(Vec v, PetscInt *lo, PetscInt *hi) { *lo = 0; *hi = (PetscInt)v->a.size(); return 0; }
static inline PetscErrorCode VecGetArray(Vec v, PetscScalar **p) { *p = v->a.data(); return 0; }
static inline PetscErrorCode VecRestoreArray(Vec, PetscScalar **) { return 0; }
static inline PetscErrorCode VecSetValues(Vec v, PetscInt n, const PetscInt *ix, const PetscScalar *y, InsertMode) {
  for (PetscInt i = 0; i < n; ++i) v->a[(size_t)ix[i]] = y[i]; return 0;
}
static inline PetscErrorCode VecAssemblyBegin(Vec) { return 0; }
static inline PetscErrorCode VecAssemblyEnd(Vec) { return 0; }
static inline PetscErrorCode VecDestroy(Vec *v) { delete *v; *v = nullptr; return 0; }
static inline PetscErrorCode TaoCreate(MPI_Comm, Tao *t) { *t = new ShimTao; shim_last_tao = *t; return 0; }
static inline PetscErrorCode TaoSetType(Tao, TaoType) { return 0; }
static inline PetscErrorCode TaoSetObjectiveAndGradientRoutine(Tao t, ShimObjGrad f, void *c) { t->objgrad = f; t->objctx = c; return 0; }
static inline PetscErrorCode TaoSetVariableBoundsRoutine(Tao t, ShimBounds f, void *c) { t->bounds = f; t->bctx = c; return 0; }
static inline PetscErrorCode TaoSetFromOptions(Tao) { return 0; }
static inline PetscErrorCode TaoSetInitialVector(Tao t, Vec x) { t->x = x; return 0; }
static inline PetscErrorCode TaoSolve(Tao t) {
  Vec g; VecDuplicate(t->x, &g);
  PetscErrorCode e = t->objgrad(t, t->x, &t->f, g, t->objctx);
  VecDestroy(&g); return e;
}
static inline PetscErrorCode TaoGetSolutionStatus(Tao t, PetscInt *, PetscReal *f, PetscReal *, PetscReal *, PetscReal *, TaoConvergedReason *r) {
  if (f) *f = t->f; if (r) *r = 0; return 0;
}
static inline PetscErrorCode TaoDestroy(Tao *t) { delete *t; *t = nullptr; return 0; }
#endif
