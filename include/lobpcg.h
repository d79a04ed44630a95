/*
 * lobpcg.h -- the BLOPEX LOBPCG solver entry points (drop-in C ABI).
 *
 * Replaces blopex_abstract/krylov/lobpcg.h:13-168.  Names, argument lists,
 * struct layouts and return codes are those of the reference so that a C
 * caller (serial_driver.c:117, HYPRE_lobpcg.c:434, the MATLAB gateway) can
 * relink against liblobpcg_gb300.so unchanged.  What runs behind them is
 * the GB300 device solver: the block vectors must be gpu_MultiVector
 * objects wrapped with the interpreter from GpuSetupInterpreter
 * (lobpcg_gb300.h); all block work, the Gram matrices, the Cholesky
 * factorisations and the Rayleigh-Ritz eigenproblem run on the GPU.
 */
#ifndef BLOPEX_GB300_LOBPCG_H
#define BLOPEX_GB300_LOBPCG_H

#include "multivector.h"
#include "fortran_interpreter.h"
#include "fortran_matrix.h"

/* exit flags, lobpcg.h:13-16 of the reference */
#define PROBLEM_SIZE_TOO_SMALL 1
#define WRONG_BLOCK_SIZE 2
#define WRONG_CONSTRAINTS 3
#define REQUESTED_ACCURACY_NOT_ACHIEVED -1

/* residual test |r_i| <= |lambda_i| * relative + absolute (lobpcg.h:18-23) */
typedef struct {
  double absolute;
  double relative;
} lobpcg_Tolerance;

/* LAPACK hooks (lobpcg.h:25-46).  The device solver accepts them for ABI
   compatibility and does not call them: its Cholesky factorisations and
   generalized eigensolver are GPU kernels. */
typedef struct {
  BlopexInt (*dpotrf)(char* uplo, BlopexInt* n, double* a, BlopexInt* lda, BlopexInt* info);
  BlopexInt (*dsygv)(BlopexInt* itype, char* jobz, char* uplo, BlopexInt* n, double* a,
                     BlopexInt* lda, double* b, BlopexInt* ldb, double* w, double* work,
                     BlopexInt* lwork, BlopexInt* info);
  BlopexInt (*zpotrf)(char* uplo, BlopexInt* n, komplex* a, BlopexInt* lda, BlopexInt* info);
  BlopexInt (*zhegv)(BlopexInt* itype, char* jobz, char* uplo, BlopexInt* n, komplex* a,
                     BlopexInt* lda, komplex* b, BlopexInt* ldb, double* w, komplex* work,
                     BlopexInt* lwork, double* rwork, BlopexInt* info);
} lobpcg_BLASLAPACKFunctions;

#ifdef __cplusplus
extern "C" {
#endif

/* small dense hooks of the generic solver (lobpcg.h:52-66); accepted by
   lobpcg_solve for ABI compatibility, not called by the device solver */
typedef struct {
  BlopexInt (*chol)(utilities_FortranMatrix* a, lobpcg_BLASLAPACKFunctions blap_fn,
                    utilities_FortranInterpreter* util);
  BlopexInt (*solveGEVP)(utilities_FortranMatrix* mtxA, utilities_FortranMatrix* mtxB,
                         utilities_FortranMatrix* eigVal, lobpcg_BLASLAPACKFunctions blap_fn,
                         utilities_FortranInterpreter* util);
} lobpcg_Interpreter;

/*
 * Solve A x = lambda B x for the sizeX smallest eigenpairs, sizeX = width of
 * blockVectorX (lobpcg.h:68-113 / lobpcg.c:332-413 of the reference).
 *   blockVectorX   initial block on entry, Ritz vectors on exit (in place)
 *   operatorA/B/T  void op(void* data, void* X, void* Y): Y = op(X) on the
 *                  active columns; X and Y are gpu_MultiVector*.  B == NULL
 *                  means B = I, T == NULL means no preconditioner.
 *   blockVectorY   constraints (may be NULL): X is kept B-orthogonal to Y
 *   lambda_values, residualNorms_values: host arrays of sizeX doubles
 *   *History_values: host sizeX x (maxIterations+1) column-major arrays with
 *                  leading dimension *_gh, or NULL
 * Returns 0 (converged), WRONG_BLOCK_SIZE, WRONG_CONSTRAINTS, or
 * REQUESTED_ACCURACY_NOT_ACHIEVED (not converged, a factorisation failed,
 * or a CUDA error occurred -- the message goes to stderr when
 * verbosityLevel > 0).
 */
int lobpcg_solve_double(mv_MultiVectorPtr blockVectorX,
                        void* operatorAData, void (*operatorA)(void*, void*, void*),
                        void* operatorBData, void (*operatorB)(void*, void*, void*),
                        void* operatorTData, void (*operatorT)(void*, void*, void*),
                        mv_MultiVectorPtr blockVectorY,
                        lobpcg_BLASLAPACKFunctions blap_fn,
                        lobpcg_Tolerance tolerance,
                        int maxIterations,
                        int verbosityLevel,
                        int* iterationNumber,
                        double* lambda_values,
                        double* lambdaHistory_values,
                        BlopexInt lambdaHistory_gh,
                        double* residualNorms_values,
                        double* residualNormsHistory_values,
                        BlopexInt residualNormsHistory_gh);

/* Generic entry (lobpcg.h:143-168): identical to lobpcg_solve_double for
   real data; `lobpcg` and `util` are accepted and not used. */
int lobpcg_solve(mv_MultiVectorPtr blockVectorX,
                 void* operatorAData, void (*operatorA)(void*, void*, void*),
                 void* operatorBData, void (*operatorB)(void*, void*, void*),
                 void* operatorTData, void (*operatorT)(void*, void*, void*),
                 mv_MultiVectorPtr blockVectorY,
                 lobpcg_BLASLAPACKFunctions blap_fn,
                 lobpcg_Tolerance tolerance,
                 int maxIterations,
                 int verbosityLevel,
                 int* iterationNumber,
                 void* lambda_values,
                 void* lambdaHistory_values,
                 BlopexInt lambdaHistory_gh,
                 double* residualNorms_values,
                 double* residualNormsHistory_values,
                 BlopexInt residualNormsHistory_gh,
                 lobpcg_Interpreter* lobpcg,
                 utilities_FortranInterpreter* util);

#ifdef __cplusplus
}
#endif

#endif
