/*
 * ref_harness.c -- test infrastructure, NOT product code.
 *
 * Drives the UNMODIFIED reference BLOPEX serial-double backend
 * (blopex_abstract/krylov/lobpcg.c + blopex_serial_double/*) so that its
 * outputs can be recorded as golden vectors and used to pin the oracle
 * restatement in lobpcg_oracle.c.  The reference sources are compiled
 * where they lie by oracle/Makefile; nothing here is copied from them.
 *
 * Operators supplied to the reference (same callback signature as
 * blopex_serial_double/pcg_multi/pcg_multi.c:167 MatMultiVec):
 *   - CSR sparse A            (ref_csr_apply)
 *   - dense A (the reference's own MatMultiVec, pcg_multi.c:167-193)
 *   - diagonal operator y = d .* x  (used for B = diag and Jacobi T)
 *
 * LAPACK: the reference calls blap_fn.dsygv / blap_fn.dpotrf
 * (lobpcg.c:36, lobpcg.c:96).  The Python side hands us the function
 * pointers from scipy.linalg.cython_lapack, so no LAPACK link is needed.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "fortran_matrix.h"
#include "fortran_interpreter.h"
#include "lobpcg.h"
#include "multi_vector.h"
#include "multivector.h"
#include "pcg_multi.h"
#include "interpreter.h"

typedef void (*lapack_dsygv_t)(int*, char*, char*, int*, double*, int*,
                               double*, int*, double*, double*, int*, int*);
typedef void (*lapack_dpotrf_t)(char*, int*, double*, int*, int*);

static lapack_dsygv_t g_dsygv = NULL;
static lapack_dpotrf_t g_dpotrf = NULL;

void ref_set_lapack(void* dsygv, void* dpotrf)
{
  g_dsygv = (lapack_dsygv_t)dsygv;
  g_dpotrf = (lapack_dpotrf_t)dpotrf;
}

static BlopexInt harness_dsygv(BlopexInt* itype, char* jobz, char* uplo,
                               BlopexInt* n, double* a, BlopexInt* lda,
                               double* b, BlopexInt* ldb, double* w,
                               double* work, BlopexInt* lwork, BlopexInt* info)
{
  g_dsygv(itype, jobz, uplo, n, a, lda, b, ldb, w, work, lwork, info);
  return 0;
}

static BlopexInt harness_dpotrf(char* uplo, BlopexInt* n, double* a,
                                BlopexInt* lda, BlopexInt* info)
{
  g_dpotrf(uplo, n, a, lda, info);
  return 0;
}

/* Optional fault injection for the failure-path goldens: the Cholesky
   (resp. the generalized eigensolver) reports INFO = 1 on its Nth call
   (1-based); 0 disables. */
static int g_potrf_fail_at = 0, g_potrf_calls = 0;
static int g_sygv_fail_at = 0, g_sygv_calls = 0;

void ref_set_faults(int potrf_fail_at, int sygv_fail_at)
{
  g_potrf_fail_at = potrf_fail_at;
  g_sygv_fail_at = sygv_fail_at;
}

static BlopexInt harness_dpotrf_faulty(char* uplo, BlopexInt* n, double* a,
                                       BlopexInt* lda, BlopexInt* info)
{
  g_potrf_calls++;
  g_dpotrf(uplo, n, a, lda, info);
  if (g_potrf_calls == g_potrf_fail_at && *info == 0) *info = 1;
  return 0;
}

static BlopexInt harness_dsygv_faulty(BlopexInt* itype, char* jobz, char* uplo,
                                      BlopexInt* n, double* a, BlopexInt* lda,
                                      double* b, BlopexInt* ldb, double* w,
                                      double* work, BlopexInt* lwork, BlopexInt* info)
{
  g_sygv_calls++;
  if (g_sygv_calls == g_sygv_fail_at) {
    *info = 1;
    return 0;
  }
  g_dsygv(itype, jobz, uplo, n, a, lda, b, ldb, w, work, lwork, info);
  return 0;
}

/* ---------------- operators on serial_Multi_Vector ---------------- */

typedef struct {
  int n;
  const int* rowptr;
  const int* colidx;
  const double* vals;
} harness_csr;

static void ref_csr_apply(void* A_, void* X_, void* Y_)
{
  harness_csr* A = (harness_csr*)A_;
  serial_Multi_Vector* X = (serial_Multi_Vector*)X_;
  serial_Multi_Vector* Y = (serial_Multi_Vector*)Y_;
  int c, r, p;
  for (c = 0; c < X->num_active_vectors; c++) {
    const double* x = X->data + (long)X->active_indices[c] * X->size;
    double* y = Y->data + (long)Y->active_indices[c] * Y->size;
    for (r = 0; r < A->n; r++) {
      double s = 0.0;
      for (p = A->rowptr[r]; p < A->rowptr[r + 1]; p++)
        s += A->vals[p] * x[A->colidx[p]];
      y[r] = s;
    }
  }
}

typedef struct {
  int n;
  const double* d;
} harness_diag;

static void ref_diag_apply(void* D_, void* X_, void* Y_)
{
  harness_diag* D = (harness_diag*)D_;
  serial_Multi_Vector* X = (serial_Multi_Vector*)X_;
  serial_Multi_Vector* Y = (serial_Multi_Vector*)Y_;
  int c, r;
  for (c = 0; c < X->num_active_vectors; c++) {
    const double* x = X->data + (long)X->active_indices[c] * X->size;
    double* y = Y->data + (long)Y->active_indices[c] * Y->size;
    for (r = 0; r < D->n; r++) y[r] = D->d[r] * x[r];
  }
}

/* X0 exactly as serial_Multi_VectorSetRandomValues produces it. */
void ref_random_block(int n, int k, int seed, double* out)
{
  serial_Multi_Vector* x = serial_Multi_VectorCreate(n, k);
  serial_Multi_VectorInitialize(x);
  serial_Multi_VectorSetRandomValues(x, seed);
  memcpy(out, x->data, sizeof(double) * (size_t)n * k);
  serial_Multi_VectorDestroy(x);
}

/*
 * One call of the reference lobpcg_solve_double.
 *   A: CSR (a_rowptr != NULL) or dense column-major n*n (a_dense).
 *   b_diag / t_diag: NULL for "no B" / "no T".
 *   Y: ny constraint vectors (column-major n*ny) or ny == 0.
 *   x0 == NULL: X0 from serial_Multi_VectorSetRandomValues(seed).
 * Returns the reference's exit flag; X (n*k) is written to x_out.
 */
int ref_solve(int n, int k,
              const int* a_rowptr, const int* a_colidx, const double* a_vals,
              const double* a_dense,
              const double* b_diag, const double* t_diag,
              int ny, const double* y,
              int seed, const double* x0,
              double atol, double rtol, int maxit, int verbosity,
              double* x_out, double* lambda, double* resnorms,
              double* lambda_hist, double* res_hist, int* iterations)
{
  serial_Multi_Vector* x = serial_Multi_VectorCreate(n, k);
  serial_Multi_Vector* ymv = NULL;
  serial_Multi_Vector* adense = NULL;
  mv_InterfaceInterpreter ii;
  mv_MultiVectorPtr xx, yy = NULL;
  lobpcg_BLASLAPACKFunctions blap;
  lobpcg_Tolerance tol;
  harness_csr acsr;
  harness_diag bd, td;
  void* adata;
  void (*aop)(void*, void*, void*);
  int flag;

  serial_Multi_VectorInitialize(x);
  if (x0 != NULL)
    memcpy(x->data, x0, sizeof(double) * (size_t)n * k);
  else
    serial_Multi_VectorSetRandomValues(x, seed);

  SerialSetupInterpreter(&ii);
  xx = mv_MultiVectorWrap(&ii, x, 0);
  if (ny > 0) {
    ymv = serial_Multi_VectorCreate(n, ny);
    serial_Multi_VectorInitialize(ymv);
    memcpy(ymv->data, y, sizeof(double) * (size_t)n * ny);
    yy = mv_MultiVectorWrap(&ii, ymv, 0);
  }

  if (a_rowptr != NULL) {
    acsr.n = n; acsr.rowptr = a_rowptr; acsr.colidx = a_colidx; acsr.vals = a_vals;
    adata = &acsr;
    aop = ref_csr_apply;
  } else {
    adense = serial_Multi_VectorCreate(n, n);
    serial_Multi_VectorInitialize(adense);
    memcpy(adense->data, a_dense, sizeof(double) * (size_t)n * n);
    adata = adense;
    aop = MatMultiVec;
  }
  bd.n = n; bd.d = b_diag;
  td.n = n; td.d = t_diag;

  memset(&blap, 0, sizeof(blap));
  g_potrf_calls = 0;
  g_sygv_calls = 0;
  blap.dsygv = g_sygv_fail_at > 0 ? harness_dsygv_faulty : harness_dsygv;
  blap.dpotrf = g_potrf_fail_at > 0 ? harness_dpotrf_faulty : harness_dpotrf;
  tol.absolute = atol;
  tol.relative = rtol;

  flag = lobpcg_solve_double(xx, adata, aop,
                             b_diag ? (void*)&bd : NULL, b_diag ? ref_diag_apply : NULL,
                             t_diag ? (void*)&td : NULL, t_diag ? ref_diag_apply : NULL,
                             yy, blap, tol, maxit, verbosity, iterations,
                             lambda, lambda_hist, k, resnorms, res_hist, k);
  fflush(stdout);
  fflush(stderr);

  memcpy(x_out, x->data, sizeof(double) * (size_t)n * k);
  mv_MultiVectorDestroy(xx);
  serial_Multi_VectorDestroy(x);
  if (yy) { mv_MultiVectorDestroy(yy); serial_Multi_VectorDestroy(ymv); }
  if (adense) serial_Multi_VectorDestroy(adense);
  return flag;
}
