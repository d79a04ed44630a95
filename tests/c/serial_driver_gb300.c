/* A C caller of the device solver, written the way the reference's
 * blopex_serial_double/driver/serial_driver.c:62-117 calls lobpcg_solve_double:
 * a 3D 7-point Dirichlet Laplacian in CSR, k Ritz pairs from a drand48 block,
 * Jacobi-free, through the mv_InterfaceInterpreter table.  Prints the
 * eigenvalues and exits 0 when the solve converged.  Compiled (and linked)
 * by tests/test_abi.py as a check that the headers are plain C99 and that
 * the library resolves every symbol a C caller uses. */
#include <stdio.h>
#include <stdlib.h>

#include "lobpcg_gb300.h"

int main(int argc, char** argv)
{
  const int g = argc > 1 ? atoi(argv[1]) : 10, k = 4;
  const long n = (long)g * g * g;
  int* rowptr = (int*)malloc(sizeof(int) * (size_t)(n + 1));
  int* colidx = (int*)malloc(sizeof(int) * (size_t)(7 * n));
  double* vals = (double*)malloc(sizeof(double) * (size_t)(7 * n));
  long nnz = 0;
  for (long r = 0; r < n; r++) {
    const long i = r % g, j = (r / g) % g, l = r / ((long)g * g);
    rowptr[r] = (int)nnz;
    const long nb[7] = {l > 0 ? r - (long)g * g : -1, j > 0 ? r - g : -1, i > 0 ? r - 1 : -1, r,
                        i < g - 1 ? r + 1 : -1, j < g - 1 ? r + g : -1,
                        l < g - 1 ? r + (long)g * g : -1};
    for (int e = 0; e < 7; e++) {
      if (nb[e] < 0) continue;
      colidx[nnz] = (int)nb[e];
      vals[nnz] = nb[e] == r ? 6.0 : -1.0;
      nnz++;
    }
  }
  rowptr[n] = (int)nnz;

  gpu_Context* ctx = gpu_ContextCreate(0, NULL);
  if (!ctx) {
    fprintf(stderr, "no device context\n");
    return 2;
  }
  gpu_Operator* A = gpu_CSRMatrixCreate(ctx, n, nnz, rowptr, colidx, vals);
  gpu_MultiVector* x = gpu_MultiVectorCreate(ctx, n, k, GPU_MV_FLOAT64);
  gpu_MultiVectorSetRandomValues(x, 1);

  mv_InterfaceInterpreter ii;
  GpuSetupInterpreter(&ii);
  mv_MultiVectorPtr xx = mv_MultiVectorWrap(&ii, x, 0);

  lobpcg_BLASLAPACKFunctions blap_fn = {0};
  lobpcg_Tolerance tol = {1e-8, 1e-50};
  double eigs[4], resid[4];
  int iterations = 0;
  const int rc = lobpcg_solve_double(xx, A, gpu_OperatorApply, NULL, NULL, NULL, NULL, NULL,
                                     blap_fn, tol, 500, 0, &iterations, eigs, NULL, 0, resid,
                                     NULL, 0);
  printf("exit %d after %d iterations\n", rc, iterations);
  for (int c = 0; c < k; c++) printf("lambda %d = %.15e  residual %.3e\n", c, eigs[c], resid[c]);

  mv_MultiVectorDestroy(xx);
  gpu_MultiVectorDestroy(x);
  gpu_OperatorDestroy(A);
  gpu_ContextDestroy(ctx);
  free(rowptr);
  free(colidx);
  free(vals);
  return rc == 0 ? 0 : 1;
}
