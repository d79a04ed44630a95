/*
 * io.c -- readers for the file formats the reference's tools and drivers use
 * to bring external problems in, so that they can feed the device solver:
 *
 *   HYPRE IJ matrix files (blopex_tools/matlab/matlab2hypre/matlab2hypreIJ.m):
 *     one file per partition, <prefix>.00000, <prefix>.00001, ...; first line
 *     "ilower iupper jlower jupper" (0-based row / column range of the
 *     partition), then one "row col value" triple per line, 0-based, rows
 *     ascending.
 *   HYPRE ParVector files (matlab2hypreParVectors.m): for vector j and
 *     partition i the file <prefix>.j.i holds the partition's row count, then
 *     its values, one per line.
 *   multivector text (serial_Multi_VectorLoad,
 *     blopex_serial_complex/multivector/multi_vector.c:668-700): "size
 *     num_vectors", then the values column by column (the complex version
 *     reads pairs "re im"; here one real value per entry, read in full double
 *     precision where the reference's %e reads a float).
 *
 * Host parsing only; the gpu_*Load* functions upload the result.
 */
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "internal.h"

typedef struct {
  long n, cap;
  long* row;
  long* col;
  double* val;
} triplets;

static int trip_push(triplets* t, long r, long c, double v)
{
  if (t->n == t->cap) {
    long cap = t->cap ? 2 * t->cap : 1024;
    long* nr = (long*)realloc(t->row, sizeof(long) * cap);
    if (!nr) return -1;
    t->row = nr;
    long* nc = (long*)realloc(t->col, sizeof(long) * cap);
    if (!nc) return -1;
    t->col = nc;
    double* nv = (double*)realloc(t->val, sizeof(double) * cap);
    if (!nv) return -1;
    t->val = nv;
    t->cap = cap;
  }
  t->row[t->n] = r;
  t->col[t->n] = c;
  t->val[t->n] = v;
  t->n++;
  return 0;
}

static void trip_free(triplets* t)
{
  free(t->row);
  free(t->col);
  free(t->val);
}

void gpu_FreeHost(void* p) { free(p); }

int gpu_ReadHypreIJ(const char* prefix, int nfiles, long* n_out, long* nnz_out, int** rowptr_out,
                    int** colidx_out, double** vals_out)
{
  triplets t;
  memset(&t, 0, sizeof(t));
  long n = 0;
  char name[4096];
  for (int f = 0; f < nfiles; f++) {
    snprintf(name, sizeof(name), "%s.%05d", prefix, f);
    FILE* fp = fopen(name, "r");
    if (!fp) {
      trip_free(&t);
      return -1;
    }
    long il, iu, jl, ju;
    if (fscanf(fp, "%ld %ld %ld %ld", &il, &iu, &jl, &ju) != 4) {
      fclose(fp);
      trip_free(&t);
      return -2;
    }
    if (iu + 1 > n) n = iu + 1;
    long r, c;
    double v;
    while (fscanf(fp, "%ld %ld %lf", &r, &c, &v) == 3) {
      if (r < il || r > iu || c < 0) {
        fclose(fp);
        trip_free(&t);
        return -3;
      }
      if (trip_push(&t, r, c, v)) {
        fclose(fp);
        trip_free(&t);
        return -4;
      }
    }
    fclose(fp);
  }
  for (long e = 0; e < t.n; e++)
    if (t.col[e] >= n) {
      trip_free(&t);
      return -3;
    }
  int* rowptr = (int*)calloc((size_t)n + 1, sizeof(int));
  int* colidx = (int*)malloc(sizeof(int) * (size_t)(t.n > 0 ? t.n : 1));
  double* vals = (double*)malloc(sizeof(double) * (size_t)(t.n > 0 ? t.n : 1));
  if (!rowptr || !colidx || !vals) {
    free(rowptr);
    free(colidx);
    free(vals);
    trip_free(&t);
    return -4;
  }
  for (long e = 0; e < t.n; e++) rowptr[t.row[e] + 1]++;
  for (long r = 0; r < n; r++) rowptr[r + 1] += rowptr[r];
  int* fill = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
  for (long r = 0; r < n; r++) fill[r] = rowptr[r];
  for (long e = 0; e < t.n; e++) {  // stable: the file order within a row
    const int pos = fill[t.row[e]]++;
    colidx[pos] = (int)t.col[e];
    vals[pos] = t.val[e];
  }
  free(fill);
  *n_out = n;
  *nnz_out = t.n;
  *rowptr_out = rowptr;
  *colidx_out = colidx;
  *vals_out = vals;
  trip_free(&t);
  return 0;
}

int gpu_ReadMultiVector(const char* path, long* n_out, int* k_out, double** data_out)
{
  FILE* fp = fopen(path, "r");
  if (!fp) return -1;
  long n;
  int k;
  if (fscanf(fp, "%ld %d", &n, &k) != 2 || n <= 0 || k < 0) {
    fclose(fp);
    return -2;
  }
  const long total = n * k;
  // either one value per entry, or the (real, imaginary) pairs that the
  // reference's loader reads (multi_vector.c:681-693 of the complex serial
  // multivector), whose imaginary parts must then be zero
  double* raw = (double*)calloc((size_t)(2 * total + 1), sizeof(double));
  if (!raw) {
    fclose(fp);
    return -4;
  }
  long j = 0;
  double v;
  while (j <= 2 * total && fscanf(fp, "%lf", &v) == 1) raw[j++] = v;
  fclose(fp);
  double* d = (double*)calloc((size_t)(total > 0 ? total : 1), sizeof(double));
  if (!d) {
    free(raw);
    return -4;
  }
  int rc = 0;
  if (j == 2 * total && total > 0) {
    for (long e = 0; e < total; e++) {
      if (raw[2 * e + 1] != 0.0) rc = -5;  // a complex entry: not a real block
      d[e] = raw[2 * e];
    }
  } else if (j >= total) {
    memcpy(d, raw, sizeof(double) * (size_t)total);
  } else {
    rc = -2;  // short file: the reference leaves the rest as initialised (zero)
  }
  free(raw);
  if (rc) {
    free(d);
    return rc;
  }
  *n_out = n;
  *k_out = k;
  *data_out = d;
  return 0;
}

int gpu_ReadHypreParVectors(const char* prefix, int k, int nfiles, long* n_out, double** data_out)
{
  char name[4096];
  long n = 0;
  /* sizes from vector 0's partitions */
  long* part = (long*)malloc(sizeof(long) * (size_t)(nfiles > 0 ? nfiles : 1));
  if (!part) return -4;
  for (int i = 0; i < nfiles; i++) {
    snprintf(name, sizeof(name), "%s.0.%d", prefix, i);
    FILE* fp = fopen(name, "r");
    if (!fp || fscanf(fp, "%ld", &part[i]) != 1 || part[i] < 0) {
      if (fp) fclose(fp);
      free(part);
      return -1;
    }
    fclose(fp);
    n += part[i];
  }
  double* d = (double*)malloc(sizeof(double) * (size_t)(n > 0 ? n : 1) * (k > 0 ? k : 1));
  if (!d) {
    free(part);
    return -4;
  }
  for (int j = 0; j < k; j++) {
    long row = 0;
    for (int i = 0; i < nfiles; i++) {
      snprintf(name, sizeof(name), "%s.%d.%d", prefix, j, i);
      FILE* fp = fopen(name, "r");
      long nr;
      if (!fp || fscanf(fp, "%ld", &nr) != 1 || nr != part[i]) {
        if (fp) fclose(fp);
        free(part);
        free(d);
        return -2;
      }
      for (long r = 0; r < nr; r++)
        if (fscanf(fp, "%lf", &d[(size_t)j * n + row + r]) != 1) {
          fclose(fp);
          free(part);
          free(d);
          return -2;
        }
      row += nr;
      fclose(fp);
    }
  }
  free(part);
  *n_out = n;
  *data_out = d;
  return 0;
}

/* ------------------------------------------------------ device loaders */

gpu_Operator* gpu_CSRMatrixLoadHypreIJ(gpu_Context* ctx, const char* prefix, int nfiles)
{
  long n, nnz;
  int *rp, *ci;
  double* va;
  int rc = gpu_ReadHypreIJ(prefix, nfiles, &n, &nnz, &rp, &ci, &va);
  if (rc) {
    gb_fail(ctx, "HYPRE IJ files %s.*: read failed (%d)", prefix, rc);
    return NULL;
  }
  gpu_Operator* op = gpu_CSRMatrixCreate(ctx, n, nnz, rp, ci, va);
  free(rp);
  free(ci);
  free(va);
  return op;
}

static gpu_MultiVector* upload_block(gpu_Context* ctx, long n, int k, double* d, int dtype)
{
  gpu_MultiVector* x = gpu_MultiVectorCreate(ctx, n, k, dtype);
  if (x && gpu_MultiVectorFromHost(x, d, n)) {
    gpu_MultiVectorDestroy(x);
    x = NULL;
  }
  free(d);
  return x;
}

gpu_MultiVector* gpu_MultiVectorLoad(gpu_Context* ctx, const char* path, int dtype)
{
  long n;
  int k;
  double* d;
  int rc = gpu_ReadMultiVector(path, &n, &k, &d);
  if (rc) {
    gb_fail(ctx, "multivector file %s: read failed (%d)", path, rc);
    return NULL;
  }
  return upload_block(ctx, n, k, d, dtype);
}

gpu_MultiVector* gpu_MultiVectorLoadHypreParVectors(gpu_Context* ctx, const char* prefix, int k,
                                                    int nfiles, int dtype)
{
  long n;
  double* d;
  int rc = gpu_ReadHypreParVectors(prefix, k, nfiles, &n, &d);
  if (rc) {
    gb_fail(ctx, "ParVector files %s.*: read failed (%d)", prefix, rc);
    return NULL;
  }
  return upload_block(ctx, n, k, d, dtype);
}
