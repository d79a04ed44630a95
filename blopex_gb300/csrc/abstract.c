/*
 * abstract.c -- host side of the BLOPEX C API that is not device work:
 *   the abstract multivector (an interpreter table + backend data), whose
 *   functions forward to the table (blopex_abstract/multivector/
 *   multivector.c:15-254 behaves the same way), and
 *   the column-major host small-matrix routines callers use to hold
 *   eigenvalue / residual histories (blopex_abstract/utilities/
 *   fortran_matrix.c, real routines only).
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "lobpcg.h"

struct mv_MultiVector {
  void* data;
  BlopexInt ownsData;
  mv_InterfaceInterpreter* interpreter;
};

void* mv_MultiVectorGetData(mv_MultiVectorPtr x) { return x ? x->data : NULL; }

mv_MultiVectorPtr mv_MultiVectorWrap(mv_InterfaceInterpreter* ii, void* data, BlopexInt ownsData)
{
  mv_MultiVectorPtr x = (mv_MultiVectorPtr)malloc(sizeof(*x));
  if (!x) return NULL;
  x->interpreter = ii;
  x->data = data;
  x->ownsData = ownsData;
  return x;
}

mv_MultiVectorPtr mv_MultiVectorCreateFromSampleVector(void* ii_, BlopexInt n, void* sample)
{
  mv_InterfaceInterpreter* ii = (mv_InterfaceInterpreter*)ii_;
  mv_MultiVectorPtr x;
  if (!ii || !ii->CreateMultiVector) return NULL;
  x = (mv_MultiVectorPtr)malloc(sizeof(*x));
  if (!x) return NULL;
  x->interpreter = ii;
  x->data = ii->CreateMultiVector(ii, n, sample);
  x->ownsData = 1;
  return x;
}

mv_MultiVectorPtr mv_MultiVectorCreateCopy(mv_MultiVectorPtr x, BlopexInt copyValues)
{
  mv_MultiVectorPtr y;
  if (!x) return NULL;
  y = (mv_MultiVectorPtr)malloc(sizeof(*y));
  if (!y) return NULL;
  y->interpreter = x->interpreter;
  y->data = x->interpreter->CopyCreateMultiVector(x->data, copyValues);
  y->ownsData = 1;
  return y;
}

void mv_MultiVectorDestroy(mv_MultiVectorPtr v)
{
  if (!v) return;
  if (v->ownsData) v->interpreter->DestroyMultiVector(v->data);
  free(v);
}

BlopexInt mv_MultiVectorWidth(mv_MultiVectorPtr v) { return v ? v->interpreter->Width(v->data) : 0; }

BlopexInt mv_MultiVectorHeight(mv_MultiVectorPtr v)
{
  return (v && v->interpreter->Height) ? v->interpreter->Height(v->data) : 0;
}

void mv_MultiVectorSetMask(mv_MultiVectorPtr v, BlopexInt* mask) { v->interpreter->SetMask(v->data, mask); }

void mv_MultiVectorClear(mv_MultiVectorPtr v) { v->interpreter->ClearMultiVector(v->data); }

void mv_MultiVectorSetRandom(mv_MultiVectorPtr v, BlopexInt seed)
{
  v->interpreter->SetRandomVectors(v->data, seed);
}

void mv_MultiVectorCopy(mv_MultiVectorPtr src, mv_MultiVectorPtr dest)
{
  src->interpreter->CopyMultiVector(src->data, dest->data);
}

void mv_MultiVectorAxpy(double a, mv_MultiVectorPtr x, mv_MultiVectorPtr y)
{
  x->interpreter->MultiAxpy(a, x->data, y->data);
}

void mv_MultiVectorByMultiVector(mv_MultiVectorPtr x, mv_MultiVectorPtr y, BlopexInt gh, BlopexInt h,
                                 BlopexInt w, void* v)
{
  x->interpreter->MultiInnerProd(x->data, y->data, gh, h, w, v);
}

void mv_MultiVectorByMultiVectorDiag(mv_MultiVectorPtr x, mv_MultiVectorPtr y, BlopexInt* mask,
                                     BlopexInt n, void* d)
{
  x->interpreter->MultiInnerProdDiag(x->data, y->data, mask, n, d);
}

void mv_MultiVectorByMatrix(mv_MultiVectorPtr x, BlopexInt gh, BlopexInt h, BlopexInt w, void* v,
                            mv_MultiVectorPtr y)
{
  x->interpreter->MultiVecMat(x->data, gh, h, w, v, y->data);
}

void mv_MultiVectorXapy(mv_MultiVectorPtr x, BlopexInt gh, BlopexInt h, BlopexInt w, void* v,
                        mv_MultiVectorPtr y)
{
  x->interpreter->MultiXapy(x->data, gh, h, w, v, y->data);
}

void mv_MultiVectorByDiagonal(mv_MultiVectorPtr x, BlopexInt* mask, BlopexInt n, void* d,
                              mv_MultiVectorPtr y)
{
  x->interpreter->MultiVecMatDiag(x->data, mask, n, d, y->data);
}

void mv_MultiVectorEval(void (*f)(void*, void*, void*), void* par, mv_MultiVectorPtr x,
                        mv_MultiVectorPtr y)
{
  x->interpreter->Eval(f, par, x->data, y->data);
}

void mv_MultiVectorPrint(mv_MultiVectorPtr x, char* tag, BlopexInt limit)
{
  x->interpreter->MultiPrint(x->data, tag, limit);
}

mv_InterfaceInterpreter* gb_mv_interpreter(mv_MultiVectorPtr x) { return x ? x->interpreter : NULL; }

/* ------------------------------------------------------------------ */
/* column-major host matrices                                          */
/* ------------------------------------------------------------------ */

#define EL(m, i, j) (((double*)(m)->value)[(i) + (j) * (m)->globalHeight])

utilities_FortranMatrix* utilities_FortranMatrixCreate(void)
{
  return (utilities_FortranMatrix*)calloc(1, sizeof(utilities_FortranMatrix));
}

void utilities_FortranMatrixAllocateData(long h, long w, utilities_FortranMatrix* mtx)
{
  if (mtx->value && mtx->ownsValues) free(mtx->value);
  mtx->value = calloc((size_t)(h > 0 ? h : 1) * (w > 0 ? w : 1), sizeof(double));
  mtx->globalHeight = h;
  mtx->height = h;
  mtx->width = w;
  mtx->ownsValues = 1;
}

void utilities_FortranMatrixWrap(void* v, long gh, long h, long w, utilities_FortranMatrix* mtx)
{
  if (mtx->value && mtx->ownsValues) free(mtx->value);
  mtx->value = v;
  mtx->globalHeight = gh;
  mtx->height = h;
  mtx->width = w;
  mtx->ownsValues = 0;
}

void utilities_FortranMatrixDestroy(utilities_FortranMatrix* mtx)
{
  if (!mtx) return;
  if (mtx->ownsValues && mtx->value) free(mtx->value);
  free(mtx);
}

long utilities_FortranMatrixGlobalHeight(utilities_FortranMatrix* m) { return m->globalHeight; }
long utilities_FortranMatrixHeight(utilities_FortranMatrix* m) { return m->height; }
long utilities_FortranMatrixWidth(utilities_FortranMatrix* m) { return m->width; }
void* utilities_FortranMatrixValues(utilities_FortranMatrix* m) { return m->value; }

void utilities_FortranMatrixClear(utilities_FortranMatrix* m)
{
  for (long j = 0; j < m->width; j++)
    for (long i = 0; i < m->height; i++) EL(m, i, j) = 0.0;
}

void utilities_FortranMatrixClearL(utilities_FortranMatrix* m)
{
  long w = m->width < m->height ? m->width : m->height;
  for (long j = 0; j < w; j++)
    for (long i = j + 1; i < m->height; i++) EL(m, i, j) = 0.0;
}

void utilities_FortranMatrixSetToIdentity(utilities_FortranMatrix* m)
{
  utilities_FortranMatrixClear(m);
  for (long j = 0; j < m->width && j < m->height; j++) EL(m, j, j) = 1.0;
}

void utilities_FortranMatrixTransposeSquare(utilities_FortranMatrix* m)
{
  for (long j = 0; j < m->width; j++)
    for (long i = j + 1; i < m->height; i++) {
      double t = EL(m, i, j);
      EL(m, i, j) = EL(m, j, i);
      EL(m, j, i) = t;
    }
}

void utilities_FortranMatrixSymmetrize(utilities_FortranMatrix* m)
{
  for (long j = 0; j < m->width; j++)
    for (long i = j + 1; i < m->height; i++) {
      double v = (EL(m, i, j) + EL(m, j, i)) * 0.5;
      EL(m, i, j) = v;
      EL(m, j, i) = v;
    }
}

void utilities_FortranMatrixCopy(utilities_FortranMatrix* src, BlopexInt t,
                                 utilities_FortranMatrix* dest)
{
  for (long j = 0; j < dest->width; j++)
    for (long i = 0; i < dest->height; i++) EL(dest, i, j) = t ? EL(src, j, i) : EL(src, i, j);
}

void utilities_FortranMatrixIndexCopy(BlopexInt* index, utilities_FortranMatrix* src, BlopexInt t,
                                      utilities_FortranMatrix* dest)
{
  for (long j = 0; j < dest->width; j++)
    for (long i = 0; i < dest->height; i++)
      EL(dest, i, j) = t ? EL(src, j, index[i] - 1) : EL(src, index[i] - 1, j);
}

void utilities_FortranMatrixSetDiagonal(utilities_FortranMatrix* m, utilities_FortranMatrix* d)
{
  for (long j = 0; j < m->width && j < m->height; j++) EL(m, j, j) = ((double*)d->value)[j];
}

void utilities_FortranMatrixGetDiagonal(utilities_FortranMatrix* m, utilities_FortranMatrix* d)
{
  for (long j = 0; j < m->width && j < m->height; j++) ((double*)d->value)[j] = EL(m, j, j);
}

void utilities_FortranMatrixAdd(double a, utilities_FortranMatrix* A, utilities_FortranMatrix* B,
                                utilities_FortranMatrix* C)
{
  for (long j = 0; j < C->width; j++)
    for (long i = 0; i < C->height; i++) EL(C, i, j) = a * EL(A, i, j) + EL(B, i, j);
}

void utilities_FortranMatrixDMultiply(utilities_FortranMatrix* d, utilities_FortranMatrix* m)
{
  for (long j = 0; j < m->width; j++)
    for (long i = 0; i < m->height; i++) EL(m, i, j) *= ((double*)d->value)[i];
}

void utilities_FortranMatrixMultiplyD(utilities_FortranMatrix* m, utilities_FortranMatrix* d)
{
  for (long j = 0; j < m->width; j++)
    for (long i = 0; i < m->height; i++) EL(m, i, j) *= ((double*)d->value)[j];
}

void utilities_FortranMatrixMultiply(utilities_FortranMatrix* A, BlopexInt tA,
                                     utilities_FortranMatrix* B, BlopexInt tB,
                                     utilities_FortranMatrix* C)
{
  long l = tA ? A->height : A->width;
  for (long j = 0; j < C->width; j++)
    for (long i = 0; i < C->height; i++) {
      double s = 0.0;
      for (long q = 0; q < l; q++) s += (tA ? EL(A, q, i) : EL(A, i, q)) * (tB ? EL(B, j, q) : EL(B, q, j));
      EL(C, i, j) = s;
    }
}

double utilities_FortranMatrixFNorm(utilities_FortranMatrix* m)
{
  double s = 0.0;
  for (long j = 0; j < m->width; j++)
    for (long i = 0; i < m->height; i++) s += EL(m, i, j) * EL(m, i, j);
  return sqrt(s);
}

double utilities_FortranMatrixAbs(utilities_FortranMatrix* m, long i, long j) { return fabs(EL(m, i - 1, j - 1)); }

void* utilities_FortranMatrixValuePtr(utilities_FortranMatrix* m, long i, long j) { return &EL(m, i - 1, j - 1); }

double utilities_FortranMatrixMaxValue(utilities_FortranMatrix* m)
{
  double v = EL(m, 0, 0);
  for (long j = 0; j < m->width; j++)
    for (long i = 0; i < m->height; i++)
      if (EL(m, i, j) > v) v = EL(m, i, j);
  return v;
}

void utilities_FortranMatrixSelectBlock(utilities_FortranMatrix* m, long iFrom, long iTo, long jFrom,
                                        long jTo, utilities_FortranMatrix* block)
{
  if (block->value && block->ownsValues) free(block->value);
  block->globalHeight = m->globalHeight;
  block->ownsValues = 0;
  if (iTo < iFrom || jTo < jFrom) {
    block->height = block->width = 0;
    block->value = NULL;
    return;
  }
  block->height = iTo - iFrom + 1;
  block->width = jTo - jFrom + 1;
  block->value = (double*)m->value + (iFrom - 1) + (jFrom - 1) * m->globalHeight;
}

void utilities_FortranMatrixUpperInv(utilities_FortranMatrix* u)
{
  long n = u->height;
  double* d = (double*)malloc(sizeof(double) * (n > 0 ? n : 1));
  for (long i = 0; i < n; i++) {
    d[i] = EL(u, i, i);
    EL(u, i, i) = 1.0 / d[i];
  }
  for (long i = n - 2; i >= 0; i--)
    for (long j = n - 1; j > i; j--) {
      double s = 0.0;
      for (long l = i + 1; l <= j; l++) s -= EL(u, i, l) * EL(u, l, j);
      EL(u, i, j) = s / d[i];
    }
  free(d);
}

BlopexInt utilities_FortranMatrixPrint(utilities_FortranMatrix* m, char fileName[])
{
  FILE* f = fopen(fileName, "w");
  if (!f) return 1;
  fprintf(f, "%ld\n%ld\n", m->height, m->width);
  for (long j = 0; j < m->width; j++)
    for (long i = 0; i < m->height; i++) fprintf(f, "%.14e\n", EL(m, i, j));
  fclose(f);
  return 0;
}
