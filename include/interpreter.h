/*
 * interpreter.h -- the multivector function table (the backend seam).
 *
 * Replaces blopex_abstract/multivector/interpreter.h:11-50.  Member order and
 * signatures are unchanged: a caller fills this table (here with
 * GpuSetupInterpreter from lobpcg_gb300.h, in the reference with
 * SerialSetupInterpreter, blopex_serial_double/pcg_multi/pcg_multi.c:207)
 * and wraps its multivector with mv_MultiVectorWrap.
 *
 * Small matrices exchanged through MultiInnerProd / MultiInnerProdDiag /
 * MultiVecMat / MultiVecMatDiag are column-major HOST arrays of doubles.
 */
#ifndef BLOPEX_GB300_INTERPRETER_H
#define BLOPEX_GB300_INTERPRETER_H

#include "fortran_options.h"

typedef struct {
  /* single-vector entries (not used by the solver) */
  void* (*CreateVector)(void* vector);
  BlopexInt (*DestroyVector)(void* vector);
  BlopexInt (*InnerProd)(void* x, void* y, void* result);
  BlopexInt (*CopyVector)(void* x, void* y);
  BlopexInt (*ClearVector)(void* x);
  BlopexInt (*SetRandomValues)(void* x, BlopexInt seed);
  BlopexInt (*ScaleVector)(double alpha, void* x);
  BlopexInt (*Axpy)(void* alpha, void* x, void* y);
  BlopexInt (*VectorSize)(void* vector);

  /* multivector entries */
  void* (*CreateMultiVector)(void*, BlopexInt n, void* vector);
  void* (*CopyCreateMultiVector)(void* x, BlopexInt copyValues);
  void (*DestroyMultiVector)(void* x);
  BlopexInt (*Width)(void* x);
  BlopexInt (*Height)(void* x);
  void (*SetMask)(void* x, BlopexInt* mask);
  void (*CopyMultiVector)(void* x, void* y);
  void (*ClearMultiVector)(void* x);
  void (*SetRandomVectors)(void* x, BlopexInt seed);
  /* v(1:h,1:w) = x' * y, column-major with leading dimension gh */
  void (*MultiInnerProd)(void* x, void* y, BlopexInt gh, BlopexInt h, BlopexInt w, void* v);
  /* diag(mask) = diag(x' * y) */
  void (*MultiInnerProdDiag)(void* x, void* y, BlopexInt* mask, BlopexInt n, void* diag);
  /* y = x * v, v is h x w column-major with leading dimension gh */
  void (*MultiVecMat)(void* x, BlopexInt gh, BlopexInt h, BlopexInt w, void* v, void* y);
  /* y = x * diag(mask) */
  void (*MultiVecMatDiag)(void* x, BlopexInt* mask, BlopexInt n, void* diag, void* y);
  /* y = y + alpha * x */
  void (*MultiAxpy)(double alpha, void* x, void* y);
  void (*MultiPrint)(void* x, char* tag, BlopexInt limit);
  /* y = y + x * v */
  void (*MultiXapy)(void* x, BlopexInt gh, BlopexInt h, BlopexInt w, void* v, void* y);
  void (*Eval)(void (*f)(void*, void*, void*), void*, void* x, void* y);
} mv_InterfaceInterpreter;

#endif
