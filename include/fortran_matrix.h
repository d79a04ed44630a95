/*
 * fortran_matrix.h -- small column-major ("Fortran") host matrices.
 *
 * Replaces blopex_abstract/utilities/fortran_matrix.h:11-175.  The struct
 * layout is kept because callers allocate and read these objects directly
 * (e.g. blopex_hypre/krylov/HYPRE_lobpcg.c:415-417 sizes the eigenvalue and
 * residual histories with utilities_FortranMatrixAllocateData).  Only the
 * real (double) routines are provided; the complex ("z") variants belong to
 * the complex solver, which this library does not implement.
 */
#ifndef BLOPEX_GB300_FORTRAN_MATRIX_H
#define BLOPEX_GB300_FORTRAN_MATRIX_H

#include "fortran_options.h"

typedef struct {
  long globalHeight; /* leading dimension */
  long height;
  long width;
  void* value;       /* column-major storage, element (i,j) at i + j*globalHeight */
  BlopexInt ownsValues;
} utilities_FortranMatrix;

#ifdef __cplusplus
extern "C" {
#endif

/* double-complex scalar, kept for ABI compatibility of lobpcg.h */
typedef struct { double real, imag; } komplex;

utilities_FortranMatrix* utilities_FortranMatrixCreate(void);
void utilities_FortranMatrixWrap(void* values, long gh, long h, long w,
                                 utilities_FortranMatrix* mtx);
void utilities_FortranMatrixDestroy(utilities_FortranMatrix* mtx);
long utilities_FortranMatrixGlobalHeight(utilities_FortranMatrix* mtx);
long utilities_FortranMatrixHeight(utilities_FortranMatrix* mtx);
long utilities_FortranMatrixWidth(utilities_FortranMatrix* mtx);
void* utilities_FortranMatrixValues(utilities_FortranMatrix* mtx);
double utilities_FortranMatrixFNorm(utilities_FortranMatrix* mtx);

void utilities_FortranMatrixAllocateData(long h, long w, utilities_FortranMatrix* mtx);
void utilities_FortranMatrixClear(utilities_FortranMatrix* mtx);
void utilities_FortranMatrixClearL(utilities_FortranMatrix* mtx);
void utilities_FortranMatrixSetToIdentity(utilities_FortranMatrix* mtx);
void utilities_FortranMatrixTransposeSquare(utilities_FortranMatrix* mtx);
void utilities_FortranMatrixSymmetrize(utilities_FortranMatrix* mtx);
void utilities_FortranMatrixCopy(utilities_FortranMatrix* src, BlopexInt t,
                                 utilities_FortranMatrix* dest);
void utilities_FortranMatrixIndexCopy(BlopexInt* index, utilities_FortranMatrix* src,
                                      BlopexInt t, utilities_FortranMatrix* dest);
void utilities_FortranMatrixSetDiagonal(utilities_FortranMatrix* mtx,
                                        utilities_FortranMatrix* d);
void utilities_FortranMatrixGetDiagonal(utilities_FortranMatrix* mtx,
                                        utilities_FortranMatrix* d);
void utilities_FortranMatrixAdd(double a, utilities_FortranMatrix* mtxA,
                                utilities_FortranMatrix* mtxB,
                                utilities_FortranMatrix* mtxC);
void utilities_FortranMatrixDMultiply(utilities_FortranMatrix* d,
                                      utilities_FortranMatrix* mtx);
void utilities_FortranMatrixMultiplyD(utilities_FortranMatrix* mtx,
                                      utilities_FortranMatrix* d);
void utilities_FortranMatrixMultiply(utilities_FortranMatrix* mtxA, BlopexInt tA,
                                     utilities_FortranMatrix* mtxB, BlopexInt tB,
                                     utilities_FortranMatrix* mtxC);
double utilities_FortranMatrixAbs(utilities_FortranMatrix* mtx, long i, long j);
void* utilities_FortranMatrixValuePtr(utilities_FortranMatrix* mtx, long i, long j);
double utilities_FortranMatrixMaxValue(utilities_FortranMatrix* mtx);
void utilities_FortranMatrixSelectBlock(utilities_FortranMatrix* mtx, long iFrom, long iTo,
                                        long jFrom, long jTo,
                                        utilities_FortranMatrix* block);
void utilities_FortranMatrixUpperInv(utilities_FortranMatrix* u);
BlopexInt utilities_FortranMatrixPrint(utilities_FortranMatrix* mtx, char fileName[]);

#ifdef __cplusplus
}
#endif

#endif
