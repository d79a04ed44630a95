/*
 * fortran_interpreter.h -- function table for the small-matrix routines.
 *
 * Replaces blopex_abstract/utilities/fortran_interpreter.h:29-74 with the
 * same member order (the table is passed by pointer to lobpcg_solve).
 */
#ifndef BLOPEX_GB300_FORTRAN_INTERPRETER_H
#define BLOPEX_GB300_FORTRAN_INTERPRETER_H

#include "fortran_matrix.h"

typedef struct {
  utilities_FortranMatrix* (*FortranMatrixCreate)(void);
  void (*FortranMatrixAllocateData)(long, long, utilities_FortranMatrix*);
  void (*FortranMatrixWrap)(void*, long, long, long, utilities_FortranMatrix*);
  void (*FortranMatrixDestroy)(utilities_FortranMatrix*);
  long (*FortranMatrixGlobalHeight)(utilities_FortranMatrix*);
  long (*FortranMatrixHeight)(utilities_FortranMatrix*);
  long (*FortranMatrixWidth)(utilities_FortranMatrix*);
  void* (*FortranMatrixValues)(utilities_FortranMatrix*);
  void (*FortranMatrixClear)(utilities_FortranMatrix*);
  void (*FortranMatrixClearL)(utilities_FortranMatrix*);
  void (*FortranMatrixSetToIdentity)(utilities_FortranMatrix*);
  void (*FortranMatrixTransposeSquare)(utilities_FortranMatrix*);
  void (*FortranMatrixSymmetrize)(utilities_FortranMatrix*);
  void (*FortranMatrixCopy)(utilities_FortranMatrix*, BlopexInt, utilities_FortranMatrix*);
  void (*FortranMatrixIndexCopy)(BlopexInt*, utilities_FortranMatrix*, BlopexInt,
                                 utilities_FortranMatrix*);
  void (*FortranMatrixSetDiagonal)(utilities_FortranMatrix*, utilities_FortranMatrix*);
  void (*FortranMatrixGetDiagonal)(utilities_FortranMatrix*, utilities_FortranMatrix*);
  void (*FortranMatrixAdd)(double, utilities_FortranMatrix*, utilities_FortranMatrix*,
                           utilities_FortranMatrix*);
  void (*FortranMatrixDMultiply)(utilities_FortranMatrix*, utilities_FortranMatrix*);
  void (*FortranMatrixMultiplyD)(utilities_FortranMatrix*, utilities_FortranMatrix*);
  void (*FortranMatrixMultiply)(utilities_FortranMatrix*, BlopexInt,
                                utilities_FortranMatrix*, BlopexInt,
                                utilities_FortranMatrix*);
  double (*FortranMatrixFNorm)(utilities_FortranMatrix*);
  double (*FortranMatrixAbs)(utilities_FortranMatrix*, long, long);
  void* (*FortranMatrixValuePtr)(utilities_FortranMatrix*, long, long);
  double (*FortranMatrixMaxValue)(utilities_FortranMatrix*);
  void (*FortranMatrixSelectBlock)(utilities_FortranMatrix*, long, long, long, long,
                                   utilities_FortranMatrix*);
  void (*FortranMatrixUpperInv)(utilities_FortranMatrix*);
  BlopexInt (*FortranMatrixPrint)(utilities_FortranMatrix*, char fileName[]);
} utilities_FortranInterpreter;

#endif
