/*
 * multivector.h -- the abstract multivector used by the solver.
 *
 * Replaces blopex_abstract/multivector/multivector.h:23-103 (same function
 * names and signatures).  An mv_MultiVectorPtr couples backend data with the
 * mv_InterfaceInterpreter table that operates on it; every function here
 * forwards to that table.
 */
#ifndef BLOPEX_GB300_MULTIVECTOR_H
#define BLOPEX_GB300_MULTIVECTOR_H

#include "fortran_options.h"
#include "interpreter.h"

typedef struct mv_MultiVector* mv_MultiVectorPtr;

#ifdef __cplusplus
extern "C" {
#endif

void* mv_MultiVectorGetData(mv_MultiVectorPtr x);
mv_MultiVectorPtr mv_MultiVectorWrap(mv_InterfaceInterpreter* ii, void* data,
                                     BlopexInt ownsData);
mv_MultiVectorPtr mv_MultiVectorCreateFromSampleVector(void* ii, BlopexInt n, void* sample);
mv_MultiVectorPtr mv_MultiVectorCreateCopy(mv_MultiVectorPtr x, BlopexInt copyValues);
void mv_MultiVectorDestroy(mv_MultiVectorPtr x);
BlopexInt mv_MultiVectorWidth(mv_MultiVectorPtr v);
BlopexInt mv_MultiVectorHeight(mv_MultiVectorPtr v);
void mv_MultiVectorSetMask(mv_MultiVectorPtr v, BlopexInt* mask);
void mv_MultiVectorClear(mv_MultiVectorPtr x);
void mv_MultiVectorSetRandom(mv_MultiVectorPtr v, BlopexInt seed);
void mv_MultiVectorCopy(mv_MultiVectorPtr src, mv_MultiVectorPtr dest);
void mv_MultiVectorAxpy(double a, mv_MultiVectorPtr x, mv_MultiVectorPtr y);
void mv_MultiVectorByMultiVector(mv_MultiVectorPtr x, mv_MultiVectorPtr y, BlopexInt gh,
                                 BlopexInt h, BlopexInt w, void* v);
void mv_MultiVectorByMultiVectorDiag(mv_MultiVectorPtr x, mv_MultiVectorPtr y,
                                     BlopexInt* mask, BlopexInt n, void* diag);
void mv_MultiVectorByMatrix(mv_MultiVectorPtr x, BlopexInt gh, BlopexInt h, BlopexInt w,
                            void* v, mv_MultiVectorPtr y);
void mv_MultiVectorXapy(mv_MultiVectorPtr x, BlopexInt gh, BlopexInt h, BlopexInt w,
                        void* v, mv_MultiVectorPtr y);
void mv_MultiVectorByDiagonal(mv_MultiVectorPtr x, BlopexInt* mask, BlopexInt n, void* diag,
                              mv_MultiVectorPtr y);
void mv_MultiVectorEval(void (*f)(void*, void*, void*), void* par, mv_MultiVectorPtr x,
                        mv_MultiVectorPtr y);
void mv_MultiVectorPrint(mv_MultiVectorPtr x, char* tag, BlopexInt limit);

#ifdef __cplusplus
}
#endif

#endif
