/*
 * fortran_options.h -- integer type and assertion macro of the BLOPEX C API.
 *
 * Replaces blopex_abstract/utilities/fortran_options.h:14-18: BlopexInt is
 * `int` unless the build overrides it (the GB300 library is built with the
 * default), and BlopexAssert maps to assert.
 */
#ifndef BLOPEX_GB300_FORTRAN_OPTIONS_H
#define BLOPEX_GB300_FORTRAN_OPTIONS_H

#ifndef BlopexInt
#define BlopexInt int
#endif

#include <assert.h>
#define BlopexAssert assert

#endif
