"""ctypes binding of liblobpcg_gb300.so (the C ABI in include/*.h).

There is no fallback: if the shared library is missing the import fails with
instructions to build it.
"""
from __future__ import annotations

import ctypes
import os

from .build import LIBDIR, LIBNAME

LIBPATH = os.path.join(LIBDIR, LIBNAME)

c_int, c_long, c_double, c_void_p = ctypes.c_int, ctypes.c_long, ctypes.c_double, ctypes.c_void_p
c_longlong = ctypes.c_longlong


class Tolerance(ctypes.Structure):
    _fields_ = [("absolute", c_double), ("relative", c_double)]


class BlasLapack(ctypes.Structure):
    _fields_ = [("dpotrf", c_void_p), ("dsygv", c_void_p), ("zpotrf", c_void_p), ("zhegv", c_void_p)]


class Options(ctypes.Structure):
    _fields_ = [("precision", c_int), ("compensated_below", c_double), ("fp64_below", c_double),
                ("fp32_stall", c_int), ("tensor_cores", c_int), ("potrf_fail_at", c_int),
                ("sygv_fail_at", c_int), ("explicit_pivot_below", c_double),
                ("fp32_accurate_op", c_int), ("recompute_ap", c_int), ("explicit_fp64", c_int),
                ("accum64", c_int),
                ("rr_method", c_int), ("fp32_precond", c_int), ("split_products", c_int),
                ("wait_polls", c_int)]


class Stats(ctypes.Structure):
    _fields_ = [("iterations_fp32", c_int), ("iterations_fp64", c_int),
                ("iterations_compensated", c_int), ("kernel_launches", c_longlong),
                ("seconds_total", c_double), ("seconds_fp32", c_double),
                ("seconds_fp64", c_double), ("final_max_residual", c_double),
                ("rr_calls", c_int), ("rr_jacobi32_sweeps", c_int), ("rr_max_cluster", c_int),
                ("rr_fallbacks", c_int), ("rr_graded", c_int),
                ("explicit_undos", c_int), ("explicit_p_drops", c_int),
                ("iterations_split", c_int), ("handover_reason", c_int),
                ("device_errors", c_int)]


class KernelTime(ctypes.Structure):
    _fields_ = [("name", ctypes.c_char * 24), ("launches", c_longlong), ("ms", c_double),
                ("bytes", c_double), ("flops", c_double)]


class GpuMultiVectorStruct(ctypes.Structure):
    _fields_ = [("data", c_void_p), ("size", c_long), ("ld", c_long), ("num_vectors", c_int),
                ("dtype", c_int), ("owns_data", c_int), ("num_active", c_int),
                ("active", ctypes.POINTER(c_int)), ("active_dev", c_void_p), ("ctx", c_void_p)]


# mv_InterfaceInterpreter: 26 function pointers
INTERPRETER_SLOTS = 26

# every exported symbol declared in include/*.h, with (restype, argtypes)
SIGNATURES = {
    # lobpcg.h
    "lobpcg_solve_double": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                    c_void_p, c_void_p, BlasLapack, Tolerance, c_int, c_int,
                                    ctypes.POINTER(c_int), c_void_p, c_void_p, c_int, c_void_p,
                                    c_void_p, c_int]),
    "lobpcg_solve": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                             c_void_p, c_void_p, BlasLapack, Tolerance, c_int, c_int,
                             ctypes.POINTER(c_int), c_void_p, c_void_p, c_int, c_void_p,
                             c_void_p, c_int, c_void_p, c_void_p]),
    # multivector.h
    "mv_MultiVectorGetData": (c_void_p, [c_void_p]),
    "mv_MultiVectorWrap": (c_void_p, [c_void_p, c_void_p, c_int]),
    "mv_MultiVectorCreateFromSampleVector": (c_void_p, [c_void_p, c_int, c_void_p]),
    "mv_MultiVectorCreateCopy": (c_void_p, [c_void_p, c_int]),
    "mv_MultiVectorDestroy": (None, [c_void_p]),
    "mv_MultiVectorWidth": (c_int, [c_void_p]),
    "mv_MultiVectorHeight": (c_int, [c_void_p]),
    "mv_MultiVectorSetMask": (None, [c_void_p, c_void_p]),
    "mv_MultiVectorClear": (None, [c_void_p]),
    "mv_MultiVectorSetRandom": (None, [c_void_p, c_int]),
    "mv_MultiVectorCopy": (None, [c_void_p, c_void_p]),
    "mv_MultiVectorAxpy": (None, [c_double, c_void_p, c_void_p]),
    "mv_MultiVectorByMultiVector": (None, [c_void_p, c_void_p, c_int, c_int, c_int, c_void_p]),
    "mv_MultiVectorByMultiVectorDiag": (None, [c_void_p, c_void_p, c_void_p, c_int, c_void_p]),
    "mv_MultiVectorByMatrix": (None, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p]),
    "mv_MultiVectorXapy": (None, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p]),
    "mv_MultiVectorByDiagonal": (None, [c_void_p, c_void_p, c_int, c_void_p, c_void_p]),
    "mv_MultiVectorEval": (None, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "mv_MultiVectorPrint": (None, [c_void_p, ctypes.c_char_p, c_int]),
    # fortran_matrix.h
    "utilities_FortranMatrixCreate": (c_void_p, []),
    "utilities_FortranMatrixWrap": (None, [c_void_p, c_long, c_long, c_long, c_void_p]),
    "utilities_FortranMatrixDestroy": (None, [c_void_p]),
    "utilities_FortranMatrixGlobalHeight": (c_long, [c_void_p]),
    "utilities_FortranMatrixHeight": (c_long, [c_void_p]),
    "utilities_FortranMatrixWidth": (c_long, [c_void_p]),
    "utilities_FortranMatrixValues": (c_void_p, [c_void_p]),
    "utilities_FortranMatrixFNorm": (c_double, [c_void_p]),
    "utilities_FortranMatrixAllocateData": (None, [c_long, c_long, c_void_p]),
    "utilities_FortranMatrixClear": (None, [c_void_p]),
    "utilities_FortranMatrixClearL": (None, [c_void_p]),
    "utilities_FortranMatrixSetToIdentity": (None, [c_void_p]),
    "utilities_FortranMatrixTransposeSquare": (None, [c_void_p]),
    "utilities_FortranMatrixSymmetrize": (None, [c_void_p]),
    "utilities_FortranMatrixCopy": (None, [c_void_p, c_int, c_void_p]),
    "utilities_FortranMatrixIndexCopy": (None, [c_void_p, c_void_p, c_int, c_void_p]),
    "utilities_FortranMatrixSetDiagonal": (None, [c_void_p, c_void_p]),
    "utilities_FortranMatrixGetDiagonal": (None, [c_void_p, c_void_p]),
    "utilities_FortranMatrixAdd": (None, [c_double, c_void_p, c_void_p, c_void_p]),
    "utilities_FortranMatrixDMultiply": (None, [c_void_p, c_void_p]),
    "utilities_FortranMatrixMultiplyD": (None, [c_void_p, c_void_p]),
    "utilities_FortranMatrixMultiply": (None, [c_void_p, c_int, c_void_p, c_int, c_void_p]),
    "utilities_FortranMatrixAbs": (c_double, [c_void_p, c_long, c_long]),
    "utilities_FortranMatrixValuePtr": (c_void_p, [c_void_p, c_long, c_long]),
    "utilities_FortranMatrixMaxValue": (c_double, [c_void_p]),
    "utilities_FortranMatrixSelectBlock": (None, [c_void_p, c_long, c_long, c_long, c_long,
                                                  c_void_p]),
    "utilities_FortranMatrixUpperInv": (None, [c_void_p]),
    "utilities_FortranMatrixPrint": (c_int, [c_void_p, ctypes.c_char_p]),
    # lobpcg_gb300.h
    "gpu_ContextCreate": (c_void_p, [c_int, c_void_p]),
    "gpu_ContextDestroy": (None, [c_void_p]),
    "gpu_ContextStream": (c_void_p, [c_void_p]),
    "gpu_ContextSynchronize": (c_int, [c_void_p]),
    "gpu_ContextGetOptions": (None, [c_void_p, ctypes.POINTER(Options)]),
    "gpu_ContextSetOptions": (c_int, [c_void_p, ctypes.POINTER(Options)]),
    "gpu_ContextGetStats": (None, [c_void_p, ctypes.POINTER(Stats)]),
    "gpu_ContextLastError": (ctypes.c_char_p, [c_void_p]),
    "gpu_ContextDeviceError": (c_int, [c_void_p, c_void_p]),
    "gpu_ContextSetProfiling": (c_int, [c_void_p, c_int]),
    "gpu_ContextKernelTimes": (c_int, [c_void_p, ctypes.POINTER(KernelTime), c_int]),
    "gpu_ContextResetKernelTimes": (None, [c_void_p]),
    "gpu_ContextTrim": (None, [c_void_p]),
    "gpu_KernelLaunchCount": (c_longlong, []),
    "gpu_MultiVectorCreate": (c_void_p, [c_void_p, c_long, c_int, c_int]),
    "gpu_MultiVectorWrapDevice": (c_void_p, [c_void_p, c_void_p, c_long, c_long, c_int, c_int]),
    "gpu_MultiVectorDestroy": (None, [c_void_p]),
    "gpu_MultiVectorFromHost": (c_int, [c_void_p, c_void_p, c_long]),
    "gpu_MultiVectorToHost": (c_int, [c_void_p, c_void_p, c_long]),
    "gpu_MultiVectorSetRandomValues": (c_int, [c_void_p, c_int]),
    "gpu_MultiVectorCopy": (c_int, [c_void_p, c_void_p]),
    "GpuSetupInterpreter": (c_int, [c_void_p]),
    "gpu_CSRMatrixCreate": (c_void_p, [c_void_p, c_long, c_long, c_void_p, c_void_p, c_void_p]),
    "gpu_Stencil7Create": (c_void_p, [c_void_p, c_int, c_int, c_int, c_void_p, c_void_p,
                                      c_void_p, c_double]),
    "gpu_Stencil5Create": (c_void_p, [c_void_p, c_int, c_int, c_void_p, c_void_p, c_double]),
    "gpu_Stencil27Create": (c_void_p, [c_void_p, c_int, c_int, c_int, c_void_p, c_double]),
    "gpu_DiagonalCreate": (c_void_p, [c_void_p, c_long, c_void_p]),
    "gpu_OperatorDiagonal": (c_int, [c_void_p, c_void_p]),
    "gpu_OperatorDestroy": (None, [c_void_p]),
    "gpu_PCGPreconditionerCreate": (c_void_p, [c_void_p, c_void_p, c_void_p, c_int]),
    "gpu_OperatorApply": (None, [c_void_p, c_void_p, c_void_p]),
    "gpu_ExplicitGram": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                 c_int, c_void_p, c_void_p, c_int]),
    "gpu_BlockUpdate": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_void_p, c_int]),
    "gpu_SplitGram": (c_int, [c_void_p, c_void_p, c_int, c_void_p, c_int]),
    "gpu_EigenvectorAdjoint": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                       c_void_p, c_void_p, c_void_p, c_void_p, c_void_p,
                                       c_double, c_int, c_void_p, c_void_p, c_void_p, c_void_p]),
    "gpu_OperatorParameterCount": (c_long, [c_void_p]),
    "gpu_OperatorGradient": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p]),
    "gpu_MassGradient": (c_int, [c_void_p, c_void_p, c_void_p, c_void_p, c_void_p, c_void_p]),
    "gpu_ReadHypreIJ": (c_int, [ctypes.c_char_p, c_int, ctypes.POINTER(c_long), ctypes.POINTER(c_long),
                                ctypes.POINTER(c_void_p), ctypes.POINTER(c_void_p),
                                ctypes.POINTER(c_void_p)]),
    "gpu_ReadMultiVector": (c_int, [ctypes.c_char_p, ctypes.POINTER(c_long), ctypes.POINTER(c_int),
                                    ctypes.POINTER(c_void_p)]),
    "gpu_ReadHypreParVectors": (c_int, [ctypes.c_char_p, c_int, c_int, ctypes.POINTER(c_long),
                                        ctypes.POINTER(c_void_p)]),
    "gpu_FreeHost": (None, [c_void_p]),
    "gpu_CSRMatrixLoadHypreIJ": (c_void_p, [c_void_p, ctypes.c_char_p, c_int]),
    "gpu_MultiVectorLoad": (c_void_p, [c_void_p, ctypes.c_char_p, c_int]),
    "gpu_MultiVectorLoadHypreParVectors": (c_void_p, [c_void_p, ctypes.c_char_p, c_int, c_int, c_int]),
    "gpu_GramNoAlloc": (c_int, [c_int, c_long, c_void_p, c_long, c_int, c_void_p, c_long, c_int,
                                c_void_p, c_int, c_void_p]),
}

_lib = None


def load() -> ctypes.CDLL:
    """Load liblobpcg_gb300.so and declare every entry point."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIBPATH):
        raise ImportError(f"{LIBPATH} is missing: build it with "
                          "`python -c 'import __graft_entry__ as g; g.build()'` "
                          "(there is no CPU fallback)")
    lib = ctypes.CDLL(LIBPATH)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def symbol_address(name: str) -> int:
    return ctypes.cast(getattr(load(), name), c_void_p).value
