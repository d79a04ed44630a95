"""Readers and writers for the reference tools' file formats (HYPRE IJ matrix
files, HYPRE ParVector files, the multivector text format), through the C ABI
readers (io.c), plus device loaders.  The writers follow
blopex_tools/matlab/matlab2hypre/matlab2hypreIJ.m and
matlab2hypreParVectors.m (one file per partition)."""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from . import solver as S


def _take(ptr, n, ctype, dtype):
    arr = np.ctypeslib.as_array(ctypes.cast(ptr, ctypes.POINTER(ctype)), shape=(n,)).astype(dtype)
    return arr


def read_hypre_ij(prefix: str, nfiles: int = 1):
    """(rowptr, colidx, vals) of the CSR matrix in <prefix>.00000 ..."""
    lib = _lib.load()
    n, nnz = ctypes.c_long(), ctypes.c_long()
    rp, ci, va = ctypes.c_void_p(), ctypes.c_void_p(), ctypes.c_void_p()
    rc = lib.gpu_ReadHypreIJ(prefix.encode(), nfiles, ctypes.byref(n), ctypes.byref(nnz),
                             ctypes.byref(rp), ctypes.byref(ci), ctypes.byref(va))
    if rc:
        raise OSError(f"HYPRE IJ files {prefix}.*: read failed ({rc})")
    try:
        return (_take(rp, n.value + 1, ctypes.c_int, np.int32),
                _take(ci, max(nnz.value, 1), ctypes.c_int, np.int32)[:nnz.value],
                _take(va, max(nnz.value, 1), ctypes.c_double, np.float64)[:nnz.value])
    finally:
        for p in (rp, ci, va):
            lib.gpu_FreeHost(p)


def write_hypre_ij(prefix: str, rowptr, colidx, vals, nfiles: int = 1) -> None:
    """The matrix as HYPRE IJ files: row partitions as matlab2hypreIJ makes
    them (the first partition takes the remainder rows)."""
    n = len(rowptr) - 1
    size, rest = divmod(n, nfiles)
    bounds = [0] + list(range(rest + size, n + 1, size)) if size else [0, n]
    for f in range(nfiles):
        lo, hi = bounds[f], bounds[f + 1]
        with open(f"{prefix}.{f:05d}", "w") as fh:
            fh.write(f"{lo} {hi - 1} {lo} {hi - 1}\n")
            for r in range(lo, hi):
                for e in range(rowptr[r], rowptr[r + 1]):
                    fh.write(f"{r} {colidx[e]} {vals[e]:.15e}\n")


def read_multivector(path: str) -> np.ndarray:
    lib = _lib.load()
    n, k, d = ctypes.c_long(), ctypes.c_int(), ctypes.c_void_p()
    rc = lib.gpu_ReadMultiVector(path.encode(), ctypes.byref(n), ctypes.byref(k), ctypes.byref(d))
    if rc:
        raise OSError(f"multivector file {path}: read failed ({rc})")
    try:
        flat = _take(d, max(n.value * k.value, 1), ctypes.c_double, np.float64)[:n.value * k.value]
        return flat.reshape((k.value, n.value)).T.copy(order="F")
    finally:
        lib.gpu_FreeHost(d)


def write_multivector(path: str, x: np.ndarray) -> None:
    x = np.asarray(x, dtype=np.float64)
    with open(path, "w") as fh:
        fh.write(f"{x.shape[0]} {x.shape[1]}\n")
        for v in x.T.ravel():
            fh.write(f"{v:.17e}\n")


def read_hypre_parvectors(prefix: str, k: int, nfiles: int = 1) -> np.ndarray:
    lib = _lib.load()
    n, d = ctypes.c_long(), ctypes.c_void_p()
    rc = lib.gpu_ReadHypreParVectors(prefix.encode(), k, nfiles, ctypes.byref(n), ctypes.byref(d))
    if rc:
        raise OSError(f"ParVector files {prefix}.*: read failed ({rc})")
    try:
        flat = _take(d, max(n.value * k, 1), ctypes.c_double, np.float64)[:n.value * k]
        return flat.reshape((k, n.value)).T.copy(order="F")
    finally:
        lib.gpu_FreeHost(d)


def write_hypre_parvectors(prefix: str, x: np.ndarray, nfiles: int = 1) -> None:
    """As matlab2hypreParVectors: <prefix>.j.i with the partition's row count
    then its values, and the INFO files <prefix>.j.INFO.i."""
    x = np.asarray(x, dtype=np.float64)
    n, k = x.shape
    size, rest = divmod(n, nfiles)
    bounds = [0] + list(range(rest + size, n + 1, size)) if size else [0, n]
    for j in range(k):
        for i in range(nfiles):
            lo, hi = bounds[i], bounds[i + 1]
            with open(f"{prefix}.{j}.{i}", "w") as fh:
                fh.write(f"{hi - lo}\n")
                for v in x[lo:hi, j]:
                    fh.write(f"{v:.15e}\n")
            with open(f"{prefix}.{j}.INFO.{i}", "w") as fh:
                fh.write("\n".join(str(t) for t in [n] + bounds[:nfiles]) + "\n")


def load_csr_hypre_ij(ctx: S.Context, prefix: str, nfiles: int = 1) -> S.Operator:
    """A device CSR operator read from HYPRE IJ files (gpu_CSRMatrixLoadHypreIJ)."""
    n = 0
    for f in range(nfiles):
        with open(f"{prefix}.{f:05d}") as fh:
            n = max(n, int(fh.readline().split()[1]) + 1)
    h = ctx.lib.gpu_CSRMatrixLoadHypreIJ(ctx.handle, prefix.encode(), nfiles)
    return S.Operator(ctx, h, n)


def load_multivector(ctx: S.Context, path: str, dtype: int = S.FLOAT64) -> S.MultiVector:
    """A device block read from the multivector text format (gpu_MultiVectorLoad)."""
    with open(path) as fh:
        n, k = (int(t) for t in fh.readline().split()[:2])
    h = ctx.lib.gpu_MultiVectorLoad(ctx.handle, path.encode(), dtype)
    if not h:
        raise S.GpuError(ctx.last_error())
    mv = S.MultiVector(ctx, n, k, dtype, handle=h)
    mv.owned = True
    return mv
