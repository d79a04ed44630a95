"""Python mirror of the BLOPEX C interface, backed by liblobpcg_gb300.so.

The objects here are thin owners of C-ABI handles:

* ``Context``      -> gpu_Context (device, stream, precision options, stats)
* ``MultiVector``  -> gpu_MultiVector (device-resident column-major block)
* ``CSRMatrix`` / ``Stencil7`` / ``Stencil5`` / ``Stencil27`` / ``Diagonal``
                   -> gpu_Operator (passed as operatorA/B/T with the
                      gpu_OperatorApply callback)
* ``lobpcg_solve_double`` calls the C entry point of the same name with the
  reference's argument meaning (blopex_abstract/krylov/lobpcg.h:68-113) and
  returns its outputs.
"""
from __future__ import annotations

import ctypes
import weakref
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib

FP64, MIXED = 0, 1
FLOAT64, FLOAT32 = 0, 1

EXIT_CONVERGED = 0
PROBLEM_SIZE_TOO_SMALL = 1
WRONG_BLOCK_SIZE = 2
WRONG_CONSTRAINTS = 3
REQUESTED_ACCURACY_NOT_ACHIEVED = -1


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


class GpuError(RuntimeError):
    pass


class Context:
    """A device, a stream and the solver options (gpu_Context)."""

    def __init__(self, device: int = 0, stream: Optional[int] = None, precision: int = FP64,
                 **options):
        self.lib = _lib.load()
        self.handle = self.lib.gpu_ContextCreate(device, stream)
        if not self.handle:
            raise GpuError(f"gpu_ContextCreate(device={device}) failed (no usable CUDA device?)")
        # device objects created on this context; closed before the context
        self._children = weakref.WeakSet()
        self.set_options(precision=precision, **options)

    def options(self) -> _lib.Options:
        o = _lib.Options()
        self.lib.gpu_ContextGetOptions(self.handle, ctypes.byref(o))
        return o

    def set_options(self, **kw) -> None:
        o = self.options()
        for key, val in kw.items():
            if not hasattr(o, key):
                raise KeyError(key)
            setattr(o, key, val)
        if self.lib.gpu_ContextSetOptions(self.handle, ctypes.byref(o)):
            raise GpuError(self.last_error())

    def stats(self) -> dict:
        s = _lib.Stats()
        self.lib.gpu_ContextGetStats(self.handle, ctypes.byref(s))
        return {f: getattr(s, f) for f, _ in s._fields_}

    def profiling(self, on: bool) -> None:
        self.lib.gpu_ContextSetProfiling(self.handle, 1 if on else 0)

    def reset_kernel_times(self) -> None:
        self.lib.gpu_ContextResetKernelTimes(self.handle)

    def kernel_times(self) -> dict:
        """{class: {launches, ms, bytes, flops}} from the CUDA-event timers."""
        buf = (_lib.KernelTime * 64)()
        n = self.lib.gpu_ContextKernelTimes(self.handle, buf, 64)
        return {buf[i].name.decode(): {"launches": buf[i].launches, "ms": buf[i].ms,
                                       "bytes": buf[i].bytes, "flops": buf[i].flops}
                for i in range(n)}

    def last_error(self) -> str:
        msg = self.lib.gpu_ContextLastError(self.handle)
        return msg.decode() if msg else ""

    def device_error(self) -> int:
        """The device error word (read and cleared): nonzero when a tcgen05 /
        TMA kernel gave up a bounded wait since the last read."""
        code = ctypes.c_int(0)
        if self.lib.gpu_ContextDeviceError(self.handle, ctypes.byref(code)):
            raise GpuError(self.last_error())
        return code.value

    def synchronize(self) -> None:
        if self.lib.gpu_ContextSynchronize(self.handle):
            raise GpuError(self.last_error())

    @property
    def stream(self) -> int:
        return self.lib.gpu_ContextStream(self.handle)

    def close(self) -> None:
        if self.handle:
            for child in list(self._children):
                child.close()
            self.lib.gpu_ContextDestroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class MultiVector:
    """A device block of n x k vectors (gpu_MultiVector)."""

    def __init__(self, ctx: Context, n: int, k: int, dtype: int = FLOAT64, handle=None):
        self.ctx = ctx
        self.lib = ctx.lib
        self.owned = handle is None
        self.handle = handle or self.lib.gpu_MultiVectorCreate(ctx.handle, n, k, dtype)
        if not self.handle:
            raise GpuError(ctx.last_error() or "gpu_MultiVectorCreate failed")
        ctx._children.add(self)

    @classmethod
    def from_host(cls, ctx: Context, x: np.ndarray, dtype: int = FLOAT64) -> "MultiVector":
        x = np.asfortranarray(x, dtype=np.float64)
        if x.ndim == 1:
            x = x[:, None]
        mv = cls(ctx, x.shape[0], x.shape[1], dtype)
        mv.upload(x)
        return mv

    @classmethod
    def wrap_device(cls, ctx: Context, ptr: int, n: int, ld: int, k: int,
                    dtype: int = FLOAT64) -> "MultiVector":
        h = ctx.lib.gpu_MultiVectorWrapDevice(ctx.handle, ptr, n, ld, k, dtype)
        if not h:
            raise GpuError(ctx.last_error())
        mv = cls(ctx, n, k, dtype, handle=h)
        mv.owned = True  # the wrapper object (not the memory) is ours
        return mv

    @property
    def struct(self) -> _lib.GpuMultiVectorStruct:
        return _lib.GpuMultiVectorStruct.from_address(self.handle)

    @property
    def shape(self):
        s = self.struct
        return (s.size, s.num_vectors)

    @property
    def ld(self) -> int:
        return self.struct.ld

    @property
    def data_ptr(self) -> int:
        return self.struct.data

    def upload(self, x: np.ndarray) -> None:
        x = np.asfortranarray(x, dtype=np.float64)
        if self.lib.gpu_MultiVectorFromHost(self.handle, _p(x), x.shape[0]):
            raise GpuError(self.ctx.last_error())

    def to_host(self) -> np.ndarray:
        n, k = self.shape
        out = np.zeros((n, k), order="F")
        if self.lib.gpu_MultiVectorToHost(self.handle, _p(out), n):
            raise GpuError(self.ctx.last_error())
        return out

    def upload_ptr(self, host_ptr: int, ldh: int) -> None:
        """Copy from caller host memory (column-major doubles, leading dim ldh)."""
        if self.lib.gpu_MultiVectorFromHost(self.handle, host_ptr, ldh):
            raise GpuError(self.ctx.last_error())

    def download_ptr(self, host_ptr: int, ldh: int) -> None:
        if self.lib.gpu_MultiVectorToHost(self.handle, host_ptr, ldh):
            raise GpuError(self.ctx.last_error())

    def copy_from(self, other: "MultiVector") -> None:
        if self.lib.gpu_MultiVectorCopy(other.handle, self.handle):
            raise GpuError(self.ctx.last_error())

    def set_random(self, seed: int) -> None:
        if self.lib.gpu_MultiVectorSetRandomValues(self.handle, seed):
            raise GpuError(self.ctx.last_error())

    def close(self) -> None:
        if self.handle and self.owned and self.ctx.handle:
            self.lib.gpu_MultiVectorDestroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Operator:
    """A device operator (gpu_Operator) used through gpu_OperatorApply."""

    def __init__(self, ctx: Context, handle: int, n: int):
        if not handle:
            raise GpuError(ctx.last_error() or "operator creation failed")
        self.ctx = ctx
        self.lib = ctx.lib
        self.handle = handle
        self.n = n
        ctx._children.add(self)

    @property
    def callback(self) -> int:
        return _lib.symbol_address("gpu_OperatorApply")

    def diagonal(self) -> np.ndarray:
        d = np.zeros(self.n)
        if self.lib.gpu_OperatorDiagonal(self.handle, _p(d)):
            raise GpuError(self.ctx.last_error())
        return d

    def apply(self, x: MultiVector, y: MultiVector) -> None:
        self.lib.gpu_OperatorApply(self.handle, x.handle, y.handle)
        err = self.ctx.last_error()
        if err:
            raise GpuError(err)

    def close(self) -> None:
        if self.handle and self.ctx.handle:
            self.lib.gpu_OperatorDestroy(self.handle)
        self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def CSRMatrix(ctx: Context, rowptr, colidx, vals) -> Operator:
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    colidx = np.ascontiguousarray(colidx, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    n = len(rowptr) - 1
    h = ctx.lib.gpu_CSRMatrixCreate(ctx.handle, n, len(vals), _p(rowptr), _p(colidx), _p(vals))
    return Operator(ctx, h, n)


def Stencil7(ctx: Context, cx, cy, cz, shift: float = 0.0) -> Operator:
    cx, cy, cz = (np.ascontiguousarray(c, dtype=np.float64) for c in (cx, cy, cz))
    nz, ny, nxp = cx.shape
    nx = nxp - 1
    h = ctx.lib.gpu_Stencil7Create(ctx.handle, nx, ny, nz, _p(cx), _p(cy), _p(cz), shift)
    return Operator(ctx, h, nx * ny * nz)


def Stencil5(ctx: Context, cx, cy, shift: float = 0.0) -> Operator:
    cx, cy = (np.ascontiguousarray(c, dtype=np.float64) for c in (cx, cy))
    ny, nxp = cx.shape
    nx = nxp - 1
    h = ctx.lib.gpu_Stencil5Create(ctx.handle, nx, ny, _p(cx), _p(cy), shift)
    return Operator(ctx, h, nx * ny)


def Stencil27(ctx: Context, nx: int, ny: int, nz: int, w, shift: float) -> Operator:
    w = np.ascontiguousarray(w, dtype=np.float64).reshape(-1)
    h = ctx.lib.gpu_Stencil27Create(ctx.handle, nx, ny, nz, _p(w), shift)
    return Operator(ctx, h, nx * ny * nz)


def Diagonal(ctx: Context, d) -> Operator:
    d = np.ascontiguousarray(d, dtype=np.float64)
    h = ctx.lib.gpu_DiagonalCreate(ctx.handle, len(d), _p(d))
    return Operator(ctx, h, len(d))


def PCGPreconditioner(ctx: Context, A: Operator, M: Optional[Operator], iterations: int) -> Operator:
    """T ~ inv(A) by `iterations` steps of CG preconditioned by M."""
    h = ctx.lib.gpu_PCGPreconditionerCreate(ctx.handle, A.handle, M.handle if M is not None else None,
                                            iterations)
    op = Operator(ctx, h, A.n)
    op.parts = (A, M)  # the device operator keeps raw pointers to these
    return op


class _Interp:
    """An mv_InterfaceInterpreter filled by GpuSetupInterpreter."""

    def __init__(self, lib):
        self.table = (ctypes.c_void_p * _lib.INTERPRETER_SLOTS)()
        lib.GpuSetupInterpreter(ctypes.addressof(self.table))

    @property
    def ptr(self) -> int:
        return ctypes.addressof(self.table)


@dataclass
class Result:
    flag: int
    iterations: int
    lam: np.ndarray
    res: np.ndarray
    lam_hist: Optional[np.ndarray]
    res_hist: Optional[np.ndarray]
    stats: dict


def lobpcg_solve_double(X: MultiVector, A: Operator, B: Optional[Operator] = None,
                        T: Optional[Operator] = None, Y: Optional[MultiVector] = None,
                        atol: float = 1e-6, rtol: float = 1e-50, maxit: int = 100,
                        verbosity: int = 0, history: bool = True) -> Result:
    """Call the C entry point lobpcg_solve_double on device blocks.

    X is overwritten with the Ritz vectors (as in the reference, which works
    in place on blockVectorX)."""
    lib = X.lib
    interp = _Interp(lib)
    xx = lib.mv_MultiVectorWrap(interp.ptr, X.handle, 0)
    yy = lib.mv_MultiVectorWrap(interp.ptr, Y.handle, 0) if Y is not None else None
    n, k = X.shape
    kk = max(k, 1)
    lam = np.zeros(kk)
    res = np.zeros(kk)
    lh = np.zeros((kk, maxit + 1), order="F") if history else None
    rh = np.zeros((kk, maxit + 1), order="F") if history else None
    it = ctypes.c_int(0)
    blap = _lib.BlasLapack()
    tol = _lib.Tolerance(atol, rtol)
    try:
        flag = lib.lobpcg_solve_double(
            xx, A.handle, A.callback,
            B.handle if B is not None else None, B.callback if B is not None else None,
            T.handle if T is not None else None, T.callback if T is not None else None,
            yy, blap, tol, maxit, verbosity, ctypes.byref(it),
            _p(lam), _p(lh) if lh is not None else None, kk,
            _p(res), _p(rh) if rh is not None else None, kk)
    finally:
        lib.mv_MultiVectorDestroy(xx)
        if yy:
            lib.mv_MultiVectorDestroy(yy)
    return Result(flag, it.value, lam[:k], res[:k], lh, rh, X.ctx.stats())
