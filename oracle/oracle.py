"""Test infrastructure: Python bindings for the oracle (NOT product code).

Two CPU implementations of the reference LOBPCG path live behind this module:

* ``liboracle.so`` -- the C restatement in ``oracle/lobpcg_oracle.c``
  (builds anywhere with gcc; used by the tests, by ``smoke()`` as the checker
  and by ``bench.py`` as the CPU baseline);
* ``_ref/libblopex_ref.so`` -- the UNMODIFIED reference sources compiled by
  ``oracle/Makefile`` together with ``ref_harness.c``.  It exists only where
  the reference checkout exists; it pins the restatement (golden vectors).

LAPACK (``dsygv``/``dpotrf``, called by the reference at
blopex_abstract/krylov/lobpcg.c:36 and :96) is taken from
``scipy.linalg.cython_lapack`` as raw function pointers.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass
from typing import Optional

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libblopex_ref.so")
# the reference checkout, when this machine has one (no default location)
REF_SRC = os.environ.get("BLOPEX_REFERENCE_DIR", "")

OP_NONE, OP_CSR, OP_DENSE, OP_DIAG, OP_STENCIL7, OP_STENCIL5, OP_STENCIL27, OP_PCG = range(8)


def build(ref: bool = True) -> None:
    """Compile the restatement (always) and the reference harness (when the
    reference checkout is present)."""
    subprocess.run(["make", "-s", "-C", HERE, "oracle"], check=True)
    if ref and REF_SRC and os.path.isdir(REF_SRC):
        subprocess.run(["make", "-s", "-C", HERE, "ref", f"REF={REF_SRC}"], check=True)


def build_ref_variants() -> None:
    """FMA-contracted and x87 builds of the reference (x86 only)."""
    subprocess.run(["make", "-s", "-C", HERE, "ref_variants", f"REF={REF_SRC}"], check=True)


def have_ref() -> bool:
    return os.path.exists(REF_SO)


def lapack_ptrs() -> tuple[int, int]:
    """Addresses of LAPACK dsygv and dpotrf (Fortran ABI, 32-bit ints)."""
    import scipy.linalg.cython_lapack as cl

    get = ctypes.pythonapi.PyCapsule_GetPointer
    get.restype = ctypes.c_void_p
    get.argtypes = [ctypes.py_object, ctypes.c_char_p]
    caps = cl.__pyx_capi__

    def ptr(name):
        cap = caps[name]
        nm = ctypes.pythonapi.PyCapsule_GetName
        nm.restype = ctypes.c_char_p
        nm.argtypes = [ctypes.py_object]
        return get(cap, nm(cap))

    return ptr("dsygv"), ptr("dpotrf")


class _OpC(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int), ("data", ctypes.c_void_p)]


class _CSR(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int), ("rowptr", ctypes.c_void_p),
                ("colidx", ctypes.c_void_p), ("vals", ctypes.c_void_p)]


class _ST7(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("cx", ctypes.c_void_p), ("cy", ctypes.c_void_p), ("cz", ctypes.c_void_p),
                ("shift", ctypes.c_double)]


class _ST5(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int),
                ("cx", ctypes.c_void_p), ("cy", ctypes.c_void_p), ("shift", ctypes.c_double)]


class _ST27(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("w", ctypes.c_void_p), ("shift", ctypes.c_double)]


class _PCG(ctypes.Structure):
    _fields_ = [("A", _OpC), ("M", _OpC), ("iters", ctypes.c_int)]


def _p(a: np.ndarray) -> int:
    return a.ctypes.data


@dataclass
class Operator:
    """An oracle operator: keeps its arrays alive next to the C struct."""
    kind: int
    struct: object = None
    keep: tuple = ()


NONE = Operator(OP_NONE)


def csr(rowptr, colidx, vals) -> Operator:
    rowptr = np.ascontiguousarray(rowptr, dtype=np.int32)
    colidx = np.ascontiguousarray(colidx, dtype=np.int32)
    vals = np.ascontiguousarray(vals, dtype=np.float64)
    s = _CSR(len(rowptr) - 1, _p(rowptr), _p(colidx), _p(vals))
    return Operator(OP_CSR, s, (rowptr, colidx, vals))


def diag(d) -> Operator:
    d = np.ascontiguousarray(d, dtype=np.float64)
    return Operator(OP_DIAG, ctypes.c_double.from_address(_p(d)), (d,))


def dense(a) -> Operator:
    a = np.asfortranarray(a, dtype=np.float64)
    return Operator(OP_DENSE, ctypes.c_double.from_address(_p(a)), (a,))


def stencil7(nx, ny, nz, cx, cy, cz, shift=0.0) -> Operator:
    cx, cy, cz = (np.ascontiguousarray(c, dtype=np.float64).ravel() for c in (cx, cy, cz))
    s = _ST7(nx, ny, nz, _p(cx), _p(cy), _p(cz), shift)
    return Operator(OP_STENCIL7, s, (cx, cy, cz))


def stencil5(nx, ny, cx, cy, shift=0.0) -> Operator:
    cx, cy = (np.ascontiguousarray(c, dtype=np.float64).ravel() for c in (cx, cy))
    s = _ST5(nx, ny, _p(cx), _p(cy), shift)
    return Operator(OP_STENCIL5, s, (cx, cy))


def stencil27(nx, ny, nz, w, shift) -> Operator:
    w = np.ascontiguousarray(w, dtype=np.float64).ravel()
    s = _ST27(nx, ny, nz, _p(w), shift)
    return Operator(OP_STENCIL27, s, (w,))


def _opc_ptr(op: Operator) -> ctypes.c_void_p:
    if op.struct is None:
        return None
    if isinstance(op.struct, ctypes.c_double):
        return ctypes.c_void_p(ctypes.addressof(op.struct))
    return ctypes.cast(ctypes.pointer(op.struct), ctypes.c_void_p)


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(ORACLE_SO):
            build(ref=False)
        L = ctypes.CDLL(ORACLE_SO)
        L.oracle_solve.restype = ctypes.c_int
        L.oracle_solve.argtypes = [
            ctypes.c_long, ctypes.c_int, _OpC, _OpC, _OpC,
            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_double, ctypes.c_double, ctypes.c_int,
            ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.POINTER(ctypes.c_int)]
        L.oracle_set_faults.argtypes = [ctypes.c_int, ctypes.c_int]
        L.oracle_apply.restype = None
        L.oracle_apply.argtypes = [ctypes.c_long, ctypes.c_int, _OpC,
                                   ctypes.c_void_p, ctypes.c_void_p]
        _lib = L
    return _lib


def _opc(op: Operator) -> _OpC:
    return _OpC(op.kind, _opc_ptr(op))


def pcg(A: Operator, M: Operator, iters: int) -> Operator:
    """T ~ inv(A) by `iters` steps of CG on A preconditioned by M (NONE: none),
    the inner preconditioner of HYPRE's LOBPCG driver with -pcgitr
    (blopex_hypre/krylov/HYPRE_lobpcg.c:317-320)."""
    s = _PCG(_opc(A), _opc(M), iters)
    return Operator(OP_PCG, s, (A, M))


@dataclass
class Result:
    flag: int
    iterations: int
    x: np.ndarray
    lam: np.ndarray
    res: np.ndarray
    lam_hist: Optional[np.ndarray]
    res_hist: Optional[np.ndarray]


def solve(A: Operator, x0: np.ndarray, B: Operator = NONE, T: Operator = NONE,
          Y: Optional[np.ndarray] = None, atol: float = 1e-6, rtol: float = 1e-50,
          maxit: int = 100, history: bool = True, potrf_fail_at: int = 0,
          sygv_fail_at: int = 0) -> Result:
    """Run the C restatement of lobpcg_solve_double (lobpcg.c:332-413).
    ``potrf_fail_at``/``sygv_fail_at`` inject INFO = 1 into the Nth call of
    the Cholesky / generalized eigensolver (host-side fault injection)."""
    x = np.array(x0, dtype=np.float64, order="F", copy=True)
    n, k = x.shape
    lam = np.zeros(max(k, 1))
    res = np.zeros(max(k, 1))
    lh = np.zeros((k, maxit + 1), order="F") if history else None
    rh = np.zeros((k, maxit + 1), order="F") if history else None
    if Y is not None:
        Y = np.asfortranarray(Y, dtype=np.float64)
    it = ctypes.c_int(0)
    sygv, potrf = lapack_ptrs()
    L = lib()
    L.oracle_set_faults(potrf_fail_at, sygv_fail_at)
    try:
        flag = L.oracle_solve(n, k, _opc(A), _opc(B), _opc(T),
                              0 if Y is None else Y.shape[1], None if Y is None else _p(Y),
                              _p(x), atol, rtol, maxit, sygv, potrf,
                              _p(lam), _p(res), None if lh is None else _p(lh),
                              None if rh is None else _p(rh), ctypes.byref(it))
    finally:
        L.oracle_set_faults(0, 0)
    return Result(flag, it.value, x, lam[:k], res[:k], lh, rh)


def apply(op: Operator, x: np.ndarray) -> np.ndarray:
    """y = op(x) column by column (CPU restatement of the operator)."""
    x = np.asfortranarray(x, dtype=np.float64)
    if x.ndim == 1:
        x = x[:, None]
    y = np.zeros_like(x, order="F")
    lib().oracle_apply(x.shape[0], x.shape[1], _opc(op), _p(x), _p(y))
    return y


# ---------------------------------------------------------------------------
# the unmodified reference (only where the reference checkout was compiled)
# ---------------------------------------------------------------------------

_ref = {}


def ref_lib(variant: str = ""):
    """The compiled reference; variant "" (plain -O2), "fma" or "x87"."""
    if variant not in _ref:
        path = REF_SO if not variant else REF_SO.replace(".so", f"_{variant}.so")
        if not os.path.exists(path):
            raise RuntimeError(f"reference harness not built ({path} missing)")
        L = ctypes.CDLL(path)
        L.ref_set_lapack.argtypes = [ctypes.c_void_p, ctypes.c_void_p]
        L.ref_random_block.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_void_p]
        L.ref_solve.restype = ctypes.c_int
        L.ref_solve.argtypes = [
            ctypes.c_int, ctypes.c_int,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_int, ctypes.c_void_p,
            ctypes.c_int, ctypes.c_void_p,
            ctypes.c_double, ctypes.c_double, ctypes.c_int, ctypes.c_int,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
            ctypes.c_void_p, ctypes.c_void_p, ctypes.POINTER(ctypes.c_int)]
        L.ref_set_faults.argtypes = [ctypes.c_int, ctypes.c_int]
        L.ref_set_lapack(*lapack_ptrs())
        _ref[variant] = L
    return _ref[variant]


def ref_random_block(n: int, k: int, seed: int) -> np.ndarray:
    out = np.zeros((n, k), order="F")
    ref_lib().ref_random_block(n, k, seed, _p(out))
    return out


def ref_solve(n: int, k: int, csr_arrays=None, dense_a=None, b_diag=None, t_diag=None,
              Y=None, seed: int = 0, x0=None, atol=1e-6, rtol=1e-50, maxit=100,
              verbosity=0, potrf_fail_at=0, sygv_fail_at=0, variant: str = "") -> Result:
    """Run the reference lobpcg_solve_double with the serial backend."""
    L = ref_lib(variant)
    keep = []

    def arr(a, dt):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=dt) if a.ndim == 1 else np.asfortranarray(a, dtype=dt)
        keep.append(a)
        return _p(a)

    rp = ci = va = None
    if csr_arrays is not None:
        rp, ci, va = (arr(csr_arrays[0], np.int32), arr(csr_arrays[1], np.int32),
                      arr(csr_arrays[2], np.float64))
    dn = arr(dense_a, np.float64) if dense_a is not None else None
    x = np.zeros((n, k), order="F")
    lam = np.zeros(max(k, 1))
    res = np.zeros(max(k, 1))
    lh = np.zeros((k, maxit + 1), order="F")
    rh = np.zeros((k, maxit + 1), order="F")
    it = ctypes.c_int(0)
    ny = 0 if Y is None else Y.shape[1]
    L.ref_set_faults(potrf_fail_at, sygv_fail_at)
    try:
        flag = L.ref_solve(n, k, rp, ci, va, dn, arr(b_diag, np.float64),
                           arr(t_diag, np.float64),
                           ny, arr(Y, np.float64) if Y is not None else None,
                           seed, arr(x0, np.float64) if x0 is not None else None,
                           atol, rtol, maxit, verbosity,
                           _p(x), _p(lam), _p(res), _p(lh), _p(rh), ctypes.byref(it))
    finally:
        L.ref_set_faults(0, 0)
    return Result(flag, it.value, x, lam[:k], res[:k], lh, rh)
