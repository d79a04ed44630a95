"""Helpers shared by the GPU tests: build solver inputs for a golden case."""
import numpy as np

from blopex_gb300 import solver as S


def operators_for(ctx, case):
    if case.csr is not None:
        A = S.CSRMatrix(ctx, *case.csr)
    else:
        # dense test matrices (diag(1..40)) go in as CSR
        a = np.asarray(case.dense)
        rows, cols = np.nonzero(a)
        order = np.lexsort((cols, rows))
        rows, cols = rows[order], cols[order]
        rowptr = np.zeros(a.shape[0] + 1, dtype=np.int64)
        np.add.at(rowptr, rows + 1, 1)
        rowptr = np.cumsum(rowptr)
        A = S.CSRMatrix(ctx, rowptr, cols, a[rows, cols])
    B = S.Diagonal(ctx, case.b_diag) if case.b_diag is not None else None
    T = S.Diagonal(ctx, case.t_diag) if case.t_diag is not None else None
    return A, B, T


def run_case(ctx, case, dtype=S.FLOAT64):
    A, B, T = operators_for(ctx, case)
    X = S.MultiVector.from_host(ctx, case.initial_block(), dtype)
    Y = S.MultiVector.from_host(ctx, case.Y, dtype) if case.Y is not None else None
    r = S.lobpcg_solve_double(X, A, B, T, Y, atol=case.atol, rtol=case.rtol, maxit=case.maxit)
    return r, X.to_host()


def subspace_angle(a, b, bmat=None):
    """Largest principal angle between span(a) and span(b) (B-inner product)."""
    if bmat is not None:
        s = np.sqrt(bmat)[:, None]
        a, b = a * s, b * s
    qa, _ = np.linalg.qr(a)
    qb, _ = np.linalg.qr(b)
    sv = np.linalg.svd(qa.T @ qb, compute_uv=False)
    return float(np.arccos(np.clip(sv.min(), -1.0, 1.0)))
