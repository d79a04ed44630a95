"""Reverse-mode derivatives of LOBPCG eigenpairs through the C ABI, and thin
torch.autograd.Function wrappers.

The device work is in adjoint.cu / operators.cu (gpu_EigenvectorAdjoint,
gpu_OperatorGradient, gpu_MassGradient): for the k computed pairs of
A x = lambda B x and a loss L(lambda, X),

    dL/dtheta = sum_i w_i' (dA/dtheta - lambda_i dB/dtheta) x_i
                - 1/2 sum_i (g_i' x_i) x_i' (dB/dtheta) x_i,
    w_i = dL/dlambda_i x_i + sum_{j != i} x_j (x_j' g_i) / (lambda_i - lambda_j),

where g_i = dL/dx_i and the sum over the spectrum outside span(X) comes from a
projected conjugate-gradient solve of (A - lambda_i B).  The forward pass
keeps only the final eigenpairs (no iteration history).  The reference has
no derivatives; these functions have no counterpart there.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import solver as S


@dataclass
class AdjointResult:
    W: S.MultiVector          # w_i = glam_i x_i + mu_i (n x k, FP64)
    xg: np.ndarray            # g_i' x_i
    iterations: int
    max_rel_residual: float


def eigenvector_adjoint(X: S.MultiVector, lam: np.ndarray, A: S.Operator,
                        G: Optional[np.ndarray] = None, glam: Optional[np.ndarray] = None,
                        B: Optional[S.Operator] = None, T: Optional[S.Operator] = None,
                        tol: float = 1e-10, maxit: int = 2000) -> AdjointResult:
    """The adjoint vectors W of the eigenpairs (lam, X) for the cotangents
    G = dL/dX (host n x k array or None) and glam = dL/dlambda."""
    ctx = X.ctx
    lib = ctx.lib
    n, k = X.shape
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    W = S.MultiVector(ctx, n, k)
    Gm = S.MultiVector.from_host(ctx, G) if G is not None else None
    gl = np.ascontiguousarray(glam, dtype=np.float64) if glam is not None else None
    xg = np.zeros(k)
    its = ctypes.c_int(0)
    res = ctypes.c_double(0.0)
    rc = lib.gpu_EigenvectorAdjoint(
        X.handle, lam.ctypes.data, Gm.handle if Gm is not None else None,
        gl.ctypes.data if gl is not None else None,
        A.handle, A.callback,
        B.handle if B is not None else None, B.callback if B is not None else None,
        T.handle if T is not None else None, T.callback if T is not None else None,
        tol, maxit, W.handle, xg.ctypes.data, ctypes.byref(its), ctypes.byref(res))
    if rc:
        raise S.GpuError(ctx.last_error())
    return AdjointResult(W, xg, its.value, res.value)


def operator_gradient(op: S.Operator, X: S.MultiVector, W: S.MultiVector) -> np.ndarray:
    """sum_i w_i' (dA/dtheta) x_i for every parameter of op (the layout of
    gpu_OperatorParameterCount)."""
    lib = op.lib
    m = lib.gpu_OperatorParameterCount(op.handle)
    g = np.zeros(max(m, 1))
    if lib.gpu_OperatorGradient(op.handle, X.handle, W.handle, g.ctypes.data):
        raise S.GpuError(op.ctx.last_error())
    return g[:m]


def mass_gradient(B: S.Operator, X: S.MultiVector, W: S.MultiVector, lam: np.ndarray,
                  xg: Optional[np.ndarray]) -> np.ndarray:
    lam = np.ascontiguousarray(lam, dtype=np.float64)
    g = np.zeros(B.n)
    xgp = np.ascontiguousarray(xg, dtype=np.float64).ctypes.data if xg is not None else None
    if B.lib.gpu_MassGradient(B.handle, X.handle, W.handle, lam.ctypes.data, xgp, g.ctypes.data):
        raise S.GpuError(B.ctx.last_error())
    return g


# --------------------------------------------------------------- autograd
try:
    import torch
except ImportError:  # pragma: no cover - torch is part of the environment
    torch = None


@dataclass
class SolveOptions:
    k: int
    atol: float = 1e-10
    maxit: int = 1000
    seed: int = 1
    precision: int = S.FP64
    adjoint_tol: float = 1e-10
    adjoint_maxit: int = 5000
    inner_cg: int = 0  # > 0: precondition with that many CG steps on A (else Jacobi)


def _preconditioner(ctx: S.Context, A: S.Operator, opts: SolveOptions) -> S.Operator:
    J = S.Diagonal(ctx, 1.0 / A.diagonal())
    if opts.inner_cg > 0:
        return S.PCGPreconditioner(ctx, A, J, opts.inner_cg)
    return J


def _solve(ctx: S.Context, A: S.Operator, B: Optional[S.Operator], T: Optional[S.Operator],
           opts: SolveOptions):
    X = S.MultiVector(ctx, A.n, opts.k)
    X.set_random(opts.seed)
    ctx.set_options(precision=opts.precision)
    left = opts.maxit
    for _ in range(8):
        r = S.lobpcg_solve_double(X, A, B=B, T=T, atol=opts.atol, rtol=1e-50, maxit=left,
                                  history=False)
        left -= r.iterations
        # near the tolerance the Gram matrix of [X R P] can lose definiteness
        # (the reference then exits with -1): restart from the current block
        if r.flag != -1 or left <= 0:
            break
    if r.flag != 0:
        raise RuntimeError(f"LOBPCG did not converge (flag {r.flag}, {r.iterations} iterations, "
                           f"max residual {np.max(r.res):.3e})")
    return X, r.lam.copy()


def _cotangents(glam, gX):
    gl = glam.detach().cpu().numpy().astype(np.float64) if glam is not None else None
    G = None
    if gX is not None:
        G = gX.detach().cpu().numpy().astype(np.float64)
        if not np.any(G):
            G = None
    return gl, G


if torch is not None:

    class Stencil5Eigs(torch.autograd.Function):
        """(lambda, X) of the 2D 5-point operator with face coefficients cx
        (ny x nx+1) and cy (ny+1 x nx); differentiable in cx and cy."""

        @staticmethod
        def forward(fctx, cx, cy, ctx: S.Context, opts: SolveOptions):
            cxn = cx.detach().cpu().numpy().astype(np.float64)
            cyn = cy.detach().cpu().numpy().astype(np.float64)
            A = S.Stencil5(ctx, cxn, cyn)
            T = _preconditioner(ctx, A, opts)
            X, lam = _solve(ctx, A, None, T, opts)
            fctx.state = (ctx, A, T, X, lam, opts, cxn.shape, cyn.shape)
            return torch.from_numpy(lam), torch.from_numpy(X.to_host())

        @staticmethod
        def backward(fctx, glam, gX):
            ctx, A, T, X, lam, opts, sx, sy = fctx.state
            gl, G = _cotangents(glam, gX)
            adj = eigenvector_adjoint(X, lam, A, G=G, glam=gl, T=T, tol=opts.adjoint_tol,
                                      maxit=opts.adjoint_maxit)
            g = operator_gradient(A, X, adj.W)
            nx_ = int(np.prod(sx))
            return (torch.from_numpy(g[:nx_].reshape(sx)), torch.from_numpy(g[nx_:].reshape(sy)),
                    None, None)

    class Stencil27MassEigs(torch.autograd.Function):
        """(lambda, X) of A x = lambda B x with A the shifted 27-point graph
        Laplacian of edge weights w (n x 13, cell-major) and B = diag(b);
        differentiable in w and b."""

        @staticmethod
        def forward(fctx, w, b, ctx: S.Context, grid, shift: float, opts: SolveOptions):
            nx, ny, nz = grid
            wn = np.ascontiguousarray(w.detach().cpu().numpy(), dtype=np.float64)
            bn = np.ascontiguousarray(b.detach().cpu().numpy(), dtype=np.float64)
            A = S.Stencil27(ctx, nx, ny, nz, wn, shift)
            B = S.Diagonal(ctx, bn)
            T = _preconditioner(ctx, A, opts)
            X, lam = _solve(ctx, A, B, T, opts)
            fctx.state = (ctx, A, B, T, X, lam, opts, wn.shape)
            return torch.from_numpy(lam), torch.from_numpy(X.to_host())

        @staticmethod
        def backward(fctx, glam, gX):
            ctx, A, B, T, X, lam, opts, sw = fctx.state
            gl, G = _cotangents(glam, gX)
            adj = eigenvector_adjoint(X, lam, A, G=G, glam=gl, B=B, T=T, tol=opts.adjoint_tol,
                                      maxit=opts.adjoint_maxit)
            gw = operator_gradient(A, X, adj.W).reshape(sw)
            gb = mass_gradient(B, X, adj.W, lam, adj.xg)
            return torch.from_numpy(gw), torch.from_numpy(gb), None, None, None, None

    class CSREigs(torch.autograd.Function):
        """(lambda, X) of a CSR matrix with a fixed pattern (rowptr, colidx);
        differentiable in the stored values (dlambda_i/da_pq = x_i[p] x_i[q])."""

        @staticmethod
        def forward(fctx, vals, ctx: S.Context, rowptr, colidx, opts: SolveOptions):
            vn = np.ascontiguousarray(vals.detach().cpu().numpy(), dtype=np.float64)
            A = S.CSRMatrix(ctx, rowptr, colidx, vn)
            d = A.diagonal()
            T = S.Diagonal(ctx, 1.0 / d) if np.all(d > 0) else None
            X, lam = _solve(ctx, A, None, T, opts)
            fctx.state = (ctx, A, T, X, lam, opts)
            return torch.from_numpy(lam), torch.from_numpy(X.to_host())

        @staticmethod
        def backward(fctx, glam, gX):
            ctx, A, T, X, lam, opts = fctx.state
            gl, G = _cotangents(glam, gX)
            adj = eigenvector_adjoint(X, lam, A, G=G, glam=gl, T=T, tol=opts.adjoint_tol,
                                      maxit=opts.adjoint_maxit)
            return torch.from_numpy(operator_gradient(A, X, adj.W)), None, None, None, None


def stencil5_faces_torch(c):
    """Face coefficients of the 5-point operator from cell coefficients c
    (ny x nx), differentiable: interior faces the mean of the two cells,
    boundary faces the cell's own value (problems.stencil5_from_cells)."""
    cx = torch.cat([c[:, :1], 0.5 * (c[:, :-1] + c[:, 1:]), c[:, -1:]], dim=1)
    cy = torch.cat([c[:1, :], 0.5 * (c[:-1, :] + c[1:, :]), c[-1:, :]], dim=0)
    return cx, cy
