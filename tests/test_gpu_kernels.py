"""Device kernels through the C ABI against the oracle / numpy (FP64 and FP32)."""
import numpy as np
import pytest

from blopex_gb300 import problems as P
from blopex_gb300 import solver as S
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = S.Context(0)
    yield c
    c.close()


def test_drand48_device_bit_exact(ctx):
    for n, k, seed in ((40, 5, 1), (8000, 10, 0), (1003, 7, 12345)):
        X = S.MultiVector(ctx, n, k)
        X.set_random(seed)
        assert np.array_equal(X.to_host(), P.drand48_block(n, k, seed))


@pytest.mark.parametrize("dtype,rtol", [(S.FLOAT64, 1e-13), (S.FLOAT32, 2e-5)])
@pytest.mark.parametrize("n,h,w", [(1, 1, 1), (37, 3, 5), (4099, 17, 33), (20000, 96, 64)])
def test_gram_matches_numpy(ctx, dtype, rtol, n, h, w):
    rng = np.random.default_rng(n + h + w)
    x = rng.standard_normal((n, h))
    y = rng.standard_normal((n, w))
    if dtype == S.FLOAT32:
        x, y = x.astype(np.float32).astype(np.float64), y.astype(np.float32).astype(np.float64)
    X = S.MultiVector.from_host(ctx, x, dtype)
    Yv = S.MultiVector.from_host(ctx, y, dtype)
    interp = S._Interp(ctx.lib)
    xx = ctx.lib.mv_MultiVectorWrap(interp.ptr, X.handle, 0)
    yy = ctx.lib.mv_MultiVectorWrap(interp.ptr, Yv.handle, 0)
    gh = h + 3
    v = np.full((gh, w), 7.0, order="F")
    ctx.lib.mv_MultiVectorByMultiVector(xx, yy, gh, h, w, v.ctypes.data)
    ref = x.T @ y
    scale = np.sqrt(np.outer((x * x).sum(0), (y * y).sum(0)))
    assert np.all(np.abs(v[:h] - ref) <= rtol * scale + 1e-300)
    assert np.all(v[h:] == 7.0)
    ctx.lib.mv_MultiVectorDestroy(xx)
    ctx.lib.mv_MultiVectorDestroy(yy)


@pytest.mark.parametrize("dtype", [S.FLOAT64, S.FLOAT32])
@pytest.mark.parametrize("n,h", [(1, 1), (300, 7), (4099, 32), (70001, 33), (20000, 64)])
def test_symmetric_gram_bit_identical(ctx, dtype, n, h):
    """X'X of one block takes the lower-triangle kernel; the same product of
    two distinct copies takes the full kernel.  Same splits, same order of
    multiply-adds: the results agree bit for bit, and X'X is symmetric."""
    rng = np.random.default_rng(n * 7 + h)
    x = rng.standard_normal((n, h))
    X = S.MultiVector.from_host(ctx, x, dtype)
    X2 = S.MultiVector.from_host(ctx, x, dtype)
    interp = S._Interp(ctx.lib)
    xx = ctx.lib.mv_MultiVectorWrap(interp.ptr, X.handle, 0)
    x2 = ctx.lib.mv_MultiVectorWrap(interp.ptr, X2.handle, 0)
    sym = np.zeros((h, h), order="F")
    full = np.zeros((h, h), order="F")
    ctx.lib.mv_MultiVectorByMultiVector(xx, xx, h, h, h, sym.ctypes.data)
    ctx.lib.mv_MultiVectorByMultiVector(xx, x2, h, h, h, full.ctypes.data)
    ctx.lib.mv_MultiVectorDestroy(xx)
    ctx.lib.mv_MultiVectorDestroy(x2)
    assert np.array_equal(sym, np.tril(full) + np.tril(full, -1).T)
    assert np.array_equal(sym, full)
    xr = x.astype(np.float32).astype(np.float64) if dtype == S.FLOAT32 else x
    np.testing.assert_allclose(sym, xr.T @ xr, rtol=0,
                               atol=(1e-13 if dtype == S.FLOAT64 else 2e-5) * n)


@pytest.mark.parametrize("dtype,rtol", [(S.FLOAT64, 1e-13), (S.FLOAT32, 2e-5)])
@pytest.mark.parametrize("n,h,w", [(5, 1, 1), (1000, 10, 10), (70001, 40, 33)])
def test_bymatrix_matches_numpy(ctx, dtype, rtol, n, h, w):
    rng = np.random.default_rng(3 * n + h)
    x = rng.standard_normal((n, h))
    c = rng.standard_normal((h + 2, w))
    if dtype == S.FLOAT32:
        x = x.astype(np.float32).astype(np.float64)
    X = S.MultiVector.from_host(ctx, x, dtype)
    Yv = S.MultiVector(ctx, n, w, dtype)
    interp = S._Interp(ctx.lib)
    xx = ctx.lib.mv_MultiVectorWrap(interp.ptr, X.handle, 0)
    yy = ctx.lib.mv_MultiVectorWrap(interp.ptr, Yv.handle, 0)
    cf = np.asfortranarray(c)
    ctx.lib.mv_MultiVectorByMatrix(xx, h + 2, h, w, cf.ctypes.data, yy)
    ref = x @ c[:h]
    scale = np.abs(x) @ np.abs(c[:h])
    assert np.all(np.abs(Yv.to_host() - ref) <= rtol * scale + 1e-300)
    ctx.lib.mv_MultiVectorDestroy(xx)
    ctx.lib.mv_MultiVectorDestroy(yy)


def _ops(ctx):
    rng = np.random.default_rng(7)
    out = []
    rp, ci, va = P.laplacian3d_csr(9, 7, 5)
    out.append((S.CSRMatrix(ctx, rp, ci, va), O.csr(rp, ci, va), 315))
    # rows of 1 to ~40 entries: the FP32 kernel's register path and its long-row loop
    m = 300
    dense = np.zeros((m, m))
    for i in range(m):
        cols = rng.choice(m, size=int(rng.integers(0, 20)), replace=False)
        dense[i, cols] = rng.standard_normal(cols.size)
    dense = dense + dense.T + np.diag(rng.uniform(1.0, 2.0, m))
    rows, cols = np.nonzero(dense)
    rp = np.searchsorted(rows, np.arange(m + 1)).astype(np.int32)
    ci = cols.astype(np.int32)
    va = dense[rows, cols]
    assert np.diff(rp).max() > 8 and np.diff(rp).min() <= 8
    out.append((S.CSRMatrix(ctx, rp, ci, va), O.csr(rp, ci, va), m))
    cx, cy, cz = P.stencil7_coefficients(11, 6, 5, seed=2)
    out.append((S.Stencil7(ctx, cx, cy, cz, 0.3), O.stencil7(11, 6, 5, cx, cy, cz, 0.3), 330))
    # several (x, y) tiles and z chunks of the blocked kernel, ragged edges
    cx, cy, cz = P.stencil7_coefficients(37, 9, 70, seed=5)
    out.append((S.Stencil7(ctx, cx, cy, cz, 0.0), O.stencil7(37, 9, 70, cx, cy, cz, 0.0), 23310))
    # nx a multiple of 4: the FP32 column-ring kernel (ragged and whole tiles)
    cx, cy, cz = P.stencil7_coefficients(44, 10, 6, seed=8)
    out.append((S.Stencil7(ctx, cx, cy, cz, 0.2), O.stencil7(44, 10, 6, cx, cy, cz, 0.2), 2640))
    cx, cy, cz = P.stencil7_coefficients(64, 40, 3, seed=9)
    out.append((S.Stencil7(ctx, cx, cy, cz, 0.0), O.stencil7(64, 40, 3, cx, cy, cz, 0.0), 7680))
    c = np.exp(rng.standard_normal((13, 17)))
    sx, sy = P.stencil5_from_cells(c)
    out.append((S.Stencil5(ctx, sx, sy, 0.1), O.stencil5(17, 13, sx, sy, 0.1), 221))
    w = P.stencil27_weights(6, 5, 7, seed=4)
    out.append((S.Stencil27(ctx, 6, 5, 7, w, 0.5), O.stencil27(6, 5, 7, w, 0.5), 210))
    d = rng.uniform(0.5, 1.5, 333)
    out.append((S.Diagonal(ctx, d), O.diag(d), 333))
    return out


@pytest.mark.parametrize("dtype,rtol", [(S.FLOAT64, 1e-13), (S.FLOAT32, 3e-6)])
def test_operators_match_oracle(ctx, dtype, rtol):
    rng = np.random.default_rng(11)
    for gop, oop, n in _ops(ctx):
        for k in (1, 3, 17):
            x = rng.standard_normal((n, k))
            if dtype == S.FLOAT32:
                x = x.astype(np.float32).astype(np.float64)
            X = S.MultiVector.from_host(ctx, x, dtype)
            Yv = S.MultiVector(ctx, n, k, dtype)
            gop.apply(X, Yv)
            ref = O.apply(oop, x)
            scale = O.apply(oop, np.abs(x)) if oop.kind == O.OP_DIAG else np.abs(ref).max()
            np.testing.assert_allclose(Yv.to_host(), ref, rtol=0, atol=rtol * np.max(scale) * 10)


def test_operator_diagonal(ctx):
    for gop, oop, n in _ops(ctx):
        e = np.zeros(n)
        d = np.empty(n)
        for i in range(n):
            e[:] = 0
            e[i] = 1
            d[i] = O.apply(oop, e)[i, 0]
        np.testing.assert_allclose(gop.diagonal(), d, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("n", [1, 5, 4099, 1000003])
def test_fp32_dot_products_fp64_accurate(ctx, n):
    """Column inner products of FP32 blocks (mv_MultiVectorByMultiVectorDiag,
    blockops.cu's FP32 path): exact products in a compensated FP32 sum
    flushed to FP64, so |error| <= 1e-12 sum |x_i y_i| although the data are
    FP32 and no FP64 arithmetic runs per element."""
    rng = np.random.default_rng(n)
    k = 7
    x = rng.standard_normal((n, k)).astype(np.float32).astype(np.float64)
    y = (rng.standard_normal((n, k)) * 10.0 ** rng.uniform(-3, 3, size=(n, 1)))
    y = y.astype(np.float32).astype(np.float64)
    X = S.MultiVector.from_host(ctx, x, S.FLOAT32)
    Y = S.MultiVector.from_host(ctx, y, S.FLOAT32)
    interp = S._Interp(ctx.lib)
    xx = ctx.lib.mv_MultiVectorWrap(interp.ptr, X.handle, 0)
    yy = ctx.lib.mv_MultiVectorWrap(interp.ptr, Y.handle, 0)
    d = np.zeros(k)
    ctx.lib.mv_MultiVectorByMultiVectorDiag(xx, yy, None, k, d.ctypes.data)
    ctx.lib.mv_MultiVectorDestroy(xx)
    ctx.lib.mv_MultiVectorDestroy(yy)
    assert ctx.last_error() == ""
    ref = np.einsum("ij,ij->j", x, y)  # products exact in FP64
    assert np.all(np.abs(d - ref) <= 1e-12 * np.einsum("ij,ij->j", np.abs(x), np.abs(y)))


def _cg_reference(A, M, X, steps):
    """The inner-CG recurrence of gpu_PCGPreconditionerCreate in FP64 numpy."""
    Y = np.zeros_like(X)
    for j in range(X.shape[1]):
        r = X[:, j].copy()
        z = M * r if M is not None else r.copy()
        p = z.copy()
        rho = r @ z
        y = np.zeros_like(r)
        for it in range(steps):
            q = A @ p
            alpha = rho / (p @ q) if rho != 0 else 0.0
            y += alpha * p
            r -= alpha * q
            if it + 1 == steps:
                break
            z = M * r if M is not None else r
            rho2 = r @ z
            beta = rho2 / rho if rho != 0 else 0.0
            p = z + beta * p
            rho = rho2
        Y[:, j] = y
    return Y


@pytest.mark.parametrize("dtype", [S.FLOAT32, S.FLOAT64])
@pytest.mark.parametrize("jacobi", [True, False])
@pytest.mark.parametrize("grid", [(13, 11, 7), (16, 16, 16)])
def test_pcg_preconditioner_matches_cg(ctx, dtype, jacobi, grid):
    """T X by the inner-CG preconditioner (FP32: the fused float4 kernels, a
    ragged n % 4 tail included; FP64: the column kernels) against the same
    recurrence in FP64 numpy."""
    import scipy.sparse as sp
    nx, ny, nz = grid
    n, w, steps = nx * ny * nz, 5, 8
    cx, cy, cz = P.stencil7_coefficients(nx, ny, nz, seed=7)
    rp, ci, va = P.stencil7_to_csr(cx, cy, cz)
    Acsr = sp.csr_matrix((va, ci, rp), shape=(n, n))
    if dtype == S.FLOAT32:
        # the FP32 operator and Jacobi weights, as the device applies them
        Acsr = sp.csr_matrix((va.astype(np.float32).astype(np.float64), ci, rp), shape=(n, n))
    M = 1.0 / P.stencil7_diagonal(cx, cy, cz)
    A = S.Stencil7(ctx, cx, cy, cz)
    Mop = S.Diagonal(ctx, M) if jacobi else None
    T = S.PCGPreconditioner(ctx, A, Mop, steps)
    rng = np.random.default_rng(n)
    x = rng.standard_normal((n, w))
    if dtype == S.FLOAT32:
        x = x.astype(np.float32).astype(np.float64)
        M = M.astype(np.float32).astype(np.float64)
    X = S.MultiVector.from_host(ctx, x, dtype)
    Y = S.MultiVector(ctx, n, w, dtype)
    T.apply(X, Y)
    ref = _cg_reference(Acsr, M if jacobi else None, x, steps)
    tol = 1e-10 if dtype == S.FLOAT64 else 2e-4
    err = np.linalg.norm(Y.to_host() - ref, axis=0) / np.linalg.norm(ref, axis=0)
    assert np.all(err <= tol), err
