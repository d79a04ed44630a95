"""The FP64-accurate split-operand tensor-core products, through the C ABI:
the block update Y = X C (+ Z) (gpu_BlockUpdate mode 2) and the Gram
G = L' [L Q_0 ..] (gpu_SplitGram), against FP64 numpy.

Error bounds follow from the splitting.  The update cuts every row of X and
every column of C into 6 digits of 7 bits (42 fraction bits below the row's /
column's power-of-two scale) and drops the digit products below level 6, so
|Y - XC| <= h * 2^-38 * rowmax|X| * colmax|C| (plus the rounding of the one
final FP64 result).  The Gram cuts each column of each 64-row chunk into 4
digits of 8 bits (32 fraction bits), so the truncation is at most 2^-29 *
64 * max|L_i| * max|Q_j| per chunk; the chunk's level 0 enters the
double-float sum over chunks exactly and the levels below it, 2^-8 smaller,
with FP32 roundings (2^-30 |L_c' Q_c|).  Integer-valued inputs split without
truncation, so those products must come out exact: that checks that the
tensor cores' FP32 accumulation of the digit products is exact."""
import numpy as np
import pytest

from blopex_gb300 import solver as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = S.Context(0)
    yield c
    c.close()


def _update(ctx, X, C, Z=None, zdtype=S.FLOAT64):
    n, h = X.shape
    w = C.shape[1]
    mx = S.MultiVector.from_host(ctx, X, S.FLOAT64)
    my = S.MultiVector(ctx, n, w, S.FLOAT64)
    mz = S.MultiVector.from_host(ctx, Z, zdtype) if Z is not None else None
    Cf = np.asfortranarray(C)
    rc = ctx.lib.gpu_BlockUpdate(mx.handle, Cf.ctypes.data, h, my.handle,
                                 mz.handle if mz is not None else None, 2)
    assert rc == 0, ctx.last_error()
    return my.to_host()


def _bound_update(X, C, Z):
    h = X.shape[1]
    rmax = np.abs(X).max(axis=1)
    cmax = np.abs(C).max(axis=0)
    b = h * 2.0 ** -38 * np.outer(rmax, cmax)
    ref = X @ C + (Z if Z is not None else 0.0)
    # FP64 rounding of the result and of numpy's own dot products
    b += 2.0 ** -52 * (np.abs(X) @ np.abs(C) * (h + 1) + (np.abs(Z) if Z is not None else 0.0))
    return ref, b


@pytest.mark.parametrize("n,h,w,z", [(1, 1, 1, None), (129, 17, 33, "f64"), (1000, 64, 64, "f32"),
                                     (100003, 64, 64, "f64"), (70000, 16, 32, None),
                                     (4097, 64, 1, "f32"), (300001, 33, 64, "f32")])
def test_split_update_matches_fp64(ctx, n, h, w, z):
    rng = np.random.default_rng(7 * n + h + w)
    X = rng.standard_normal((n, h))
    C = rng.standard_normal((h, w))
    Z = None
    if z == "f64":
        Z = rng.standard_normal((n, w))
    elif z == "f32":
        Z = rng.standard_normal((n, w)).astype(np.float32).astype(np.float64)
    Y = _update(ctx, X, C, Z, S.FLOAT64 if z == "f64" else S.FLOAT32)
    ref, b = _bound_update(X, C, Z)
    assert np.all(np.isfinite(Y))
    err = np.abs(Y - ref)
    assert np.all(err <= b), (err / b).max()


def test_split_update_wide_range_and_zeros(ctx):
    """Rows and columns spread over 40 decades, zero rows, a zero column and a
    correction Z much larger than the product on some rows."""
    rng = np.random.default_rng(11)
    n, h, w = 20000, 64, 48
    X = rng.standard_normal((n, h)) * 10.0 ** rng.uniform(-20, 20, size=(n, 1))
    X[::97] = 0.0
    X[:, 5] *= 1e-12
    C = rng.standard_normal((h, w)) * 10.0 ** rng.uniform(-10, 10, size=(1, w))
    C[:, 7] = 0.0
    Z = rng.standard_normal((n, w)) * 10.0 ** rng.uniform(-30, 30, size=(n, 1))
    Y = _update(ctx, X, C, Z, S.FLOAT64)
    ref, b = _bound_update(X, C, Z)
    err = np.abs(Y - ref)
    assert np.all(err <= b), (err / b).max()
    assert np.array_equal(Y[::97], Z[::97])


def test_split_update_fp32_z_wide_range(ctx):
    """An FP32 Z joins the product's exact integer in its units: Z far below
    the product (rounded at half a unit), comparable to it, far above it (the
    FP64 fallback), on zero rows of X and on a zero column of C."""
    rng = np.random.default_rng(13)
    n, h, w = 30000, 64, 40
    X = rng.standard_normal((n, h)) * 10.0 ** rng.uniform(-8, 8, size=(n, 1))
    X[::101] = 0.0
    C = rng.standard_normal((h, w))
    C[:, 3] = 0.0
    Z = rng.standard_normal((n, w)) * 10.0 ** rng.uniform(-30, 30, size=(n, 1))
    Z = Z.astype(np.float32).astype(np.float64)
    Y = _update(ctx, X, C, Z, S.FLOAT32)
    ref, b = _bound_update(X, C, Z)
    err = np.abs(Y - ref)
    assert np.all(err <= b), (err / b).max()
    assert np.array_equal(Y[::101], Z[::101])
    assert np.array_equal(Y[:, 3], Z[:, 3])


def test_split_update_exact_on_integers(ctx):
    """Small integers split without truncation: the result must be exact."""
    rng = np.random.default_rng(5)
    n, h, w = 50000, 64, 64
    X = rng.integers(-1000, 1001, size=(n, h)).astype(np.float64)
    C = rng.integers(-1000, 1001, size=(h, w)).astype(np.float64)
    Z = rng.integers(-10 ** 6, 10 ** 6, size=(n, w)).astype(np.float64)
    Y = _update(ctx, X, C, Z, S.FLOAT64)
    assert np.array_equal(Y, X @ C + Z)


def _gram(ctx, L, Qs, ldt=S.FLOAT64):
    h = L.shape[1]
    ml = S.MultiVector.from_host(ctx, L, ldt)
    mqs = [S.MultiVector.from_host(ctx, q, dt) for q, dt in Qs]
    import ctypes
    arr = (ctypes.c_void_p * max(1, len(mqs)))(*[m.handle for m in mqs])
    wtot = h + sum(q.shape[1] for q, _ in Qs)
    G = np.zeros((h, wtot), order="F")
    rc = ctx.lib.gpu_SplitGram(ml.handle, arr, len(mqs), G.ctypes.data, h)
    assert rc == 0, ctx.last_error()
    return G


def _bound_gram(L, R):
    n = L.shape[0]
    b = np.zeros((L.shape[1], R.shape[1]))
    c = np.zeros_like(b)
    for r0 in range(0, n, 64):
        ml = np.abs(L[r0:r0 + 64]).max(axis=0)
        mr = np.abs(R[r0:r0 + 64]).max(axis=0)
        b += 64.0 * np.outer(ml, mr)
        c += np.abs(L[r0:r0 + 64].T @ R[r0:r0 + 64])
    return 2.0 ** -29 * b + 2.0 ** -30 * c + 2.0 ** -50 * (np.abs(L).T @ np.abs(R))


@pytest.mark.parametrize("n,h,widths", [(64, 1, []), (1000, 8, [(8, "f32")]),
                                        (100003, 64, [(64, "f32"), (64, "f32")]),
                                        (262144, 32, [(17, "f64"), (64, "f32")]),
                                        (4099, 64, [(1, "f32"), (3, "f64"), (64, "f32")]),
                                        # narrow blocks of one dtype share tiles
                                        (50000, 16, [(8, "f32"), (8, "f32"), (20, "f32"), (30, "f32")]),
                                        (20000, 8, [(5, "f32"), (7, "f32"), (9, "f32"), (11, "f32")]),
                                        (7000, 5, [(3, "f64"), (2, "f64"), (4, "f32")])])
def test_split_gram_matches_fp64(ctx, n, h, widths):
    rng = np.random.default_rng(n + h)
    L = rng.standard_normal((n, h)) * np.exp(rng.standard_normal((1, h)))
    Qs = []
    for w, dt in widths:
        q = rng.standard_normal((n, w))
        if dt == "f32":
            q = q.astype(np.float32).astype(np.float64)
        Qs.append((q, S.FLOAT32 if dt == "f32" else S.FLOAT64))
    G = _gram(ctx, L, Qs)
    R = np.hstack([L] + [q for q, _ in Qs])
    ref = L.T @ R
    b = _bound_gram(L, R)
    assert np.all(np.isfinite(G))
    err = np.abs(G - ref)
    assert np.all(err <= b), (err / b).max()


def test_split_gram_unbiased_on_long_positive_sums(ctx):
    """Diagonal entries of L'L over 2^22 rows: sums of positive terms, where
    truncating accumulators lose a fixed fraction; here the relative error
    must stay near the digit resolution."""
    rng = np.random.default_rng(3)
    n, h = 1 << 22, 16
    L = rng.uniform(0.5, 1.0, size=(n, h))
    G = _gram(ctx, L, [])
    ref = np.einsum("ij,ij->j", L, L)
    rel = np.abs(np.diag(G) - ref) / ref
    assert rel.max() < 1e-8, rel.max()


def test_split_gram_exact_on_integers(ctx):
    rng = np.random.default_rng(9)
    n, h = 10000, 64
    L = rng.integers(-50, 51, size=(n, h)).astype(np.float64)
    Q = rng.integers(-50, 51, size=(n, 40)).astype(np.float32).astype(np.float64)
    G = _gram(ctx, L, [(Q, S.FLOAT32)])
    assert np.array_equal(G, L.T @ np.hstack([L, Q]))


def test_split_gram_fp32_left_block(ctx):
    """L FP32 (the mixed mode's R and P blocks, nearly dependent columns):
    R'[R AR] to the same bound."""
    rng = np.random.default_rng(21)
    n = 200003
    base = rng.standard_normal((n, 4))
    L = (base @ rng.standard_normal((4, 40)) + 1e-4 * rng.standard_normal((n, 40)))
    L = L.astype(np.float32).astype(np.float64)
    Q = rng.standard_normal((n, 64)).astype(np.float32).astype(np.float64)
    G = _gram(ctx, L, [(Q, S.FLOAT32)], ldt=S.FLOAT32)
    R = np.hstack([L, Q])
    err = np.abs(G - L.T @ R)
    assert np.all(err <= _bound_gram(L, R)), (err / _bound_gram(L, R)).max()
