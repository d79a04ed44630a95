"""gpu_GramNoAlloc: the Gram product for callers that cannot allocate device
memory on this path (e.g. inside another framework's memory pool, or where
a cudaMalloc's implicit synchronisation is not acceptable).  It is checked
through the C ABI against the allocating Gram entry point
(mv_MultiVectorByMultiVector on the GPU interpreter) on two calls in a row,
so that scratch contents left by the first call cannot leak into the
second.  This file is collected last on purpose."""
import ctypes

import numpy as np
import pytest

from blopex_gb300 import solver as S

pytestmark = pytest.mark.gpu


def _gram_allocating(ctx, X, Y, h, w):
    interp = S._Interp(ctx.lib)
    xx = ctx.lib.mv_MultiVectorWrap(interp.ptr, X.handle, 0)
    yy = ctx.lib.mv_MultiVectorWrap(interp.ptr, Y.handle, 0)
    v = np.zeros((h, w), order="F")
    ctx.lib.mv_MultiVectorByMultiVector(xx, yy, h, h, w, v.ctypes.data)
    ctx.lib.mv_MultiVectorDestroy(xx)
    ctx.lib.mv_MultiVectorDestroy(yy)
    return v


@pytest.mark.parametrize("dtype,rtol", [(S.FLOAT64, 1e-13), (S.FLOAT32, 2e-5)])
def test_gram_noalloc_matches_allocating_entry_point(dtype, rtol):
    ctx = S.Context(0)
    lib = ctx.lib
    rng = np.random.default_rng(5)
    # two calls in a row, different shapes; the third is the widest block,
    # where the fixed array holds only 3 split-k partial sums and so limits
    # the row splits below what the SM count would choose
    shapes = [(300001, 32, 32), (70003, 17, 96), (200003, 384, 384)]
    for n, h, w in shapes:
        x = rng.standard_normal((n, h))
        y = rng.standard_normal((n, w))
        X = S.MultiVector.from_host(ctx, x, dtype)
        Y = S.MultiVector.from_host(ctx, y, dtype)
        G = S.MultiVector(ctx, h, w, S.FLOAT64)  # device output block, ld >= h
        rc = lib.gpu_GramNoAlloc(dtype, n, X.data_ptr, X.ld, h, Y.data_ptr, Y.ld, w,
                                 G.data_ptr, G.ld, ctx.stream)
        assert rc == 0
        got = G.to_host()
        ref = _gram_allocating(ctx, X, Y, h, w)
        xs = x if dtype == S.FLOAT64 else x.astype(np.float32).astype(np.float64)
        ys = y if dtype == S.FLOAT64 else y.astype(np.float32).astype(np.float64)
        scale = np.sqrt(np.outer((xs * xs).sum(0), (ys * ys).sum(0)))
        assert np.all(np.abs(got - ref) <= rtol * scale)
    ctx.close()


def test_gram_noalloc_rejects_sizes_beyond_the_maximum():
    ctx = S.Context(0)
    X = S.MultiVector(ctx, 1000, 4)
    G = S.MultiVector(ctx, 400, 4)
    lib = ctx.lib
    assert lib.gpu_GramNoAlloc(S.FLOAT64, 1000, X.data_ptr, X.ld, 385, X.data_ptr, X.ld, 4,
                               G.data_ptr, G.ld, ctx.stream) == -2
    assert lib.gpu_GramNoAlloc(S.FLOAT64, 1000, X.data_ptr, X.ld, 4, X.data_ptr, 10, 4,
                               G.data_ptr, G.ld, ctx.stream) == -1
    ctx.close()
