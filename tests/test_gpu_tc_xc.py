"""The tensor-core block update Y = X C (+ Z) (tcgen05, compensated TF32)
against FP64 numpy and the CUDA-core kernel, through the C ABI
(gpu_BlockUpdate).  The compensated products carry FP32 accuracy; the
accumulation over the h <= 128 input columns is short."""
import numpy as np
import pytest

from blopex_gb300 import solver as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = S.Context(0)
    yield c
    c.close()


def _update(ctx, X, C, Z, mode, w):
    n = X.shape[0]
    mx = S.MultiVector.from_host(ctx, X, S.FLOAT32)
    my = S.MultiVector(ctx, n, w, S.FLOAT32)
    mz = S.MultiVector.from_host(ctx, Z, S.FLOAT32) if Z is not None else None
    Cf = np.asfortranarray(C)
    rc = ctx.lib.gpu_BlockUpdate(mx.handle, Cf.ctypes.data, C.shape[0], my.handle,
                                 mz.handle if mz is not None else None, mode)
    assert rc == 0, ctx.last_error()
    return my.to_host()


@pytest.mark.parametrize("n,h,w,with_z", [(4096, 32, 32, False), (100003, 128, 64, True),
                                          (70001, 64, 64, True), (5000, 17, 20, False),
                                          (300000, 96, 48, True), (129, 1, 1, True),
                                          (1000, 128, 33, False)])
def test_tc_block_update_matches_reference(ctx, n, h, w, with_z):
    rng = np.random.default_rng(n + h + w)
    X = rng.standard_normal((n, h)).astype(np.float32).astype(np.float64)
    C = rng.standard_normal((h, w))
    Z = rng.standard_normal((n, w)).astype(np.float32).astype(np.float64) if with_z else None
    ref = X @ C.astype(np.float32).astype(np.float64) + (Z if with_z else 0.0)
    # the dot-product error bound scale: sum_c |X_rc| |C_cj| (+ |Z_rj|)
    scale = np.abs(X) @ np.abs(C) + (np.abs(Z) if with_z else 0.0)
    Y1 = _update(ctx, X, C, Z, 1, w)
    Y0 = _update(ctx, X, C, Z, 0, w)
    e1 = np.abs(Y1 - ref) / scale
    e0 = np.abs(Y0 - ref) / scale
    assert np.all(np.isfinite(Y1))
    assert e1.max() < 2e-6, e1.max()
    assert e0.max() < 2e-6, e0.max()
