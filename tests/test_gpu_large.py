"""Parity at the benchmark sizes (128^3).

* The FP64 path against the unmodified reference's first iterations on the
  128^3 plain-FP64 configuration (7-point Laplacian CSR, k = 32, Jacobi) and
  on the variable-coefficient stencil at 128^3 (k = 64, Jacobi): the
  eigenvalue and residual histories of every iteration
  (lobpcg.c:1288-1316), to 1e-10 relative where the reference's own plain,
  FMA and x87 builds agree and within three times their spread where they
  do not (they part after ~10 iterations on these problems).
* The mixed mode against the FP64 path on the variable-coefficient stencil at
  128^3 (k = 64, 20 inner CG steps, tol 1e-8): both converge, the eigenvalues
  agree to 1e-10, the eigenvector blocks span the same space (largest
  principal angle) and X'X = I.
"""
import hashlib
import json
import os

import numpy as np
import pytest

from blopex_gb300 import problems as P
from blopex_gb300 import solver as S
from tests.golden import cases as C

pytestmark = pytest.mark.gpu

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def ctx():
    c = S.Context(0)
    yield c
    c.close()


def _sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def _check_input(g, key, a):
    """Integer inputs and the drand48 block are bit-identical on every host;
    exp(N(0,1)) coefficients carry numpy's platform-dependent last bit, so a
    floating-point input whose hash differs must match the fixture's
    fingerprint (two weighted sums) to 1e-12."""
    if _sha(a) == g["inputs_sha256"][key]:
        return
    assert np.asarray(a).dtype.kind == "f", key
    v = np.ascontiguousarray(a, dtype=np.float64).ravel()
    w = (np.arange(v.size) % 97 + 1.0) / 97.0
    got = np.array([np.sum(v), np.dot(v, w)])
    ref = np.array(g["inputs_fingerprint"][key])
    np.testing.assert_allclose(got, ref, rtol=1e-12, err_msg=key)


def _envelope(g, key):
    """Per-iteration reference value and tolerance: 1e-10 relative, or three
    times the spread of the reference's three builds, whichever is larger."""
    runs = [np.array(g[key])] + [np.array(v[key]) for v in g["variants"].values()]
    ref = runs[0]
    scale = np.maximum(np.abs(ref), 1e-300)
    spread = np.max([np.abs(r - ref) / scale for r in runs[1:]], axis=0)
    return ref, scale, np.maximum(1e-10, 3.0 * spread)


@pytest.mark.parametrize("name", C.LARGE_NAMES)
def test_fp64_histories_match_reference_at_size(ctx, name):
    with open(os.path.join(HERE, name + ".json")) as f:
        g = json.load(f)
    case = C.build(name)
    rp, ci, va = case.csr
    x0 = case.initial_block()
    assert _sha(rp) == g["inputs_sha256"]["rowptr"]
    assert _sha(ci) == g["inputs_sha256"]["colidx"]
    assert _sha(x0) == g["inputs_sha256"]["x0"]
    _check_input(g, "vals", va)
    _check_input(g, "t_diag", case.t_diag)
    A = S.CSRMatrix(ctx, rp, ci, va)
    T = S.Diagonal(ctx, case.t_diag)
    X = S.MultiVector.from_host(ctx, x0)
    ctx.set_options(precision=S.FP64)
    r = S.lobpcg_solve_double(X, A, T=T, atol=case.atol, rtol=case.rtol, maxit=case.maxit,
                              history=True)
    assert r.flag == g["flag"] and r.iterations == g["iterations"], (r.flag, r.iterations)
    its = r.iterations + 1
    lam = r.lam_hist[:, :its].T
    res = r.res_hist[:, :its].T
    lref, lscale, ltol = _envelope(g, "lambda_hist")
    rref, rscale, rtol = _envelope(g, "res_hist")
    lerr = np.abs(lam - lref) / lscale
    rerr = np.abs(res - rref) / rscale
    assert np.all(lerr <= ltol), (np.argwhere(lerr > ltol)[:5], lerr.max())
    # residual norms: the same bar, at least 1e-8 relative (a norm loses the
    # cancellation its entries carry)
    rtol = np.maximum(rtol, 1e-8)
    assert np.all(rerr <= rtol), (np.argwhere(rerr > rtol)[:5], rerr.max())
    # the first iterations, where the builds agree to ~1e-13, at 1e-10
    assert np.max(lerr[:5]) <= 1e-10


def test_mixed_meets_tolerance_against_fp64_at_size(ctx):
    g = 128
    cx, cy, cz = P.stencil7_coefficients(g, g, g, seed=2)
    A = S.Stencil7(ctx, cx, cy, cz)
    T = S.PCGPreconditioner(ctx, A, S.Diagonal(ctx, 1.0 / P.stencil7_diagonal(cx, cy, cz)), 20)
    n, k = g ** 3, 64
    out = {}
    for mode in ("fp64", "mixed"):
        X = S.MultiVector(ctx, n, k)
        X.set_random(2)
        ctx.set_options(precision=S.FP64 if mode == "fp64" else S.MIXED)
        r = S.lobpcg_solve_double(X, A, T=T, atol=1e-8, rtol=1e-50, maxit=1000, history=False)
        assert r.flag == 0, (mode, r.iterations, ctx.last_error())
        assert np.max(r.res) <= 1e-8
        out[mode] = (X, r)
    (Xf, rf), (Xm, rm) = out["fp64"], out["mixed"]
    np.testing.assert_allclose(rm.lam, rf.lam, rtol=1e-10)
    assert rm.stats["iterations_split"] > 0  # the split-operand phase did the work
    # largest principal angle between the blocks, and X'X - I of the mixed one
    xf, xm = Xf.to_host(), Xm.to_host()
    d = xm - xf @ (xf.T @ xm)
    sin_max = np.sqrt(max(np.linalg.eigvalsh(d.T @ d)[-1], 0.0))
    # the wanted block is separated from the rest of the spectrum: with
    # residuals <= 1e-8 the angle is bounded by res / gap
    assert sin_max < 1e-4, sin_max
    assert np.linalg.norm(xm.T @ xm - np.eye(k)) < 1e-10
