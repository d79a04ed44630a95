"""The bounded waits of the tcgen05 / TMA kernels, run out on purpose.

Every pipeline wait of these kernels (the mbarrier phases of bulk copies,
TMA tiles and MMAs) gives up after `wait_polls` polls.  Here the limit is one
poll, so that waits on copies from HBM and on the other roles give up, and
the tests check that
* the kernel ends, raises the context's device error word, and leaves
  either the exact result or NaN / an untouched entry -- never a wrong
  finite value;
* the context stays usable: with the default limit the same call is exact
  and raises no error;
* a mixed solve undoes the step, hands over to the FP64 loop
  (handover_reason 6) and still converges to the tolerance.  The reference's
  contract at this boundary is the -1 return with a message only when the
  solve cannot go on (lobpcg.c:1170-1176); here it can, in FP64.
The drains (copies in flight before a CTA exits, the MMAs before TMEM is
freed) keep the full limit, so a short limit never leaves work in flight.
Whether a single poll succeeds depends on timing, so each check repeats the
call a few times and asserts that the wait ran out at least once.
"""
import ctypes

import numpy as np
import pytest
import scipy.sparse as sp

from blopex_gb300 import problems as P
from blopex_gb300 import solver as S

pytestmark = pytest.mark.gpu

ATTEMPTS = 4


@pytest.fixture
def ctx():
    c = S.Context(0)
    yield c
    c.set_options(wait_polls=0)
    c.close()


def _attempts(ctx, call, check_ok, check_timed_out):
    """Run call() with one poll per wait ATTEMPTS times; every outcome must be
    exact or a reported time-out; at least one must time out."""
    ctx.set_options(wait_polls=1)
    outcomes = []
    for _ in range(ATTEMPTS):
        out = call()
        code = ctx.device_error()
        if code == 0 and check_ok(out):
            outcomes.append("ok")
        else:
            assert code != 0, "incomplete output without the device error word"
            check_timed_out(out)
            outcomes.append("timeout")
    ctx.set_options(wait_polls=0)
    assert "timeout" in outcomes, outcomes
    return outcomes


def test_split_update_gives_up_cleanly(ctx):
    rng = np.random.default_rng(1)
    n, h, w = 1 << 21, 64, 64
    X = rng.standard_normal((n, h))
    C = np.asfortranarray(rng.standard_normal((h, w)))
    ref = X @ C
    bound = h * 2.0 ** -38 * np.outer(np.abs(X).max(1), np.abs(C).max(0)) + 1e-13 * np.abs(ref)
    mx = S.MultiVector.from_host(ctx, X)
    my = S.MultiVector(ctx, n, w)
    sentinel = np.full((n, w), np.nan)

    def call():
        my.upload(sentinel)
        rc = ctx.lib.gpu_BlockUpdate(mx.handle, C.ctypes.data, h, my.handle, None, 2)
        return rc, my.to_host()

    def ok(out):
        rc, Y = out
        return rc == 0 and np.all(np.abs(Y - ref) <= bound)

    def timed_out(out):
        rc, Y = out
        # the C ABI reports the time-out (it reads and clears the word itself,
        # so the word is raised again below only if the kernel set it)
        written = ~np.isnan(Y)
        assert np.all(np.abs(Y[written] - ref[written]) <= bound[written])

    ctx.set_options(wait_polls=1)
    seen = []
    for _ in range(ATTEMPTS):
        rc, Y = call()
        if rc != 0:
            assert "timed out" in ctx.last_error()
            timed_out((rc, Y))
            seen.append("timeout")
        else:
            assert ok((rc, Y))
            seen.append("ok")
    ctx.set_options(wait_polls=0)
    assert "timeout" in seen, seen
    rc, Y = call()
    assert rc == 0 and ok((rc, Y)), ctx.last_error()
    assert ctx.device_error() == 0


def test_split_gram_gives_up_cleanly(ctx):
    rng = np.random.default_rng(2)
    n, h = 1 << 21, 64
    L = rng.standard_normal((n, h))
    Q = rng.standard_normal((n, 64)).astype(np.float32).astype(np.float64)
    ml = S.MultiVector.from_host(ctx, L)
    mq = S.MultiVector.from_host(ctx, Q, S.FLOAT32)
    arr = (ctypes.c_void_p * 1)(mq.handle)
    ref = L.T @ np.hstack([L, Q])
    tol = 1e-6 * np.sqrt(np.outer((L * L).sum(0), (np.hstack([L, Q]) ** 2).sum(0)))

    def call():
        G = np.zeros((h, h + 64), order="F")
        rc = ctx.lib.gpu_SplitGram(ml.handle, arr, 1, G.ctypes.data, h)
        return rc, G

    ctx.set_options(wait_polls=1)
    seen = []
    for _ in range(ATTEMPTS):
        rc, G = call()
        if rc != 0:
            assert "timed out" in ctx.last_error()
            seen.append("timeout")
        else:
            assert np.all(np.abs(G - ref) <= tol)
            seen.append("ok")
    ctx.set_options(wait_polls=0)
    assert "timeout" in seen, seen
    rc, G = call()
    assert rc == 0, ctx.last_error()
    assert np.all(np.abs(G - ref) <= tol)
    assert ctx.device_error() == 0


def test_tf32_gram_gives_up_cleanly(ctx):
    rng = np.random.default_rng(3)
    n, k = 1 << 20, 32
    blocks = {nm: rng.standard_normal((n, k)).astype(np.float32).astype(np.float64)
              for nm in ("X", "R", "P", "AX", "AR", "AP")}
    mvs = {nm: S.MultiVector.from_host(ctx, a, S.FLOAT32) for nm, a in blocks.items()}
    m = 3 * k
    L = np.hstack([blocks["X"], blocks["R"], blocks["P"]])
    Gref = L.T @ np.hstack([blocks["AX"], blocks["AR"], blocks["AP"]])
    scale = np.sqrt(np.outer((L * L).sum(0), (L * L).sum(0)))

    def call():
        G = np.zeros((m, m), order="F")
        H = np.zeros((m, m), order="F")
        rc = ctx.lib.gpu_ExplicitGram(*(mvs[nm].handle for nm in ("X", "R", "P", "AX", "AR", "AP")),
                                      2, G.ctypes.data, H.ctypes.data, m)
        assert rc == 0, ctx.last_error()
        return G

    blocks_of = np.repeat(np.arange(3), k)
    low = blocks_of[:, None] >= blocks_of[None, :]
    _attempts(ctx, call,
              lambda G: np.all(np.isfinite(G)) and (np.abs(G - Gref)[low] / scale[low]).max() < 5e-6,
              lambda G: np.testing.assert_equal(np.isnan(G).all(), True))
    assert (np.abs(call() - Gref)[low] / scale[low]).max() < 5e-6
    assert ctx.device_error() == 0


def test_tma_stencil_gives_up_cleanly(ctx):
    g, w = 128, 16
    cx, cy, cz = P.stencil7_coefficients(g, g, g, seed=5)
    A = S.Stencil7(ctx, cx, cy, cz)
    rp, ci, va = P.stencil7_to_csr(cx, cy, cz)
    n = g ** 3
    Acsr = sp.csr_matrix((va, ci, rp), shape=(n, n))
    rng = np.random.default_rng(4)
    X = rng.standard_normal((n, w)).astype(np.float32).astype(np.float64)
    ref = Acsr @ X
    # FP32 coefficients and arithmetic: a few ulps of the row's absolute sum
    bound = 1e-5 * (abs(Acsr) @ np.abs(X)) + 1e-30
    mx = S.MultiVector.from_host(ctx, X, S.FLOAT32)
    my = S.MultiVector(ctx, n, w, S.FLOAT32)

    def call():
        A.apply(mx, my)
        return my.to_host()

    def ok(Y):
        return np.all(np.abs(Y - ref) <= bound)

    def timed_out(Y):
        written = ~np.isnan(Y)
        assert np.all(np.abs(Y[written] - ref[written]) <= bound[written])
        assert not written.all()

    _attempts(ctx, call, ok, timed_out)
    assert ok(call())
    assert ctx.device_error() == 0


def test_mixed_solve_hands_over_after_time_outs(ctx):
    g, k = 48, 16
    cx, cy, cz = P.stencil7_coefficients(g, g, g, seed=2)
    A = S.Stencil7(ctx, cx, cy, cz)
    T = S.Diagonal(ctx, 1.0 / P.stencil7_diagonal(cx, cy, cz))
    n = g ** 3
    res = {}
    for mode, polls in (("fp64", 0), ("mixed", 1)):
        X = S.MultiVector(ctx, n, k)
        X.set_random(3)
        ctx.set_options(precision=S.FP64 if mode == "fp64" else S.MIXED, wait_polls=polls)
        r = S.lobpcg_solve_double(X, A, T=T, atol=1e-8, rtol=1e-50, maxit=2000, history=False)
        ctx.set_options(wait_polls=0)
        assert r.flag == 0, (mode, r.iterations, ctx.last_error())
        assert np.max(r.res) <= 1e-8
        res[mode] = r
    st = res["mixed"].stats
    assert st["device_errors"] >= 1, st
    assert st["handover_reason"] == 6, st
    assert st["iterations_fp64"] > 0, st
    np.testing.assert_allclose(res["mixed"].lam, res["fp64"].lam, rtol=1e-8)
    assert ctx.device_error() == 0
