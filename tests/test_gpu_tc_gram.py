"""The tensor-core (tcgen05) Gram kernel of the explicit iteration against
the CUDA-core FP32 kernel and against FP64 numpy, through the C ABI
(gpu_ExplicitGram).  TF32 products carry ~2^-10 relative error; the
compensated 3xTF32 mode reaches FP32-level accuracy on entries with mixed
signs.  Accumulation in TMEM rounds toward zero, so long sums of positive
terms (the diagonal of H) drift by ~1e-5 relative over a CTA's rows; the
solver takes the diagonal blocks it relies on from the Rayleigh-Ritz
identities instead (X'X = I, X'AX = diag(lambda)), as the reference does."""
import numpy as np
import pytest

from blopex_gb300 import solver as S

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    c = S.Context(0)
    yield c
    c.close()


def _sym_apply(d, v):
    """A symmetric operator (diagonal plus circulant neighbours): the kernel
    computes the lower blocks of G and mirrors the upper ones, which is exact
    only for symmetric A."""
    return d[:, None] * v + np.roll(v, 1, axis=0) + np.roll(v, -1, axis=0)


def _blocks(ctx, n, k, nR, nP, seed):
    rng = np.random.default_rng(seed)
    d = rng.uniform(1.0, 3.0, n)
    mats = {}
    for name, w in (("X", k), ("R", nR), ("P", nP)):
        a = rng.standard_normal((n, max(w, 1))).astype(np.float32).astype(np.float64)
        mats[name] = a[:, :w]
        mats["A" + name] = _sym_apply(d, mats[name]).astype(np.float32).astype(np.float64)
    mvs = {nm: (S.MultiVector.from_host(ctx, a, S.FLOAT32) if a.shape[1] else None)
           for nm, a in mats.items()}
    return mats, mvs


def _explicit(ctx, mvs, m, mode):
    G = np.zeros((m, m), order="F")
    H = np.zeros((m, m), order="F")
    h = lambda nm: mvs[nm].handle if mvs[nm] is not None else None
    rc = ctx.lib.gpu_ExplicitGram(h("X"), h("R"), h("P"), h("AX"), h("AR"), h("AP"), mode,
                                  G.ctypes.data, H.ctypes.data, m)
    assert rc == 0, ctx.last_error()
    return G, H


@pytest.mark.parametrize("n,k,nR,nP", [(4096, 32, 32, 32), (100003, 32, 17, 17), (70001, 64, 64, 64),
                                       (33333, 64, 40, 40), (5000, 20, 20, 0), (300000, 64, 64, 0)])
def test_tc_gram_matches_reference(ctx, n, k, nR, nP):
    mats, mvs = _blocks(ctx, n, k, nR, nP, seed=n + k)
    m = k + nR + nP
    L = np.hstack([mats["X"], mats["R"], mats["P"]])
    Rg = np.hstack([mats["AX"], mats["AR"], mats["AP"]])
    Gref, Href = L.T @ Rg, L.T @ L
    # lower blocks are computed directly, upper ones mirrored: compare the
    # symmetric parts (the solver symmetrises G and H)
    sym = lambda a: 0.5 * (a + a.T)
    scaleG = np.sqrt(np.outer((L * L).sum(0), (Rg * Rg).sum(0)))
    scaleH = np.sqrt(np.outer((L * L).sum(0), (L * L).sum(0)))
    G0, H0 = _explicit(ctx, mvs, m, 0)
    for mode, tol in ((1, 4e-3), (2, 5e-6)):
        G, H = _explicit(ctx, mvs, m, mode)
        eg = np.abs(sym(G) - sym(Gref)) / (0.5 * (scaleG + scaleG.T))
        eh = np.abs(H - Href) / scaleH
        off = ~np.eye(m, dtype=bool)
        assert eg[off].max() < tol, (mode, eg[off].max())
        assert eh[off].max() < tol, (mode, eh[off].max())
        # diagonals: sums of positive terms, truncating accumulation
        assert np.diag(eh).max() < max(tol, 1e-4), (mode, np.diag(eh).max())
        # the lower block triangle is exact to the same tolerance without symmetrising
        blocks = np.repeat(np.arange(3), [k, nR, nP])
        low = blocks[:, None] >= blocks[None, :]
        low &= off
        assert (np.abs(G - Gref)[low] / scaleG[low]).max() < tol
    # the CUDA-core kernel (FP32 data, FP64 sums) is FP32-accurate
    assert (np.abs(G0 - Gref) / scaleG).max() < 1e-5
