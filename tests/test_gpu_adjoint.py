"""Reverse-mode derivatives of the eigenpairs (adjoint module) through the C
ABI and the torch.autograd.Function wrappers, against

  * dense FP64 references: torch.linalg.eigh autograd on the assembled
    matrices (the generalized problem through B^-1/2 A B^-1/2),
  * FP64 central finite differences of the device solver itself,

at 1e-6 relative.  Loss: sum of the k eigenvalues plus the squared overlap of
x_1 with a fixed random vector (invariant to the sign of x_1)."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from blopex_gb300 import adjoint as AD  # noqa: E402
from blopex_gb300 import problems as P  # noqa: E402
from blopex_gb300 import solver as S  # noqa: E402

pytestmark = pytest.mark.gpu
RTOL = 1e-6


@pytest.fixture(scope="module")
def ctx():
    c = S.Context(0)
    yield c
    c.close()


def loss_of(lam, X, v):
    v = v / torch.linalg.norm(v)
    return lam.sum() + (X[:, 0] @ v) ** 2


# --------------------------------------------------------- dense builders
def dense_stencil5(cx, cy):
    ny, nx = cy.shape[0] - 1, cx.shape[1] - 1
    n = nx * ny
    j, i = np.meshgrid(np.arange(ny), np.arange(nx), indexing="ij")
    i, j = i.ravel(), j.ravel()
    c = i + nx * j
    A = torch.zeros(n, n, dtype=torch.float64)
    ti, tj = torch.from_numpy(i), torch.from_numpy(j)
    cw, ce = cx[tj, ti], cx[tj, ti + 1]
    cs, cn = cy[tj, ti], cy[tj + 1, ti]
    idx = torch.arange(n)
    A = A.index_put((idx, idx), cw + ce + cs + cn, accumulate=True)
    m = torch.from_numpy(i > 0)
    A = A.index_put((torch.from_numpy(c)[m], torch.from_numpy(c)[m] - 1), -cw[m], accumulate=True)
    tc = torch.from_numpy(c)
    m = torch.from_numpy(i < nx - 1)
    A = A.index_put((tc[m], tc[m] + 1), -ce[m], accumulate=True)
    m = torch.from_numpy(j > 0)
    A = A.index_put((tc[m], tc[m] - nx), -cs[m], accumulate=True)
    m = torch.from_numpy(j < ny - 1)
    A = A.index_put((tc[m], tc[m] + nx), -cn[m], accumulate=True)
    return A


def dense_stencil27(grid, w, shift):
    nx, ny, nz = grid
    n = nx * ny * nz
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    c = i + nx * (j + ny * k)
    A = torch.eye(n, dtype=torch.float64) * shift
    for e, (di, dj, dk) in enumerate(P.STENCIL27_OFFSETS):
        i2, j2, k2 = i + di, j + dj, k + dk
        ok = (i2 >= 0) & (i2 < nx) & (j2 >= 0) & (j2 < ny) & (k2 >= 0) & (k2 < nz)
        a = torch.from_numpy(c[ok])
        b = torch.from_numpy((i2 + nx * (j2 + ny * k2))[ok])
        we = w[a, e]
        A = A.index_put((a, a), we, accumulate=True)
        A = A.index_put((b, b), we, accumulate=True)
        A = A.index_put((a, b), -we, accumulate=True)
        A = A.index_put((b, a), -we, accumulate=True)
    return A


def dense_eigs(A, k, b=None):
    if b is None:
        lam, V = torch.linalg.eigh(A)
        return lam[:k], V[:, :k]
    s = 1.0 / torch.sqrt(b)
    lam, V = torch.linalg.eigh(s[:, None] * A * s[None, :])
    return lam[:k], s[:, None] * V[:, :k]


# ------------------------------------------------------------------ tests
def _theta(ny, nx, seed):
    return torch.from_numpy(0.5 * P.gaussian_random_field(nx, ny, 0.2, seed))


def _stencil5_loss(ctx, theta, opts, v, device_solver=True):
    c = torch.exp(theta)
    cx, cy = AD.stencil5_faces_torch(c)
    if device_solver:
        lam, X = AD.Stencil5Eigs.apply(cx, cy, ctx, opts)
    else:
        lam, X = dense_eigs(dense_stencil5(cx, cy), opts.k)
    return loss_of(lam, X, v)


def test_stencil5_gradient_matches_dense_eigh(ctx):
    ny, nx, k = 10, 12, 4
    opts = AD.SolveOptions(k=k, atol=1e-11, maxit=2000)
    v = torch.from_numpy(np.random.default_rng(5).standard_normal(nx * ny))
    th = _theta(ny, nx, 3).requires_grad_(True)
    L = _stencil5_loss(ctx, th, opts, v)
    (g,) = torch.autograd.grad(L, th)
    th2 = th.detach().clone().requires_grad_(True)
    L2 = _stencil5_loss(ctx, th2, opts, v, device_solver=False)
    (g2,) = torch.autograd.grad(L2, th2)
    assert abs(L.item() - L2.item()) < 1e-9 * abs(L2.item())
    err = (g - g2).abs().max() / g2.abs().max()
    assert err < RTOL, float(err)


def test_eigenvalue_only_gradient(ctx):
    """dL/dtheta for L = sum lambda (no eigenvector term: the adjoint solve is
    skipped) equals the dense reference."""
    ny, nx, k = 9, 11, 3
    opts = AD.SolveOptions(k=k, atol=1e-11, maxit=2000)
    th = _theta(ny, nx, 7).requires_grad_(True)
    c = torch.exp(th)
    cx, cy = AD.stencil5_faces_torch(c)
    lam, _ = AD.Stencil5Eigs.apply(cx, cy, ctx, opts)
    (g,) = torch.autograd.grad(lam.sum(), th)
    th2 = th.detach().clone().requires_grad_(True)
    cx2, cy2 = AD.stencil5_faces_torch(torch.exp(th2))
    lam2, _ = dense_eigs(dense_stencil5(cx2, cy2), k)
    (g2,) = torch.autograd.grad(lam2.sum(), th2)
    assert ((g - g2).abs().max() / g2.abs().max()) < RTOL


def test_generalized_27point_mass_gradient(ctx):
    """A = 27-point graph Laplacian of edge weights + shift, B = diag(b):
    gradients in the weights and in b against the dense generalized eigh."""
    grid, k, shift = (5, 5, 4), 4, 0.5
    n = grid[0] * grid[1] * grid[2]
    opts = AD.SolveOptions(k=k, atol=1e-11, maxit=3000)
    rng = np.random.default_rng(11)
    w = torch.from_numpy(rng.uniform(0.5, 1.5, (n, 13))).requires_grad_(True)
    b = torch.from_numpy(rng.uniform(0.5, 1.5, n)).requires_grad_(True)
    v = torch.from_numpy(rng.standard_normal(n))
    lam, X = AD.Stencil27MassEigs.apply(w, b, ctx, grid, shift, opts)
    gw, gb = torch.autograd.grad(loss_of(lam, X, v), (w, b))
    w2 = w.detach().clone().requires_grad_(True)
    b2 = b.detach().clone().requires_grad_(True)
    lam2, X2 = dense_eigs(dense_stencil27(grid, w2, shift), k, b2)
    gw2, gb2 = torch.autograd.grad(loss_of(lam2, X2, v), (w2, b2))
    assert ((gw - gw2).abs().max() / gw2.abs().max()) < RTOL
    assert ((gb - gb2).abs().max() / gb2.abs().max()) < RTOL


def test_csr_value_gradient(ctx):
    """dlambda_i / da_pq = x_i[p] x_i[q] on the stored pattern."""
    rp, ci, va = P.laplacian3d_csr(6, 5, 4)
    rng = np.random.default_rng(2)
    va = va * (1.0 + 0.1 * rng.standard_normal(len(va)))
    # keep it symmetric: symmetrise the perturbed values through the dense form
    n = len(rp) - 1
    D = np.zeros((n, n))
    for r in range(n):
        D[r, ci[rp[r]:rp[r + 1]]] = va[rp[r]:rp[r + 1]]
    D = 0.5 * (D + D.T)
    va = np.array([D[r, c] for r in range(n) for c in ci[rp[r]:rp[r + 1]]])
    k = 4
    opts = AD.SolveOptions(k=k, atol=1e-11, maxit=2000)
    vals = torch.from_numpy(va).requires_grad_(True)
    lam, X = AD.CSREigs.apply(vals, ctx, rp, ci, opts)
    wts = torch.tensor([1.0, 2.0, -1.0, 0.5], dtype=torch.float64)
    (g,) = torch.autograd.grad((wts * lam).sum(), vals)
    lamd, V = np.linalg.eigh(D)
    rows = np.repeat(np.arange(n), np.diff(rp))
    ref = sum(wts[i].item() * V[rows, i] * V[ci, i] for i in range(k))
    assert np.max(np.abs(g.numpy() - ref)) / np.max(np.abs(ref)) < RTOL


def _richardson(f, h):
    """Central differences at h and h/2 combined to O(h^4)."""
    d1 = (f(h) - f(-h)) / (2 * h)
    d2 = (f(h / 2) - f(-h / 2)) / h
    return (4.0 * d2 - d1) / 3.0


def _directions(g, rng, count):
    """Unit directions mixing the gradient direction with a random one, so the
    directional derivative is not small against the difference noise."""
    for _ in range(count):
        r = torch.from_numpy(rng.standard_normal(tuple(g.shape)))
        d = g / torch.linalg.norm(g) + 0.5 * r / torch.linalg.norm(r)
        yield d / torch.linalg.norm(d)


def test_stencil5_gradcheck_device_finite_differences(ctx):
    """FP64 central differences of the device solver itself (16 x 16, forward
    converged to residual 1e-12)."""
    ny = nx = 16
    opts = AD.SolveOptions(k=4, atol=1e-12, maxit=6000)
    rng = np.random.default_rng(13)
    v = torch.from_numpy(rng.standard_normal(nx * ny))
    th0 = torch.from_numpy(0.5 * P.gaussian_random_field(nx, ny, 0.1, 3))
    th = th0.clone().requires_grad_(True)
    (g,) = torch.autograd.grad(_stencil5_loss(ctx, th, opts, v), th)
    for d in _directions(g, rng, 2):
        with torch.no_grad():
            fd = _richardson(lambda t: _stencil5_loss(ctx, th0 + t * d, opts, v).item(), 1e-2)
        an = float((g * d).sum())
        assert abs(fd - an) <= RTOL * abs(an), (fd, an, abs(fd - an) / abs(an))


def test_stencil5_gradcheck_64x64(ctx):
    """The differentiation case's FP64 gradcheck size: 64 x 64 cells, k = 8,
    GRF coefficients (length 0.1, seed 3).  LOBPCG in FP64 stalls near
    residual 1e-10 on this operator, so the differences are taken of the
    exact loss (dense FP64 eigh of the assembled matrix, Richardson-
    extrapolated); the adjoint gradient uses the device solver."""
    ny = nx = 64
    k = 8
    opts = AD.SolveOptions(k=k, atol=3e-10, maxit=6000)
    rng = np.random.default_rng(13)
    v = torch.from_numpy(rng.standard_normal(nx * ny))
    th0 = torch.from_numpy(0.5 * P.gaussian_random_field(nx, ny, 0.1, 3))
    th = th0.clone().requires_grad_(True)
    L = _stencil5_loss(ctx, th, opts, v)
    (g,) = torch.autograd.grad(L, th)
    dev = "cuda" if torch.cuda.is_available() else "cpu"

    def exact(t):
        with torch.no_grad():
            cx, cy = AD.stencil5_faces_torch(torch.exp(th0 + t * d))
            lam, X = dense_eigs(dense_stencil5(cx, cy).to(dev), k)
            return loss_of(lam.cpu(), X.cpu(), v).item()

    d = torch.zeros_like(th0)
    assert abs(exact(0.0) - L.item()) <= 1e-9 * abs(L.item())
    for d in _directions(g, rng, 2):
        fd = _richardson(exact, 1e-2)
        an = float((g * d).sum())
        assert abs(fd - an) <= RTOL * abs(an), (fd, an, abs(fd - an) / abs(an))


def test_inner_cg_preconditioner_solve_and_gradient(ctx):
    """LOBPCG preconditioned by an inner CG (the -pcgitr preconditioner) and
    the flexible adjoint solve with the same preconditioner give the dense
    reference's eigenvalues and gradient."""
    ny, nx, k = 10, 12, 4
    opts = AD.SolveOptions(k=k, atol=1e-11, maxit=2000, inner_cg=8)
    v = torch.from_numpy(np.random.default_rng(5).standard_normal(nx * ny))
    th = _theta(ny, nx, 3).requires_grad_(True)
    L = _stencil5_loss(ctx, th, opts, v)
    (g,) = torch.autograd.grad(L, th)
    th2 = th.detach().clone().requires_grad_(True)
    L2 = _stencil5_loss(ctx, th2, opts, v, device_solver=False)
    (g2,) = torch.autograd.grad(L2, th2)
    assert abs(L.item() - L2.item()) < 1e-9 * abs(L2.item())
    assert ((g - g2).abs().max() / g2.abs().max()) < RTOL
