"""Seeded synthetic inputs for the solver (host-side builders, numpy).

These build the operators and initial blocks the solver is run on; they do
no part of the eigensolver's arithmetic.  All layouts match the device
operators in ``csrc/operators.cu``:

* cells are numbered ``i + nx*(j + ny*k)`` (x fastest);
* 3D 7-point face coefficients: ``cx[k, j, i]`` for the x-face between cells
  i-1 and i (shape nz x ny x (nx+1)), likewise ``cy`` (nz x (ny+1) x nx) and
  ``cz`` ((nz+1) x ny x nx); faces on the boundary couple to a Dirichlet zero;
* 27-point weights: 13 per cell, one per "forward" neighbour offset in
  ``STENCIL27_OFFSETS`` (edges leaving the grid do not exist).

The initial block ``drand48_block`` reproduces the reference's
``serial_Multi_VectorSetRandomValues`` (blopex_serial_double/multivector/
multi_vector.c:165-184): ``srand48(seed)`` then ``2*drand48()-1`` column by
column.
"""
from __future__ import annotations

import numpy as np

STENCIL27_OFFSETS = np.array(
    [[1, 0, 0], [-1, 1, 0], [0, 1, 0], [1, 1, 0],
     [-1, -1, 1], [0, -1, 1], [1, -1, 1],
     [-1, 0, 1], [0, 0, 1], [1, 0, 1],
     [-1, 1, 1], [0, 1, 1], [1, 1, 1]], dtype=np.int64)

_M48 = (1 << 48) - 1
_A48 = 0x5DEECE66D
_C48 = 0xB


def _lcg_jump(steps: int) -> tuple[int, int]:
    """(A, C) with state_{t+steps} = A*state_t + C mod 2^48."""
    a, c = 1, 0
    ba, bc = _A48, _C48
    s = steps
    while s:
        if s & 1:
            a, c = (a * ba) & _M48, (c * ba + bc) & _M48
        ba, bc = (ba * ba) & _M48, (bc * ba + bc) & _M48
        s >>= 1
    return a, c


def drand48_stream(count: int, seed: int) -> np.ndarray:
    """The first ``count`` values of drand48() after srand48(seed), exactly."""
    state0 = ((seed & 0xFFFFFFFF) << 16) | 0x330E
    block = 1 << 16
    # coefficients for 1..block steps ahead
    A = np.empty(block, dtype=np.uint64)
    C = np.empty(block, dtype=np.uint64)
    a, c = 1, 0
    for t in range(block):
        a, c = (a * _A48) & _M48, (c * _A48 + _C48) & _M48
        A[t], C[t] = a, c
    out = np.empty(count, dtype=np.float64)
    state = state0
    mask = np.uint64(_M48)
    for start in range(0, count, block):
        m = min(block, count - start)
        st = (A[:m] * np.uint64(state) + C[:m]) & mask  # wraps mod 2^64, exact mod 2^48
        out[start:start + m] = st.astype(np.float64) / float(1 << 48)
        state = int(st[m - 1])
    return out


def drand48_block(n: int, k: int, seed: int) -> np.ndarray:
    """X0 (n x k, column-major) = 2*drand48()-1 after srand48(seed)."""
    v = drand48_stream(n * k, seed)
    return np.asfortranarray((2.0 * v - 1.0).reshape(k, n).T)


def laplacian3d_csr(nx: int, ny: int, nz: int):
    """7-point Dirichlet Laplacian (diag 6, off-diagonals -1), CSR int32/f64,
    column indices ascending within each row."""
    n = nx * ny * nz
    idx = np.arange(n, dtype=np.int64).reshape(nz, ny, nx)
    cols = []
    for dk, dj, di in ((-1, 0, 0), (0, -1, 0), (0, 0, -1), (0, 0, 0), (0, 0, 1), (0, 1, 0), (1, 0, 0)):
        c = np.full((nz, ny, nx), -1, dtype=np.int64)
        ks = slice(max(0, -dk), nz - max(0, dk))
        js = slice(max(0, -dj), ny - max(0, dj))
        is_ = slice(max(0, -di), nx - max(0, di))
        kd = slice(max(0, dk), nz + min(0, dk))
        jd = slice(max(0, dj), ny + min(0, dj))
        id_ = slice(max(0, di), nx + min(0, di))
        c[ks, js, is_] = idx[kd, jd, id_]
        cols.append(c.reshape(n))
    cols = np.stack(cols, axis=1)  # n x 7, ascending order by construction
    vals = np.where(cols == np.arange(n)[:, None], 6.0, -1.0)
    valid = cols >= 0
    counts = valid.sum(axis=1)
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.cumsum(counts, out=rowptr[1:])
    return (rowptr.astype(np.int32), cols[valid].astype(np.int32), vals[valid].astype(np.float64))


def laplacian_eigs(dims, count: int) -> np.ndarray:
    """Smallest ``count`` eigenvalues of the Dirichlet Laplacian on a grid
    with ``dims`` interior points per axis: sums of 4 sin^2(pi j / (2(m+1)))."""
    per = []
    for m in dims:
        j = np.arange(1, min(m, count) + 1)
        per.append(4.0 * np.sin(np.pi * j / (2.0 * (m + 1))) ** 2)
    tot = per[0]
    for p in per[1:]:
        tot = np.add.outer(tot, p).ravel()
    return np.sort(tot)[:count]


def stencil7_coefficients(nx: int, ny: int, nz: int, seed: int, dtype=np.float64):
    """Face coefficients exp(g), g ~ N(0,1) i.i.d. (numpy PCG64, ``seed``),
    drawn in the order cx, cy, cz."""
    rng = np.random.default_rng(seed)
    cx = np.exp(rng.standard_normal((nz, ny, nx + 1))).astype(dtype)
    cy = np.exp(rng.standard_normal((nz, ny + 1, nx))).astype(dtype)
    cz = np.exp(rng.standard_normal((nz + 1, ny, nx))).astype(dtype)
    return cx, cy, cz


def stencil7_constant(nx: int, ny: int, nz: int, value: float = 1.0):
    """Unit face coefficients: the plain 7-point Dirichlet Laplacian."""
    return (np.full((nz, ny, nx + 1), value), np.full((nz, ny + 1, nx), value),
            np.full((nz + 1, ny, nx), value))


def stencil7_diagonal(cx, cy, cz, shift: float = 0.0) -> np.ndarray:
    """Diagonal of the 7-point operator (sum of the six incident faces)."""
    d = (cx[:, :, :-1] + cx[:, :, 1:] + cy[:, :-1, :] + cy[:, 1:, :]
         + cz[:-1, :, :] + cz[1:, :, :] + shift)
    return np.ascontiguousarray(d).ravel()


def stencil7_to_csr(cx, cy, cz, shift: float = 0.0):
    """Assemble the 7-point operator as CSR (for small checks)."""
    nz, ny, nxp = cx.shape
    nx = nxp - 1
    n = nx * ny * nz
    rows, cols, vals = [], [], []
    idx = np.arange(n).reshape(nz, ny, nx)
    diag = stencil7_diagonal(cx, cy, cz, shift)
    rows.append(np.arange(n)); cols.append(np.arange(n)); vals.append(diag)
    # x neighbours (interior faces only)
    f = cx[:, :, 1:-1]
    rows += [idx[:, :, :-1].ravel(), idx[:, :, 1:].ravel()]
    cols += [idx[:, :, 1:].ravel(), idx[:, :, :-1].ravel()]
    vals += [-f.ravel(), -f.ravel()]
    f = cy[:, 1:-1, :]
    rows += [idx[:, :-1, :].ravel(), idx[:, 1:, :].ravel()]
    cols += [idx[:, 1:, :].ravel(), idx[:, :-1, :].ravel()]
    vals += [-f.ravel(), -f.ravel()]
    f = cz[1:-1, :, :]
    rows += [idx[:-1].ravel(), idx[1:].ravel()]
    cols += [idx[1:].ravel(), idx[:-1].ravel()]
    vals += [-f.ravel(), -f.ravel()]
    return coo_to_csr(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))


def coo_to_csr(n, rows, cols, vals):
    order = np.lexsort((cols, rows))
    rows, cols, vals = rows[order], cols[order], vals[order]
    rowptr = np.zeros(n + 1, dtype=np.int64)
    np.add.at(rowptr, rows + 1, 1)
    np.cumsum(rowptr, out=rowptr)
    return rowptr.astype(np.int32), cols.astype(np.int32), vals.astype(np.float64)


def csr_to_dense(rowptr, colidx, vals, n):
    a = np.zeros((n, n))
    for r in range(n):
        a[r, colidx[rowptr[r]:rowptr[r + 1]]] = vals[rowptr[r]:rowptr[r + 1]]
    return a


def csr_diagonal(rowptr, colidx, vals):
    n = len(rowptr) - 1
    rows = np.repeat(np.arange(n), np.diff(rowptr))
    d = np.zeros(n)
    m = rows == colidx
    d[rows[m]] = vals[m]
    return d


def stencil5_from_cells(c: np.ndarray):
    """2D 5-point diffusion from cell coefficients c (ny x nx): an interior
    face takes the arithmetic mean of its two cells, a boundary face the
    value of its one cell (Dirichlet zero outside)."""
    ny, nx = c.shape
    cx = np.empty((ny, nx + 1))
    cx[:, 1:-1] = 0.5 * (c[:, :-1] + c[:, 1:])
    cx[:, 0] = c[:, 0]
    cx[:, -1] = c[:, -1]
    cy = np.empty((ny + 1, nx))
    cy[1:-1, :] = 0.5 * (c[:-1, :] + c[1:, :])
    cy[0, :] = c[0, :]
    cy[-1, :] = c[-1, :]
    return cx, cy


def gaussian_random_field(nx: int, ny: int, length: float, seed: int) -> np.ndarray:
    """Smooth GRF on the unit square (cell centres), squared-exponential
    covariance exp(-r^2 / (2 length^2)), unit variance, sampled spectrally on
    a periodic grid twice the size (numpy PCG64, ``seed``)."""
    rng = np.random.default_rng(seed)
    mx, my = 2 * nx, 2 * ny
    kx = np.fft.fftfreq(mx, d=1.0 / nx)  # wavenumbers for a domain of length 2
    ky = np.fft.fftfreq(my, d=1.0 / ny)
    KX, KY = np.meshgrid(kx, ky)
    k2 = (2 * np.pi) ** 2 * (KX ** 2 + KY ** 2) / 4.0
    spec = np.exp(-0.5 * length ** 2 * k2)
    noise = rng.standard_normal((my, mx))
    field = np.fft.ifft2(np.fft.fft2(noise) * np.sqrt(spec)).real
    field = field[:ny, :nx]
    return (field - field.mean()) / field.std()


def stencil27_weights(nx: int, ny: int, nz: int, seed: int) -> np.ndarray:
    """13 edge weights per cell, U[0.5, 1.5] (numpy PCG64, ``seed``)."""
    rng = np.random.default_rng(seed)
    return rng.uniform(0.5, 1.5, size=(nx * ny * nz, 13))


def mass_diagonal(n: int, seed: int) -> np.ndarray:
    """Lumped mass B = diag(U[0.5, 1.5]) (numpy PCG64, ``seed``)."""
    return np.random.default_rng(seed).uniform(0.5, 1.5, size=n)


def stencil27_to_csr(nx: int, ny: int, nz: int, w: np.ndarray, shift: float):
    """Assemble the shifted 27-point graph Laplacian as CSR (small checks)."""
    n = nx * ny * nz
    k, j, i = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    i, j, k = i.ravel(), j.ravel(), k.ravel()
    c = i + nx * (j + ny * k)
    rows, cols, vals = [], [], []
    diag = np.full(n, float(shift))
    for e, (di, dj, dk) in enumerate(STENCIL27_OFFSETS):
        i2, j2, k2 = i + di, j + dj, k + dk
        ok = (i2 >= 0) & (i2 < nx) & (j2 >= 0) & (j2 < ny) & (k2 >= 0) & (k2 < nz)
        a, b = c[ok], (i2 + nx * (j2 + ny * k2))[ok]
        wv = np.asarray(w).reshape(n, 13)[a, e]
        rows += [a, b]
        cols += [b, a]
        vals += [-wv, -wv]
        np.add.at(diag, a, wv)
        np.add.at(diag, b, wv)
    rows.append(np.arange(n)); cols.append(np.arange(n)); vals.append(diag)
    return coo_to_csr(n, np.concatenate(rows), np.concatenate(cols), np.concatenate(vals))
