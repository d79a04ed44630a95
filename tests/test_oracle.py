"""The oracle (C restatement) against the golden vectors recorded from the
unmodified reference, plus the input generators it is fed with."""
import hashlib
import json
import os

import numpy as np
import pytest

from blopex_gb300 import problems as P
from oracle import oracle as O
from tests.golden import cases as C

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def load(name):
    with open(os.path.join(GOLDEN, f"{name}.json")) as f:
        return json.load(f)


def oracle_run(case):
    A = O.csr(*case.csr) if case.csr is not None else O.dense(case.dense)
    B = O.diag(case.b_diag) if case.b_diag is not None else O.NONE
    T = O.diag(case.t_diag) if case.t_diag is not None else O.NONE
    return O.solve(A, case.initial_block(), B=B, T=T, Y=case.Y, atol=case.atol,
                   rtol=case.rtol, maxit=case.maxit, potrf_fail_at=case.potrf_fail_at,
                   sygv_fail_at=case.sygv_fail_at)


@pytest.mark.parametrize("name", C.NAMES)
def test_golden_inputs_pinned(name):
    g = load(name)
    case = C.build(name)
    for key, val in case.arrays().items():
        assert sha(val) == g["inputs_sha256"][key], key


@pytest.mark.parametrize("name", C.NAMES)
def test_oracle_matches_reference_golden(name):
    g = load(name)
    case = C.build(name)
    r = oracle_run(case)
    assert r.flag == g["flag"]
    assert r.iterations == g["iterations"]
    ncol = g["iterations"] + 1
    if g["k"] and g["lambda_hist"]:
        np.testing.assert_allclose(r.lam_hist[:, :ncol].T, np.array(g["lambda_hist"]),
                                   rtol=1e-12, atol=1e-14)
        np.testing.assert_allclose(r.res_hist[:, :ncol].T, np.array(g["res_hist"]),
                                   rtol=1e-9, atol=1e-14)
    if g["flag"] == 0 or g["iterations"] > 0:
        np.testing.assert_allclose(r.lam, g["lambda"], rtol=1e-12)


def test_wrong_block_size():
    case = C.build("wrong_block_size")
    r = O.solve(O.dense(case.dense), np.zeros((40, 0), order="F"), maxit=10)
    assert r.flag == 2 and r.iterations == 0


def test_laplacian_known_answer():
    g = load("lap20_k10_maxit1000")
    np.testing.assert_allclose(g["lambda"], P.laplacian_eigs((20, 20, 20), 10), rtol=1e-10)
    g = load("serial_driver")
    np.testing.assert_allclose(g["lambda"], [1, 2, 3, 4, 5], rtol=1e-10)


def test_constraints_known_answer():
    g = load("constraints_diag40")
    np.testing.assert_allclose(g["lambda"], [3, 4, 5], rtol=1e-10)


def test_generalized_against_dense_eigh():
    import scipy.linalg as sl
    g = load("gen27_8_k4")
    case = C.build("gen27_8_k4")
    A = P.csr_to_dense(*case.csr, case.n)
    w = sl.eigh(A, np.diag(case.b_diag), eigvals_only=True)[:4]
    np.testing.assert_allclose(g["lambda"], w, rtol=1e-10)


def test_drand48_matches_reference_stream():
    x = P.drand48_block(40, 5, 1)
    g = load("serial_driver")
    assert sha(x) == g["inputs_sha256"]["x0"]
    # the first values of the POSIX sequence after srand48(0)
    v = P.drand48_stream(3, 0)
    state = (0 << 16) | 0x330E
    for i in range(3):
        state = (0x5DEECE66D * state + 0xB) % (1 << 48)
        assert v[i] == state / float(1 << 48)


def test_laplacian_csr_generator():
    rp, ci, va = P.laplacian3d_csr(5, 4, 3)
    n = 60
    A = P.csr_to_dense(rp, ci, va, n)
    assert np.allclose(A, A.T)
    w = np.linalg.eigvalsh(A)[:6]
    np.testing.assert_allclose(w, P.laplacian_eigs((5, 4, 3), 6), rtol=1e-12)


def test_stencil_operators_match_csr():
    rng = np.random.default_rng(0)
    cx, cy, cz = P.stencil7_coefficients(5, 4, 3, seed=1)
    x = rng.standard_normal((60, 3))
    y1 = O.apply(O.stencil7(5, 4, 3, cx, cy, cz, shift=0.25), x)
    y2 = O.apply(O.csr(*P.stencil7_to_csr(cx, cy, cz, shift=0.25)), x)
    np.testing.assert_allclose(y1, y2, rtol=1e-13, atol=1e-13)
    w = P.stencil27_weights(4, 3, 5, seed=2)
    y1 = O.apply(O.stencil27(4, 3, 5, w, 0.5), x)
    y2 = O.apply(O.csr(*P.stencil27_to_csr(4, 3, 5, w, 0.5)), x)
    np.testing.assert_allclose(y1, y2, rtol=1e-13, atol=1e-13)
    c = np.exp(rng.standard_normal((6, 10)))
    sx, sy = P.stencil5_from_cells(c)
    y1 = O.apply(O.stencil5(10, 6, sx, sy), x)
    # assemble the 5-point operator as a 7-point one with nz = 1
    cz = np.zeros((2, 6, 10))
    y2 = O.apply(O.stencil7(10, 6, 1, sx[None], sy[None], cz), x)
    np.testing.assert_allclose(y1, y2, rtol=1e-13, atol=1e-13)


@pytest.mark.parametrize("jacobi", [True, False])
def test_pcg_preconditioner_recurrence(jacobi):
    """The oracle's inner-CG preconditioner (HYPRE -pcgitr semantics) against
    the same recurrence in numpy, column by column, and T r = A^-1 r once the
    steps exceed n (CG on an SPD matrix is exact in n steps, up to rounding)."""
    cx, cy, cz = P.stencil7_coefficients(5, 4, 3, seed=8)
    rp, ci, va = P.stencil7_to_csr(cx, cy, cz)
    n = 60
    A = np.zeros((n, n))
    for r in range(n):
        A[r, ci[rp[r]:rp[r + 1]]] = va[rp[r]:rp[r + 1]]
    M = 1.0 / np.diag(A)
    x = np.random.default_rng(4).standard_normal((n, 3))

    def ref(steps):
        out = np.zeros_like(x)
        for j in range(x.shape[1]):
            r = x[:, j].copy()
            z = M * r if jacobi else r.copy()
            p = z.copy()
            rho = r @ z
            y = np.zeros(n)
            for it in range(steps):
                q = A @ p
                pq = p @ q
                alpha = rho / pq if (pq != 0 and rho != 0) else 0.0
                y += alpha * p
                r -= alpha * q
                if it + 1 == steps:
                    break
                z = M * r if jacobi else r
                rho2 = r @ z
                beta = rho2 / rho if (rho != 0 and rho2 != 0) else 0.0
                p = z + beta * p
                rho = rho2
            out[:, j] = y
        return out

    Mop = O.diag(M) if jacobi else O.NONE
    for steps in (1, 5, 12):
        T = O.pcg(O.csr(rp, ci, va), Mop, steps)
        np.testing.assert_allclose(O.apply(T, x), ref(steps), rtol=1e-12, atol=1e-14)
    T = O.pcg(O.csr(rp, ci, va), Mop, 2 * n)
    np.testing.assert_allclose(O.apply(T, x), np.linalg.solve(A, x), rtol=1e-8)
