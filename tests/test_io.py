"""The reference tools' file formats (HYPRE IJ / ParVector files, multivector
text): host readers of the C ABI on CPU, device loaders on the GPU."""
import os

import numpy as np
import pytest

from blopex_gb300 import io as IO
from blopex_gb300 import problems as P
from blopex_gb300 import solver as S


@pytest.mark.parametrize("nfiles", [1, 3])
def test_hypre_ij_roundtrip(tmp_path, nfiles):
    rp, ci, va = P.laplacian3d_csr(5, 4, 3)
    va = va * np.random.default_rng(1).uniform(0.5, 1.5, len(va))
    prefix = str(tmp_path / "A")
    IO.write_hypre_ij(prefix, rp, ci, va, nfiles)
    rp2, ci2, va2 = IO.read_hypre_ij(prefix, nfiles)
    np.testing.assert_array_equal(rp2, rp)
    np.testing.assert_array_equal(ci2, ci)
    np.testing.assert_allclose(va2, va, rtol=1e-15)


def test_multivector_and_parvectors_roundtrip(tmp_path):
    x = np.random.default_rng(2).standard_normal((37, 4))
    IO.write_multivector(str(tmp_path / "x.txt"), x)
    np.testing.assert_array_equal(IO.read_multivector(str(tmp_path / "x.txt")), x)
    IO.write_hypre_parvectors(str(tmp_path / "v"), x, nfiles=3)
    np.testing.assert_allclose(IO.read_hypre_parvectors(str(tmp_path / "v"), 4, 3), x, rtol=1e-15)


FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "hypre")


def test_hand_written_reference_layout_files():
    """Files written by hand in the layout of the reference's tools, not by
    this package's writers: matlab2hypreIJ.m (three row partitions, the
    first taking the remainder row -- part = [0 3 5 7] for n = 7 -- a header
    "ilower iupper jlower jupper" per file, 0-based "row col value" lines in
    %16.15e), matlab2hypreParVectors.m (<prefix>.j.i with the row count then
    the values, INFO files [n part(1:p)]) and the multivector text loader
    (blopex_serial_complex/multivector/multi_vector.c:681-693, "n k" then
    (real, imaginary) pairs column by column)."""
    d = np.diag([2.0, 2.5, 3.0, 3.5, 4.0, 4.5, 5.0])
    A = d - np.eye(7, k=1) - np.eye(7, k=-1)
    A[0, 6] = A[6, 0] = 0.3333333333333333
    rp, ci, va = IO.read_hypre_ij(os.path.join(FIX, "A"), 3)
    dense = np.zeros((7, 7))
    for r in range(7):
        dense[r, ci[rp[r]:rp[r + 1]]] = va[rp[r]:rp[r + 1]]
    np.testing.assert_array_equal(dense, A)
    assert rp[-1] == 21
    V = IO.read_hypre_parvectors(os.path.join(FIX, "v"), 2, 3)
    np.testing.assert_array_equal(V[:, 0], np.arange(1, 8) * 0.125)
    np.testing.assert_array_equal(V[:, 1], [-1.0, 0.5, 1e-3, 2.5e10, -3.75, 0.0, 1e-300])
    ref = np.array([[1.5, 4.0], [-2.25, 5.0], [3.0e-05, 6.0]])
    np.testing.assert_array_equal(IO.read_multivector(os.path.join(FIX, "x_pairs.txt")), ref)
    np.testing.assert_array_equal(IO.read_multivector(os.path.join(FIX, "x_real.txt")), ref)
    with pytest.raises(OSError, match=r"\(-5\)"):
        IO.read_multivector(os.path.join(FIX, "x_complex.txt"))


def test_reader_errors(tmp_path):
    with pytest.raises(OSError, match=r"\(-1\)"):
        IO.read_hypre_ij(str(tmp_path / "missing"))
    (tmp_path / "bad.00000").write_text("0 2 0\n")
    with pytest.raises(OSError, match=r"\(-2\)"):
        IO.read_hypre_ij(str(tmp_path / "bad"))
    (tmp_path / "oob.00000").write_text("0 1 0 1\n0 0 1.0\n5 0 1.0\n")
    with pytest.raises(OSError, match=r"\(-3\)"):
        IO.read_hypre_ij(str(tmp_path / "oob"))
    (tmp_path / "short.txt").write_text("3 2\n1.0\n2.0\n")
    with pytest.raises(OSError, match=r"\(-2\)"):
        IO.read_multivector(str(tmp_path / "short.txt"))


@pytest.mark.gpu
def test_loaded_problem_solves_like_the_original(tmp_path):
    ctx = S.Context(0)
    try:
        rp, ci, va = P.laplacian3d_csr(10, 9, 8)
        prefix = str(tmp_path / "lap")
        IO.write_hypre_ij(prefix, rp, ci, va, nfiles=2)
        x0 = P.drand48_block(len(rp) - 1, 5, 3)
        IO.write_multivector(str(tmp_path / "x0.txt"), x0)
        A1 = S.CSRMatrix(ctx, rp, ci, va)
        A2 = IO.load_csr_hypre_ij(ctx, prefix, nfiles=2)
        X1 = S.MultiVector.from_host(ctx, x0)
        X2 = IO.load_multivector(ctx, str(tmp_path / "x0.txt"))
        ctx.set_options(precision=S.FP64)
        r1 = S.lobpcg_solve_double(X1, A1, atol=1e-9, maxit=500)
        r2 = S.lobpcg_solve_double(X2, A2, atol=1e-9, maxit=500)
        assert r1.flag == r2.flag == 0 and r1.iterations == r2.iterations
        np.testing.assert_array_equal(r1.lam, r2.lam)
    finally:
        ctx.close()
