"""The seeded problem instances behind the golden fixtures.

Each case rebuilds its inputs from the generators in
``blopex_gb300.problems``; ``make_golden.py`` records the reference's
outputs for them and the tests replay them against the oracle and the GPU.
"""
from __future__ import annotations

from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from blopex_gb300 import problems as P


@dataclass
class Case:
    name: str
    description: str
    n: int
    k: int
    seed: int
    atol: float
    rtol: float
    maxit: int
    csr: Optional[tuple] = None
    dense: Optional[np.ndarray] = None
    b_diag: Optional[np.ndarray] = None
    t_diag: Optional[np.ndarray] = None
    Y: Optional[np.ndarray] = None
    x0: Optional[np.ndarray] = None
    verbosity: int = 0
    potrf_fail_at: int = 0
    sygv_fail_at: int = 0
    extra: dict = field(default_factory=dict)

    def initial_block(self) -> np.ndarray:
        if self.x0 is not None:
            return np.asfortranarray(self.x0)
        return P.drand48_block(self.n, self.k, self.seed)

    def arrays(self) -> dict:
        out = {"x0": self.initial_block()}
        if self.csr is not None:
            out.update(rowptr=self.csr[0], colidx=self.csr[1], vals=self.csr[2])
        if self.dense is not None:
            out["dense"] = np.asfortranarray(self.dense)
        for key in ("b_diag", "t_diag", "Y"):
            v = getattr(self, key)
            if v is not None:
                out[key] = np.asfortranarray(v)
        return out


def _diag40():
    return np.diag(np.arange(1.0, 41.0))


def build(name: str) -> Case:
    if name == "serial_driver":
        return Case(name, "diag(1..40), k=5, X0 seed 1, tol 1e-6 abs, maxit 100, verbosity 2 "
                    "(blopex_serial_double/driver/serial_driver.c:44-117)",
                    40, 5, 1, 1e-6, 1e-50, 100, dense=_diag40(), verbosity=2)
    if name == "serial_driver_v1":
        return Case(name, "as serial_driver with verbosity 1", 40, 5, 1, 1e-6, 1e-50, 100,
                    dense=_diag40(), verbosity=1)
    if name == "lap20_k10":
        return Case(name, "3D 7-point Dirichlet Laplacian 20^3 CSR, k=10, X0 seed 0, tol 1e-6, "
                    "maxit 100, no T", 8000, 10, 0, 1e-6, 1e-50, 100,
                    csr=P.laplacian3d_csr(20, 20, 20))
    if name == "lap20_k10_maxit1000":
        return Case(name, "as lap20_k10 with maxit 1000 (converges)", 8000, 10, 0, 1e-6, 1e-50,
                    1000, csr=P.laplacian3d_csr(20, 20, 20))
    if name == "st7vc_12_k6_jacobi":
        cx, cy, cz = P.stencil7_coefficients(12, 12, 12, seed=2)
        csr = P.stencil7_to_csr(cx, cy, cz)
        return Case(name, "variable-coefficient 7-point 12^3 (faces exp(N(0,1)) seed 2) as CSR, "
                    "k=6, Jacobi T, X0 seed 5, tol 1e-8, maxit 300", 1728, 6, 5, 1e-8, 1e-50,
                    300, csr=csr, t_diag=1.0 / P.stencil7_diagonal(cx, cy, cz))
    if name == "gen27_8_k4":
        w = P.stencil27_weights(8, 8, 8, seed=4)
        csr = P.stencil27_to_csr(8, 8, 8, w, shift=0.5)
        return Case(name, "generalized: 27-point 8^3 (weights U[0.5,1.5] seed 4, shift 0.5) as "
                    "CSR, B = diag(U[0.5,1.5] seed 14), k=4, X0 seed 6, tol 1e-8, maxit 300",
                    512, 4, 6, 1e-8, 1e-50, 300, csr=csr, b_diag=P.mass_diagonal(512, seed=14))
    if name == "constraints_diag40":
        Y = np.zeros((40, 2))
        Y[0, 0] = 1.0
        Y[1, 1] = 1.0
        return Case(name, "diag(1..40) with constraints e1, e2, k=3, X0 seed 7, tol 1e-8",
                    40, 3, 7, 1e-8, 1e-50, 100, dense=_diag40(), Y=Y)
    if name == "all_paths_lap6":
        csr = P.laplacian3d_csr(6, 6, 6)
        n = 216
        Y = P.drand48_block(n, 2, 11)
        return Case(name, "Laplacian 6^3 CSR with B = diag(U[0.5,1.5] seed 21), Jacobi T = "
                    "1/diag(A), 2 random constraints (drand48 seed 11), k=3, X0 seed 8, "
                    "tol 1e-8, rtol 1e-9", n, 3, 8, 1e-8, 1e-9, 200, csr=csr,
                    b_diag=P.mass_diagonal(n, seed=21), t_diag=np.full(n, 1.0 / 6.0), Y=Y)
    if name == "lap10_k1":
        return Case(name, "Laplacian 10^3 CSR, k=1, X0 seed 3, tol 1e-8, maxit 500",
                    1000, 1, 3, 1e-8, 1e-50, 500, csr=P.laplacian3d_csr(10, 10, 10))
    if name == "wrong_block_size":
        # Not a golden: the reference aborts here on an assert in
        # utilities_FortranMatrixWrap (fortran_matrix.c:139) before reaching
        # the WRONG_BLOCK_SIZE return at lobpcg.c:689-698.
        return Case(name, "k=0: WRONG_BLOCK_SIZE (lobpcg.c:689-698)", 40, 0, 1, 1e-6, 1e-50,
                    10, dense=_diag40())
    if name == "bad_initial_block":
        x0 = P.drand48_block(40, 4, 1)
        x0[:, 3] = x0[:, 1]
        return Case(name, "two equal columns in X0: the first orthonormalisation fails "
                    "(lobpcg.c:857-862)", 40, 4, 1, 1e-6, 1e-50, 100, dense=_diag40(), x0=x0)
    if name == "wrong_constraints":
        Y = np.zeros((40, 2))
        Y[3, 0] = 1.0
        Y[3, 1] = 1.0
        return Case(name, "linearly dependent constraints: WRONG_CONSTRAINTS (lobpcg.c:720-739)",
                    40, 3, 7, 1e-8, 1e-50, 100, dense=_diag40(), Y=Y)
    if name == "fail_p_orth":
        return Case(name, "Laplacian 8^3, k=4: the 4th Cholesky (P block, iteration 2) reports "
                    "failure -> sizeP = 0 restart (lobpcg.c:1056-1063)", 512, 4, 9, 1e-8, 1e-50,
                    60, csr=P.laplacian3d_csr(8, 8, 8), potrf_fail_at=4)
    if name == "fail_r_orth":
        return Case(name, "Laplacian 8^3, k=4: the 3rd Cholesky (R block, iteration 2) reports "
                    "failure -> exit -1 (lobpcg.c:1027-1034)", 512, 4, 9, 1e-8, 1e-50, 60,
                    csr=P.laplacian3d_csr(8, 8, 8), potrf_fail_at=3)
    if name == "fail_gevp":
        return Case(name, "Laplacian 8^3, k=4: the 4th Rayleigh-Ritz solve reports failure "
                    "(lobpcg.c:1167-1176)", 512, 4, 9, 1e-8, 1e-50, 60,
                    csr=P.laplacian3d_csr(8, 8, 8), sygv_fail_at=4)
    if name == "lap128_k32_jacobi_it30":
        n = 128 ** 3
        return Case(name, "the 128^3 plain-FP64 configuration for its first 30 iterations: 7-point "
                    "Laplacian 128^3 CSR (n=2097152), k=32, Jacobi T = 1/diag(A) = I/6, X0 seed 1, "
                    "tol 1e-8, maxit 30", n, 32, 1, 1e-8, 1e-50, 30,
                    csr=P.laplacian3d_csr(128, 128, 128), t_diag=np.full(n, 1.0 / 6.0))
    if name == "st7vc128_k64_jacobi_it20":
        cx, cy, cz = P.stencil7_coefficients(128, 128, 128, seed=2)
        return Case(name, "the variable-coefficient stencil configuration at 128^3 for its first "
                    "20 iterations: faces exp(N(0,1)) seed 2 (assembled as CSR), k=64, Jacobi T, "
                    "X0 seed 2, tol 1e-8, maxit 20", 128 ** 3, 64, 2, 1e-8, 1e-50, 20,
                    csr=P.stencil7_to_csr(cx, cy, cz),
                    t_diag=1.0 / P.stencil7_diagonal(cx, cy, cz))
    raise KeyError(name)


NAMES = ["serial_driver", "serial_driver_v1", "lap20_k10", "lap20_k10_maxit1000",
         "st7vc_12_k6_jacobi", "gen27_8_k4", "constraints_diag40", "all_paths_lap6",
         "lap10_k1", "bad_initial_block", "wrong_constraints",
         "fail_p_orth", "fail_r_orth", "fail_gevp"]

# Cases at the benchmark sizes (128^3): each reference run takes tens of
# minutes on one core, so they are generated separately (make_golden.py
# --large) and replayed only by the GPU tests.
LARGE_NAMES = ["lap128_k32_jacobi_it30", "st7vc128_k64_jacobi_it20"]
