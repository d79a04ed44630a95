"""The drop-in boundary from plain C: tests/c/serial_driver_gb300.c calls
lobpcg_solve_double through the mv_InterfaceInterpreter table, the way the
reference's serial driver does, on a 3D 7-point Dirichlet Laplacian g^3;
its eigenvalues are checked against the analytic spectrum."""
import os
import re
import shutil
import subprocess

import numpy as np
import pytest

from blopex_gb300 import _lib

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_c_caller_solves_the_laplacian(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    libdir = os.path.dirname(_lib.LIBPATH)
    exe = tmp_path / "serial_driver_gb300"
    build = subprocess.run(
        ["gcc", "-std=c99", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"),
         os.path.join(ROOT, "tests", "c", "serial_driver_gb300.c"), "-L", libdir, "-llobpcg_gb300",
         "-Wl,-rpath," + libdir, "-o", str(exe)], capture_output=True, text=True)
    assert build.returncode == 0, build.stderr
    g = 10
    run = subprocess.run([str(exe), str(g)], capture_output=True, text=True, timeout=300)
    assert run.returncode == 0, run.stdout + run.stderr
    lam = [float(v) for v in re.findall(r"lambda \d+ = (\S+)", run.stdout)]
    res = [float(v) for v in re.findall(r"residual (\S+)", run.stdout)]
    # Dirichlet 7-point Laplacian on g^3: sum over axes of 2 - 2 cos(p pi / (g + 1))
    t = 2.0 - 2.0 * np.cos(np.arange(1, g + 1) * np.pi / (g + 1))
    exact = np.sort((t[:, None, None] + t[None, :, None] + t[None, None, :]).ravel())[:4]
    np.testing.assert_allclose(lam, exact, rtol=1e-10)
    assert len(res) == 4 and max(res) <= 1e-8
