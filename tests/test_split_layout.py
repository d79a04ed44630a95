"""The split Gram's staging layout, checked on the CPU.

oz_gram.cu stages each 64-row chunk of up to 128 columns in shared memory:
a run of equally spaced columns arrives as one 2-D TMA tile, every other
column by its own bulk copy.  The host decides that layout (ozg_layout) and
every TMA destination in it; a wrong offset would make the kernel write
outside its buffer.  tests/c/oz_layout_check.cu compiles the kernel file's
host code with the library calls stubbed and a checking stand-in for the
driver's tensor-map encoder, and verifies the layout's invariants on random
blocks (contiguous, masked, scattered, merged; FP32 and FP64).  No GPU.
"""
import os
import shutil
import subprocess

import pytest

from blopex_gb300 import build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_staging_layout_invariants(tmp_path):
    nvcc = os.path.join(build._cuda_home(), "bin", "nvcc")
    if not os.path.exists(nvcc) and shutil.which("nvcc") is None:
        pytest.skip("nvcc not available")
    exe = str(tmp_path / "oz_layout_check")
    cmd = [nvcc if os.path.exists(nvcc) else "nvcc", *build.ARCH, "-std=c++17", "-O1",
           "-I", build.CSRC, "-I", build.INCLUDE,
           os.path.join(ROOT, "tests", "c", "oz_layout_check.cu"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([exe, "60000"], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok:"), r.stdout
